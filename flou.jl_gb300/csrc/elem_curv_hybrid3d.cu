// Element kernels, 3D Euler on general (curvilinear / unstructured) elements: hybrid operator.
#include "flou_internal.cuh"
namespace flou {
cudaError_t launch_elem_curv_hybrid3d(const ElemLaunch& L, const ElemParams& P, cudaStream_t s) {
    if (L.eq != FLOU_EQ_EULER) return cudaErrorInvalidValue;
    return launch_elem_dim_curv_hybrid<3>(L.n, L.tp, P, s, L.prepare);
}
}  // namespace flou
