// Element kernels with general (curvilinear / unstructured) geometry, 2D: Euler and linear
// advection, strong form and split form (LGL).
#include "flou_internal.cuh"
namespace flou {
cudaError_t launch_elem_curv2d(const ElemLaunch& L, const ElemParams& P, cudaStream_t s) {
    if (L.eq == FLOU_EQ_EULER) return launch_elem_dim_curv<2, FLOU_EQ_EULER>(L.n, L.vol, L.tp, P, s, L.prepare);
    if (L.eq == FLOU_EQ_LINEAR_ADVECTION)
        return launch_elem_dim_curv<2, FLOU_EQ_LINEAR_ADVECTION>(L.n, L.vol, L.tp, P, s, L.prepare);
    return cudaErrorInvalidValue;
}
}  // namespace flou
