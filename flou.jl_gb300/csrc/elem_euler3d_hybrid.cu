// Element kernels, 3D Euler, hybrid (telescopic split form blended with subcell FV) operator.
#include "flou_internal.cuh"
namespace flou {
cudaError_t launch_elem_euler3d_hybrid(const ElemLaunch& L, const ElemParams& P, cudaStream_t s) {
    return launch_elem_dim<3, FLOU_EQ_EULER, FLOU_OP_HYBRID>(L.n, L.vol, L.tp, L.lgl, P, s, L.prepare);
}
}  // namespace flou
