// Element kernels, 2D Euler (all volume operators).
#include "flou_internal.cuh"
namespace flou {
cudaError_t launch_elem_euler2d(const ElemLaunch& L, const ElemParams& P, cudaStream_t s) {
    return launch_elem_dim<2, FLOU_EQ_EULER>(L.n, L.vol, L.tp, L.lgl, P, s, L.prepare);
}
}  // namespace flou
