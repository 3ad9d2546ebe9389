// Element kernels, 1D Euler on Gauss nodes: entropy-projected split and hybrid operators.
#include "flou_internal.cuh"
namespace flou {
cudaError_t launch_elem_gauss1d(const ElemLaunch& L, const ElemParams& P, cudaStream_t s) {
    return L.vol == FLOU_OP_HYBRID ? launch_elem_gauss_dim<1, FLOU_OP_HYBRID>(L.n, L.tp, P, s, L.prepare)
                                   : launch_elem_gauss_dim<1, FLOU_OP_SPLIT>(L.n, L.tp, P, s, L.prepare);
}
}  // namespace flou
