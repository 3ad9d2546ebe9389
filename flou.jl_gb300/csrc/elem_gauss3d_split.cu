// Element kernels, 3D Euler on Gauss nodes: entropy-projected split operator.
#include "flou_internal.cuh"
namespace flou {
cudaError_t launch_elem_gauss3d_split(const ElemLaunch& L, const ElemParams& P, cudaStream_t s) {
    return launch_elem_gauss_dim<3, FLOU_OP_SPLIT>(L.n, L.tp, P, s, L.prepare);
}
}  // namespace flou
