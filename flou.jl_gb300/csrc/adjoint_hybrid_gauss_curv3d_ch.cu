// Hybrid-operator element VJP kernels of the discrete adjoint on Gauss nodes, general geometry,
// 3D, one two-point flux (adjoint_kernels.cuh).
#include "adjoint_kernels.cuh"
namespace flou {
cudaError_t launch_adj_hybrid_gauss_curv3d_ch(int n, const AdjElemParams& P, cudaStream_t s) {
    return launch_adj_split_tp<3, FLOU_TP_CHANDRASHEKAR, true, true, true>(n, P, s);
}
}  // namespace flou
