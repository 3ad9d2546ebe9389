// Hybrid-operator element VJP kernels of the discrete adjoint on Gauss nodes, general geometry,
// 2D (adjoint_kernels.cuh).
#include "adjoint_kernels.cuh"
namespace flou {
cudaError_t launch_adj_hybrid_gauss_curv2d(int n, int tp, const AdjElemParams& P, cudaStream_t s) {
    return launch_adj_split<2, true, true, true>(n, tp, P, s);
}
}  // namespace flou
