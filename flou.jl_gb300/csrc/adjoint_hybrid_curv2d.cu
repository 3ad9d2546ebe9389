// Hybrid-operator element VJP kernels of the discrete adjoint on general geometry, 2D
// (adjoint_kernels.cuh): subcell FV fluxes in the uploaded subcell frames.
#include "adjoint_kernels.cuh"
namespace flou {
cudaError_t launch_adj_hybrid_curv2d(int n, int tp, const AdjElemParams& P, cudaStream_t s) {
    return launch_adj_split<2, true, false, true>(n, tp, P, s);
}
}  // namespace flou
