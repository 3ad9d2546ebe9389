// Hybrid-operator element VJP kernels of the discrete adjoint, 1D and 2D (adjoint_kernels.cuh).
#include "adjoint_kernels.cuh"
namespace flou {
cudaError_t launch_adj_hybrid_12d(int dim, int n, int tp, const AdjElemParams& P, cudaStream_t s) {
    return dim == 1 ? launch_adj_split<1, false, false, true>(n, tp, P, s)
                    : launch_adj_split<2, false, false, true>(n, tp, P, s);
}
}  // namespace flou
