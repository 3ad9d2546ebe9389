// Split-form element VJP kernels of the discrete adjoint on Gauss nodes, 1D and 2D
// (adjoint_kernels.cuh): the entropy-projected coupling of each line transposed.
#include "adjoint_kernels.cuh"
namespace flou {
cudaError_t launch_adj_split_gauss(int dim, int n, int tp, const AdjElemParams& P, cudaStream_t s) {
    return dim == 1 ? launch_adj_split<1, false, true>(n, tp, P, s) : launch_adj_split<2, false, true>(n, tp, P, s);
}
}  // namespace flou
