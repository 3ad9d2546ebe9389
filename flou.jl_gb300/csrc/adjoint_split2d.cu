// Split-form element VJP kernels of the discrete adjoint, 2D (adjoint_kernels.cuh).
#include "adjoint_kernels.cuh"
namespace flou {
cudaError_t launch_adj_split_2d(int n, int tp, const AdjElemParams& P, cudaStream_t s) {
    return launch_adj_split<2>(n, tp, P, s);
}
}  // namespace flou
