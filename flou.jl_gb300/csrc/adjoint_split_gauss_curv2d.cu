// Split-form element VJP kernels of the discrete adjoint on Gauss nodes and general geometry, 2D
// (adjoint_kernels.cuh): the projected states' metric from the subcell interfaces.
#include "adjoint_kernels.cuh"
namespace flou {
cudaError_t launch_adj_split_gauss_curv2d(int n, int tp, const AdjElemParams& P, cudaStream_t s) {
    return launch_adj_split<2, true, true, false>(n, tp, P, s);
}
}  // namespace flou
