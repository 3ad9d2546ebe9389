// Split-form element VJP kernels of the discrete adjoint on Gauss nodes and general geometry, 3D
// (adjoint_kernels.cuh).
#include "adjoint_kernels.cuh"
namespace flou {
cudaError_t launch_adj_split_gauss_curv3d(int n, int tp, const AdjElemParams& P, cudaStream_t s) {
    return launch_adj_split<3, true, true, false>(n, tp, P, s);
}
}  // namespace flou
