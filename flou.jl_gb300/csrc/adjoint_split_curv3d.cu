// Split-form element VJP kernels of the discrete adjoint on general geometry, 3D
// (adjoint_kernels.cuh): pair fluxes along the averaged metric columns.
#include "adjoint_kernels.cuh"
namespace flou {
cudaError_t launch_adj_split_curv3d(int n, int tp, const AdjElemParams& P, cudaStream_t s) {
    return launch_adj_split<3, true>(n, tp, P, s);
}
}  // namespace flou
