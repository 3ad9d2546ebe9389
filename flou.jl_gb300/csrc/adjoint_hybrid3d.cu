// Hybrid-operator element VJP kernels of the discrete adjoint, 3D (adjoint_kernels.cuh).
#include "adjoint_kernels.cuh"
namespace flou {
cudaError_t launch_adj_hybrid3d(int n, int tp, const AdjElemParams& P, cudaStream_t s) {
    return launch_adj_split<3, false, false, true>(n, tp, P, s);
}
}  // namespace flou
