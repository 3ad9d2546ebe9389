// Strong-form element VJP kernels of the discrete adjoint for a basis without exact end-node
// injection (Gauss nodes; adjoint_kernels.cuh): every node takes the trace cotangents through l.
#include "adjoint_kernels.cuh"
namespace flou {
cudaError_t launch_adj_elem_gauss(int dim, int n, bool curv, const AdjElemParams& P, cudaStream_t s) {
    if (curv) return dim == 2 ? launch_adj_elem<2, true, true>(n, P, s) : launch_adj_elem<3, true, true>(n, P, s);
    if (dim == 1) return launch_adj_elem<1, false, true>(n, P, s);
    if (dim == 2) return launch_adj_elem<2, false, true>(n, P, s);
    return launch_adj_elem<3, false, true>(n, P, s);
}
}  // namespace flou
