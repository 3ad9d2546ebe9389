// Strong-form element VJP kernels of the discrete adjoint (adjoint_kernels.cuh).
#include "adjoint_kernels.cuh"
namespace flou {
cudaError_t launch_adj_elem_gauss(int dim, int n, bool curv, const AdjElemParams& P, cudaStream_t s);
cudaError_t launch_adj_elem_dim(int dim, int n, bool curv, bool gauss, const AdjElemParams& P, cudaStream_t s) {
    if (gauss) return launch_adj_elem_gauss(dim, n, curv, P, s);
    if (curv) return dim == 2 ? launch_adj_elem<2, true>(n, P, s) : launch_adj_elem<3, true>(n, P, s);
    if (dim == 1) return launch_adj_elem<1>(n, P, s);
    if (dim == 2) return launch_adj_elem<2>(n, P, s);
    return launch_adj_elem<3>(n, P, s);
}
}  // namespace flou
namespace flou {
cudaError_t launch_adj_split_1d(int n, int tp, const AdjElemParams& P, cudaStream_t s);
cudaError_t launch_adj_split_2d(int n, int tp, const AdjElemParams& P, cudaStream_t s);
cudaError_t launch_adj_split_3d(int n, int tp, const AdjElemParams& P, cudaStream_t s);
cudaError_t launch_adj_split_curv2d(int n, int tp, const AdjElemParams& P, cudaStream_t s);
cudaError_t launch_adj_split_curv3d(int n, int tp, const AdjElemParams& P, cudaStream_t s);
cudaError_t launch_adj_split_gauss(int dim, int n, int tp, const AdjElemParams& P, cudaStream_t s);
cudaError_t launch_adj_split_gauss3d(int n, int tp, const AdjElemParams& P, cudaStream_t s);
cudaError_t launch_adj_hybrid_12d(int dim, int n, int tp, const AdjElemParams& P, cudaStream_t s);
cudaError_t launch_adj_hybrid_curv2d(int n, int tp, const AdjElemParams& P, cudaStream_t s);
cudaError_t launch_adj_hybrid3d_ch(int n, const AdjElemParams& P, cudaStream_t s);
cudaError_t launch_adj_hybrid3d_kg(int n, const AdjElemParams& P, cudaStream_t s);
cudaError_t launch_adj_hybrid3d_std(int n, const AdjElemParams& P, cudaStream_t s);
cudaError_t launch_adj_hybrid_curv3d_ch(int n, const AdjElemParams& P, cudaStream_t s);
cudaError_t launch_adj_hybrid_curv3d_kg(int n, const AdjElemParams& P, cudaStream_t s);
cudaError_t launch_adj_hybrid_curv3d_std(int n, const AdjElemParams& P, cudaStream_t s);
cudaError_t launch_adj_split_gauss_curv2d(int n, int tp, const AdjElemParams& P, cudaStream_t s);
cudaError_t launch_adj_split_gauss_curv3d(int n, int tp, const AdjElemParams& P, cudaStream_t s);
// The hybrid operator's element VJP: one translation unit per dimension (and per two-point flux in 3D).
static cudaError_t launch_adj_hybrid(int dim, int n, int tp, bool curv, const AdjElemParams& P, cudaStream_t s) {
    if (dim < 3 && !curv) return launch_adj_hybrid_12d(dim, n, tp, P, s);
    if (dim == 2) return launch_adj_hybrid_curv2d(n, tp, P, s);
    if (tp == FLOU_TP_KENNEDY_GRUBER) return curv ? launch_adj_hybrid_curv3d_kg(n, P, s) : launch_adj_hybrid3d_kg(n, P, s);
    if (tp == FLOU_TP_STD_AVERAGE) return curv ? launch_adj_hybrid_curv3d_std(n, P, s) : launch_adj_hybrid3d_std(n, P, s);
    return curv ? launch_adj_hybrid_curv3d_ch(n, P, s) : launch_adj_hybrid3d_ch(n, P, s);
}
cudaError_t launch_adj_split_dim(int dim, int n, int tp, bool curv, bool gauss, bool hybrid, const AdjElemParams& P,
                                 cudaStream_t s) {
    if (hybrid) return launch_adj_hybrid(dim, n, tp, curv, P, s);
    if (gauss && curv)
        return dim == 2 ? launch_adj_split_gauss_curv2d(n, tp, P, s) : launch_adj_split_gauss_curv3d(n, tp, P, s);
    if (gauss) return dim == 3 ? launch_adj_split_gauss3d(n, tp, P, s) : launch_adj_split_gauss(dim, n, tp, P, s);
    if (curv) return dim == 2 ? launch_adj_split_curv2d(n, tp, P, s) : launch_adj_split_curv3d(n, tp, P, s);
    if (dim == 1) return launch_adj_split_1d(n, tp, P, s);
    if (dim == 2) return launch_adj_split_2d(n, tp, P, s);
    return launch_adj_split_3d(n, tp, P, s);
}
}  // namespace flou
