// Hybrid-operator element VJP kernels of the discrete adjoint on Gauss nodes, 1D and 2D (Cartesian),
// and the dispatch of both element passes (adjoint_kernels.cuh).
#include "adjoint_kernels.cuh"
namespace flou {
cudaError_t launch_adj_hybrid_gauss3d_ch(int n, const AdjElemParams& P, cudaStream_t s);
cudaError_t launch_adj_hybrid_gauss3d_kg(int n, const AdjElemParams& P, cudaStream_t s);
cudaError_t launch_adj_hybrid_gauss3d_std(int n, const AdjElemParams& P, cudaStream_t s);
cudaError_t launch_adj_hybrid_gauss_curv2d(int n, int tp, const AdjElemParams& P, cudaStream_t s);
cudaError_t launch_adj_hybrid_gauss_curv3d_ch(int n, const AdjElemParams& P, cudaStream_t s);
cudaError_t launch_adj_hybrid_gauss_curv3d_kg(int n, const AdjElemParams& P, cudaStream_t s);
cudaError_t launch_adj_hybrid_gauss_curv3d_std(int n, const AdjElemParams& P, cudaStream_t s);

cudaError_t launch_adj_hybrid_gauss(int dim, int n, int tp, bool curv, const AdjElemParams& P, cudaStream_t s) {
    if (curv && dim == 2) return launch_adj_hybrid_gauss_curv2d(n, tp, P, s);
    if (curv) {
        if (tp == FLOU_TP_KENNEDY_GRUBER) return launch_adj_hybrid_gauss_curv3d_kg(n, P, s);
        if (tp == FLOU_TP_STD_AVERAGE) return launch_adj_hybrid_gauss_curv3d_std(n, P, s);
        return launch_adj_hybrid_gauss_curv3d_ch(n, P, s);
    }
    if (dim == 1) return launch_adj_split<1, false, true, true>(n, tp, P, s);
    if (dim == 2) return launch_adj_split<2, false, true, true>(n, tp, P, s);
    if (tp == FLOU_TP_KENNEDY_GRUBER) return launch_adj_hybrid_gauss3d_kg(n, P, s);
    if (tp == FLOU_TP_STD_AVERAGE) return launch_adj_hybrid_gauss3d_std(n, P, s);
    return launch_adj_hybrid_gauss3d_ch(n, P, s);
}

cudaError_t launch_adj_hybrid_gauss_finish(int dim, int n, bool curv, const AdjElemParams& P, cudaStream_t s) {
    if (curv) return dim == 2 ? launch_adj_hybrid_gauss_finish_t<2, true>(n, P, s)
                              : launch_adj_hybrid_gauss_finish_t<3, true>(n, P, s);
    if (dim == 1) return launch_adj_hybrid_gauss_finish_t<1>(n, P, s);
    if (dim == 2) return launch_adj_hybrid_gauss_finish_t<2>(n, P, s);
    return launch_adj_hybrid_gauss_finish_t<3>(n, P, s);
}
}  // namespace flou
