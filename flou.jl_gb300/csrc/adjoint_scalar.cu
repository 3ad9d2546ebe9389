// The discrete adjoint of the scalar equations (adjoint_kernels.cuh): linear advection 1D-3D,
// Burgers 1D; strong form (Gauss-Lobatto or Gauss nodes) and the split form; linear advection
// also on general geometry.
#include "adjoint_kernels.cuh"
namespace flou {
namespace {
template <int DIM, int EQ, bool CURV>
cudaError_t scalar_face(bool gauss, int grid, int tb, const AdjFaceParams& F, cudaStream_t s) {
    if (gauss) adj_face_scalar_kernel<DIM, EQ, true, CURV><<<grid, tb, 0, s>>>(F);
    else adj_face_scalar_kernel<DIM, EQ, false, CURV><<<grid, tb, 0, s>>>(F);
    return cudaGetLastError();
}
template <int DIM, int N, int EQ, bool SPLIT, bool G, bool CURV>
cudaError_t scalar_elem_n(const AdjElemParams& P, cudaStream_t s) {
    using S = Shape<DIM, N>;
    const size_t smem = sizeof(double) * (S::NOPS + S::NN);
    const int grid = (P.nelem + S::EPB - 1) / S::EPB;
    adj_elem_scalar_kernel<DIM, N, EQ, SPLIT, G, CURV><<<grid, S::BLOCK, smem, s>>>(P);
    return cudaGetLastError();
}
template <int DIM, int EQ, bool SPLIT, bool G, bool CURV>
cudaError_t scalar_elem(int n, const AdjElemParams& P, cudaStream_t s) {
    switch (n) {
        case 2: return scalar_elem_n<DIM, 2, EQ, SPLIT, G, CURV>(P, s);
        case 3: return scalar_elem_n<DIM, 3, EQ, SPLIT, G, CURV>(P, s);
        case 4: return scalar_elem_n<DIM, 4, EQ, SPLIT, G, CURV>(P, s);
        case 5: return scalar_elem_n<DIM, 5, EQ, SPLIT, G, CURV>(P, s);
        case 6: return scalar_elem_n<DIM, 6, EQ, SPLIT, G, CURV>(P, s);
        case 7: return scalar_elem_n<DIM, 7, EQ, SPLIT, G, CURV>(P, s);
        case 8: return scalar_elem_n<DIM, 8, EQ, SPLIT, G, CURV>(P, s);
        default: return cudaErrorInvalidValue;
    }
}
template <int DIM, int EQ, bool CURV>
cudaError_t scalar_dim(int n, bool split, bool gauss, int grid, int tb, const AdjFaceParams& F,
                       const AdjElemParams& P, cudaStream_t s) {
    cudaError_t e = scalar_face<DIM, EQ, CURV>(gauss, grid, tb, F, s);
    if (e != cudaSuccess) return e;
    if (split) return scalar_elem<DIM, EQ, true, false, CURV>(n, P, s);
    return gauss ? scalar_elem<DIM, EQ, false, true, CURV>(n, P, s) : scalar_elem<DIM, EQ, false, false, CURV>(n, P, s);
}
}  // namespace
cudaError_t launch_adj_scalar(int dim, int eq, int n, bool split, bool gauss, bool curv, int grid, int tb,
                              const AdjFaceParams& F, const AdjElemParams& P, cudaStream_t s) {
    if (eq == FLOU_EQ_BURGERS) return scalar_dim<1, FLOU_EQ_BURGERS, false>(n, split, gauss, grid, tb, F, P, s);
    if (curv)
        return dim == 2 ? scalar_dim<2, FLOU_EQ_LINEAR_ADVECTION, true>(n, split, gauss, grid, tb, F, P, s)
                        : scalar_dim<3, FLOU_EQ_LINEAR_ADVECTION, true>(n, split, gauss, grid, tb, F, P, s);
    if (dim == 1) return scalar_dim<1, FLOU_EQ_LINEAR_ADVECTION, false>(n, split, gauss, grid, tb, F, P, s);
    if (dim == 2) return scalar_dim<2, FLOU_EQ_LINEAR_ADVECTION, false>(n, split, gauss, grid, tb, F, P, s);
    return scalar_dim<3, FLOU_EQ_LINEAR_ADVECTION, false>(n, split, gauss, grid, tb, F, P, s);
}
}  // namespace flou
