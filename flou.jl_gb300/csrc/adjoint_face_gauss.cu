// Face VJP kernels of the discrete adjoint for a basis without exact end-node injection (Gauss
// nodes, strong form; adjoint_kernels.cuh): interpolated traces and the full-line lift transpose,
// on Cartesian (1D-3D) and general (2D, 3D) geometry.
#include "adjoint_kernels.cuh"
namespace flou {
static cudaError_t launch_adj_face_gauss_cart(int dim, int kind, int grid, int tb, const AdjFaceParams& F, cudaStream_t s) {
    switch (dim * 8 + kind) {
        case 8: adj_face_kernel<1, 0, false, true><<<grid, tb, 0, s>>>(F); break;
        case 9: adj_face_kernel<1, 1, false, true><<<grid, tb, 0, s>>>(F); break;
        case 10: adj_face_kernel<1, 2, false, true><<<grid, tb, 0, s>>>(F); break;
        case 11: adj_face_kernel<1, 3, false, true><<<grid, tb, 0, s>>>(F); break;
        case 12: adj_face_kernel<1, 4, false, true><<<grid, tb, 0, s>>>(F); break;
        case 13: adj_face_kernel<1, 5, false, true><<<grid, tb, 0, s>>>(F); break;
        case 14: adj_face_kernel<1, 6, false, true><<<grid, tb, 0, s>>>(F); break;
        case 15: adj_face_kernel<1, 7, false, true><<<grid, tb, 0, s>>>(F); break;
        case 16: adj_face_kernel<2, 0, false, true><<<grid, tb, 0, s>>>(F); break;
        case 17: adj_face_kernel<2, 1, false, true><<<grid, tb, 0, s>>>(F); break;
        case 18: adj_face_kernel<2, 2, false, true><<<grid, tb, 0, s>>>(F); break;
        case 19: adj_face_kernel<2, 3, false, true><<<grid, tb, 0, s>>>(F); break;
        case 20: adj_face_kernel<2, 4, false, true><<<grid, tb, 0, s>>>(F); break;
        case 21: adj_face_kernel<2, 5, false, true><<<grid, tb, 0, s>>>(F); break;
        case 22: adj_face_kernel<2, 6, false, true><<<grid, tb, 0, s>>>(F); break;
        case 23: adj_face_kernel<2, 7, false, true><<<grid, tb, 0, s>>>(F); break;
        case 24: adj_face_kernel<3, 0, false, true><<<grid, tb, 0, s>>>(F); break;
        case 25: adj_face_kernel<3, 1, false, true><<<grid, tb, 0, s>>>(F); break;
        case 26: adj_face_kernel<3, 2, false, true><<<grid, tb, 0, s>>>(F); break;
        case 27: adj_face_kernel<3, 3, false, true><<<grid, tb, 0, s>>>(F); break;
        case 28: adj_face_kernel<3, 4, false, true><<<grid, tb, 0, s>>>(F); break;
        case 29: adj_face_kernel<3, 5, false, true><<<grid, tb, 0, s>>>(F); break;
        case 30: adj_face_kernel<3, 6, false, true><<<grid, tb, 0, s>>>(F); break;
        case 31: adj_face_kernel<3, 7, false, true><<<grid, tb, 0, s>>>(F); break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}
static cudaError_t launch_adj_face_gauss_curv(int dim, int kind, int grid, int tb, const AdjFaceParams& F, cudaStream_t s) {
    switch (dim * 8 + kind) {
        case 16: adj_face_kernel<2, 0, true, true><<<grid, tb, 0, s>>>(F); break;
        case 17: adj_face_kernel<2, 1, true, true><<<grid, tb, 0, s>>>(F); break;
        case 18: adj_face_kernel<2, 2, true, true><<<grid, tb, 0, s>>>(F); break;
        case 19: adj_face_kernel<2, 3, true, true><<<grid, tb, 0, s>>>(F); break;
        case 20: adj_face_kernel<2, 4, true, true><<<grid, tb, 0, s>>>(F); break;
        case 21: adj_face_kernel<2, 5, true, true><<<grid, tb, 0, s>>>(F); break;
        case 22: adj_face_kernel<2, 6, true, true><<<grid, tb, 0, s>>>(F); break;
        case 23: adj_face_kernel<2, 7, true, true><<<grid, tb, 0, s>>>(F); break;
        case 24: adj_face_kernel<3, 0, true, true><<<grid, tb, 0, s>>>(F); break;
        case 25: adj_face_kernel<3, 1, true, true><<<grid, tb, 0, s>>>(F); break;
        case 26: adj_face_kernel<3, 2, true, true><<<grid, tb, 0, s>>>(F); break;
        case 27: adj_face_kernel<3, 3, true, true><<<grid, tb, 0, s>>>(F); break;
        case 28: adj_face_kernel<3, 4, true, true><<<grid, tb, 0, s>>>(F); break;
        case 29: adj_face_kernel<3, 5, true, true><<<grid, tb, 0, s>>>(F); break;
        case 30: adj_face_kernel<3, 6, true, true><<<grid, tb, 0, s>>>(F); break;
        case 31: adj_face_kernel<3, 7, true, true><<<grid, tb, 0, s>>>(F); break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}
cudaError_t launch_adj_face_gauss(int dim, int kind, bool curv, int grid, int tb, const AdjFaceParams& F,
                                  cudaStream_t s) {
    return curv ? launch_adj_face_gauss_curv(dim, kind, grid, tb, F, s)
                : launch_adj_face_gauss_cart(dim, kind, grid, tb, F, s);
}
}  // namespace flou
