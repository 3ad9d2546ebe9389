// Face VJP kernels of the discrete adjoint (adjoint_kernels.cuh), every dimension and flux kind.
#include "adjoint_kernels.cuh"
namespace flou {
cudaError_t launch_adj_face_curv(int dim, int kind, int grid, int tb, const AdjFaceParams& F, cudaStream_t s);
cudaError_t launch_adj_face_gauss(int dim, int kind, bool curv, int grid, int tb, const AdjFaceParams& F,
                                  cudaStream_t s);
static cudaError_t launch_adj_face_plain(int dim, int kind, int grid, int tb, const AdjFaceParams& F, cudaStream_t s) {
    switch (dim * 8 + kind) {
        case 8: adj_face_kernel<1, 0, false, false><<<grid, tb, 0, s>>>(F); break;
        case 9: adj_face_kernel<1, 1, false, false><<<grid, tb, 0, s>>>(F); break;
        case 10: adj_face_kernel<1, 2, false, false><<<grid, tb, 0, s>>>(F); break;
        case 11: adj_face_kernel<1, 3, false, false><<<grid, tb, 0, s>>>(F); break;
        case 12: adj_face_kernel<1, 4, false, false><<<grid, tb, 0, s>>>(F); break;
        case 13: adj_face_kernel<1, 5, false, false><<<grid, tb, 0, s>>>(F); break;
        case 14: adj_face_kernel<1, 6, false, false><<<grid, tb, 0, s>>>(F); break;
        case 15: adj_face_kernel<1, 7, false, false><<<grid, tb, 0, s>>>(F); break;
        case 16: adj_face_kernel<2, 0, false, false><<<grid, tb, 0, s>>>(F); break;
        case 17: adj_face_kernel<2, 1, false, false><<<grid, tb, 0, s>>>(F); break;
        case 18: adj_face_kernel<2, 2, false, false><<<grid, tb, 0, s>>>(F); break;
        case 19: adj_face_kernel<2, 3, false, false><<<grid, tb, 0, s>>>(F); break;
        case 20: adj_face_kernel<2, 4, false, false><<<grid, tb, 0, s>>>(F); break;
        case 21: adj_face_kernel<2, 5, false, false><<<grid, tb, 0, s>>>(F); break;
        case 22: adj_face_kernel<2, 6, false, false><<<grid, tb, 0, s>>>(F); break;
        case 23: adj_face_kernel<2, 7, false, false><<<grid, tb, 0, s>>>(F); break;
        case 24: adj_face_kernel<3, 0, false, false><<<grid, tb, 0, s>>>(F); break;
        case 25: adj_face_kernel<3, 1, false, false><<<grid, tb, 0, s>>>(F); break;
        case 26: adj_face_kernel<3, 2, false, false><<<grid, tb, 0, s>>>(F); break;
        case 27: adj_face_kernel<3, 3, false, false><<<grid, tb, 0, s>>>(F); break;
        case 28: adj_face_kernel<3, 4, false, false><<<grid, tb, 0, s>>>(F); break;
        case 29: adj_face_kernel<3, 5, false, false><<<grid, tb, 0, s>>>(F); break;
        case 30: adj_face_kernel<3, 6, false, false><<<grid, tb, 0, s>>>(F); break;
        case 31: adj_face_kernel<3, 7, false, false><<<grid, tb, 0, s>>>(F); break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}
cudaError_t launch_adj_face(int dim, int kind, bool curv, bool gauss, int grid, int tb, const AdjFaceParams& F,
                            cudaStream_t s) {
    if (gauss) return launch_adj_face_gauss(dim, kind, curv, grid, tb, F, s);
    if (curv) return launch_adj_face_curv(dim, kind, grid, tb, F, s);
    return launch_adj_face_plain(dim, kind, grid, tb, F, s);
}
}  // namespace flou
