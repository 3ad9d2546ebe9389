// Face VJP kernels of the discrete adjoint on general geometry (adjoint_kernels.cuh): the slave
// trace through the orientation, per-node frames, surface Jacobians and 1/J; 2D and 3D.
#include "adjoint_kernels.cuh"
namespace flou {
cudaError_t launch_adj_face_curv(int dim, int kind, int grid, int tb, const AdjFaceParams& F, cudaStream_t s) {
    switch (dim * 8 + kind) {
        case 16: adj_face_kernel<2, 0, true, false><<<grid, tb, 0, s>>>(F); break;
        case 17: adj_face_kernel<2, 1, true, false><<<grid, tb, 0, s>>>(F); break;
        case 18: adj_face_kernel<2, 2, true, false><<<grid, tb, 0, s>>>(F); break;
        case 19: adj_face_kernel<2, 3, true, false><<<grid, tb, 0, s>>>(F); break;
        case 20: adj_face_kernel<2, 4, true, false><<<grid, tb, 0, s>>>(F); break;
        case 21: adj_face_kernel<2, 5, true, false><<<grid, tb, 0, s>>>(F); break;
        case 22: adj_face_kernel<2, 6, true, false><<<grid, tb, 0, s>>>(F); break;
        case 23: adj_face_kernel<2, 7, true, false><<<grid, tb, 0, s>>>(F); break;
        case 24: adj_face_kernel<3, 0, true, false><<<grid, tb, 0, s>>>(F); break;
        case 25: adj_face_kernel<3, 1, true, false><<<grid, tb, 0, s>>>(F); break;
        case 26: adj_face_kernel<3, 2, true, false><<<grid, tb, 0, s>>>(F); break;
        case 27: adj_face_kernel<3, 3, true, false><<<grid, tb, 0, s>>>(F); break;
        case 28: adj_face_kernel<3, 4, true, false><<<grid, tb, 0, s>>>(F); break;
        case 29: adj_face_kernel<3, 5, true, false><<<grid, tb, 0, s>>>(F); break;
        case 30: adj_face_kernel<3, 6, true, false><<<grid, tb, 0, s>>>(F); break;
        case 31: adj_face_kernel<3, 7, true, false><<<grid, tb, 0, s>>>(F); break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}
}  // namespace flou
