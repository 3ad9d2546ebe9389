// Face kernels (traces, boundary states, numerical fluxes) for every dimension and equation.
#include "flou_internal.cuh"
namespace flou {
template <int DIM, int EQ>
static cudaError_t launch_face_t(bool lgl, const FaceParams& P, cudaStream_t s) {
    int64_t nthreads = (int64_t)P.nfaces * P.nfd;
    if (nthreads == 0) return cudaSuccess;
    const int tb = face_block_size(nthreads);
    int grid = (int)((nthreads + tb - 1) / tb);
    if (lgl) face_kernel<DIM, EQ, true><<<grid, tb, 0, s>>>(P);
    else face_kernel<DIM, EQ, false><<<grid, tb, 0, s>>>(P);
    return cudaGetLastError();
}
cudaError_t launch_face(int dim, int eq, bool lgl, const FaceParams& P, cudaStream_t s) {
    if (eq == FLOU_EQ_EULER) {
        if (dim == 1) return launch_face_t<1, FLOU_EQ_EULER>(lgl, P, s);
        if (dim == 2) return launch_face_t<2, FLOU_EQ_EULER>(lgl, P, s);
        return launch_face_t<3, FLOU_EQ_EULER>(lgl, P, s);
    }
    if (eq == FLOU_EQ_BURGERS) return launch_face_t<1, FLOU_EQ_BURGERS>(lgl, P, s);
    if (dim == 1) return launch_face_t<1, FLOU_EQ_LINEAR_ADVECTION>(lgl, P, s);
    if (dim == 2) return launch_face_t<2, FLOU_EQ_LINEAR_ADVECTION>(lgl, P, s);
    return launch_face_t<3, FLOU_EQ_LINEAR_ADVECTION>(lgl, P, s);
}
// General geometry: the slave trace through master2slave, per-node frames and surface Jacobians.
template <int DIM, int EQ>
static cudaError_t launch_face_curv_t(bool lgl, const FaceParams& P, cudaStream_t s) {
    int64_t nthreads = (int64_t)P.nfaces * P.nfd;
    if (nthreads == 0) return cudaSuccess;
    const int tb = face_block_size(nthreads);
    int grid = (int)((nthreads + tb - 1) / tb);
    if (lgl) face_kernel<DIM, EQ, true, true><<<grid, tb, 0, s>>>(P);
    else face_kernel<DIM, EQ, false, true><<<grid, tb, 0, s>>>(P);
    return cudaGetLastError();
}
cudaError_t launch_face_curv(int dim, int eq, bool lgl, const FaceParams& P, cudaStream_t s) {
    if (eq == FLOU_EQ_EULER) return dim == 2 ? launch_face_curv_t<2, FLOU_EQ_EULER>(lgl, P, s)
                                             : launch_face_curv_t<3, FLOU_EQ_EULER>(lgl, P, s);
    if (eq == FLOU_EQ_LINEAR_ADVECTION)
        return dim == 2 ? launch_face_curv_t<2, FLOU_EQ_LINEAR_ADVECTION>(lgl, P, s)
                        : launch_face_curv_t<3, FLOU_EQ_LINEAR_ADVECTION>(lgl, P, s);
    return cudaErrorInvalidValue;
}
cudaError_t launch_elem(const ElemLaunch& L, const ElemParams& P, cudaStream_t s) {
    if (L.curv && !L.lgl) return L.dim == 2 ? launch_elem_curv_gauss2d(L, P, s) : launch_elem_curv_gauss3d(L, P, s);
    if (L.curv && L.vol == FLOU_OP_HYBRID)
        return L.dim == 2 ? launch_elem_curv_hybrid2d(L, P, s) : launch_elem_curv_hybrid3d(L, P, s);
    if (L.curv) return L.dim == 2 ? launch_elem_curv2d(L, P, s) : launch_elem_curv3d(L, P, s);
    if (L.eq != FLOU_EQ_EULER) return launch_elem_scalar(L, P, s);
    if (!L.lgl && L.vol != FLOU_OP_STRONG) {   // entropy-projected Gauss-node operators
        if (L.dim == 1) return launch_elem_gauss1d(L, P, s);
        if (L.dim == 2) return launch_elem_gauss2d(L, P, s);
        return L.vol == FLOU_OP_HYBRID ? launch_elem_gauss3d_hybrid(L, P, s) : launch_elem_gauss3d_split(L, P, s);
    }
    if (L.dim == 1) return launch_elem_euler1d(L, P, s);
    if (L.dim == 2) return launch_elem_euler2d(L, P, s);
    if (L.vol == FLOU_OP_STRONG) return launch_elem_euler3d_strong(L, P, s);
    return L.vol == FLOU_OP_HYBRID ? launch_elem_euler3d_hybrid(L, P, s) : launch_elem_euler3d_split(L, P, s);
}
}  // namespace flou
