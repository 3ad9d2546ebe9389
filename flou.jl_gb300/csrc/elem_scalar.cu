// Element kernels of the scalar equations: linear advection (1D-3D) and Burgers (1D).
#include "flou_internal.cuh"
namespace flou {
cudaError_t launch_elem_scalar(const ElemLaunch& L, const ElemParams& P, cudaStream_t s) {
    if (L.eq == FLOU_EQ_BURGERS) {
        if (L.dim != 1) return cudaErrorInvalidValue;
        return launch_elem_dim<1, FLOU_EQ_BURGERS>(L.n, L.vol, L.tp, L.lgl, P, s, L.prepare);
    }
    switch (L.dim) {
        case 1: return launch_elem_dim<1, FLOU_EQ_LINEAR_ADVECTION>(L.n, L.vol, L.tp, L.lgl, P, s, L.prepare);
        case 2: return launch_elem_dim<2, FLOU_EQ_LINEAR_ADVECTION>(L.n, L.vol, L.tp, L.lgl, P, s, L.prepare);
        case 3: return launch_elem_dim<3, FLOU_EQ_LINEAR_ADVECTION>(L.n, L.vol, L.tp, L.lgl, P, s, L.prepare);
        default: return cudaErrorInvalidValue;
    }
}
}  // namespace flou
