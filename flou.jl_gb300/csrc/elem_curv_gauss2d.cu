// Element kernels, 2D on general (curvilinear / unstructured) elements with a basis without
// boundary nodes: the strong form and the entropy-projected split and hybrid forms.
#include "flou_internal.cuh"
namespace flou {
cudaError_t launch_elem_curv_gauss2d(const ElemLaunch& L, const ElemParams& P, cudaStream_t s) {
    if (L.eq == FLOU_EQ_EULER) return launch_elem_dim_curv_gauss<2, FLOU_EQ_EULER>(L.n, L.vol, L.tp, P, s, L.prepare);
    if (L.eq == FLOU_EQ_LINEAR_ADVECTION)
        return launch_elem_dim_curv_gauss<2, FLOU_EQ_LINEAR_ADVECTION>(L.n, L.vol, L.tp, P, s, L.prepare);
    return cudaErrorInvalidValue;
}
}  // namespace flou
