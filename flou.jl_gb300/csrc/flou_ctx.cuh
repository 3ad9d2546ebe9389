// flou_ctx.cuh -- the context object behind the C ABI's flou_ctx* and the helpers that other
// translation units (the batched launch) share with flou_api.cu.
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "flou_internal.cuh"

using flou::MAXBC;

struct flou_ctx {
    flou_config cfg;
    int nv = 0, n = 0, npe = 0, nfd = 0;
    bool lgl = false;               // l_l = e_1, l_r = e_n exactly: the kernels skip the zero terms
    bool bnodes = false;            // the basis has boundary nodes (hasboundaries), to round-off
    bool lift_ends = false;         // and ∂g vanishes off the end nodes (DGSEM; not a VCJH correction)
    bool diag_roundoff = false;     // every diagonal entry of D♯ is round-off (an SBP operator's D♯ = 2D - B)
    std::string err;
    cudaStream_t own_stream = nullptr, stream = nullptr;
    bool have_ops = false, have_mesh = false, have_geom = false;
    int nelem = 0, nfaces = 0;
    int64_t ndofs = 0, nfdofs = 0;
    std::vector<double> omega;              // quadrature weights (1D)
    std::vector<double> h_invJ, h_J;        // per element
    int nbcs = 0;
    int bc_kind[flou::MAXBC] = {0};
    double bc_state[flou::MAXBC][5] = {{0}};
    std::vector<int8_t> h_face_bc;
    std::vector<int32_t> h_face_elem;   // packed face -> element table (host copy)
    // device buffers
    double* d_ops = nullptr;        // Ds, D♯, l_l, l_r, dg_l, dg_r
    int32_t* d_elem_face = nullptr;
    int32_t* d_face_elem = nullptr;
    int8_t* d_face_bc = nullptr;
    double* d_faceJ = nullptr;
    double* d_invJ = nullptr;
    double* d_Ja = nullptr;
    double* d_dx = nullptr;         // per-element CFL length (vol / n^d)^(1/d)
    double* d_Fn = nullptr;         // face-flux scratch
    double* d_U = nullptr;          // RK stage scratch
    double* d_Qh = nullptr;         // staging for host-pointer calls
    double* d_dQh = nullptr;
    double* d_c = nullptr;          // optional per-element LxF dissipation scale
    // HybridDivOperator: 1D weights, subcell FV flux, blending constant
    double* d_omega1 = nullptr;
    bool have_hybrid = false;
    int fvflux = 0, fvavg = 0;
    double fvintensity = 1.0, blend = 0.0;
    // general (curvilinear / unstructured) geometry: the CURV kernels
    bool curv = false;
    bool any_orient = false;        // some face has a non-zero master2slave orientation
    double* d_invJn = nullptr;      // [ndofs]
    double* d_Jan = nullptr;        // [dim*dim][ndofs]
    double* d_frames = nullptr;     // [9][nfdofs]
    double* d_faceJn = nullptr;     // [nfdofs]
    uint8_t* d_orient = nullptr;    // [nfaces]
    double* d_Jn = nullptr;         // [ndofs] J (limiter, monitors)
    int32_t* d_status = nullptr;    // [flags, lowest element]
    unsigned long long* d_dtmin = nullptr;
    // Zhang-Shu limiter and integral monitors (limiter.cu)
    int limiter = 0;                // FLOU_LIMITER_*
    double lim_min = 0.0;
    double* d_Jel = nullptr;        // J per element
    double* d_wtp = nullptr;        // tensor-product quadrature weights [npe]
    int mon_mask = 0, mon_cap = 0;  // monitors recorded after every flou_step step
    double* d_mon = nullptr;        // [mon_cap][2]: kinetic energy, entropy
    int32_t* d_moncount = nullptr;  // [0]: steps recorded, [1]: single-evaluation slot counter
    double* d_monpart = nullptr;    // block partial sums
    double* d_monval = nullptr;     // single evaluation [2]
    // step method of flou_step: 0 stages = Shu-Osher SSP-RK3, else a 2N-storage method
    int lsrk_s = 0;
    double lsrk_A[FLOU_MAX_LSRK_STAGES], lsrk_B[FLOU_MAX_LSRK_STAGES];
    double* d_bcfield = nullptr;    // [nv][nfdofs] FLOU_BC_STATE_FIELD states
    // subcell-interface geometry of general elements (flou_set_subgrid): [9][ns] frames, [ns] J
    double* d_subfr = nullptr;
    double* d_subJ = nullptr;
    // CFL-limited stepping (flou_step_cfl): the step state lives on the device
    double* d_cfl = nullptr;        // [0] t, [1] dt of the step (0 once t reached tfinal), [2] tfinal,
                                    // [3] dtmax, [4] steps taken, [5] 1 when no positive dt was found
    unsigned long long* d_cflmin = nullptr;   // ordered-bit minimum of the CFL bound
    const double* d_gate = nullptr;           // &d_cfl[1] while the CFL step is captured
    cudaGraph_t cfl_graph = nullptr;
    cudaGraphExec_t cfl_exec = nullptr;
    double* cfl_Q = nullptr;
    double cfl_value = 0.0;
    // graph cache for flou_step
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t gexec = nullptr;
    double* g_Q = nullptr;
    double g_dt = 0.0;
};


namespace flou {
int ctx_fail(flou_ctx* c, int code, const char* msg);
int ctx_cuda_fail(flou_ctx* c, cudaError_t e, const char* what);
int ctx_prepare(flou_ctx* c);   // set-up complete, face and stage buffers allocated
FaceParams ctx_face_params(const flou_ctx* c, const double* Q);
ElemParams ctx_elem_params(const flou_ctx* c, const double* Q, const double* Q0, double* out, int mode, double dt,
                           double a0, double a1);
ElemLaunch ctx_elem_launch(const flou_ctx* c);
int ctx_stage(flou_ctx* c, cudaStream_t s, const double* Q, const double* Q0, double* out, int mode, double dt,
              double a0, double a1, double* Fn = nullptr);   // Fn: face-flux scratch (NULL: the context's)
int ctx_check_status(flou_ctx* c);
// limiter.cu: the stage limiter on Q (no-op when off) and the per-step monitor record
int ctx_limit(flou_ctx* c, cudaStream_t s, double* Q);
// The limiter's VJP at the pre-limiter state V: A (cotangent of the limited state) becomes that of
// V; with K set, K = kK K + kb A afterwards.
int ctx_limit_vjp(flou_ctx* c, cudaStream_t s, const double* V, double* A, double* K, double kK, double kb);
int ctx_record_monitors(flou_ctx* c, cudaStream_t s, const double* Q);
void ctx_free_limiter(flou_ctx* c);
void drop_step_graph(flou_ctx* c);   // settings that change the captured step
}  // namespace flou
