// flou_api.cu -- the C ABI of libflou_cuda (include/flou_cuda.h): context lifecycle,
// host-side validation and compression of the set-up arrays, the residual, SSP-RK3
// stepping replayed as a CUDA graph, the CFL time step and the FP64 peak probe.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "flou_ctx.cuh"

using namespace flou;

namespace {

int fail(flou_ctx* c, int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    if (c) c->err = buf;
    return code;
}

int cuda_fail(flou_ctx* c, cudaError_t e, const char* what) {
    if (e == cudaErrorMemoryAllocation) return fail(c, FLOU_ERR_OOM, "%s: %s", what, cudaGetErrorString(e));
    return fail(c, FLOU_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

#define CK(call, what)                                  \
    do {                                                \
        cudaError_t _e = (call);                        \
        if (_e != cudaSuccess) return cuda_fail(c, _e, what); \
    } while (0)

template <class T>
int upload(flou_ctx* c, T** dst, const T* src, size_t count, const char* what) {
    if (*dst) { cudaFree(*dst); *dst = nullptr; }
    if (count == 0) return FLOU_OK;
    CK(cudaMalloc((void**)dst, count * sizeof(T)), what);
    CK(cudaMemcpy(*dst, src, count * sizeof(T), cudaMemcpyHostToDevice), what);
    return FLOU_OK;
}

int ensure(flou_ctx* c, double** buf, size_t count, const char* what) {
    if (*buf) return FLOU_OK;
    CK(cudaMalloc((void**)buf, count * sizeof(double)), what);
    return FLOU_OK;
}

void drop_graph(flou_ctx* c) {
    if (c->gexec) cudaGraphExecDestroy(c->gexec);
    if (c->graph) cudaGraphDestroy(c->graph);
    c->gexec = nullptr;
    c->graph = nullptr;
    c->g_Q = nullptr;
    if (c->cfl_exec) cudaGraphExecDestroy(c->cfl_exec);
    if (c->cfl_graph) cudaGraphDestroy(c->cfl_graph);
    c->cfl_exec = nullptr;
    c->cfl_graph = nullptr;
    c->cfl_Q = nullptr;
}

// Every set-up check a residual needs, with no allocation: flou_rhs (through ready) and
// flou_rhs_noalloc accept exactly the same contexts.
int validate(flou_ctx* c) {
    if (!c) return FLOU_ERR_ARG;
    if (!c->have_ops) return fail(c, FLOU_ERR_STATE, "flou_set_operators has not been called");
    if (!c->have_mesh) return fail(c, FLOU_ERR_STATE, "flou_set_mesh has not been called");
    if (!c->have_geom) return fail(c, FLOU_ERR_STATE, "flou_set_geometry has not been called");
    if (c->cfg.volume_op == FLOU_OP_HYBRID && !c->have_hybrid)
        return fail(c, FLOU_ERR_STATE, "flou_set_hybrid has not been called (hybrid operator)");
    if (c->curv && !c->d_subJ &&
        (c->cfg.volume_op == FLOU_OP_HYBRID || (c->cfg.volume_op == FLOU_OP_SPLIT && !c->bnodes)))
        return fail(c, FLOU_ERR_STATE, "flou_set_subgrid has not been called (general geometry: the hybrid "
                                       "operator, or the split form on a basis without boundary nodes)");
    for (int f = 0; f < c->nfaces; ++f) {
        int b = c->h_face_bc[f];
        if (b >= 0 && (b >= c->nbcs || c->bc_kind[b] == 0))
            return fail(c, FLOU_ERR_STATE, "boundary index %d of face %d has no boundary condition", b + 1, f + 1);
        if (b >= 0 && c->bc_kind[b] == FLOU_BC_STATE_FIELD && !c->d_bcfield)
            return fail(c, FLOU_ERR_STATE, "flou_set_bc_field has not been called (boundary %d)", b + 1);
    }
    return FLOU_OK;
}

int ready(flou_ctx* c) {
    int r = validate(c);
    if (r) return r;
    return ensure(c, &c->d_Fn, (size_t)c->nfdofs * c->nv, "face-flux buffer");
}

FaceParams face_params(const flou_ctx* c, const double* Q) {
    FaceParams P;
    memset(&P, 0, sizeof(P));
    P.Q = Q;
    P.Fn = c->d_Fn;
    P.face_elem = c->d_face_elem;
    P.faceJ = c->d_faceJ;
    P.face_bc = c->d_face_bc;
    P.bc_field = c->d_bcfield;
    P.l = c->d_ops + 2 * c->n * c->n;
    P.elem_c = c->d_c;
    P.ndofs = c->ndofs;
    P.nfdofs = c->nfdofs;
    P.nfaces = c->nfaces;
    P.n = c->n;
    P.npe = c->npe;
    P.nfd = c->nfd;
    P.frames = c->d_frames;
    P.faceJn = c->d_faceJn;
    P.orient = c->d_orient;
    P.status = c->d_status;
    P.numflux = c->cfg.numflux;
    P.lxf_avg = c->cfg.numflux_avg;
    P.intensity = c->cfg.numflux_intensity;
    P.gamma = c->cfg.gamma;
    for (int d = 0; d < 3; ++d) P.adv[d] = c->cfg.advection[d];
    for (int b = 0; b < MAXBC; ++b) {
        P.bc_kind[b] = c->bc_kind[b];
        for (int k = 0; k < 5; ++k) P.bc_state[b][k] = c->bc_state[b][k];
    }
    return P;
}

ElemParams elem_params(const flou_ctx* c, const double* Q, const double* Q0, double* out, int mode, double dt,
                       double a0, double a1) {
    ElemParams P;
    memset(&P, 0, sizeof(P));
    P.Q = Q;
    P.Q0 = Q0;
    P.out = out;
    P.Fn = c->d_Fn;
    P.elem_face = c->d_elem_face;
    P.elem_invJ = c->d_invJ;
    P.elem_Ja = c->d_Ja;
    P.ops = c->d_ops;
    P.ndofs = c->ndofs;
    P.nfdofs = c->nfdofs;
    P.nelem = c->nelem;
    P.mode = mode;
    P.dt = dt;
    P.a0 = a0;
    P.a1 = a1;
    P.aux = mode == 3 ? const_cast<double*>(Q0) : nullptr;   // the 2N register travels in Q0's slot
    P.dtp = c->d_gate;
    P.lift_ends = c->lift_ends ? 1 : 0;
    P.diag_roundoff = c->diag_roundoff ? 1 : 0;
    P.subfr = c->d_subfr;
    P.subJ = c->d_subJ;
    P.gamma = c->cfg.gamma;
    for (int d = 0; d < 3; ++d) P.adv[d] = c->cfg.advection[d];
    P.status = c->d_status;
    P.omega1 = c->d_omega1;
    P.fvflux = c->fvflux;
    P.fvavg = c->fvavg;
    P.fvintensity = c->fvintensity;
    P.blend = c->blend;
    P.invJn = c->d_invJn;
    P.Jan = c->d_Jan;
    P.orient = c->d_orient;
    return P;
}

ElemLaunch elem_launch(const flou_ctx* c) {
    ElemLaunch L;
    L.dim = c->cfg.dim;
    L.eq = c->cfg.equation;
    L.n = c->n;
    L.vol = c->cfg.volume_op;
    L.tp = c->cfg.twopoint_flux;
    // the strong form takes the specialised path only on exact end-node operators; the split and
    // hybrid kernels follow the basis type (their Gauss-Lobatto lift reads the end entries only)
    L.lgl = c->cfg.volume_op == FLOU_OP_STRONG ? c->lgl : c->bnodes;
    L.prepare = false;
    L.curv = c->curv;
    return L;
}

// One residual evaluation followed by the stage combination selected by `mode`.
// Fn: face-flux scratch of this stage (NULL: the context's own).  Stages that may run
// concurrently on different streams need different face-flux buffers.
int stage(flou_ctx* c, cudaStream_t s, const double* Q, const double* Q0, double* out, int mode, double dt,
          double a0, double a1, double* Fn = nullptr) {
    FaceParams fp = face_params(c, Q);
    ElemParams ep = elem_params(c, Q, Q0, out, mode, dt, a0, a1);
    if (Fn) {
        fp.Fn = Fn;
        ep.Fn = Fn;
    }
    cudaError_t e = c->curv ? launch_face_curv(c->cfg.dim, c->cfg.equation, c->lgl, fp, s)
                            : launch_face(c->cfg.dim, c->cfg.equation, c->lgl, fp, s);
    if (e != cudaSuccess) return cuda_fail(c, e, "face kernel launch");
    e = launch_elem(elem_launch(c), ep, s);
    if (e != cudaSuccess) return cuda_fail(c, e, "element kernel launch");
    return FLOU_OK;
}

// One SSP-RK3 step; with a limiter set, it acts after every stage (OrdinaryDiffEq's
// stage_limiter!, FlouTime.jl:136-148), and the selected monitors are recorded after the step.
int rk3_step(flou_ctx* c, cudaStream_t s, double* Q, double dt) {
    int r;
    if ((r = stage(c, s, Q, Q, c->d_U, 1, dt, 0.0, 1.0))) return r;
    if ((r = ctx_limit(c, s, c->d_U))) return r;
    if ((r = stage(c, s, c->d_U, Q, c->d_U, 2, dt, 0.75, 0.25))) return r;
    if ((r = ctx_limit(c, s, c->d_U))) return r;
    if ((r = stage(c, s, c->d_U, Q, Q, 2, dt, 1.0 / 3.0, 2.0 / 3.0))) return r;
    if ((r = ctx_limit(c, s, Q))) return r;
    return ctx_record_monitors(c, s, Q);
}

// One step of a 2N-storage Runge-Kutta method (Williamson 1980; OrdinaryDiffEq's LowStorageRK2N
// with williamson_condition = false, the ORK256 of test/tests.jl:19): every stage is one residual
// whose element epilogue updates k = A_i k + dt L(u) in d_U and u = u + B_i k in place.
int lsrk_step(flou_ctx* c, cudaStream_t s, double* Q, double dt) {
    int r;
    for (int st = 0; st < c->lsrk_s; ++st) {
        if ((r = stage(c, s, Q, c->d_U, Q, 3, dt, st == 0 ? 0.0 : c->lsrk_A[st], c->lsrk_B[st]))) return r;
        if ((r = ctx_limit(c, s, Q))) return r;
    }
    return ctx_record_monitors(c, s, Q);
}

int step_once(flou_ctx* c, cudaStream_t s, double* Q, double dt) {
    return c->lsrk_s ? lsrk_step(c, s, Q, dt) : rk3_step(c, s, Q, dt);
}

int check_status(flou_ctx* c) {
    int32_t st[2];
    CK(cudaMemcpyAsync(st, c->d_status, sizeof(st), cudaMemcpyDeviceToHost, c->stream), "status read");
    CK(cudaStreamSynchronize(c->stream), "stream synchronize");
    if (st[0]) {
        int32_t init[2] = {0, 0x7fffffff};
        cudaMemcpy(c->d_status, init, sizeof(init), cudaMemcpyHostToDevice);
        if (st[0] & 4)
            return fail(c, FLOU_ERR_INDEX, "a device index check failed (element %d; FLOU_CUDA_CHECKED build)", st[1]);
        return fail(c, FLOU_ERR_NONPHYSICAL, "non-physical or non-finite state in element %d", st[1]);
    }
    return FLOU_OK;
}

__global__ void max_dt_kernel(const double* Q, const double* dx, int64_t ndofs, int npe, int dim, int eq,
                              double gamma, double a0, double a1, double a2, double cfl,
                              unsigned long long* out) {
    int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    double v = INFINITY;
    if (g < ndofs) {
        double h = dx[g / npe];
        if (eq == FLOU_EQ_LINEAR_ADVECTION) {
            v = cfl * h / sqrt(a0 * a0 + a1 * a1 + a2 * a2);
        } else if (eq == FLOU_EQ_BURGERS) {
            v = cfl * h / Q[g];   // no abs, as Burgers.jl:35-37
        } else {
            double rho = Q[g];
            double m[3] = {Q[ndofs + g], dim > 1 ? Q[2 * ndofs + g] : 0.0, dim > 2 ? Q[3 * ndofs + g] : 0.0};
            double E = Q[(dim + 1) * ndofs + g];
            double s = m[0] * m[0] + m[1] * m[1] + m[2] * m[2];
            double p = (gamma - 1.0) * (E - s / (2.0 * rho));
            double a = sqrt(gamma * p / rho);
            double u = m[0] / rho, vv = m[1] / rho, w = m[2] / rho;
            double speed = dim == 1 ? fabs(u) : sqrt(u * u + vv * vv + w * w);
            v = cfl * h / (speed + a);
        }
        if (!(v == v)) v = 0.0;   // NaN -> report 0 so the caller sees a broken state
    }
    // warp/block min of positive doubles through their ordered bit patterns
    for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
    __shared__ double sm[32];
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x < 32) {
        v = (threadIdx.x < (blockDim.x + 31) / 32) ? sm[threadIdx.x] : INFINITY;
        for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
        if (threadIdx.x == 0) {
            double w = v < 0.0 ? 0.0 : v;
            atomicMin(out, (unsigned long long)__double_as_longlong(w));
        }
    }
}

// Step control of CFL-limited stepping (get_cfl_callback, FlouTime.jl:92-105, with OrdinaryDiffEq
// landing the last step on tfinal): dt = min(CFL bound, dtmax), cut to tfinal - t; dt = 0 once t
// has reached tfinal, after which every kernel of the step returns at once.  A bound that is not
// positive (a broken state) ends the run and raises S[5].
__global__ void cfl_control_kernel(double* S, unsigned long long* bound) {
    double b = __longlong_as_double((long long)*bound);
    double t = S[0], tf = S[2];
    double dt = fmin(b, S[3]);
    if (!(t < tf)) {
        dt = 0.0;
    } else if (!(dt > 0.0)) {
        dt = 0.0;
        S[5] = 1.0;
        t = tf;
    } else if (t + dt >= tf) {
        dt = tf - t;
        t = tf;
    } else {
        t = t + dt;
    }
    S[0] = t;
    S[1] = dt;
    if (dt > 0.0) S[4] = S[4] + 1.0;
    *bound = (unsigned long long)__double_as_longlong(INFINITY);
}

// Throughput probe: independent FMA chains per thread, eight per thread for ILP.
__global__ void fma_probe_kernel(double* sink, int iters, double x) {
    double a0 = x, a1 = x + 1, a2 = x + 2, a3 = x + 3, a4 = x + 4, a5 = x + 5, a6 = x + 6, a7 = x + 7;
    const double m = 0.999999999, b = 1e-9;
    for (int i = 0; i < iters; ++i) {
        a0 = fma(a0, m, b); a1 = fma(a1, m, b); a2 = fma(a2, m, b); a3 = fma(a3, m, b);
        a4 = fma(a4, m, b); a5 = fma(a5, m, b); a6 = fma(a6, m, b); a7 = fma(a7, m, b);
    }
    double s = ((a0 + a1) + (a2 + a3)) + ((a4 + a5) + (a6 + a7));
    if (s == 1234.5678) sink[threadIdx.x] = s;   // never true; keeps the chains alive
}

// Accuracy of rcp_refined and sqrt_refined against the correctly rounded 1/x and sqrt(x): the
// largest error in units of 2^-53 relative over n doubles with random mantissas and exponents in
// [2^-40, 2^40] (splitmix64 of the sample index), one (rcp, sqrt) pair per block in out.
// Launched with 256 threads per block.
__global__ void refined_math_kernel(long long n, double* out) {
    double mr = 0.0, ms = 0.0;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        unsigned long long z = (unsigned long long)t + 0x9E3779B97F4A7C15ull;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        const unsigned long long ex = 1023ull - 40ull + (z >> 52) % 81ull;
        const double x = __longlong_as_double((long long)((ex << 52) | (z & 0xFFFFFFFFFFFFFull)));
        const double r = 1.0 / x, q = sqrt(x);
        mr = fmax(mr, fabs(rcp_refined(x) - r) / (r * 0x1p-53));
        ms = fmax(ms, fabs(sqrt_refined(x) - q) / (q * 0x1p-53));
    }
    __shared__ double red[2][256];
    red[0][threadIdx.x] = mr;
    red[1][threadIdx.x] = ms;
    __syncthreads();
    for (int h = 128; h > 0; h >>= 1) {
        if ((int)threadIdx.x < h) {
            red[0][threadIdx.x] = fmax(red[0][threadIdx.x], red[0][threadIdx.x + h]);
            red[1][threadIdx.x] = fmax(red[1][threadIdx.x], red[1][threadIdx.x + h]);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        out[2 * blockIdx.x] = red[0][0];
        out[2 * blockIdx.x + 1] = red[1][0];
    }
}

// FP64 tensor-core probe: eight independent m8n8k4 DMMA chains per warp (mma.sync with f64
// operands, the only FP64 matrix instruction of sm_103a; tcgen05 has no f64 kind).  Each
// instruction does 8*8*4 multiply-adds for the warp.
__global__ void dmma_probe_kernel(double* sink, int iters, double x) {
    double a = 1e-3 * x, b = 1e-3 * x + 1e-6 * (threadIdx.x & 31);
    double c[8][2];
#pragma unroll
    for (int k = 0; k < 8; ++k) c[k][0] = c[k][1] = 1e-3 * k;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < 8; ++k)
            asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0, %1}, {%2}, {%3}, {%0, %1};"
                         : "+d"(c[k][0]), "+d"(c[k][1])
                         : "d"(a), "d"(b));
    }
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < 8; ++k) s += c[k][0] + c[k][1];
    if (s == 1234.5678) sink[threadIdx.x] = s;   // never true; keeps the chains alive
}

// Validates Flou's 1-based connectivity and packs it for the kernels (no CUDA involved):
//   ef[e*2d + k] = (face << 1) | side,  fe[2f + s] = (elem << 3) | local position (-1: none),
//   fb[f] = boundary index (0-based) or -1.
int validate_pack_mesh(int dim, int32_t nelem, int32_t nfaces, const int32_t* faceinds, const int32_t* facepos,
                       const int32_t* eleminds, const int32_t* elempos, const uint8_t* orientation,
                       const int32_t* bdface_index, std::vector<int32_t>& ef, std::vector<int32_t>& fe,
                       std::vector<int8_t>& fb, std::string& msg) {
    char buf[256];
    auto bad = [&](int code, const char* fmt, int a, int b, int c2, int d) {
        snprintf(buf, sizeof(buf), fmt, a, b, c2, d);
        msg = buf;
        return code;
    };
    if (dim < 1 || dim > 3) return bad(FLOU_ERR_ARG, "invalid dimension %d", dim, 0, 0, 0);
    int nfpe = 2 * dim;
    if (nelem <= 0 || nfaces <= 0 || nelem >= (1 << 27))
        return bad(FLOU_ERR_ARG, "invalid sizes nelem=%d nfaces=%d", nelem, nfaces, 0, 0);
    if (!faceinds || !facepos || !eleminds || !elempos || !orientation || !bdface_index)
        return bad(FLOU_ERR_ARG, "null connectivity pointer", 0, 0, 0, 0);
    ef.assign((size_t)nelem * nfpe, 0);
    fe.assign((size_t)nfaces * 2, -1);
    fb.assign(nfaces, -1);
    const int maxo = dim == 1 ? 0 : (dim == 2 ? 1 : 7);   // master2slave: StdSegment / StdQuad
    for (int f = 0; f < nfaces; ++f) {
        if (orientation[f] > maxo)
            return bad(FLOU_ERR_ARG, "face %d has orientation %d; a %dD face takes 0..%d", f + 1,
                       (int)orientation[f], dim, maxo);
        for (int s = 0; s < 2; ++s) {
            int e = eleminds[2 * f + s], p = elempos[2 * f + s];
            if (s == 1 && e == 0) continue;
            if (e < 1 || e > nelem || p < 1 || p > nfpe)
                return bad(FLOU_ERR_ARG, "face %d side %d: element %d / position %d out of range", f + 1, s + 1, e, p);
            if (faceinds[(size_t)(e - 1) * nfpe + p - 1] != f + 1 || facepos[(size_t)(e - 1) * nfpe + p - 1] != s + 1)
                return bad(FLOU_ERR_ARG, "face %d side %d is not face %d of element %d in faceinds/facepos", f + 1,
                           s + 1, p, e);
            fe[2 * f + s] = ((e - 1) << 3) | (p - 1);
        }
        int b = bdface_index[f];
        if (eleminds[2 * f + 1] == 0) {
            if (b < 1 || b > MAXBC) return bad(FLOU_ERR_ARG, "boundary face %d has boundary index %d", f + 1, b, 0, 0);
            fb[f] = (int8_t)(b - 1);
        } else if (b != 0) {
            return bad(FLOU_ERR_ARG, "interior face %d has boundary index %d", f + 1, b, 0, 0);
        }
    }
    for (int e = 0; e < nelem; ++e)
        for (int k = 0; k < nfpe; ++k) {
            int f = faceinds[(size_t)e * nfpe + k], s = facepos[(size_t)e * nfpe + k];
            if (f < 1 || f > nfaces || s < 1 || s > 2)
                return bad(FLOU_ERR_ARG, "element %d face %d: face %d / side %d out of range", e + 1, k + 1, f, s);
            if (eleminds[2 * (f - 1) + s - 1] != e + 1 || elempos[2 * (f - 1) + s - 1] != k + 1)
                return bad(FLOU_ERR_ARG, "element %d face %d does not point back through eleminds/elempos", e + 1,
                           k + 1, 0, 0);
            ef[(size_t)e * nfpe + k] = ((f - 1) << 1) | (s - 1);
        }
    return FLOU_OK;
}

// Validates the geometry (J > 0 at every node, finite metric, unit face normals, positive
// surface Jacobians) and computes dx[nelem], get_max_dt's length scale (Σ J ω / n^d)^(1/d)
// (MultielementDiscontinuous.jl:169-171).  When the geometry is Cartesian (J and a diagonal
// metric constant per element, one surface Jacobian per face, the Cartesian frame of the face's
// master side) it is also compressed: invJ[nelem], Jd[nelem*dim], fJ[nfaces]; otherwise
// *cartesian is false and the kernels read the per-node arrays.
int validate_pack_geometry(int dim, int n, int32_t nelem, int32_t nfaces, const double* omega,
                           const std::vector<int32_t>& fe, const double* J, const double* Ja, const double* frames,
                           const double* face_J, std::vector<double>& invJ, std::vector<double>& Jd,
                           std::vector<double>& fJ, std::vector<double>& dx, bool* cartesian, std::string& msg) {
    char buf[256];
    auto bad = [&](int code, const char* fmt, int a) {
        snprintf(buf, sizeof(buf), fmt, a);
        msg = buf;
        return code;
    };
    if (!J || !Ja || !frames || !face_J || !omega) return bad(FLOU_ERR_ARG, "null geometry pointer%.0d", 0);
    int npe = ipow(n, dim), nfd = ipow(n, dim - 1);
    bool cart = true;
    invJ.assign(nelem, 0.0);
    Jd.assign((size_t)nelem * dim, 0.0);
    fJ.assign(nfaces, 0.0);
    dx.assign(nelem, 0.0);
    for (int e = 0; e < nelem; ++e) {
        const double* Je = J + (size_t)e * npe;
        const double* Me = Ja + (size_t)e * npe * dim * dim;
        for (int i = 0; i < npe; ++i) {
            if (!(Je[i] > 0.0) || !std::isfinite(Je[i])) return bad(FLOU_ERR_ARG, "element %d: J <= 0", e + 1);
            if (Je[i] != Je[0]) cart = false;
            for (int q = 0; q < dim * dim; ++q) {
                double v = Me[(size_t)i * dim * dim + q];
                if (!std::isfinite(v)) return bad(FLOU_ERR_ARG, "element %d: non-finite metric", e + 1);
                bool diag = (q % (dim + 1)) == 0;
                if ((!diag && v != 0.0) || v != Me[q]) cart = false;
            }
        }
        invJ[e] = 1.0 / Je[0];
        for (int d = 0; d < dim; ++d) Jd[(size_t)e * dim + d] = Me[d * (dim + 1)];
        double vol = 0.0;
        for (int i = 0; i < npe; ++i) {
            double w = 1.0;
            int r = i;
            for (int d = 0; d < dim; ++d) { w *= omega[r % n]; r /= n; }
            vol += Je[i] * w;
        }
        double h = vol / npe;
        dx[e] = dim == 1 ? h : (dim == 2 ? std::sqrt(h) : std::cbrt(h));
    }
    for (int f = 0; f < nfaces; ++f) {
        FrameTab T = frame_of(dim, fe[2 * f] & 7);
        for (int m = 0; m < nfd; ++m) {
            size_t idx = (size_t)f * nfd + m;
            if (!(face_J[idx] > 0.0) || !std::isfinite(face_J[idx]))
                return bad(FLOU_ERR_ARG, "face %d: surface Jacobian <= 0", f + 1);
            if (face_J[idx] != face_J[(size_t)f * nfd]) cart = false;
            const double* fr = frames + idx * 9;
            double nn = 0.0;
            for (int q = 0; q < 9; ++q)
                if (!std::isfinite(fr[q])) return bad(FLOU_ERR_ARG, "face %d: non-finite frame", f + 1);
            for (int q = 0; q < dim; ++q) nn += fr[q] * fr[q];
            if (std::fabs(nn - 1.0) > 1e-10) return bad(FLOU_ERR_ARG, "face %d: the normal is not a unit vector", f + 1);
            for (int q = 0; q < 3; ++q) {
                bool ok = (q >= dim || (fr[q] == T.n[q] && fr[3 + q] == T.t[q] && (dim < 3 || fr[6 + q] == T.b[q])));
                if (!ok) cart = false;
            }
        }
        fJ[f] = face_J[(size_t)f * nfd];
    }
    *cartesian = cart;
    return FLOU_OK;
}

}  // namespace

namespace flou {
int ctx_fail(flou_ctx* c, int code, const char* msg) { return fail(c, code, "%s", msg); }
int ctx_cuda_fail(flou_ctx* c, cudaError_t e, const char* what) { return cuda_fail(c, e, what); }
int ctx_prepare(flou_ctx* c) {
    int r = ready(c);
    if (r) return r;
    return ensure(c, &c->d_U, (size_t)c->ndofs * c->nv, "stage buffer");
}
FaceParams ctx_face_params(const flou_ctx* c, const double* Q) { return face_params(c, Q); }
ElemParams ctx_elem_params(const flou_ctx* c, const double* Q, const double* Q0, double* out, int mode, double dt,
                           double a0, double a1) {
    return elem_params(c, Q, Q0, out, mode, dt, a0, a1);
}
ElemLaunch ctx_elem_launch(const flou_ctx* c) { return elem_launch(c); }
int ctx_stage(flou_ctx* c, cudaStream_t s, const double* Q, const double* Q0, double* out, int mode, double dt,
              double a0, double a1, double* Fn) {
    return stage(c, s, Q, Q0, out, mode, dt, a0, a1, Fn);
}
int ctx_check_status(flou_ctx* c) { return check_status(c); }
void drop_step_graph(flou_ctx* c) { drop_graph(c); }
}  // namespace flou

extern "C" {

const char* flou_last_error(const flou_ctx* c) { return c ? c->err.c_str() : "null context"; }

int32_t flou_create(const flou_config* cfg, flou_ctx** out) {
    if (!cfg || !out) return FLOU_ERR_ARG;
    *out = nullptr;
    if (cfg->dim < 1 || cfg->dim > 3) return FLOU_ERR_ARG;
    if (cfg->nnodes < 2 || cfg->nnodes > MAXN) return FLOU_ERR_ARG;
    if (cfg->equation < 0 || cfg->equation > 2) return FLOU_ERR_ARG;
    if (cfg->equation == FLOU_EQ_BURGERS && cfg->dim != 1) return FLOU_ERR_ARG;
    if (cfg->volume_op != FLOU_OP_STRONG && cfg->volume_op != FLOU_OP_SPLIT && cfg->volume_op != FLOU_OP_HYBRID)
        return FLOU_ERR_ARG;
    if (cfg->volume_op == FLOU_OP_HYBRID && cfg->equation != FLOU_EQ_EULER) return FLOU_ERR_UNSUPPORTED;
    if (cfg->numflux < 0 || cfg->numflux > 6) return FLOU_ERR_ARG;
    if (cfg->numflux_avg != FLOU_NF_STD_AVERAGE && cfg->numflux_avg != FLOU_NF_CHANDRASHEKAR) return FLOU_ERR_ARG;
    if (cfg->equation != FLOU_EQ_EULER && cfg->numflux != FLOU_NF_STD_AVERAGE && cfg->numflux != FLOU_NF_LXF)
        return FLOU_ERR_UNSUPPORTED;
    if (cfg->equation == FLOU_EQ_EULER && !(cfg->gamma > 1.0)) return FLOU_ERR_ARG;
    flou_ctx* c = new flou_ctx();
    c->cfg = *cfg;
    c->n = cfg->nnodes;
    c->nv = cfg->equation == FLOU_EQ_EULER ? cfg->dim + 2 : 1;
    c->npe = ipow(c->n, cfg->dim);
    c->nfd = ipow(c->n, cfg->dim - 1);
    cudaError_t e = cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete c;
        return FLOU_ERR_CUDA;
    }
    c->stream = c->own_stream;
    e = cudaMalloc((void**)&c->d_status, 2 * sizeof(int32_t));
    if (e != cudaSuccess) {
        cudaStreamDestroy(c->own_stream);
        delete c;
        return FLOU_ERR_OOM;
    }
    int32_t init[2] = {0, 0x7fffffff};
    cudaMemcpy(c->d_status, init, sizeof(init), cudaMemcpyHostToDevice);
    *out = c;
    return FLOU_OK;
}

int32_t flou_destroy(flou_ctx* c) {
    if (!c) return FLOU_ERR_ARG;
    drop_graph(c);
    void* bufs[] = {c->d_ops, c->d_elem_face, c->d_face_elem, c->d_face_bc, c->d_faceJ, c->d_invJ, c->d_Ja, c->d_dx,
                    c->d_Fn, c->d_U, c->d_Qh, c->d_dQh, c->d_status, c->d_dtmin, c->d_c, c->d_invJn, c->d_Jan,
                    c->d_frames, c->d_faceJn, c->d_orient, c->d_Jn, c->d_omega1, c->d_cfl, c->d_cflmin,
                    c->d_subfr, c->d_subJ, c->d_bcfield};
    for (void* b : bufs)
        if (b) cudaFree(b);
    ctx_free_limiter(c);
    if (c->own_stream) cudaStreamDestroy(c->own_stream);
    delete c;
    return FLOU_OK;
}

int32_t flou_set_stream(flou_ctx* c, void* stream) {
    if (!c) return FLOU_ERR_ARG;
    c->stream = stream ? (cudaStream_t)stream : c->own_stream;
    return FLOU_OK;
}

int32_t flou_set_operators(flou_ctx* c, const double* D, const double* Ds, const double* Dsharp, const double* omega,
                           const double* l_l, const double* l_r, const double* dg_l, const double* dg_r) {
    if (!c) return FLOU_ERR_ARG;
    if (!D || !Ds || !Dsharp || !omega || !l_l || !l_r || !dg_l || !dg_r)
        return fail(c, FLOU_ERR_ARG, "null operator pointer");
    int n = c->n;
    std::vector<double> ops(2 * n * n + 4 * n);
    std::copy(Ds, Ds + n * n, ops.begin());
    std::copy(Dsharp, Dsharp + n * n, ops.begin() + n * n);
    std::copy(l_l, l_l + n, ops.begin() + 2 * n * n);
    std::copy(l_r, l_r + n, ops.begin() + 2 * n * n + n);
    std::copy(dg_l, dg_l + n, ops.begin() + 2 * n * n + 2 * n);
    std::copy(dg_r, dg_r + n, ops.begin() + 2 * n * n + 3 * n);
    for (double v : ops)
        if (!std::isfinite(v)) return fail(c, FLOU_ERR_ARG, "non-finite operator entry");
    // A basis with boundary nodes (Gauss-Lobatto) injects the end nodes: l_l = e_1,
    // l_r = e_n and ∂g vanishes off the ends, exactly.  Then the kernels skip the zero terms
    // (bitwise the same result); any other basis takes the general interpolation path.
    bool lgl = l_l[0] == 1.0 && l_r[n - 1] == 1.0;
    for (int i = 0; i < n; ++i) {
        if (i != 0 && (l_l[i] != 0.0 || dg_l[i] != 0.0)) lgl = false;
        if (i != n - 1 && (l_r[i] != 0.0 || dg_r[i] != 0.0)) lgl = false;
    }
    // Whether the basis has boundary nodes (the reference's hasboundaries, a property of the node
    // type) decides the split and hybrid operators' coupling to the faces.  Operators fitted the
    // way the reference builds them carry round-off in the entries that vanish on Gauss-Lobatto
    // nodes, so this test has a tolerance; Gauss nodes are far from it.
    bool bnodes = fabs(l_l[0] - 1.0) < 1e-10 && fabs(l_r[n - 1] - 1.0) < 1e-10;
    bool lift_ends = true;   // ∂g vanishes off the end nodes (DGSEM on Gauss-Lobatto nodes; not VCJH)
    for (int i = 0; i < n; ++i) {
        if (i != 0 && fabs(l_l[i]) > 1e-10) bnodes = false;
        if (i != n - 1 && fabs(l_r[i]) > 1e-10) bnodes = false;
        if (i != 0 && fabs(dg_l[i]) > 1e-10 * fabs(dg_l[0])) lift_ends = false;
        if (i != n - 1 && fabs(dg_r[i]) > 1e-10 * fabs(dg_r[n - 1])) lift_ends = false;
    }
    // Without boundary nodes the split and hybrid operators couple the volume to the faces
    // through entropy-projected states (OpDivergence.jl:301-437, 614-780): Euler only, since
    // the scalar equations have no entropy variables in the reference.
    // The hybrid operator on a basis with boundary nodes sums 2 ω_l D_lk F♯ (OpDivergence.jl:557-
    // 604), whatever the reconstruction: its telescoped form uses 2D - B with the corner B of
    // DGSEM (-1/ω_1, 1/ω_n), which equals the given D♯ only when ∂g acts on the end nodes alone.
    if (c->cfg.volume_op == FLOU_OP_HYBRID && bnodes) {
        for (int j = 0; j < n; ++j)
            for (int i = 0; i < n; ++i) ops[n * n + i + j * n] = 2.0 * D[i + j * n];
        ops[n * n] += 1.0 / omega[0];
        ops[n * n + (n - 1) + (n - 1) * n] -= 1.0 / omega[n - 1];
    }
    // Whether every diagonal entry of the (possibly replaced) D♯ is round-off against its row:
    // true for an SBP operator (2 ω_i D_ii = B_ii), false for a VCJH correction.
    bool diag_roundoff = true;
    for (int i = 0; i < n; ++i) {
        double rowmax = 0.0;
        for (int j = 0; j < n; ++j) rowmax = fmax(rowmax, fabs(ops[n * n + i + j * n]));
        if (fabs(ops[n * n + i + i * n]) > 1e-14 * rowmax) diag_roundoff = false;
    }
    if (c->cfg.volume_op != FLOU_OP_STRONG && !bnodes && c->cfg.equation != FLOU_EQ_EULER)
        return fail(c, FLOU_ERR_UNSUPPORTED,
                    "the split-form and hybrid operators of the scalar equations need a basis with boundary "
                    "nodes (the Gauss-node path projects the entropy variables of the Euler equations)");
    int r = upload(c, &c->d_ops, ops.data(), ops.size(), "operator upload");
    if (r) return r;
    if ((r = upload(c, &c->d_omega1, omega, (size_t)n, "operator upload"))) return r;
    c->lgl = lgl;
    c->bnodes = bnodes;
    c->lift_ends = bnodes && lift_ends;
    c->diag_roundoff = diag_roundoff;
    c->omega.assign(omega, omega + n);
    c->have_ops = true;
    drop_graph(c);
    return FLOU_OK;
}

int32_t flou_set_mesh(flou_ctx* c, int32_t nelem, int32_t nfaces, const int32_t* faceinds, const int32_t* facepos,
                      const int32_t* eleminds, const int32_t* elempos, const uint8_t* orientation,
                      const int32_t* bdface_index) {
    if (!c) return FLOU_ERR_ARG;
    std::vector<int32_t> ef, fe;
    std::vector<int8_t> fb;
    std::string msg;
    int r = validate_pack_mesh(c->cfg.dim, nelem, nfaces, faceinds, facepos, eleminds, elempos, orientation,
                               bdface_index, ef, fe, fb, msg);
    if (r) return fail(c, r, "%s", msg.c_str());
    if ((r = upload(c, &c->d_elem_face, ef.data(), ef.size(), "mesh upload"))) return r;
    if ((r = upload(c, &c->d_face_elem, fe.data(), fe.size(), "mesh upload"))) return r;
    if ((r = upload(c, &c->d_face_bc, fb.data(), fb.size(), "mesh upload"))) return r;
    if ((r = upload(c, &c->d_orient, orientation, (size_t)nfaces, "mesh upload"))) return r;
    c->any_orient = false;
    for (int f = 0; f < nfaces; ++f) c->any_orient |= orientation[f] != 0;
    c->curv = false;
    // sizes changed: drop size-dependent buffers
    double** sized[] = {&c->d_Fn, &c->d_U, &c->d_Qh, &c->d_dQh, &c->d_c};
    for (double** b : sized)
        if (*b) { cudaFree(*b); *b = nullptr; }
    c->h_face_bc = fb;
    c->h_face_elem = fe;
    c->nelem = nelem;
    c->nfaces = nfaces;
    c->ndofs = (int64_t)nelem * c->npe;
    c->nfdofs = (int64_t)nfaces * c->nfd;
    c->have_mesh = true;
    c->have_geom = false;
    drop_graph(c);
    return FLOU_OK;
}

int32_t flou_set_bcs(flou_ctx* c, int32_t nbcs, const int32_t* kinds, const double* states) {
    if (!c) return FLOU_ERR_ARG;
    if (nbcs < 0 || nbcs > MAXBC) return fail(c, FLOU_ERR_ARG, "at most %d boundary conditions", MAXBC);
    if (nbcs > 0 && !kinds) return fail(c, FLOU_ERR_ARG, "null kinds");
    for (int b = 0; b < nbcs; ++b) {
        int k = kinds[b];
        if (k != FLOU_BC_OUTFLOW && k != FLOU_BC_INFLOW && k != FLOU_BC_SLIP && k != FLOU_BC_STATE_FIELD)
            return fail(c, FLOU_ERR_ARG, "unknown boundary condition kind %d", k);
        if (k == FLOU_BC_SLIP && c->cfg.equation != FLOU_EQ_EULER)
            return fail(c, FLOU_ERR_ARG, "slip walls apply to the Euler equations only");
        if (k == FLOU_BC_INFLOW && !states) return fail(c, FLOU_ERR_ARG, "inflow condition without a state");
    }
    c->nbcs = nbcs;
    for (int b = 0; b < MAXBC; ++b) {
        c->bc_kind[b] = b < nbcs ? kinds[b] : 0;
        for (int k = 0; k < 5; ++k) c->bc_state[b][k] = (b < nbcs && states) ? states[b * 5 + k] : 0.0;
    }
    drop_graph(c);
    return FLOU_OK;
}

int32_t flou_set_bc_field(flou_ctx* c, const double* states) {
    if (!c) return FLOU_ERR_ARG;
    if (!c->have_mesh) return fail(c, FLOU_ERR_STATE, "flou_set_mesh must come before flou_set_bc_field");
    if (!states) return fail(c, FLOU_ERR_ARG, "null boundary states");
    const size_t nf = (size_t)c->nfdofs;
    std::vector<double> soa((size_t)c->nv * nf);
    for (size_t i = 0; i < nf; ++i)
        for (int k = 0; k < c->nv; ++k) {
            double v = states[5 * i + k];
            if (!std::isfinite(v)) return fail(c, FLOU_ERR_ARG, "non-finite boundary state at face node %zu", i);
            soa[k * nf + i] = v;
        }
    int r = upload(c, &c->d_bcfield, soa.data(), soa.size(), "boundary-state upload");
    if (r) return r;
    drop_graph(c);
    return FLOU_OK;
}

int32_t flou_set_geometry(flou_ctx* c, const double* J, const double* Ja, const double* frames, const double* face_J) {
    if (!c) return FLOU_ERR_ARG;
    if (!c->have_mesh) return fail(c, FLOU_ERR_STATE, "flou_set_mesh must come before flou_set_geometry");
    if (!c->have_ops) return fail(c, FLOU_ERR_STATE, "flou_set_operators must come before flou_set_geometry");
    std::vector<double> invJ, Jd, fJ, dx;
    std::string msg;
    bool cart = true;
    int r = validate_pack_geometry(c->cfg.dim, c->n, c->nelem, c->nfaces, c->omega.data(), c->h_face_elem, J, Ja,
                                   frames, face_J, invJ, Jd, fJ, dx, &cart, msg);
    if (r) return fail(c, r, "%s", msg.c_str());
    bool curv = !cart || c->any_orient;
    if (curv && c->cfg.dim == 1)
        return fail(c, FLOU_ERR_UNSUPPORTED, "1D geometry must have J constant per element and the Cartesian frames");
    if (curv && c->cfg.equation == FLOU_EQ_BURGERS)
        return fail(c, FLOU_ERR_UNSUPPORTED, "Burgers' equation is 1D");
    std::vector<double> Jel(c->nelem);
    for (int e = 0; e < c->nelem; ++e) Jel[e] = J[(size_t)e * c->npe];
    if ((r = upload(c, &c->d_Jel, Jel.data(), Jel.size(), "geometry upload"))) return r;
    if (curv) {   // per-node arrays, struct-of-arrays for coalesced reads
        int d = c->cfg.dim;
        size_t nd = (size_t)c->ndofs, nf = (size_t)c->nfdofs;
        std::vector<double> invJn(nd), Jan(nd * d * d), fr(nf * 9);
        for (size_t g = 0; g < nd; ++g) {
            invJn[g] = 1.0 / J[g];
            for (int q = 0; q < d * d; ++q) Jan[q * nd + g] = Ja[g * d * d + q];
        }
        for (size_t g = 0; g < nf; ++g)
            for (int q = 0; q < 9; ++q) fr[q * nf + g] = frames[g * 9 + q];
        if ((r = upload(c, &c->d_invJn, invJn.data(), nd, "geometry upload"))) return r;
        if ((r = upload(c, &c->d_Jan, Jan.data(), Jan.size(), "geometry upload"))) return r;
        if ((r = upload(c, &c->d_frames, fr.data(), fr.size(), "geometry upload"))) return r;
        if ((r = upload(c, &c->d_faceJn, face_J, nf, "geometry upload"))) return r;
        if ((r = upload(c, &c->d_Jn, J, nd, "geometry upload"))) return r;
    }
    c->curv = curv;
    if ((r = upload(c, &c->d_invJ, invJ.data(), invJ.size(), "geometry upload"))) return r;
    if ((r = upload(c, &c->d_Ja, Jd.data(), Jd.size(), "geometry upload"))) return r;
    if ((r = upload(c, &c->d_faceJ, fJ.data(), fJ.size(), "geometry upload"))) return r;
    if ((r = upload(c, &c->d_dx, dx.data(), dx.size(), "geometry upload"))) return r;
    c->have_geom = true;
    drop_graph(c);
    return FLOU_OK;
}

int32_t flou_set_hybrid(flou_ctx* c, int32_t fvflux, int32_t fvflux_avg, double fvflux_intensity, double blend) {
    if (!c) return FLOU_ERR_ARG;
    if (c->cfg.volume_op != FLOU_OP_HYBRID) return fail(c, FLOU_ERR_STATE, "the context's operator is not hybrid");
    if (fvflux < 0 || fvflux > 6 || (fvflux_avg != FLOU_NF_STD_AVERAGE && fvflux_avg != FLOU_NF_CHANDRASHEKAR))
        return fail(c, FLOU_ERR_ARG, "invalid subcell flux %d / %d", fvflux, fvflux_avg);
    if (!std::isfinite(fvflux_intensity) || !std::isfinite(blend) || blend < 0.0)
        return fail(c, FLOU_ERR_ARG, "invalid intensity or blending constant");
    c->fvflux = fvflux;
    c->fvavg = fvflux_avg;
    c->fvintensity = fvflux_intensity;
    c->blend = blend;
    c->have_hybrid = true;
    drop_graph(c);
    return FLOU_OK;
}

int32_t flou_set_integrator(flou_ctx* c, int32_t nstages, const double* A, const double* B) {
    if (!c) return FLOU_ERR_ARG;
    if (nstages == 0) {
        c->lsrk_s = 0;
        drop_graph(c);
        return FLOU_OK;
    }
    if (nstages < 1 || nstages > FLOU_MAX_LSRK_STAGES || !A || !B)
        return fail(c, FLOU_ERR_ARG, "a 2N-storage method takes 1..%d stages and its A and B coefficients",
                    FLOU_MAX_LSRK_STAGES);
    for (int i = 0; i < nstages; ++i)
        if (!std::isfinite(B[i]) || (i > 0 && !std::isfinite(A[i])))
            return fail(c, FLOU_ERR_ARG, "non-finite coefficient in stage %d", i + 1);
    c->lsrk_s = nstages;
    for (int i = 0; i < nstages; ++i) {
        c->lsrk_A[i] = i ? A[i] : 0.0;
        c->lsrk_B[i] = B[i];
    }
    drop_graph(c);
    return FLOU_OK;
}

int32_t flou_set_subgrid(flou_ctx* c, const double* frames, const double* jac) {
    if (!c) return FLOU_ERR_ARG;
    if (!c->have_ops || !c->have_mesh) return fail(c, FLOU_ERR_STATE, "flou_set_subgrid needs the operators and the mesh");
    if (!frames || !jac) return fail(c, FLOU_ERR_ARG, "null subgrid array");
    const int d = c->cfg.dim, n = c->n;
    const size_t ns = (size_t)c->nelem * d * c->nfd * (n + 1);
    for (size_t i = 0; i < ns; ++i) {
        const double* f = frames + 9 * i;
        double nn = 0.0;
        for (int q = 0; q < d; ++q) nn += f[q] * f[q];
        if (!(jac[i] > 0.0) || !std::isfinite(jac[i]) || !(fabs(nn - 1.0) < 1e-10))
            return fail(c, FLOU_ERR_ARG, "subgrid point %zu: the surface Jacobian must be positive and the normal a "
                                         "unit vector", i);
    }
    std::vector<double> soa(9 * ns);
    for (size_t i = 0; i < ns; ++i)
        for (int q = 0; q < 9; ++q) soa[q * ns + i] = frames[9 * i + q];
    int r;
    if ((r = upload(c, &c->d_subfr, soa.data(), soa.size(), "subgrid upload"))) return r;
    if ((r = upload(c, &c->d_subJ, jac, ns, "subgrid upload"))) return r;
    drop_graph(c);
    return FLOU_OK;
}

int32_t flou_set_dissipation(flou_ctx* c, const double* celem, int32_t ptr_kind) {
    if (!c) return FLOU_ERR_ARG;
    if (!c->have_mesh) return fail(c, FLOU_ERR_STATE, "flou_set_mesh must come before flou_set_dissipation");
    if (c->cfg.numflux != FLOU_NF_LXF)
        return fail(c, FLOU_ERR_UNSUPPORTED, "a per-element dissipation scale applies to the LxF flux only");
    if (!celem) {
        if (c->d_c) cudaFree(c->d_c);
        c->d_c = nullptr;
        drop_graph(c);
        return FLOU_OK;
    }
    if (!c->d_c) CK(cudaMalloc((void**)&c->d_c, c->nelem * sizeof(double)), "dissipation upload");
    CK(cudaMemcpy(c->d_c, celem, c->nelem * sizeof(double),
                  ptr_kind == FLOU_PTR_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice),
       "dissipation upload");
    drop_graph(c);
    return FLOU_OK;
}

int32_t flou_sizes(const flou_ctx* c, int64_t* ndofs, int32_t* nvars, int32_t* nelem, int32_t* nfaces) {
    if (!c) return FLOU_ERR_ARG;
    if (ndofs) *ndofs = c->ndofs;
    if (nvars) *nvars = c->nv;
    if (nelem) *nelem = c->nelem;
    if (nfaces) *nfaces = c->nfaces;
    return FLOU_OK;
}

int32_t flou_rhs(flou_ctx* c, double* dQ, const double* Q, double t, int32_t ptr_kind) {
    (void)t;   // no time-dependent boundary condition on this path
    int r = ready(c);
    if (r) return r;
    if (!dQ || !Q) return fail(c, FLOU_ERR_ARG, "null state pointer");
    size_t bytes = (size_t)c->ndofs * c->nv * sizeof(double);
    if (ptr_kind == FLOU_PTR_HOST) {
        if ((r = ensure(c, &c->d_Qh, (size_t)c->ndofs * c->nv, "staging buffer"))) return r;
        if ((r = ensure(c, &c->d_dQh, (size_t)c->ndofs * c->nv, "staging buffer"))) return r;
        CK(cudaMemcpyAsync(c->d_Qh, Q, bytes, cudaMemcpyHostToDevice, c->stream), "state upload");
        if ((r = stage(c, c->stream, c->d_Qh, c->d_Qh, c->d_dQh, 0, 0.0, 0.0, 0.0))) return r;
        CK(cudaMemcpyAsync(dQ, c->d_dQh, bytes, cudaMemcpyDeviceToHost, c->stream), "residual download");
    } else if (ptr_kind == FLOU_PTR_DEVICE) {
        if ((r = stage(c, c->stream, Q, Q, dQ, 0, 0.0, 0.0, 0.0))) return r;
    } else {
        return fail(c, FLOU_ERR_ARG, "unknown pointer kind %d", ptr_kind);
    }
    return check_status(c);
}

int32_t flou_step_async(flou_ctx* c, double* Q, double dt, double t0, int32_t nsteps, int32_t ptr_kind) {
    (void)t0;
    int r = ready(c);
    if (r) return r;
    if (!Q) return fail(c, FLOU_ERR_ARG, "null state pointer");
    if (nsteps < 0 || !std::isfinite(dt)) return fail(c, FLOU_ERR_ARG, "invalid nsteps/dt");
    if (nsteps == 0) return FLOU_OK;
    if ((r = ensure(c, &c->d_U, (size_t)c->ndofs * c->nv, "stage buffer"))) return r;
    size_t bytes = (size_t)c->ndofs * c->nv * sizeof(double);
    double* Qd = Q;
    if (ptr_kind == FLOU_PTR_HOST) {
        if ((r = ensure(c, &c->d_Qh, (size_t)c->ndofs * c->nv, "staging buffer"))) return r;
        CK(cudaMemcpyAsync(c->d_Qh, Q, bytes, cudaMemcpyHostToDevice, c->stream), "state upload");
        Qd = c->d_Qh;
    } else if (ptr_kind != FLOU_PTR_DEVICE) {
        return fail(c, FLOU_ERR_ARG, "unknown pointer kind %d", ptr_kind);
    }
    if (!c->gexec || c->g_Q != Qd || c->g_dt != dt) {
        drop_graph(c);
        ElemLaunch L = elem_launch(c);
        L.prepare = true;
        cudaError_t pe = launch_elem(L, elem_params(c, Qd, Qd, c->d_U, 1, dt, 0.0, 1.0), c->own_stream);
        if (pe != cudaSuccess) return cuda_fail(c, pe, "element kernel set-up");
        CK(cudaStreamBeginCapture(c->own_stream, cudaStreamCaptureModeThreadLocal), "graph capture");
        int rr = step_once(c, c->own_stream, Qd, dt);
        cudaGraph_t g = nullptr;
        cudaError_t ce = cudaStreamEndCapture(c->own_stream, &g);
        if (rr) { if (g) cudaGraphDestroy(g); return rr; }
        if (ce != cudaSuccess) return cuda_fail(c, ce, "graph capture");
        c->graph = g;
        CK(cudaGraphInstantiate(&c->gexec, g, 0), "graph instantiate");
        c->g_Q = Qd;
        c->g_dt = dt;
    }
    for (int s = 0; s < nsteps; ++s) CK(cudaGraphLaunch(c->gexec, c->stream), "graph launch");
    if (ptr_kind == FLOU_PTR_HOST)
        CK(cudaMemcpyAsync(Q, c->d_Qh, bytes, cudaMemcpyDeviceToHost, c->stream), "state download");
    return FLOU_OK;
}

int32_t flou_step_cfl(flou_ctx* c, double* Q, double t0, double tfinal, double cfl, double dtmax, int64_t max_steps,
                      int32_t ptr_kind, int64_t* nsteps, double* t_out) {
    int r = ready(c);
    if (r) return r;
    if (!Q) return fail(c, FLOU_ERR_ARG, "null state pointer");
    if (!std::isfinite(t0) || !std::isfinite(tfinal) || !(cfl > 0.0) || !std::isfinite(cfl) || std::isnan(dtmax) ||
        !(dtmax > 0.0) || max_steps < 0)
        return fail(c, FLOU_ERR_ARG, "invalid t0/tfinal/cfl/dtmax/max_steps");
    if (nsteps) *nsteps = 0;
    if (t_out) *t_out = t0;
    if ((r = ensure(c, &c->d_U, (size_t)c->ndofs * c->nv, "stage buffer"))) return r;
    if (!c->d_cfl) CK(cudaMalloc((void**)&c->d_cfl, 8 * sizeof(double)), "CFL state");
    if (!c->d_cflmin) CK(cudaMalloc((void**)&c->d_cflmin, sizeof(unsigned long long)), "CFL state");
    size_t bytes = (size_t)c->ndofs * c->nv * sizeof(double);
    double* Qd = Q;
    if (ptr_kind == FLOU_PTR_HOST) {
        if ((r = ensure(c, &c->d_Qh, (size_t)c->ndofs * c->nv, "staging buffer"))) return r;
        CK(cudaMemcpyAsync(c->d_Qh, Q, bytes, cudaMemcpyHostToDevice, c->stream), "state upload");
        Qd = c->d_Qh;
    } else if (ptr_kind != FLOU_PTR_DEVICE) {
        return fail(c, FLOU_ERR_ARG, "unknown pointer kind %d", ptr_kind);
    }
    double S[8] = {t0, 0.0, tfinal, dtmax, 0.0, 0.0, 0.0, 0.0};
    unsigned long long inf;
    double dinf = INFINITY;
    memcpy(&inf, &dinf, sizeof(inf));
    CK(cudaMemcpyAsync(c->d_cfl, S, sizeof(S), cudaMemcpyHostToDevice, c->stream), "CFL state");
    CK(cudaMemcpyAsync(c->d_cflmin, &inf, sizeof(inf), cudaMemcpyHostToDevice, c->stream), "CFL state");
    if (!c->cfl_exec || c->cfl_Q != Qd || c->cfl_value != cfl) {
        drop_graph(c);
        ElemLaunch L = elem_launch(c);
        L.prepare = true;
        cudaError_t pe = launch_elem(L, elem_params(c, Qd, Qd, c->d_U, 1, 0.0, 0.0, 1.0), c->own_stream);
        if (pe != cudaSuccess) return cuda_fail(c, pe, "element kernel set-up");
        CK(cudaStreamBeginCapture(c->own_stream, cudaStreamCaptureModeThreadLocal), "graph capture");
        int grid = (int)((c->ndofs + 255) / 256);
        const double* a = c->cfg.advection;
        max_dt_kernel<<<grid, 256, 0, c->own_stream>>>(Qd, c->d_dx, c->ndofs, c->npe, c->cfg.dim, c->cfg.equation,
                                                       c->cfg.gamma, a[0], a[1], a[2], cfl, c->d_cflmin);
        cfl_control_kernel<<<1, 1, 0, c->own_stream>>>(c->d_cfl, c->d_cflmin);
        c->d_gate = c->d_cfl + 1;
        int rr = step_once(c, c->own_stream, Qd, 0.0);
        c->d_gate = nullptr;
        cudaGraph_t g = nullptr;
        cudaError_t ce = cudaStreamEndCapture(c->own_stream, &g);
        if (rr) { if (g) cudaGraphDestroy(g); return rr; }
        if (ce != cudaSuccess) return cuda_fail(c, ce, "graph capture");
        c->cfl_graph = g;
        CK(cudaGraphInstantiate(&c->cfl_exec, g, 0), "graph instantiate");
        c->cfl_Q = Qd;
        c->cfl_value = cfl;
    }
    // Launch steps in batches sized from the last dt, reading the device state between batches;
    // never more than max_steps in all.
    int64_t done_steps = 0;
    double last_dt = 0.0;
    while (done_steps < max_steps) {
        int64_t k = 1;
        if (last_dt > 0.0) {
            double left = (tfinal - S[0]) / last_dt;
            k = left > 255.0 ? 256 : (int64_t)left + 1;
        }
        if (k > max_steps - done_steps) k = max_steps - done_steps;
        for (int64_t i = 0; i < k; ++i) CK(cudaGraphLaunch(c->cfl_exec, c->stream), "graph launch");
        CK(cudaMemcpyAsync(S, c->d_cfl, sizeof(S), cudaMemcpyDeviceToHost, c->stream), "CFL state");
        CK(cudaStreamSynchronize(c->stream), "stream synchronize");
        done_steps = (int64_t)S[4];
        last_dt = S[1];
        if (!(S[0] < tfinal) || S[5] != 0.0) break;
    }
    if (nsteps) *nsteps = done_steps;
    if (t_out) *t_out = S[0];
    if ((r = check_status(c))) return r;
    if (S[5] != 0.0)
        return fail(c, FLOU_ERR_NONPHYSICAL, "no positive CFL time step at t = %.17g", S[0]);
    if (ptr_kind == FLOU_PTR_HOST) {
        CK(cudaMemcpyAsync(Q, c->d_Qh, bytes, cudaMemcpyDeviceToHost, c->stream), "state download");
        CK(cudaStreamSynchronize(c->stream), "stream synchronize");
    }
    return FLOU_OK;
}

int32_t flou_wait(flou_ctx* c) {
    if (!c) return FLOU_ERR_ARG;
    return check_status(c);
}

int32_t flou_step(flou_ctx* c, double* Q, double dt, double t0, int32_t nsteps, int32_t ptr_kind) {
    int r = flou_step_async(c, Q, dt, t0, nsteps, ptr_kind);
    if (r) return r;
    if (nsteps == 0) return FLOU_OK;
    return check_status(c);
}

int32_t flou_max_dt(flou_ctx* c, const double* Q, double cfl, double* dt, int32_t ptr_kind) {
    int r = ready(c);
    if (r) return r;
    if (!Q || !dt) return fail(c, FLOU_ERR_ARG, "null pointer");
    const double* Qd = Q;
    size_t bytes = (size_t)c->ndofs * c->nv * sizeof(double);
    if (ptr_kind == FLOU_PTR_HOST) {
        if ((r = ensure(c, &c->d_Qh, (size_t)c->ndofs * c->nv, "staging buffer"))) return r;
        CK(cudaMemcpyAsync(c->d_Qh, Q, bytes, cudaMemcpyHostToDevice, c->stream), "state upload");
        Qd = c->d_Qh;
    }
    if (!c->d_dtmin) CK(cudaMalloc((void**)&c->d_dtmin, sizeof(unsigned long long)), "dt buffer");
    double inf = INFINITY;
    unsigned long long init;
    memcpy(&init, &inf, sizeof(init));
    CK(cudaMemcpyAsync(c->d_dtmin, &init, sizeof(init), cudaMemcpyHostToDevice, c->stream), "dt init");
    int grid = (int)((c->ndofs + 255) / 256);
    const double* a = c->cfg.advection;
    max_dt_kernel<<<grid, 256, 0, c->stream>>>(Qd, c->d_dx, c->ndofs, c->npe, c->cfg.dim, c->cfg.equation,
                                               c->cfg.gamma, a[0], a[1], a[2], cfl, c->d_dtmin);
    CK(cudaGetLastError(), "dt kernel");
    unsigned long long res;
    CK(cudaMemcpyAsync(&res, c->d_dtmin, sizeof(res), cudaMemcpyDeviceToHost, c->stream), "dt read");
    CK(cudaStreamSynchronize(c->stream), "stream synchronize");
    memcpy(dt, &res, sizeof(double));
    return FLOU_OK;
}

int32_t flou_take_status(flou_ctx* c, int32_t* flags, int32_t* elem) {
    if (!c) return FLOU_ERR_ARG;
    int32_t st[2];
    CK(cudaStreamSynchronize(c->stream), "stream synchronize");
    CK(cudaMemcpy(st, c->d_status, sizeof(st), cudaMemcpyDeviceToHost), "status read");
    int32_t init[2] = {0, 0x7fffffff};
    CK(cudaMemcpy(c->d_status, init, sizeof(init), cudaMemcpyHostToDevice), "status reset");
    if (flags) *flags = st[0];
    if (elem) *elem = st[0] ? st[1] : 0;
    return FLOU_OK;
}

int32_t flou_time_kernels(flou_ctx* c, const double* Q, int32_t nrep, double* face_ms, double* elem_ms) {
    int r = ready(c);
    if (r) return r;
    if (!Q || nrep <= 0 || !face_ms || !elem_ms) return fail(c, FLOU_ERR_ARG, "invalid arguments");
    if ((r = ensure(c, &c->d_U, (size_t)c->ndofs * c->nv, "stage buffer"))) return r;
    if ((r = ensure(c, &c->d_dQh, (size_t)c->ndofs * c->nv, "stage buffer"))) return r;
    cudaEvent_t ev[4];
    for (auto& e : ev) CK(cudaEventCreate(&e), "event create");
    double tf = 0.0, te = 0.0;
    for (int it = 0; it < nrep; ++it) {
        for (int mode = 1; mode <= 3; ++mode) {
            CK(cudaEventRecord(ev[0], c->stream), "event record");
            cudaError_t e = c->curv ? launch_face_curv(c->cfg.dim, c->cfg.equation, c->lgl, face_params(c, Q), c->stream)
                                    : launch_face(c->cfg.dim, c->cfg.equation, c->lgl, face_params(c, Q), c->stream);
            if (e != cudaSuccess) return cuda_fail(c, e, "face kernel launch");
            CK(cudaEventRecord(ev[1], c->stream), "event record");
            // stage 1: U = Q + dt L; stages 2, 3: out = a0 Q0 + a1 (U + dt L) (written to scratch)
            ElemParams P = mode == 1 ? elem_params(c, Q, Q, c->d_U, 1, 1e-9, 0.0, 1.0)
                                     : elem_params(c, Q, Q, c->d_dQh, 2, 1e-9, mode == 2 ? 0.75 : 1.0 / 3.0,
                                                   mode == 2 ? 0.25 : 2.0 / 3.0);
            CK(cudaEventRecord(ev[2], c->stream), "event record");
            e = launch_elem(elem_launch(c), P, c->stream);
            if (e != cudaSuccess) return cuda_fail(c, e, "element kernel launch");
            CK(cudaEventRecord(ev[3], c->stream), "event record");
            CK(cudaEventSynchronize(ev[3]), "event synchronize");
            float a = 0.f, b = 0.f;
            cudaEventElapsedTime(&a, ev[0], ev[1]);
            cudaEventElapsedTime(&b, ev[2], ev[3]);
            tf += a;
            te += b;
        }
    }
    for (auto& e : ev) cudaEventDestroy(e);
    *face_ms = tf / (3.0 * nrep);
    *elem_ms = te / (3.0 * nrep);
    return check_status(c);
}

static int32_t copy_msg(const std::string& m, char* out, int32_t len) {
    if (out && len > 0) {
        size_t k = std::min((size_t)(len - 1), m.size());
        memcpy(out, m.data(), k);
        out[k] = 0;
    }
    return 0;
}

int32_t flou_check_mesh(int32_t dim, int32_t nelem, int32_t nfaces, const int32_t* faceinds, const int32_t* facepos,
                        const int32_t* eleminds, const int32_t* elempos, const uint8_t* orientation,
                        const int32_t* bdface_index, char* msg, int32_t msglen) {
    std::vector<int32_t> ef, fe;
    std::vector<int8_t> fb;
    std::string m;
    int r = validate_pack_mesh(dim, nelem, nfaces, faceinds, facepos, eleminds, elempos, orientation, bdface_index, ef,
                               fe, fb, m);
    copy_msg(m, msg, msglen);
    return r;
}

int32_t flou_check_geometry(int32_t dim, int32_t nnodes, int32_t nelem, int32_t nfaces, const int32_t* elempos,
                            const double* omega, const double* J, const double* Ja, const double* frames,
                            const double* face_J, char* msg, int32_t msglen) {
    if (!elempos || nfaces <= 0 || nelem <= 0 || nnodes < 2 || nnodes > MAXN || dim < 1 || dim > 3) {
        copy_msg("invalid arguments", msg, msglen);
        return FLOU_ERR_ARG;
    }
    std::vector<int32_t> fe((size_t)nfaces * 2, -1);
    for (int f = 0; f < nfaces; ++f) fe[2 * f] = elempos[2 * f] - 1;   // only the master position is used
    std::vector<double> invJ, Jd, fJ, dx;
    std::string m;
    bool cart = true;
    int r = validate_pack_geometry(dim, nnodes, nelem, nfaces, omega, fe, J, Ja, frames, face_J, invJ, Jd, fJ, dx,
                                   &cart, m);
    copy_msg(m, msg, msglen);
    return r;
}

int32_t flou_fp64_peak(double* gflops) {
    if (!gflops) return FLOU_ERR_ARG;
    flou_ctx* c = nullptr;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return FLOU_ERR_CUDA;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return FLOU_ERR_CUDA;
    double* sink = nullptr;
    CK(cudaMalloc((void**)&sink, 1024 * sizeof(double)), "probe buffer");
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    const int iters = 1 << 14, threads = 256, blocks = sms * 8;
    fma_probe_kernel<<<blocks, threads>>>(sink, 64, 1.0);   // warm-up
    cudaEventRecord(a);
    fma_probe_kernel<<<blocks, threads>>>(sink, iters, 1.0);
    cudaEventRecord(b);
    cudaError_t e = cudaEventSynchronize(b);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaFree(sink);
    if (e != cudaSuccess) return FLOU_ERR_CUDA;
    double flops = 2.0 * 8.0 * (double)iters * threads * blocks;
    *gflops = flops / (ms * 1e-3) / 1e9;
    return FLOU_OK;
}

int32_t flou_check_refined_math(int64_t nsamples, double* rcp_err, double* sqrt_err) {
    if (!rcp_err || !sqrt_err || nsamples < 1) return FLOU_ERR_ARG;
    flou_ctx* c = nullptr;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return FLOU_ERR_CUDA;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return FLOU_ERR_CUDA;
    const int blocks = sms * 4;
    double* d = nullptr;
    CK(cudaMalloc((void**)&d, 2 * (size_t)blocks * sizeof(double)), "check buffer");
    refined_math_kernel<<<blocks, 256>>>((long long)nsamples, d);
    std::vector<double> h(2 * (size_t)blocks);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpy(h.data(), d, h.size() * sizeof(double), cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) return FLOU_ERR_CUDA;
    double a = 0.0, b = 0.0;
    for (int k = 0; k < blocks; ++k) {
        a = std::max(a, h[2 * k]);
        b = std::max(b, h[2 * k + 1]);
    }
    *rcp_err = a;
    *sqrt_err = b;
    return FLOU_OK;
}

int32_t flou_fp64_dmma_peak(double* gflops) {
    if (!gflops) return FLOU_ERR_ARG;
    flou_ctx* c = nullptr;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return FLOU_ERR_CUDA;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return FLOU_ERR_CUDA;
    double* sink = nullptr;
    CK(cudaMalloc((void**)&sink, 1024 * sizeof(double)), "probe buffer");
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    const int iters = 1 << 12, threads = 256, blocks = sms * 8;
    dmma_probe_kernel<<<blocks, threads>>>(sink, 16, 1.0);   // warm-up
    cudaEventRecord(a);
    dmma_probe_kernel<<<blocks, threads>>>(sink, iters, 1.0);
    cudaEventRecord(b);
    cudaError_t e = cudaEventSynchronize(b);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaFree(sink);
    if (e != cudaSuccess) return FLOU_ERR_CUDA;
    double flops = 2.0 * 8.0 * 8.0 * 4.0 * 8.0 * (double)iters * (threads / 32) * blocks;
    *gflops = flops / (ms * 1e-3) / 1e9;
    return FLOU_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------------------
// Residual without any device allocation.
//
// flou_rhs allocates its face-flux buffer lazily with cudaMalloc on the first call.  Some
// callers cannot allow that: a Julia caller whose device memory is owned by CUDA.jl's
// memory pool, or a PyTorch caller whose caching allocator has already reserved the free
// memory, may see that cudaMalloc fail (or may forbid allocations outside their pool once
// the solve has started).  flou_rhs_noalloc computes the same residual with its face
// fluxes in the fixed array below, which is part of the library image: every GPU that
// loads libflou_cuda holds these 8 MiB until the process exits.
//
// Contract: device pointers only; nfaces * n^(d-1) * nvars must not exceed
// FLOU_NOALLOC_MAX_FACE_VALUES.  All calls (from every context) share the array, so calls
// that overlap on the GPU race on it; serialise them (one stream, or events).  The array
// keeps the last call's contents; nothing in it has to start at zero, because the face
// kernel overwrites every value it later reads.  The first call on a device looks up the
// array's device address (cudaGetSymbolAddress) for that device; make that first call
// before any stream capture.  The address is cached per device for the life of the
// process; cudaDeviceReset destroys every context's memory and the library's module on
// that device, so after a reset neither old contexts nor this cache may be used (a process
// that resets a device must not call flou_rhs_noalloc on it again).
// ---------------------------------------------------------------------------------------
#define FLOU_NOALLOC_MAX_FACE_VALUES (1 << 20)

static __device__ __align__(256) double g_noalloc_face_flux[FLOU_NOALLOC_MAX_FACE_VALUES];

namespace {
constexpr int kMaxDevices = 64;
// Written once per device; concurrent first calls from several host threads store the same
// address, so a relaxed atomic is enough.
std::atomic<double*> g_noalloc_ptr[kMaxDevices] = {};

// Once per device, with that device current: the device address of the scratch array.
// Returns nullptr (and sets *err) when the lookup fails.
double* noalloc_scratch(cudaError_t* err) {
    int dev = 0;
    *err = cudaGetDevice(&dev);
    if (*err != cudaSuccess) return nullptr;
    if (dev < 0 || dev >= kMaxDevices) {
        *err = cudaErrorInvalidDevice;
        return nullptr;
    }
    double* cached = g_noalloc_ptr[dev].load(std::memory_order_relaxed);
    if (!cached) {
        void* p = nullptr;
        *err = cudaGetSymbolAddress(&p, g_noalloc_face_flux);
        if (*err != cudaSuccess) return nullptr;
        cached = (double*)p;
        g_noalloc_ptr[dev].store(cached, std::memory_order_relaxed);
    }
    return cached;
}
}  // namespace

extern "C" int32_t flou_rhs_noalloc(flou_ctx* c, double* dQ, const double* Q, double t) {
    (void)t;
    int r = validate(c);
    if (r) return r;
    if (!dQ || !Q) return fail(c, FLOU_ERR_ARG, "null state pointer");
    int64_t need = c->nfdofs * c->nv;
    if (need > FLOU_NOALLOC_MAX_FACE_VALUES)
        return fail(c, FLOU_ERR_ARG,
                    "flou_rhs_noalloc: the mesh has %lld face values (nfaces x n^(d-1) x nvars); the fixed "
                    "scratch holds at most %d",
                    (long long)need, FLOU_NOALLOC_MAX_FACE_VALUES);
    cudaError_t e = cudaSuccess;
    double* scratch = noalloc_scratch(&e);
    if (!scratch) return cuda_fail(c, e, "flou_rhs_noalloc scratch address");
    FaceParams fp = face_params(c, Q);
    fp.Fn = scratch;
    e = c->curv ? launch_face_curv(c->cfg.dim, c->cfg.equation, c->lgl, fp, c->stream)
                : launch_face(c->cfg.dim, c->cfg.equation, c->lgl, fp, c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "face kernel launch");
    ElemParams ep = elem_params(c, Q, Q, dQ, 0, 0.0, 0.0, 0.0);
    ep.Fn = scratch;
    e = launch_elem(elem_launch(c), ep, c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "element kernel launch");
    return check_status(c);
}
