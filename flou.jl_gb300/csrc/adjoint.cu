// adjoint.cu -- host side of the discrete adjoint: the adjoint of one SSP-RK3 stage (face and
// element VJP kernels of adjoint_kernels.cuh), the binomial checkpoint schedule, the
// single-instance reverse sweep on four streams, the lockstep batched reverse sweep under one
// memory budget, and the C ABI (flou_rhs_vjp, flou_adjoint_solve, flou_adjoint_solve_batch).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "adjoint_kernels.cuh"

namespace flou {

// Terminal functional J = 1/2 Σ w_i (ρ_i - ρt_i)²: seed Ū (density column) and per-block partials.
__global__ void functional_kernel(const double* Q, const double* rho_t, const double* w, int64_t ndofs, int nv,
                                  double* Ubar, double* partial) {
    int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    double j = 0.0;
    if (g < ndofs) {
        double r = Q[g] - rho_t[g];
        Ubar[g] = w[g] * r;
        for (int k = 1; k < nv; ++k) Ubar[k * ndofs + g] = 0.0;
        j = 0.5 * w[g] * (r * r);
    }
    for (int o = 16; o > 0; o >>= 1) j += __shfl_xor_sync(0xffffffffu, j, o);
    __shared__ double sm[32];
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = j;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int k = 0; k < (int)(blockDim.x + 31) / 32; ++k) s += sm[k];
        partial[blockIdx.x] = s;
    }
}

// y = a x (the first reverse stage of a 2N-storage step: k̄ = B_s Ū)
__global__ void scale_kernel(double* y, const double* x, double a, int64_t n) {
    int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (g < n) y[g] = a * x[g];
}

}  // namespace flou

using namespace flou;

namespace {

struct AdjBuffers {
    double *QbL = nullptr, *QbR = nullptr, *Ibar = nullptr;
    // the hybrid operator on Gauss nodes: the forward face fluxes at U, their cotangents by side
    // of the face, and the first element pass's partial node cotangents
    double *Fn = nullptr, *FbS = nullptr, *Tq = nullptr;
};

// The hybrid operator on a basis without boundary nodes: its stage takes two element passes.
bool hybrid_gauss(const flou_ctx* c) {
    return c->cfg.equation == FLOU_EQ_EULER && c->cfg.volume_op == FLOU_OP_HYBRID && !c->bnodes;
}

// The flux kind of adj_face_kernel / numflux_vjp for an interface flux (numflux, central part),
// -1 for one the adjoint does not differentiate.
int flux_kind(int nf, int avg) {
    const int ch = avg == FLOU_NF_CHANDRASHEKAR ? 1 : 0;
    if (nf == FLOU_NF_HLLC) return 3;
    if (nf == FLOU_NF_HLL) return 2;
    if (avg != FLOU_NF_STD_AVERAGE && avg != FLOU_NF_CHANDRASHEKAR) return -1;
    if (nf == FLOU_NF_SCALAR_DISSIPATION) return 4 + ch;
    if (nf == FLOU_NF_MATRIX_DISSIPATION) return 6 + ch;
    if (nf == FLOU_NF_LXF) return ch;
    return -1;
}
int fv_kind(const flou_ctx* c) { return flux_kind(c->fvflux, c->fvavg); }

// The scalar equations (linear advection, Burgers): the strong form on either node set or the
// split form with the arithmetic-mean two-point flux, the LxF or central interface flux.
int adj_supported_scalar(flou_ctx* c) {
    const flou_config& k = c->cfg;
    const bool vol = k.volume_op == FLOU_OP_STRONG ||
                     (k.volume_op == FLOU_OP_SPLIT && k.twopoint_flux == FLOU_TP_STD_AVERAGE);
    const bool nf = k.numflux == FLOU_NF_STD_AVERAGE ||
                    (k.numflux == FLOU_NF_LXF && k.numflux_avg == FLOU_NF_STD_AVERAGE);
    if (!vol || !nf)
        return ctx_fail(c, FLOU_ERR_UNSUPPORTED, "the adjoint of the scalar equations covers the strong form and the "
                                                 "split form with the StdAverage two-point flux, with the LxF or "
                                                 "StdAverage interface flux");
    return FLOU_OK;
}

int adj_supported(flou_ctx* c) {
    const flou_config& k = c->cfg;
    if (k.equation != FLOU_EQ_EULER) return adj_supported_scalar(c);
    bool vol = k.volume_op == FLOU_OP_STRONG ||
               ((k.volume_op == FLOU_OP_SPLIT || k.volume_op == FLOU_OP_HYBRID) &&
                (k.twopoint_flux == FLOU_TP_CHANDRASHEKAR || k.twopoint_flux == FLOU_TP_KENNEDY_GRUBER ||
                 k.twopoint_flux == FLOU_TP_STD_AVERAGE));
    bool nf = ((k.numflux == FLOU_NF_LXF || k.numflux == FLOU_NF_SCALAR_DISSIPATION ||
                k.numflux == FLOU_NF_MATRIX_DISSIPATION) &&
               (k.numflux_avg == FLOU_NF_STD_AVERAGE || k.numflux_avg == FLOU_NF_CHANDRASHEKAR)) ||
              k.numflux == FLOU_NF_HLL || k.numflux == FLOU_NF_HLLC;
    if (k.equation != FLOU_EQ_EULER || !vol || !nf)
        return ctx_fail(c, FLOU_ERR_UNSUPPORTED, "the adjoint covers the Euler equations with the strong form or "
                                                 "the split form (Chandrashekar, Kennedy-Gruber or StdAverage), and the "
                                                 "LxF, Scalar- or MatrixDissipation (StdAverage or ChandrasekharAverage), "
                                                 "HLL or HLLC interface flux");
    if (k.volume_op == FLOU_OP_SPLIT && c->bnodes && !c->lift_ends)
        return ctx_fail(c, FLOU_ERR_UNSUPPORTED, "the adjoint of the split form needs the DGSEM lift on a basis "
                                                 "with boundary nodes");
    if (k.volume_op == FLOU_OP_SPLIT && !c->bnodes && !adj_split_tile_fits(k.dim, c->n, k.twopoint_flux, true, false))
        return ctx_fail(c, FLOU_ERR_UNSUPPORTED, "the Gauss-node split adjoint tile exceeds shared memory");
    if (k.volume_op == FLOU_OP_HYBRID) {
        if (c->bnodes && !c->lift_ends)
            return ctx_fail(c, FLOU_ERR_UNSUPPORTED, "the adjoint of the hybrid operator covers Gauss-Lobatto and "
                                                     "Gauss nodes");
        if (fv_kind(c) < 0)
            return ctx_fail(c, FLOU_ERR_UNSUPPORTED, "the hybrid operator's subcell flux must be LxF, "
                                                     "Scalar- or MatrixDissipation (StdAverage or "
                                                     "ChandrasekharAverage), HLL or HLLC for the adjoint");
        if (!adj_split_tile_fits(k.dim, c->n, k.twopoint_flux, !c->bnodes, true))
            return ctx_fail(c, FLOU_ERR_UNSUPPORTED, "the hybrid adjoint tile exceeds shared memory");
    }
    return FLOU_OK;
}

int alloc_adj(flou_ctx* c, AdjBuffers& B) {
    size_t nf = (size_t)c->nfdofs * c->nv;
    cudaError_t e = cudaMalloc((void**)&B.QbL, nf * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc((void**)&B.QbR, nf * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc((void**)&B.Ibar, (size_t)c->nfdofs * sizeof(double));
    if (hybrid_gauss(c)) {
        if (e == cudaSuccess) e = cudaMalloc((void**)&B.Fn, nf * sizeof(double));
        if (e == cudaSuccess) e = cudaMalloc((void**)&B.FbS, 2 * nf * sizeof(double));
        if (e == cudaSuccess) e = cudaMalloc((void**)&B.Tq, (size_t)c->ndofs * c->nv * sizeof(double));
    }
    if (e != cudaSuccess) return ctx_cuda_fail(c, e, "adjoint buffers");
    return FLOU_OK;
}

void free_adj(AdjBuffers& B) {
    if (B.QbL) cudaFree(B.QbL);
    if (B.QbR) cudaFree(B.QbR);
    if (B.Ibar) cudaFree(B.Ibar);
    if (B.Fn) cudaFree(B.Fn);
    if (B.FbS) cudaFree(B.FbS);
    if (B.Tq) cudaFree(B.Tq);
    B = AdjBuffers();
}

// One transposed residual, fused with an adjoint stage combination:
//   Aout = alpha Ain + beta B + (∂L/∂U)(U)ᵀ (s_lam Ain);  B = gamma_B B + delta_B Ain (writeB)
//   cbar += (∂L/∂c)ᵀ (s_lam Ain)
int adj_stage(flou_ctx* c, AdjBuffers& Bf, cudaStream_t s, const double* U, const double* Ain, double* Aout,
              double* Bacc, double* cbar, double s_lam, double alpha, double beta, int readB, int writeB,
              double gamma_B, double delta_B, double* K = nullptr, double kA = 0.0, double kB = 0.0) {
    AdjFaceParams F;
    memset(&F, 0, sizeof(F));
    F.status = c->d_status;
    F.U = U;
    F.Ain = Ain;
    F.s_lam = s_lam;
    F.QbL = Bf.QbL;
    F.QbR = Bf.QbR;
    F.Ibar = Bf.Ibar;
    F.face_elem = c->d_face_elem;
    F.faceJ = c->d_faceJ;
    F.face_bc = c->d_face_bc;
    F.invJ = c->d_invJ;
    F.ops = c->d_ops;
    F.elem_c = c->d_c;
    F.frames = c->d_frames;
    F.faceJn = c->d_faceJn;
    F.orient = c->d_orient;
    F.invJn = c->d_invJn;
    F.intensity = c->cfg.numflux_intensity;
    F.gamma = c->cfg.gamma;
    F.ndofs = c->ndofs;
    F.nfdofs = c->nfdofs;
    F.nfaces = c->nfaces;
    F.n = c->n;
    F.npe = c->npe;
    F.nfd = c->nfd;
    for (int b = 0; b < MAXBC; ++b) {
        F.bc_kind[b] = c->bc_kind[b];
        for (int k = 0; k < 5; ++k) F.bc_state[b][k] = c->bc_state[b][k];
    }
    F.bc_field = c->d_bcfield;
    int64_t nth = (int64_t)c->nfaces * c->nfd;
    const int tb = face_block_size(nth);
    int grid = (int)((nth + tb - 1) / tb);
    int dim = c->cfg.dim;
    const int kind = flux_kind(c->cfg.numflux, c->cfg.numflux_avg);
    // interpolated traces and the full-line lift: the strong form on a basis without exact end-node
    // injection, the split form on a basis without boundary nodes (the forward's general paths)
    const bool gauss = c->cfg.volume_op == FLOU_OP_STRONG ? !c->lgl : !c->bnodes;
    const bool scalar = c->cfg.equation != FLOU_EQ_EULER;
    for (int d = 0; d < 3; ++d) F.adv[d] = c->cfg.advection[d];
    F.lxf = c->cfg.numflux == FLOU_NF_LXF ? 1 : 0;
    const bool hg = hybrid_gauss(c);
    if (hg && !(Bf.Fn && Bf.FbS && Bf.Tq))
        return ctx_fail(c, FLOU_ERR_STATE, "the Gauss-node hybrid adjoint stage has no face-flux buffers");
    cudaError_t e = scalar || hg ? cudaSuccess : launch_adj_face(dim, kind, c->curv, gauss, grid, tb, F, s);
    if (e != cudaSuccess) return ctx_cuda_fail(c, e, "adjoint face kernel");
    AdjElemParams P;
    memset(&P, 0, sizeof(P));
    P.status = c->d_status;
    P.U = U;
    P.Ain = Ain;
    P.Aout = Aout;
    P.B = Bacc;
    P.QbL = Bf.QbL;
    P.QbR = Bf.QbR;
    P.Ibar = Bf.Ibar;
    P.cbar = c->d_c ? cbar : nullptr;
    P.elem_face = c->d_elem_face;
    P.face_elem = c->d_face_elem;
    P.invJ = c->d_invJ;
    P.Ja = c->d_Ja;
    P.invJn = c->d_invJn;
    P.Jan = c->d_Jan;
    P.orient = c->d_orient;
    P.ops = c->d_ops;
    P.ndofs = c->ndofs;
    P.nfdofs = c->nfdofs;
    P.nelem = c->nelem;
    P.s_lam = s_lam;
    P.alpha = alpha;
    P.beta = beta;
    P.gamma_B = gamma_B;
    P.delta_B = delta_B;
    P.readB = readB;
    P.writeB = writeB;
    P.gamma = c->cfg.gamma;
    P.K = K;
    P.kA = kA;
    P.kB = kB;
    P.omega1 = c->d_omega1;
    P.fvkind = c->cfg.volume_op == FLOU_OP_HYBRID ? fv_kind(c) : 0;
    P.fvflux = c->fvflux;
    P.fvavg = c->fvavg;
    P.fvintensity = c->fvintensity;
    P.blend = c->blend;
    P.subfr = c->d_subfr;
    P.subJ = c->d_subJ;
    for (int d = 0; d < 3; ++d) P.adv[d] = c->cfg.advection[d];
    if (scalar) {
        e = launch_adj_scalar(dim, c->cfg.equation, c->n, c->cfg.volume_op == FLOU_OP_SPLIT, gauss, c->curv, grid, tb,
                              F, P, s);
        if (e != cudaSuccess) return ctx_cuda_fail(c, e, "adjoint kernels (scalar equation)");
        return FLOU_OK;
    }
    if (hg) {   // forward face fluxes, element pass 1, the face VJP with its cotangents, pass 2
        FaceParams fp = ctx_face_params(c, U);
        fp.Fn = Bf.Fn;
        e = c->curv ? launch_face_curv(dim, c->cfg.equation, c->lgl, fp, s)
                    : launch_face(dim, c->cfg.equation, c->lgl, fp, s);
        if (e == cudaSuccess) e = cudaMemsetAsync(Bf.FbS, 0, 2 * (size_t)c->nfdofs * c->nv * sizeof(double), s);
        if (e != cudaSuccess) return ctx_cuda_fail(c, e, "adjoint forward face fluxes");
        P.FnU = Bf.Fn;
        P.FbS = Bf.FbS;
        P.Tq = Bf.Tq;
        e = launch_adj_hybrid_gauss(dim, c->n, c->cfg.twopoint_flux, c->curv, P, s);
        if (e != cudaSuccess) return ctx_cuda_fail(c, e, "adjoint element kernel");
        F.FbS = Bf.FbS;
        e = launch_adj_face(dim, kind, c->curv, gauss, grid, tb, F, s);
        if (e != cudaSuccess) return ctx_cuda_fail(c, e, "adjoint face kernel");
        e = launch_adj_hybrid_gauss_finish(dim, c->n, c->curv, P, s);
    } else if (c->cfg.volume_op != FLOU_OP_STRONG) {
        e = launch_adj_split_dim(dim, c->n, c->cfg.twopoint_flux, c->curv, gauss,
                                 c->cfg.volume_op == FLOU_OP_HYBRID, P, s);
    } else {
        e = launch_adj_elem_dim(dim, c->n, c->curv, gauss, P, s);
    }
    if (e != cudaSuccess) return ctx_cuda_fail(c, e, "adjoint element kernel");
    return FLOU_OK;
}

// Optimal binomial checkpointing split (Griewank & Walther's problem): minimal number of
// forward steps to reverse n steps from a stored state with s free snapshot slots, by dynamic
// programming over the position m of the next snapshot:
//   cost(n, s) = min_m m + cost(n - m, s - 1) + cost(m, s),  cost(1, s) = 0,  cost(n, 0) = n(n-1)/2.
struct Schedule {
    int n, s;
    std::vector<long long> cost;
    std::vector<int> split;
    long long& C(int nn, int ss) { return cost[(size_t)nn * (s + 1) + ss]; }
    int& M(int nn, int ss) { return split[(size_t)nn * (s + 1) + ss]; }
    // Binomial rule when the table is too large: with r the least repetition number such that
    // C(ss + r, ss) >= nn, put the snapshot so that the remainder fits C(ss - 1 + r, ss - 1).
    int split_of(int nn, int ss) {
        if (dp) return M(nn, ss);
        if (ss >= nn - 1) return 1;
        auto binom = [](int a, int b) {
            double v = 1.0;
            for (int i = 1; i <= b; ++i) v = v * (a - b + i) / i;
            return v;
        };
        int r = 0;
        while (binom(ss + r, ss) < nn) ++r;
        int m = nn - (int)std::min<double>(binom(ss - 1 + r, ss - 1), nn - 1);
        return std::max(1, std::min(nn - 1, m));
    }
    bool dp = true;
    Schedule(int n_, int s_) : n(n_), s(std::min(s_, std::max(n_ - 1, 0))) {
        if (s >= n - 1) {   // every state can be kept: advance one step per snapshot
            dp = false;
            return;
        }
        if ((double)n * n * (s + 1) > 2e8) {   // too large for the table: binomial rule below
            dp = false;
            return;
        }
        cost.assign((size_t)(n + 1) * (s + 1), 0);
        split.assign((size_t)(n + 1) * (s + 1), 0);
        for (int nn = 0; nn <= n; ++nn) C(nn, 0) = (long long)nn * (nn - 1) / 2;
        for (int ss = 1; ss <= s; ++ss)
            for (int nn = 2; nn <= n; ++nn) {
                long long best = -1;
                int bm = 1;
                for (int m = 1; m < nn; ++m) {
                    long long v = m + C(nn - m, ss - 1) + C(m, ss);
                    if (best < 0 || v < best) { best = v; bm = m; }
                }
                C(nn, ss) = best;
                M(nn, ss) = bm;
            }
    }
};

// ---- one time step, forward and reverse, for both solvers ----
// SSP-RK3 (Shu-Osher) or the context's 2N-storage method; with the Zhang-Shu limiter after every
// stage when the context has it.  A reverse step keeps the step's stage states: SSP-RK3 U1, U2
// (with the limiter also the states before it, V1, V2, V3); a 2N-storage method u_1 .. u_(s-1)
// (with the limiter also v_1 .. v_s).
bool has_limiter(const flou_ctx* c) { return c->limiter == FLOU_LIMITER_ZHANG_SHU; }

int stage_count(const flou_ctx* c) {
    const int s = c->lsrk_s;
    return s ? (has_limiter(c) ? 2 * s - 1 : s - 1) : (has_limiter(c) ? 5 : 2);
}

// One 2N-storage stage (0-based st) from u: k = A_st k + dt L(u) in K, out = u + B_st k.
int lsrk_stage(flou_ctx* c, cudaStream_t s, double dt, const double* u, double* K, double* out, int st, double* Fn) {
    return ctx_stage(c, s, u, K, out, 3, dt, st == 0 ? 0.0 : c->lsrk_A[st], c->lsrk_B[st], Fn);
}

int limit_if(flou_ctx* c, cudaStream_t s, double* Q) { return has_limiter(c) ? ctx_limit(c, s, Q) : FLOU_OK; }

// dst <- the limited copy of src
int limited_copy(flou_ctx* c, cudaStream_t s, double* dst, const double* src) {
    cudaError_t e = cudaMemcpyAsync(dst, src, (size_t)c->ndofs * c->nv * sizeof(double), cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) return ctx_cuda_fail(c, e, "stage copy");
    return limit_if(c, s, dst);
}

// k steps in place; R is a state-sized register (the SSP-RK3 stage, the 2N-storage k).
int advance_steps(flou_ctx* c, cudaStream_t s, double dt, double* Q, double* R, double* Fn, int k) {
    for (int i = 0; i < k; ++i) {
        int r;
        if (c->lsrk_s) {
            for (int st = 0; st < c->lsrk_s; ++st) {
                if ((r = lsrk_stage(c, s, dt, Q, R, Q, st, Fn))) return r;
                if ((r = limit_if(c, s, Q))) return r;
            }
        } else {
            if ((r = ctx_stage(c, s, Q, Q, R, 1, dt, 0.0, 1.0, Fn))) return r;
            if ((r = limit_if(c, s, R))) return r;
            if ((r = ctx_stage(c, s, R, Q, R, 2, dt, 0.75, 0.25, Fn))) return r;
            if ((r = limit_if(c, s, R))) return r;
            if ((r = ctx_stage(c, s, R, Q, Q, 2, dt, 1.0 / 3.0, 2.0 / 3.0, Fn))) return r;
            if ((r = limit_if(c, s, Q))) return r;
        }
    }
    return FLOU_OK;
}

// The stage states of the step from X into SX (stage_count buffers) with the register K; for a
// 2N-storage method and seedT set, also the step's result U^n (the functional's state).
int stage_states(flou_ctx* c, cudaStream_t s, double dt, const double* X, double* const* SX, double* K, double* Fn,
                 double* seedT) {
    int r;
    const int ns = c->lsrk_s;
    if (ns && has_limiter(c)) {   // v_(i+1) from u_i, u_(i+1) its limited copy
        const double* u = X;
        for (int st = 0; st < ns; ++st) {
            double* v = SX[ns - 1 + st];
            if ((r = lsrk_stage(c, s, dt, u, K, v, st, Fn))) return r;
            if (st + 1 < ns && (r = limited_copy(c, s, SX[st], v))) return r;
            u = SX[st];
        }
        if (seedT && (r = limited_copy(c, s, seedT, SX[2 * ns - 2]))) return r;
    } else if (ns) {
        const double* u = X;
        for (int st = 0; st + 1 < ns; ++st) {
            if ((r = lsrk_stage(c, s, dt, u, K, SX[st], st, Fn))) return r;
            u = SX[st];
        }
        if (seedT && (r = lsrk_stage(c, s, dt, u, K, seedT, ns - 1, Fn))) return r;
    } else if (has_limiter(c)) {   // V1, U1 = L(V1), V2, U2 = L(V2), V3
        if ((r = ctx_stage(c, s, X, X, SX[2], 1, dt, 0.0, 1.0, Fn))) return r;
        if ((r = limited_copy(c, s, SX[0], SX[2]))) return r;
        if ((r = ctx_stage(c, s, SX[0], X, SX[3], 2, dt, 0.75, 0.25, Fn))) return r;
        if ((r = limited_copy(c, s, SX[1], SX[3]))) return r;
        if ((r = ctx_stage(c, s, SX[1], X, SX[4], 2, dt, 1.0 / 3.0, 2.0 / 3.0, Fn))) return r;
    } else {
        if ((r = ctx_stage(c, s, X, X, SX[0], 1, dt, 0.0, 1.0, Fn))) return r;
        if ((r = ctx_stage(c, s, SX[0], X, SX[1], 2, dt, 0.75, 0.25, Fn))) return r;
    }
    return FLOU_OK;
}

// SSP-RK3: the step's result U^n into T from its stage states (the 2N-storage methods form it in
// stage_states).
int final_state(flou_ctx* c, cudaStream_t s, double dt, const double* X, double* const* SX, double* T, double* Fn) {
    if (has_limiter(c)) return limited_copy(c, s, T, SX[4]);   // U^n = L(V3)
    return ctx_stage(c, s, SX[1], X, T, 2, dt, 1.0 / 3.0, 2.0 / 3.0, Fn);
}

// The adjoint of one step: A holds Ū^(k+1) on entry and Ū^k on exit; T and B are scratch.
// SSP-RK3 (Ū2 = ⅔V̄3 + VJP(U2; ⅔dt V̄3), B = ⅓V̄3; Ū1 = ¼V̄2 + VJP(U1; ¼dt V̄2), B += ¾V̄2;
// Ū0 = V̄1 + B + VJP(U0; dt V̄1), with V̄ = Ū without the limiter, its VJP at V with it).
// A 2N-storage step (Williamson form; stage i from u_i: k_i = A_i k_(i-1) + dt L(u_i),
// u_(i+1) = u_i + B_i k_i, A_0 = 0), reverse stage i with k̄ = k̄_i + B_i Ū(i+1) in T:
//   Ū_i = Ū_(i+1) + dt (∂L/∂u)(u_i)ᵀ k̄,  then T = A_i k̄ + B_(i-1) Ū_i for stage i-1
// (the element kernel's epilogue forms the next k̄ in place); the last stage starts from
// k̄ = B_(s-1) Ū; A_0 = 0 leaves nothing to carry into the previous step.  With the limiter
// (u_(i+1) = L(v_(i+1))), Ū_(i+1) first becomes V̄_(i+1) through the limiter's VJP, which also
// adds B_i V̄_(i+1) to the register (the epilogue then carries A_i k̄ alone).
int reverse_stages(flou_ctx* c, AdjBuffers& ab, cudaStream_t s, double dt, const double* X, double* const* SX,
                   double* A, double* T, double* B, double* cbar) {
    int r;
    const bool lim = has_limiter(c);
    const int ns = c->lsrk_s;
    if (ns) {
        if (lim) {
            if ((r = ctx_limit_vjp(c, s, SX[2 * ns - 2], A, T, 0.0, c->lsrk_B[ns - 1]))) return r;
        } else {
            const int64_t n = c->ndofs * c->nv;
            scale_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(T, A, c->lsrk_B[ns - 1], n);
            cudaError_t e = cudaGetLastError();
            if (e != cudaSuccess) return ctx_cuda_fail(c, e, "adjoint register");
        }
        for (int i = ns - 1; i >= 0; --i) {
            const double* u = i == 0 ? X : SX[i - 1];
            if ((r = adj_stage(c, ab, s, u, T, A, A, cbar, dt, 0.0, 1.0, 1, 0, 0.0, 0.0, i > 0 ? T : nullptr,
                               c->lsrk_A[i], (i > 0 && !lim) ? c->lsrk_B[i - 1] : 0.0)))
                return r;
            if (lim && i > 0 && (r = ctx_limit_vjp(c, s, SX[ns - 2 + i], A, T, 1.0, c->lsrk_B[i - 1]))) return r;
        }
        return FLOU_OK;
    }
    if (lim && (r = ctx_limit_vjp(c, s, SX[4], A, nullptr, 0.0, 0.0))) return r;
    if ((r = adj_stage(c, ab, s, SX[1], A, T, B, cbar, (2.0 / 3.0) * dt, 2.0 / 3.0, 0.0, 0, 1, 0.0, 1.0 / 3.0)))
        return r;
    if (lim && (r = ctx_limit_vjp(c, s, SX[3], T, nullptr, 0.0, 0.0))) return r;
    if ((r = adj_stage(c, ab, s, SX[0], T, A, B, cbar, 0.25 * dt, 0.25, 0.0, 0, 1, 1.0, 0.75))) return r;
    if (lim && (r = ctx_limit_vjp(c, s, SX[2], A, nullptr, 0.0, 0.0))) return r;
    return adj_stage(c, ab, s, X, A, A, B, cbar, dt, 1.0, 1.0, 1, 0, 0.0, 0.0);
}

// Single-instance reverse sweep on four streams.  Two forward streams `sf[0..1]` take turns: each
// places snapshots and recomputes the state U^k that a reverse step needs, into one of NB X
// buffers; the stage stream `ss` forms that step's two stage states U^(k,1), U^(k,2); the adjoint
// stream `sa` runs the three adjoint stages.  None of the recomputation depends on the adjoint,
// so while the adjoint stream reverses step k+1, the stage stream forms the stages of step k and
// the forward streams recompute U^(k-1) and U^(k-2) side by side: four chains of one-wave kernels
// share the GPU.  Events order every hand-over: X filled (ready) -> stages filled (sready) ->
// consumed (done); per snapshot, the event of its last placement (written) and of the last copy
// each forward stream made from it (read), so a slot is only rewritten after its readers and
// only read after its writer.  Each stream has its own stage and face-flux scratch.
struct Solver {
    static constexpr int NB = 3, NF = 2;
    flou_ctx* c;
    cudaStream_t sa = nullptr, ss = nullptr;
    cudaStream_t sf[NF] = {};
    double dt;
    int nsteps;
    std::vector<double*> slot;          // snapshot states; slot[0] = U^0
    std::vector<int> free_slots;
    std::vector<cudaEvent_t> written;   // [slot]
    std::vector<cudaEvent_t> read;      // [slot * NF + f]
    double* X[NB] = {};
    // stage states of a reverse step: SSP-RK3 U^(k,1), U^(k,2); a 2N-storage method u_1 .. u_(s-1)
    std::vector<double*> SX[NB];
    double* Kss = nullptr;            // the stage stream's 2N register
    cudaEvent_t ready[NB] = {}, sready[NB] = {}, done[NB] = {};
    bool used[NB] = {};
    int xi = 0, fi = 0;
    double* F1[NF] = {};                                           // forward streams: stage scratch
    double* Fnf[NF] = {};                                          // and face fluxes
    double* Fns = nullptr;                                         // stage stream: face flux
    double *A = nullptr, *Bacc = nullptr, *T = nullptr;            // adjoint stream
    double* cbar = nullptr;
    const double* rho_t;
    const double* w;
    double* partial = nullptr;
    double* h_partial = nullptr;
    int nblk = 0;
    bool seeded = false;
    long long advances = 0;
    AdjBuffers ab;
    Schedule* sch = nullptr;
    size_t bytes = 0;

    int cuda(cudaError_t e, const char* what) { return e == cudaSuccess ? FLOU_OK : ctx_cuda_fail(c, e, what); }
    int wait(cudaStream_t s, cudaEvent_t e) { return cuda(cudaStreamWaitEvent(s, e, 0), "event wait"); }
    int record(cudaEvent_t e, cudaStream_t s) { return cuda(cudaEventRecord(e, s), "event record"); }
    int next_f() {
        int f = fi;
        fi = (fi + 1) % NF;
        return f;
    }
    // dst <- slot si on forward stream f, after the slot's writer; marks the read
    int copy_from(int f, double* dst, int si) {
        int r;
        if ((r = wait(sf[f], written[si]))) return r;
        if ((r = cuda(cudaMemcpyAsync(dst, slot[si], bytes, cudaMemcpyDeviceToDevice, sf[f]), "state copy"))) return r;
        return record(read[(size_t)si * NF + f], sf[f]);
    }
    int advance(int f, double* Q, int k) {   // k steps in place on forward stream f (F1[f]: its register)
        int r = advance_steps(c, sf[f], dt, Q, F1[f], Fnf[f], k);
        advances += k;
        return r;
    }
    // slot sj <- U^(i0+m) advanced from slot si (a snapshot placement)
    int place(int sj, int si, int m) {
        int r;
        int f = next_f();
        for (int g = 0; g < NF; ++g)   // earlier readers of sj, on either forward stream
            if ((r = wait(sf[f], read[(size_t)sj * NF + g]))) return r;
        if ((r = wait(sf[f], written[sj]))) return r;
        if ((r = copy_from(f, slot[sj], si))) return r;
        if ((r = advance(f, slot[sj], m))) return r;
        return record(written[sj], sf[f]);
    }
    // U^(i0+k) from snapshot si into the next buffer set, its stage states, then the reverse step
    // i0+k on them.
    int step_from(int si, int k, int kstep) {
        int r;
        int b = xi;
        xi = (xi + 1) % NB;
        int f = next_f();
        if (used[b] && (r = wait(sf[f], done[b]))) return r;
        if ((r = copy_from(f, X[b], si))) return r;
        if ((r = advance(f, X[b], k))) return r;
        if ((r = record(ready[b], sf[f]))) return r;
        // the stage stream (ready[b] comes after the forward stream's wait for done[b], so the stage
        // buffers are free again); for the last step of a 2N-storage method also U^n, into T, which
        // the adjoint stream has not used yet
        if ((r = wait(ss, ready[b]))) return r;
        const bool seed = kstep == nsteps - 1 && !seeded;
        if ((r = stage_states(c, ss, dt, X[b], SX[b].data(), Kss, Fns, seed && c->lsrk_s ? T : nullptr))) return r;
        if ((r = record(sready[b], ss))) return r;
        if ((r = wait(sa, sready[b]))) return r;
        if ((r = backward_step(kstep, b))) return r;
        used[b] = true;
        return record(done[b], sa);
    }
    // Reverse one step from U^k (X[b]) and its stage states: the adjoint of U^(k+1) is in A on
    // entry and that of U^k on exit (adjoint stream).
    int backward_step(int k, int b) {
        int r;
        if (!seeded) {   // the last step: U^n, the functional and its gradient seed
            if (k != nsteps - 1) return ctx_fail(c, FLOU_ERR_STATE, "adjoint schedule out of order");
            if (!c->lsrk_s && (r = final_state(c, sa, dt, X[b], SX[b].data(), T, nullptr))) return r;
            functional_kernel<<<nblk, 256, 0, sa>>>(T, rho_t, w, c->ndofs, c->nv, A, partial);
            if ((r = cuda(cudaGetLastError(), "functional"))) return r;
            if ((r = cuda(cudaMemcpyAsync(h_partial, partial, nblk * sizeof(double), cudaMemcpyDeviceToHost, sa),
                          "functional")))
                return r;
            seeded = true;
        }
        return reverse_stages(c, ab, sa, dt, X[b], SX[b].data(), A, T, Bacc, cbar);
    }
    // U^i0 is in slot[si]; ns free snapshot slots may be used; reverses steps i0 .. i0+n-1.
    int rev(int i0, int n, int ns, int si) {
        int r;
        if (n <= 0) return FLOU_OK;
        if (n == 1) return step_from(si, 0, i0);
        if (ns == 0 || free_slots.empty()) {
            for (int k = n - 1; k >= 0; --k)
                if ((r = step_from(si, k, i0 + k))) return r;
            return FLOU_OK;
        }
        int m = sch->split_of(n, std::min(ns, sch->s));
        if (m < 1 || m >= n) m = n / 2;
        int sj = free_slots.back();
        free_slots.pop_back();
        if ((r = place(sj, si, m))) return r;
        if ((r = rev(i0 + m, n - m, ns - 1, sj))) return r;
        free_slots.push_back(sj);
        return rev(i0, m, ns, si);
    }
};

// Lockstep reverse sweep of many independent solves under one device-memory budget.  All
// instances follow one checkpoint schedule (same number of steps, each its own dt), so a
// snapshot holds every instance's state at one step and the budget sets the number of
// snapshots for the whole batch.  Instance i runs on stream stream_of[i]: its operations stay
// ordered, while instances on other streams overlap with it.  The step scratch (X, S1, S2, T, B
// and the face cotangents) is per stream, sized for the largest instance on that stream; the
// adjoint state of instance i lives in the caller's gradient buffer and its initial state is
// read from the caller's Q0 (snapshot 0).  Each instance steps with its own context's method
// (SSP-RK3 or its 2N-storage method, with or without the limiter).
struct BatchSolver {
    struct Scratch {
        double *X = nullptr, *T = nullptr, *B = nullptr, *K = nullptr;   // K: the stepping register
        std::vector<double*> SX;                                          // stage states
        AdjBuffers ab;
    };
    int n = 0, nsteps = 0;
    std::vector<flou_ctx*> c;
    std::vector<double> dt;
    std::vector<cudaStream_t> st;
    std::vector<int> stream_of;
    std::vector<size_t> bytes, off;          // state bytes of instance i, its offset in a snapshot
    size_t snap_bytes = 0;
    std::vector<const double*> q0;
    std::vector<double*> slot;               // slot[0] unused (the caller's Q0), 1..s snapshots
    std::vector<int> free_slots;
    std::vector<Scratch> scr;
    std::vector<double*> A, cbar;
    std::vector<const double*> rho_t, w;
    std::vector<size_t> poff;
    std::vector<int> nblk;
    double* partial = nullptr;               // device, Σ nblk
    double* h_partial = nullptr;             // pinned host copy
    std::vector<char> seeded;
    long long advances = 0;                  // forward steps per instance (the same for all)
    Schedule* sch = nullptr;
    int failed = -1;

    cudaStream_t S(int i) const { return st[stream_of[i]]; }
    Scratch& W(int i) { return scr[stream_of[i]]; }
    const double* snap(int si, int i) const { return si == 0 ? q0[i] : slot[si] + off[i] / sizeof(double); }
    double* snapw(int si, int i) { return slot[si] + off[i] / sizeof(double); }
    int fail_at(int i, int r) {
        if (failed < 0) failed = i;
        return r;
    }
    int copy(double* dst, const double* src, int i) {
        cudaError_t e = cudaMemcpyAsync(dst, src, bytes[i], cudaMemcpyDeviceToDevice, S(i));
        return e == cudaSuccess ? FLOU_OK : fail_at(i, ctx_cuda_fail(c[i], e, "state copy"));
    }
    int advance(double* Q, int k, int i) {
        int r = advance_steps(c[i], S(i), dt[i], Q, W(i).K, nullptr, k);
        return r ? fail_at(i, r) : FLOU_OK;
    }
    // U^k of instance i is in its stream's X; A[i] holds the adjoint of U^(k+1) on entry and
    // that of U^k on exit.
    int backward_step(int k, int i) {
        flou_ctx* ci = c[i];
        Scratch& w_ = W(i);
        cudaStream_t s = S(i);
        double h = dt[i];
        int r;
        const bool seed = !seeded[i];
        if ((r = stage_states(ci, s, h, w_.X, w_.SX.data(), w_.K, nullptr, seed && ci->lsrk_s ? w_.T : nullptr)))
            return fail_at(i, r);
        if (seed) {
            if (k != nsteps - 1) return fail_at(i, ctx_fail(ci, FLOU_ERR_STATE, "adjoint schedule out of order"));
            if (!ci->lsrk_s && (r = final_state(ci, s, h, w_.X, w_.SX.data(), w_.T, nullptr))) return fail_at(i, r);
            functional_kernel<<<nblk[i], 256, 0, s>>>(w_.T, rho_t[i], w[i], ci->ndofs, ci->nv, A[i], partial + poff[i]);
            cudaError_t e = cudaGetLastError();
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(h_partial + poff[i], partial + poff[i], nblk[i] * sizeof(double),
                                    cudaMemcpyDeviceToHost, s);
            if (e != cudaSuccess) return fail_at(i, ctx_cuda_fail(ci, e, "functional"));
            seeded[i] = 1;
        }
        if ((r = reverse_stages(ci, w_.ab, s, h, w_.X, w_.SX.data(), A[i], w_.T, w_.B, cbar[i]))) return fail_at(i, r);
        return FLOU_OK;
    }
    // Every instance's U^i0 is in snapshot si; ns free snapshots; reverses steps i0 .. i0+m-1.
    int rev(int i0, int m, int ns, int si) {
        int r;
        if (m <= 0) return FLOU_OK;
        if (m == 1) {
            for (int i = 0; i < n; ++i) {
                if ((r = copy(W(i).X, snap(si, i), i))) return r;
                if ((r = backward_step(i0, i))) return r;
            }
            return FLOU_OK;
        }
        if (ns == 0 || free_slots.empty()) {
            for (int k = m - 1; k >= 0; --k) {
                for (int i = 0; i < n; ++i) {
                    if ((r = copy(W(i).X, snap(si, i), i))) return r;
                    if ((r = advance(W(i).X, k, i))) return r;
                    if ((r = backward_step(i0 + k, i))) return r;
                }
                advances += k;
            }
            return FLOU_OK;
        }
        int mm = sch->split_of(m, std::min(ns, sch->s));
        if (mm < 1 || mm >= m) mm = m / 2;
        int sj = free_slots.back();
        free_slots.pop_back();
        for (int i = 0; i < n; ++i) {
            if ((r = copy(snapw(sj, i), snap(si, i), i))) return r;
            if ((r = advance(snapw(sj, i), mm, i))) return r;
        }
        advances += mm;
        if ((r = rev(i0 + mm, m - mm, ns - 1, sj))) return r;
        free_slots.push_back(sj);
        return rev(i0, mm, ns, si);
    }
};

}  // namespace

extern "C" {

int32_t flou_rhs_vjp(flou_ctx* c, double* Qbar, double* cbar, const double* Q, const double* lambda) {
    if (!c) return FLOU_ERR_ARG;
    int r = ctx_prepare(c);
    if (r) return r;
    if ((r = adj_supported(c))) return r;
    if (!Qbar || !Q || !lambda) return ctx_fail(c, FLOU_ERR_ARG, "null pointer");
    AdjBuffers B;
    if ((r = alloc_adj(c, B))) return r;
    cudaStream_t s = c->stream;
    if (cbar && c->d_c) {
        cudaError_t e = cudaMemsetAsync(cbar, 0, c->nelem * sizeof(double), s);
        if (e != cudaSuccess) { free_adj(B); return ctx_cuda_fail(c, e, "cbar reset"); }
    }
    r = adj_stage(c, B, s, Q, lambda, Qbar, nullptr, cbar, 1.0, 0.0, 0.0, 0, 0, 0.0, 0.0);
    cudaError_t e = cudaStreamSynchronize(s);
    free_adj(B);
    if (r) return r;
    if (e != cudaSuccess) return ctx_cuda_fail(c, e, "vjp");
    return ctx_check_status(c);
}

int32_t flou_adjoint_solve(flou_ctx* c, const double* Q0, double dt, int32_t nsteps, int32_t nsnap,
                           const double* rho_target, const double* weights, double* J, double* dJdQ0, double* dJdc,
                           int64_t* forward_steps) {
    if (!c) return FLOU_ERR_ARG;
    int r = ctx_prepare(c);
    if (r) return r;
    if ((r = adj_supported(c))) return r;
    if (!Q0 || !rho_target || !weights || !dJdQ0 || nsteps < 1 || nsnap < 0 || !std::isfinite(dt))
        return ctx_fail(c, FLOU_ERR_ARG, "invalid arguments");
    if (dJdc && !c->d_c)
        return ctx_fail(c, FLOU_ERR_STATE, "dJ/dc needs the per-element dissipation scale (flou_set_dissipation)");
    Solver S;
    S.c = c;
    S.sa = c->stream;
    S.dt = dt;
    S.nsteps = nsteps;
    S.rho_t = rho_target;
    S.w = weights;
    S.bytes = (size_t)c->ndofs * c->nv * sizeof(double);
    S.nblk = (int)((c->ndofs + 255) / 256);
    S.A = dJdQ0;   // the adjoint state lives in the output
    int nslots = std::min(nsnap, std::max(nsteps - 1, 0));
    std::vector<double*> owned;
    cudaError_t e = cudaStreamCreateWithFlags(&S.ss, cudaStreamNonBlocking);
    for (int f = 0; f < Solver::NF && e == cudaSuccess; ++f) e = cudaStreamCreateWithFlags(&S.sf[f], cudaStreamNonBlocking);
    auto dalloc = [&](double** p, size_t b) {
        if (e != cudaSuccess) return;
        e = cudaMalloc((void**)p, b);
        if (e == cudaSuccess) owned.push_back(*p);
    };
    S.slot.assign(nslots + 1, nullptr);
    for (int i = 0; i <= nslots; ++i) dalloc(&S.slot[i], S.bytes);
    const int nst = stage_count(c);
    for (int i = 0; i < Solver::NB; ++i) {
        dalloc(&S.X[i], S.bytes);
        S.SX[i].assign(nst, nullptr);
        for (int j = 0; j < nst; ++j) dalloc(&S.SX[i][j], S.bytes);
    }
    if (c->lsrk_s) dalloc(&S.Kss, S.bytes);
    double** bufs[] = {&S.Bacc, &S.T};
    for (double** b : bufs) dalloc(b, S.bytes);
    for (int f = 0; f < Solver::NF; ++f) {
        dalloc(&S.F1[f], S.bytes);
        dalloc(&S.Fnf[f], (size_t)c->nfdofs * c->nv * sizeof(double));
    }
    dalloc(&S.Fns, (size_t)c->nfdofs * c->nv * sizeof(double));
    S.written.assign(nslots + 1, nullptr);
    S.read.assign((size_t)(nslots + 1) * Solver::NF, nullptr);
    for (auto& ev : S.written)
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
    for (auto& ev : S.read)
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
    dalloc(&S.partial, S.nblk * sizeof(double));
    for (int i = 0; i < Solver::NB && e == cudaSuccess; ++i) {
        e = cudaEventCreateWithFlags(&S.ready[i], cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&S.sready[i], cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&S.done[i], cudaEventDisableTiming);
    }
    if (e == cudaSuccess) e = cudaMallocHost((void**)&S.h_partial, S.nblk * sizeof(double));
    if (e == cudaSuccess && dJdc) S.cbar = dJdc;
    int rr = FLOU_OK;
    if (e != cudaSuccess) rr = ctx_cuda_fail(c, e, "adjoint storage");
    if (!rr) rr = alloc_adj(c, S.ab);
    if (!rr && S.cbar) {
        e = cudaMemsetAsync(S.cbar, 0, c->nelem * sizeof(double), S.sa);
        if (e != cudaSuccess) rr = ctx_cuda_fail(c, e, "cbar reset");
    }
    Schedule sch(nsteps, nslots);
    S.sch = &sch;
    for (int i = 1; i <= nslots; ++i) S.free_slots.push_back(i);
    if (!rr) {   // the forward streams start after what the caller queued on the context's stream
        cudaEvent_t ev;
        e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventRecord(ev, S.sa);
        for (int f = 0; f < Solver::NF && e == cudaSuccess; ++f) e = cudaStreamWaitEvent(S.sf[f], ev, 0);
        if (e == cudaSuccess) cudaEventDestroy(ev);
        if (e != cudaSuccess) rr = ctx_cuda_fail(c, e, "stream order");
    }
    if (!rr) {
        e = cudaMemcpyAsync(S.slot[0], Q0, S.bytes, cudaMemcpyDeviceToDevice, S.sf[0]);
        if (e == cudaSuccess) e = cudaEventRecord(S.written[0], S.sf[0]);
        if (e != cudaSuccess) rr = ctx_cuda_fail(c, e, "state copy");
    }
    if (!rr) rr = S.rev(0, nsteps, nslots, 0);
    cudaError_t e1 = cudaSuccess;
    for (int f = 0; f < Solver::NF; ++f)
        if (S.sf[f]) {
            cudaError_t ef = cudaStreamSynchronize(S.sf[f]);
            if (e1 == cudaSuccess) e1 = ef;
        }
    cudaError_t e3 = S.ss ? cudaStreamSynchronize(S.ss) : cudaSuccess;
    cudaError_t e2 = cudaStreamSynchronize(S.sa);
    if (e1 == cudaSuccess) e1 = e3;
    if (!rr && (e1 != cudaSuccess || e2 != cudaSuccess))
        rr = ctx_cuda_fail(c, e1 != cudaSuccess ? e1 : e2, "adjoint solve");
    double Jv = 0.0;
    if (!rr)
        for (int b = 0; b < S.nblk; ++b) Jv += S.h_partial[b];
    free_adj(S.ab);
    for (int i = 0; i < Solver::NB; ++i) {
        if (S.ready[i]) cudaEventDestroy(S.ready[i]);
        if (S.sready[i]) cudaEventDestroy(S.sready[i]);
        if (S.done[i]) cudaEventDestroy(S.done[i]);
    }
    for (auto ev : S.written)
        if (ev) cudaEventDestroy(ev);
    for (auto ev : S.read)
        if (ev) cudaEventDestroy(ev);
    if (S.h_partial) cudaFreeHost(S.h_partial);
    for (double* p : owned) cudaFree(p);
    for (int f = 0; f < Solver::NF; ++f)
        if (S.sf[f]) cudaStreamDestroy(S.sf[f]);
    if (S.ss) cudaStreamDestroy(S.ss);
    if (rr) return rr;
    if (J) *J = Jv;
    if (forward_steps) *forward_steps = S.advances;
    return ctx_check_status(c);
}

int32_t flou_adjoint_solve_batch(int32_t n, flou_ctx* const* ctxs, double* const* Q0, const double* dt,
                                 int32_t nsteps, int64_t budget_bytes, int32_t nstreams,
                                 double* const* rho_target, double* const* weights, double* J,
                                 double* const* dJdQ0, double* const* dJdc, int64_t* forward_steps,
                                 int32_t* nsnap) {
    if (n < 1 || !ctxs || !Q0 || !dt || !rho_target || !weights || !dJdQ0 || nsteps < 1) return FLOU_ERR_ARG;
    for (int i = 0; i < n; ++i)
        if (!ctxs[i]) return FLOU_ERR_ARG;
    auto fail_all = [&](int code, const std::string& msg) {
        for (int i = 0; i < n; ++i) ctxs[i]->err = msg;
        return code;
    };
    int dev0 = -1;
    if (cudaGetDevice(&dev0) != cudaSuccess) return fail_all(FLOU_ERR_CUDA, "no CUDA device");
    for (int i = 0; i < n; ++i) {
        flou_ctx* c = ctxs[i];
        int r = ctx_prepare(c);
        if (!r) r = adj_supported(c);
        if (!r && (!Q0[i] || !rho_target[i] || !weights[i] || !dJdQ0[i] || !std::isfinite(dt[i])))
            r = ctx_fail(c, FLOU_ERR_ARG, "invalid arguments");
        if (!r && dJdc && dJdc[i] && !c->d_c)
            r = ctx_fail(c, FLOU_ERR_STATE, "dJ/dc needs the per-element dissipation scale (flou_set_dissipation)");
        if (r) return fail_all(r, "instance " + std::to_string(i) + ": " + c->err);
    }
    BatchSolver B;
    B.n = n;
    B.nsteps = nsteps;
    B.c.assign(ctxs, ctxs + n);
    B.dt.assign(dt, dt + n);
    B.bytes.resize(n);
    B.off.resize(n);
    B.q0.assign(Q0, Q0 + n);
    B.A.assign(dJdQ0, dJdQ0 + n);
    B.cbar.assign(n, nullptr);
    for (int i = 0; i < n; ++i) {
        if (dJdc) B.cbar[i] = dJdc[i];
        B.rho_t.push_back(rho_target[i]);
        B.w.push_back(weights[i]);
        B.bytes[i] = (size_t)ctxs[i]->ndofs * ctxs[i]->nv * sizeof(double);
        B.off[i] = B.snap_bytes;
        B.snap_bytes += (B.bytes[i] + 255) / 256 * 256;
        B.nblk.push_back((int)((ctxs[i]->ndofs + 255) / 256));
        B.poff.push_back(i ? B.poff[i - 1] + B.nblk[i - 1] : 0);
    }
    size_t npart = B.poff[n - 1] + B.nblk[n - 1];
    // streams: largest instances first, each to the stream with the least work so far
    int S = std::max(1, std::min(nstreams > 0 ? nstreams : 8, n));
    std::vector<int> order(n);
    for (int i = 0; i < n; ++i) order[i] = i;
    std::sort(order.begin(), order.end(), [&](int a, int b) { return B.bytes[a] > B.bytes[b]; });
    std::vector<double> load(S, 0.0);
    std::vector<size_t> maxb(S, 0), maxf(S, 0), maxfd(S, 0), maxst(S, 0);
    std::vector<char> any2n(S, 0);   // a stream with a 2N-storage instance needs its own register
    std::vector<char> anyhg(S, 0);   // and one with a Gauss-node hybrid instance its face-flux buffers
    B.stream_of.assign(n, 0);
    for (int i : order) {
        int s = (int)(std::min_element(load.begin(), load.end()) - load.begin());
        B.stream_of[i] = s;
        load[s] += (double)B.bytes[i];
        maxb[s] = std::max(maxb[s], B.bytes[i]);
        maxf[s] = std::max(maxf[s], (size_t)ctxs[i]->nfdofs * ctxs[i]->nv);
        maxfd[s] = std::max(maxfd[s], (size_t)ctxs[i]->nfdofs);
        maxst[s] = std::max(maxst[s], (size_t)stage_count(ctxs[i]));
        if (ctxs[i]->lsrk_s) any2n[s] = 1;
        if (hybrid_gauss(ctxs[i])) anyhg[s] = 1;
    }
    size_t fixed = npart * sizeof(double);
    for (int s = 0; s < S; ++s)
        fixed += (3 + maxst[s] + any2n[s] + anyhg[s]) * maxb[s] + ((2 + 3 * anyhg[s]) * maxf[s] + maxfd[s]) *
                                                                   sizeof(double);
    if (budget_bytes < 0 || (size_t)budget_bytes < fixed)
        return fail_all(FLOU_ERR_ARG, "device-memory budget below the " + std::to_string(fixed) +
                                          " bytes of step scratch the batch needs");
    int nslots = (int)std::min<size_t>((size_t)std::max(nsteps - 1, 0), ((size_t)budget_bytes - fixed) / B.snap_bytes);
    std::vector<void*> owned;
    cudaError_t e = cudaSuccess;
    auto dalloc = [&](void** p, size_t b) {
        if (e != cudaSuccess) return;
        e = cudaMalloc(p, b);
        if (e == cudaSuccess) owned.push_back(*p);
    };
    B.st.assign(S, nullptr);
    for (int s = 0; s < S && e == cudaSuccess; ++s) e = cudaStreamCreateWithFlags(&B.st[s], cudaStreamNonBlocking);
    B.scr.resize(S);
    for (int s = 0; s < S; ++s) {
        BatchSolver::Scratch& w = B.scr[s];
        double** bufs[] = {&w.X, &w.T, &w.B};
        for (double** b : bufs) dalloc((void**)b, maxb[s]);
        w.SX.assign(maxst[s], nullptr);
        for (double*& b : w.SX) dalloc((void**)&b, maxb[s]);
        // SSP-RK3 steps and forms its stage states one after the other on the stream, so its
        // stepping register can be the first stage state; a 2N-storage register lives on
        if (any2n[s]) dalloc((void**)&w.K, maxb[s]);
        else w.K = w.SX[0];
        dalloc((void**)&w.ab.QbL, maxf[s] * sizeof(double));
        dalloc((void**)&w.ab.QbR, maxf[s] * sizeof(double));
        dalloc((void**)&w.ab.Ibar, std::max<size_t>(maxfd[s], 1) * sizeof(double));
        if (anyhg[s]) {
            dalloc((void**)&w.ab.Fn, maxf[s] * sizeof(double));
            dalloc((void**)&w.ab.FbS, 2 * maxf[s] * sizeof(double));
            dalloc((void**)&w.ab.Tq, maxb[s]);
        }
    }
    dalloc((void**)&B.partial, npart * sizeof(double));
    B.slot.assign(nslots + 1, nullptr);
    for (int j = 1; j <= nslots; ++j) dalloc((void**)&B.slot[j], B.snap_bytes);
    if (e == cudaSuccess) e = cudaMallocHost((void**)&B.h_partial, npart * sizeof(double));
    int rr = FLOU_OK;
    if (e != cudaSuccess) rr = fail_all(FLOU_ERR_OOM, std::string("batched adjoint storage: ") + cudaGetErrorString(e));
    for (int i = 0; i < n && !rr; ++i)
        if (B.cbar[i]) {
            e = cudaMemsetAsync(B.cbar[i], 0, ctxs[i]->nelem * sizeof(double), B.S(i));
            if (e != cudaSuccess) rr = fail_all(FLOU_ERR_CUDA, "cbar reset");
        }
    // the callers' inputs may still be in flight on the contexts' own streams
    for (int i = 0; i < n && !rr; ++i)
        if (cudaStreamSynchronize(ctxs[i]->stream) != cudaSuccess) rr = fail_all(FLOU_ERR_CUDA, "stream synchronize");
    Schedule sch(nsteps, nslots);
    B.sch = &sch;
    B.seeded.assign(n, 0);
    for (int j = 1; j <= nslots; ++j) B.free_slots.push_back(j);
    if (!rr) {
        rr = B.rev(0, nsteps, nslots, 0);
        if (rr && B.failed >= 0) fail_all(rr, "instance " + std::to_string(B.failed) + ": " + ctxs[B.failed]->err);
    }
    for (int s = 0; s < S; ++s)
        if (B.st[s]) {
            cudaError_t es = cudaStreamSynchronize(B.st[s]);
            if (es != cudaSuccess && !rr) rr = fail_all(FLOU_ERR_CUDA, std::string("batched adjoint: ") + cudaGetErrorString(es));
        }
    if (!rr) {
        for (int i = 0; i < n; ++i) {
            double j = 0.0;
            for (int b = 0; b < B.nblk[i]; ++b) j += B.h_partial[B.poff[i] + b];
            if (J) J[i] = j;
        }
        if (forward_steps) *forward_steps = B.advances;
        if (nsnap) *nsnap = nslots;
        for (int i = 0; i < n && !rr; ++i) {
            int r = ctx_check_status(ctxs[i]);
            if (r) rr = fail_all(r, "instance " + std::to_string(i) + ": " + ctxs[i]->err);
        }
    }
    if (B.h_partial) cudaFreeHost(B.h_partial);
    for (void* p : owned) cudaFree(p);
    for (cudaStream_t s : B.st)
        if (s) cudaStreamDestroy(s);
    return rr;
}

}  // extern "C"
