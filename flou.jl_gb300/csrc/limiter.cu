// limiter.cu -- the Zhang-Shu positivity limiter and the integral monitors of the Euler
// equations (src/FlouSpatial/Equations/Euler.jl:541-654), as the stage limiter and the monitor
// callbacks of Flou's time integration (src/FlouTime/FlouTime.jl:107-148).
//
// Limiter: one warp per element.  A division-free test first skips elements whose density and
// pressure are above the minimum everywhere (the reference changes nothing there); otherwise
// pass 1 forms the element mean Q̄ = Σ Jω Q / Σ Jω and the minimum density, pass 2 the mean and
// minimum of the pressure of the density-limited nodes, pass 3 writes the limited element.  The warp reductions are
// butterfly shuffles: IEEE addition is commutative, so every lane ends with the same bits and
// the result does not depend on scheduling.  Run after every stage inside the step graph, the
// pass reads the state once more; FP64 is the limit on GB300, hence the division-free test.
//
// Monitors: per-block partial sums of Jω f(Q) (f = kinetic energy or mathematical entropy) in a
// fixed reduction order, then one block sums the partials in a fixed order and appends the
// values to a device buffer, so monitors can be recorded after every step of a graph replay
// without a host round trip.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <vector>

#include "flou_ctx.cuh"

namespace flou {

struct LimParams {
    double* Q;
    const double* J;   // per element
    const double* Jn;  // per node (general geometry) or null
    const double* w;   // tensor quadrature weights [npe]
    int64_t ndofs;
    int nelem, npe;
    double minval, gamma;
    const double* gate;   // CFL stepping: *gate == 0 once the run is over (skip)
};

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ double warp_min(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

template <int DIM>
__device__ __forceinline__ double node_pressure(double r, const double* Q, int64_t ndofs, int64_t g, double g1) {
    double ke = 0.0;
#pragma unroll
    for (int k = 0; k < DIM; ++k) {
        double m = Q[(1 + k) * ndofs + g];
        ke = fma(m, m, ke);
    }
    return g1 * (Q[(DIM + 1) * ndofs + g] - ke / (2.0 * r));
}

template <int DIM>
__global__ void __launch_bounds__(256) zhang_shu_kernel(LimParams P) {
    constexpr int NV = DIM + 2;
    const int lane = threadIdx.x & 31;
    const int warp = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5);
    const int nwarps = (int)((gridDim.x * (int64_t)blockDim.x) >> 5);
    const double g1 = P.gamma - 1.0;
    if (P.gate && *P.gate == 0.0) return;
    for (int e = warp; e < P.nelem; e += nwarps) {
        const double Je = P.J[e];
        const int64_t b = (int64_t)e * P.npe;
        // Fast exit.  With m = min(minval, mean), θ > 1 (no change) exactly when the minimum is
        // above minval: density when ρ_min > minval, pressure when p_min > minval, i.e. when
        // 2ρ((γ-1)E - minval) > (γ-1)|ρv|² at every node (no division).  Elements that clear
        // both tests by a relative margin of 1e-12 are left alone; the others take the full
        // computation below, as the reference writes it.
        bool clear = true;
        for (int i = lane; i < P.npe; i += 32) {
            double r = P.Q[b + i];
            double ke = 0.0;
#pragma unroll
            for (int k = 0; k < DIM; ++k) {
                double mk = P.Q[(1 + k) * P.ndofs + b + i];
                ke = fma(mk, mk, ke);
            }
            double E = P.Q[(DIM + 1) * P.ndofs + b + i];
            double lhs = 2.0 * r * fma(g1, E, -P.minval), rhs = g1 * ke;
            double tol = 1e-12 * (fabs(2.0 * r * g1 * E) + fabs(2.0 * r * P.minval) + rhs);
            clear = clear && r > 0.0 && (r - P.minval > 1e-12 * fabs(P.minval) + 1e-300) && (lhs - rhs > tol);
        }
        if (__all_sync(0xffffffffu, clear)) continue;
        double S[NV], vol = 0.0, rmin = INFINITY;
#pragma unroll
        for (int k = 0; k < NV; ++k) S[k] = 0.0;
        for (int i = lane; i < P.npe; i += 32) {
            double jw = (P.Jn ? P.Jn[b + i] : Je) * P.w[i];
            vol += jw;
#pragma unroll
            for (int k = 0; k < NV; ++k) S[k] = fma(jw, P.Q[k * P.ndofs + b + i], S[k]);
            rmin = fmin(rmin, P.Q[b + i]);
        }
        vol = warp_sum(vol);
        rmin = warp_min(rmin);
        double Qm[NV];
#pragma unroll
        for (int k = 0; k < NV; ++k) Qm[k] = warp_sum(S[k]) / vol;
        // density (Euler.jl:628-637)
        double m = fmin(P.minval, Qm[0]);
        double th1 = fabs((Qm[0] - m) / (Qm[0] - rmin));
        bool l1 = th1 <= 1.0;
        // pressure of the density-limited nodes (Euler.jl:639-652)
        double ps = 0.0, pmin = INFINITY;
        for (int i = lane; i < P.npe; i += 32) {
            double r = P.Q[b + i];
            if (l1) r = th1 * (r - Qm[0]) + Qm[0];
            double p = node_pressure<DIM>(r, P.Q, P.ndofs, b + i, g1);
            ps = fma((P.Jn ? P.Jn[b + i] : Je) * P.w[i], p, ps);
            pmin = fmin(pmin, p);
        }
        double pbar = warp_sum(ps) / vol;
        pmin = warp_min(pmin);
        double m2 = fmin(P.minval, pbar);
        double th2 = fabs((pbar - m2) / (pbar - pmin));
        bool l2 = th2 <= 1.0;
        if (!l1 && !l2) continue;
        for (int i = lane; i < P.npe; i += 32) {
            double q[NV];
#pragma unroll
            for (int k = 0; k < NV; ++k) q[k] = P.Q[k * P.ndofs + b + i];
            if (l1) q[0] = th1 * (q[0] - Qm[0]) + Qm[0];
            if (l2) {
#pragma unroll
                for (int k = 0; k < NV; ++k) q[k] = th2 * (q[k] - Qm[k]) + Qm[k];
            }
#pragma unroll
            for (int k = 0; k < NV; ++k) P.Q[k * P.ndofs + b + i] = q[k];
        }
    }
}

// Partial sums over blocks of nodes of Jω f(Q): [0] kinetic energy |ρv|²/(2ρ) (FlouCommon/Euler.jl:162-175),
// [1] mathematical entropy -ρ s/(γ-1), s = log p - γ log ρ (FlouCommon/Euler.jl:202-217).
// The limiter's VJP (reverse mode through zhang_shu_kernel, for the discrete adjoint of a limited
// time step), one warp per element.  V is the state before the limiter; A holds the cotangent of
// the limited state on entry and that of V on exit.  The forward quantities are recomputed from V:
// the mean Q̄, the first minimal density node, θ₁ = |N₁/D₁| (N₁ = ρ̄ - min(minval, ρ̄), D₁ = ρ̄ -
// ρ_min), the pressures of the density-limited nodes, their mean and first minimal node, θ₂.  In
// reverse: Q'' = Q̄ + θ₂ (Q' - Q̄) gives Q̄' = θ₂ Ā, Q̄̄ += (1-θ₂) Σ Ā and θ̄₂ = Σ Ā·(Q' - Q̄); θ₂'s
// derivative (sign-bit convention for |·|) reaches p̄ and p_min when m = minval (when m = p̄ the
// numerator is identically zero); the pressures take their cotangents to (ρ', m, E); the density
// step is reversed the same way, and the mean's cotangent spreads back with Jω/vol.  Elements the
// limiter leaves alone (the forward's fast exit, or neither θ ≤ 1) pass A through.  With K set,
// K = kK K + kb A after A is formed (the 2N-storage register of the reverse sweep), every node.
struct LimVjpParams {
    const double* V;
    double* A;
    double* K;
    double kK, kb;
    const double* J;
    const double* Jn;
    const double* w;
    int64_t ndofs;
    int nelem, npe;
    double minval, gamma;
};

__device__ __forceinline__ void warp_argmin(double& v, int& idx) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const double ov = __shfl_xor_sync(0xffffffffu, v, o);
        const int oi = __shfl_xor_sync(0xffffffffu, idx, o);
        if (ov < v || (ov == v && oi < idx)) {
            v = ov;
            idx = oi;
        }
    }
}

template <int DIM>
__global__ void __launch_bounds__(256) zhang_shu_vjp_kernel(LimVjpParams P) {
    constexpr int NV = DIM + 2;
    const int lane = threadIdx.x & 31;
    const int warp = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5);
    const int nwarps = (int)((gridDim.x * (int64_t)blockDim.x) >> 5);
    const double g1 = P.gamma - 1.0;
    auto sgn = [](double x) { return signbit(x) ? -1.0 : 1.0; };
    for (int e = warp; e < P.nelem; e += nwarps) {
        const double Je = P.J[e];
        const int64_t b = (int64_t)e * P.npe;
        bool clear = true;   // the forward's fast exit, on the same state
        for (int i = lane; i < P.npe; i += 32) {
            double r = P.V[b + i];
            double ke = 0.0;
#pragma unroll
            for (int k = 0; k < DIM; ++k) {
                double mk = P.V[(1 + k) * P.ndofs + b + i];
                ke = fma(mk, mk, ke);
            }
            double E = P.V[(DIM + 1) * P.ndofs + b + i];
            double lhs = 2.0 * r * fma(g1, E, -P.minval), rhs = g1 * ke;
            double tol = 1e-12 * (fabs(2.0 * r * g1 * E) + fabs(2.0 * r * P.minval) + rhs);
            clear = clear && r > 0.0 && (r - P.minval > 1e-12 * fabs(P.minval) + 1e-300) && (lhs - rhs > tol);
        }
        bool pass = __all_sync(0xffffffffu, clear);
        double S[NV], vol = 0.0, rmin = INFINITY, Qm[NV];
        int i1 = P.npe, j2 = P.npe;
        double th1 = 2.0, th2 = 2.0, r1 = 0.0, r2 = 0.0, N1 = 0.0, D1 = 1.0, N2 = 0.0, D2 = 1.0;
        bool l1 = false, l2 = false, mmean1 = false, mmean2 = false;
        if (!pass) {
#pragma unroll
            for (int k = 0; k < NV; ++k) S[k] = 0.0;
            for (int i = lane; i < P.npe; i += 32) {
                double jw = (P.Jn ? P.Jn[b + i] : Je) * P.w[i];
                vol += jw;
#pragma unroll
                for (int k = 0; k < NV; ++k) S[k] = fma(jw, P.V[k * P.ndofs + b + i], S[k]);
                if (P.V[b + i] < rmin) {
                    rmin = P.V[b + i];
                    i1 = i;
                }
            }
            vol = warp_sum(vol);
            warp_argmin(rmin, i1);
#pragma unroll
            for (int k = 0; k < NV; ++k) Qm[k] = warp_sum(S[k]) / vol;
            const double m = fmin(P.minval, Qm[0]);
            mmean1 = Qm[0] < P.minval;
            N1 = Qm[0] - m;
            D1 = Qm[0] - rmin;
            r1 = N1 / D1;
            th1 = fabs(r1);
            l1 = th1 <= 1.0;
            double ps = 0.0, pmin = INFINITY;
            for (int i = lane; i < P.npe; i += 32) {
                double r = P.V[b + i];
                if (l1) r = th1 * (r - Qm[0]) + Qm[0];
                double p = node_pressure<DIM>(r, P.V, P.ndofs, b + i, g1);
                ps = fma((P.Jn ? P.Jn[b + i] : Je) * P.w[i], p, ps);
                if (p < pmin) {
                    pmin = p;
                    j2 = i;
                }
            }
            const double pbar = warp_sum(ps) / vol;
            warp_argmin(pmin, j2);
            const double m2 = fmin(P.minval, pbar);
            mmean2 = pbar < P.minval;
            N2 = pbar - m2;
            D2 = pbar - pmin;
            r2 = N2 / D2;
            th2 = fabs(r2);
            l2 = th2 <= 1.0;
            pass = !l1 && !l2;
        }
        if (pass) {
            if (P.K)
                for (int i = lane; i < P.npe; i += 32)
#pragma unroll
                    for (int k = 0; k < NV; ++k) {
                        const int64_t o = k * P.ndofs + b + i;
                        P.K[o] = fma(P.kK, P.K[o], P.kb * P.A[o]);
                    }
            continue;
        }
        // pressure step: the sums of Ā and Ā·(Q' - Q̄)
        double sA[NV], t2 = 0.0;
#pragma unroll
        for (int k = 0; k < NV; ++k) sA[k] = 0.0;
        if (l2) {
            for (int i = lane; i < P.npe; i += 32) {
#pragma unroll
                for (int k = 0; k < NV; ++k) {
                    double q = P.V[k * P.ndofs + b + i];
                    if (k == 0 && l1) q = th1 * (q - Qm[0]) + Qm[0];
                    const double a = P.A[k * P.ndofs + b + i];
                    sA[k] += a;
                    t2 = fma(a, q - Qm[k], t2);
                }
            }
#pragma unroll
            for (int k = 0; k < NV; ++k) sA[k] = warp_sum(sA[k]);
            t2 = warp_sum(t2);
        }
        const double rb2 = l2 ? t2 * sgn(r2) : 0.0;
        const double pbb = (l2 && !mmean2) ? rb2 * (1.0 / D2 - N2 / (D2 * D2)) : 0.0;
        const double pmb = (l2 && !mmean2) ? rb2 * N2 / (D2 * D2) : 0.0;
        double Qmb[NV];
#pragma unroll
        for (int k = 0; k < NV; ++k) Qmb[k] = l2 ? (1.0 - th2) * sA[k] : 0.0;
        // Q̄' (with the pressures' cotangents), then the density step
        double sR = 0.0, t1 = 0.0;
        for (int i = lane; i < P.npe; i += 32) {
            double qb[NV], q[NV];
#pragma unroll
            for (int k = 0; k < NV; ++k) {
                q[k] = P.V[k * P.ndofs + b + i];
                const double a = P.A[k * P.ndofs + b + i];
                qb[k] = l2 ? th2 * a : a;
            }
            const double rho0 = q[0];
            const double rp = l1 ? th1 * (q[0] - Qm[0]) + Qm[0] : q[0];
            const double jw = (P.Jn ? P.Jn[b + i] : Je) * P.w[i];
            const double pb = pbb * jw / vol + (i == j2 ? pmb : 0.0);
            if (pb != 0.0) {   // p = (γ-1)(E - |m|²/(2ρ'))
                double ke = 0.0;
#pragma unroll
                for (int k = 0; k < DIM; ++k) ke = fma(q[1 + k], q[1 + k], ke);
                const double ir = 1.0 / rp;
                qb[0] = fma(pb * g1 * 0.5 * ke, ir * ir, qb[0]);
#pragma unroll
                for (int k = 0; k < DIM; ++k) qb[1 + k] = fma(-pb * g1 * ir, q[1 + k], qb[1 + k]);
                qb[DIM + 1] = fma(pb, g1, qb[DIM + 1]);
            }
            if (l1) {
                sR += qb[0];
                t1 = fma(qb[0], rho0 - Qm[0], t1);
                qb[0] *= th1;
            }
#pragma unroll
            for (int k = 0; k < NV; ++k) P.A[k * P.ndofs + b + i] = qb[k];
        }
        double rminb = 0.0;
        if (l1) {
            sR = warp_sum(sR);
            t1 = warp_sum(t1);
            const double rb1 = t1 * sgn(r1);
            Qmb[0] = fma(1.0 - th1, sR, Qmb[0]);
            if (!mmean1) {
                Qmb[0] = fma(rb1, 1.0 / D1 - N1 / (D1 * D1), Qmb[0]);
                rminb = rb1 * N1 / (D1 * D1);
            }
        }
        for (int i = lane; i < P.npe; i += 32) {   // the mean's cotangent, the minimal node's
            const double sj = (P.Jn ? P.Jn[b + i] : Je) * P.w[i] / vol;
#pragma unroll
            for (int k = 0; k < NV; ++k) {
                const int64_t o = k * P.ndofs + b + i;
                double a = fma(Qmb[k], sj, P.A[o]);
                if (k == 0 && i == i1) a += rminb;
                P.A[o] = a;
                if (P.K) P.K[o] = fma(P.kK, P.K[o], P.kb * a);
            }
        }
    }
}


template <int DIM>
__global__ void __launch_bounds__(256) monitor_partial_kernel(const double* Q, const double* J, const double* Jn,
                                                              const double* w, int64_t ndofs, int npe, double gamma,
                                                              int mask, double* partial) {
    int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    double ke = 0.0, ent = 0.0;
    if (g < ndofs) {
        int64_t e = g / npe;
        double jw = (Jn ? Jn[g] : J[e]) * w[g - e * npe];
        double r = Q[g];
        double m2 = 0.0;
#pragma unroll
        for (int k = 0; k < DIM; ++k) {
            double m = Q[(1 + k) * ndofs + g];
            m2 = fma(m, m, m2);
        }
        if (mask & 1) ke = jw * (m2 / (2.0 * r));
        if (mask & 2) {
            double p = (gamma - 1.0) * (Q[(DIM + 1) * ndofs + g] - m2 / (2.0 * r));
            double s = log(p) - gamma * log(r);
            ent = jw * (-r * s / (gamma - 1.0));
        }
    }
    __shared__ double sm[2][8];
    ke = warp_sum(ke);
    ent = warp_sum(ent);
    int wid = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
        sm[0][wid] = ke;
        sm[1][wid] = ent;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0.0, c = 0.0;
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) {
            a += sm[0][k];
            c += sm[1][k];
        }
        partial[blockIdx.x] = a;
        partial[gridDim.x + blockIdx.x] = c;
    }
}

// One block: fixed-order sums of the partials, appended at slot *count (if below cap).
// `times` (cap entries behind the values) receives *tdev, the device time after the step (CFL
// stepping), or NaN when the time is known on the host.
__global__ void __launch_bounds__(256) monitor_final_kernel(const double* partial, int nblk, double* out,
                                                            int32_t* count, int cap, const double* gate,
                                                            double* times, const double* tdev) {
    if (gate && *gate == 0.0) return;   // CFL stepping past tfinal: no step, no record
    double a = 0.0, c = 0.0;
    for (int i = threadIdx.x; i < nblk; i += blockDim.x) {
        a += partial[i];
        c += partial[nblk + i];
    }
    __shared__ double sm[2][8];
    a = warp_sum(a);
    c = warp_sum(c);
    int wid = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
        sm[0][wid] = a;
        sm[1][wid] = c;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double x = 0.0, y = 0.0;
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) {
            x += sm[0][k];
            y += sm[1][k];
        }
        int slot = *count;
        if (slot < cap) {
            out[2 * slot] = x;
            out[2 * slot + 1] = y;
            if (times) times[slot] = tdev ? *tdev : __longlong_as_double(0x7ff8000000000000LL);
        }
        *count = slot + 1;
    }
}

namespace {

int lfail(flou_ctx* c, int code, const char* fmt, ...) {
    char buf[256];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    c->err = buf;
    return code;
}

int lcuda(flou_ctx* c, cudaError_t e, const char* what) {
    return e == cudaSuccess ? FLOU_OK : lfail(c, FLOU_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

// Tensor-product quadrature weights per element node, x fastest: ω_z (ω_y ω_x).
int ensure_weights(flou_ctx* c) {
    if (c->d_wtp) return FLOU_OK;
    int n = c->n, d = c->cfg.dim;
    std::vector<double> w(c->npe);
    for (int i = 0; i < c->npe; ++i) {
        int x = i % n, y = (i / n) % n, z = i / (n * n);
        double v = c->omega[x];
        if (d > 1) v = c->omega[y] * v;
        if (d > 2) v = c->omega[z] * v;
        w[i] = v;
    }
    int r = lcuda(c, cudaMalloc((void**)&c->d_wtp, w.size() * sizeof(double)), "quadrature weights");
    if (r) return r;
    return lcuda(c, cudaMemcpy(c->d_wtp, w.data(), w.size() * sizeof(double), cudaMemcpyHostToDevice),
                 "quadrature weights");
}

int monitor_blocks(const flou_ctx* c) { return (int)((c->ndofs + 255) / 256); }

int ensure_monitor_buffers(flou_ctx* c) {
    int r = ensure_weights(c);
    if (r) return r;
    if (!c->d_monpart) {
        r = lcuda(c, cudaMalloc((void**)&c->d_monpart, 2 * (size_t)monitor_blocks(c) * sizeof(double)),
                  "monitor buffers");
        if (r) return r;
    }
    if (!c->d_monval) {
        r = lcuda(c, cudaMalloc((void**)&c->d_monval, 2 * sizeof(double)), "monitor buffers");
        if (r) return r;
    }
    if (!c->d_moncount) {
        r = lcuda(c, cudaMalloc((void**)&c->d_moncount, 2 * sizeof(int32_t)), "monitor buffers");
        if (!r) r = lcuda(c, cudaMemset(c->d_moncount, 0, 2 * sizeof(int32_t)), "monitor buffers");
        if (r) return r;
    }
    return FLOU_OK;
}

int launch_monitors(flou_ctx* c, cudaStream_t s, const double* Q, int mask, double* out, int32_t* count, int cap) {
    int nb = monitor_blocks(c);
    int d = c->cfg.dim;
    const double* Jn = c->curv ? c->d_Jn : nullptr;
    if (d == 1) monitor_partial_kernel<1><<<nb, 256, 0, s>>>(Q, c->d_Jel, Jn, c->d_wtp, c->ndofs, c->npe, c->cfg.gamma, mask, c->d_monpart);
    else if (d == 2) monitor_partial_kernel<2><<<nb, 256, 0, s>>>(Q, c->d_Jel, Jn, c->d_wtp, c->ndofs, c->npe, c->cfg.gamma, mask, c->d_monpart);
    else monitor_partial_kernel<3><<<nb, 256, 0, s>>>(Q, c->d_Jel, Jn, c->d_wtp, c->ndofs, c->npe, c->cfg.gamma, mask, c->d_monpart);
    bool rec = count == c->d_moncount;   // the per-step record (not a single evaluation)
    monitor_final_kernel<<<1, 256, 0, s>>>(c->d_monpart, nb, out, count, cap, rec ? c->d_gate : nullptr,
                                           rec ? out + 2 * (size_t)cap : nullptr,
                                           rec && c->d_gate ? c->d_gate - 1 : nullptr);
    return lcuda(c, cudaGetLastError(), "monitor kernels");
}

bool ready_for(flou_ctx* c, const char* what) {
    if (!c->have_geom || !c->have_ops) {
        lfail(c, FLOU_ERR_STATE, "%s needs the operators and the geometry", what);
        return false;
    }
    if (c->cfg.equation != FLOU_EQ_EULER) {
        lfail(c, FLOU_ERR_UNSUPPORTED, "%s applies to the Euler equations", what);
        return false;
    }
    return true;
}

}  // namespace

int ctx_limit(flou_ctx* c, cudaStream_t s, double* Q) {
    if (c->limiter != FLOU_LIMITER_ZHANG_SHU) return FLOU_OK;
    LimParams P;
    P.Q = Q;
    P.J = c->d_Jel;
    P.Jn = c->curv ? c->d_Jn : nullptr;
    P.w = c->d_wtp;
    P.ndofs = c->ndofs;
    P.nelem = c->nelem;
    P.npe = c->npe;
    P.minval = c->lim_min;
    P.gamma = c->cfg.gamma;
    P.gate = c->d_gate;
    int grid = (c->nelem + 7) / 8;   // 8 warps per block, one element per warp
    int d = c->cfg.dim;
    if (d == 1) zhang_shu_kernel<1><<<grid, 256, 0, s>>>(P);
    else if (d == 2) zhang_shu_kernel<2><<<grid, 256, 0, s>>>(P);
    else zhang_shu_kernel<3><<<grid, 256, 0, s>>>(P);
    return lcuda(c, cudaGetLastError(), "limiter kernel");
}

int ctx_limit_vjp(flou_ctx* c, cudaStream_t s, const double* V, double* A, double* K, double kK, double kb) {
    LimVjpParams P;
    P.V = V;
    P.A = A;
    P.K = K;
    P.kK = kK;
    P.kb = kb;
    P.J = c->d_Jel;
    P.Jn = c->curv ? c->d_Jn : nullptr;
    P.w = c->d_wtp;
    P.ndofs = c->ndofs;
    P.nelem = c->nelem;
    P.npe = c->npe;
    P.minval = c->lim_min;
    P.gamma = c->cfg.gamma;
    int grid = (c->nelem + 7) / 8;
    int d = c->cfg.dim;
    if (d == 1) zhang_shu_vjp_kernel<1><<<grid, 256, 0, s>>>(P);
    else if (d == 2) zhang_shu_vjp_kernel<2><<<grid, 256, 0, s>>>(P);
    else zhang_shu_vjp_kernel<3><<<grid, 256, 0, s>>>(P);
    return lcuda(c, cudaGetLastError(), "limiter VJP kernel");
}

int ctx_record_monitors(flou_ctx* c, cudaStream_t s, const double* Q) {
    if (!c->mon_mask) return FLOU_OK;
    return launch_monitors(c, s, Q, c->mon_mask, c->d_mon, c->d_moncount, c->mon_cap);
}

void ctx_free_limiter(flou_ctx* c) {
    void* bufs[] = {c->d_Jel, c->d_wtp, c->d_mon, c->d_moncount, c->d_monpart, c->d_monval};
    for (void* b : bufs)
        if (b) cudaFree(b);
    c->d_Jel = c->d_wtp = c->d_mon = c->d_monpart = c->d_monval = nullptr;
    c->d_moncount = nullptr;
}

}  // namespace flou

using namespace flou;

extern "C" {

int32_t flou_set_limiter(flou_ctx* c, int32_t kind, double minval) {
    if (!c) return FLOU_ERR_ARG;
    if (kind == FLOU_LIMITER_NONE) {
        c->limiter = kind;
        drop_step_graph(c);
        return FLOU_OK;
    }
    if (kind != FLOU_LIMITER_ZHANG_SHU) return lfail(c, FLOU_ERR_ARG, "unknown limiter %d", kind);
    if (!ready_for(c, "the Zhang-Shu limiter")) return (int)(c->cfg.equation != FLOU_EQ_EULER ? FLOU_ERR_UNSUPPORTED : FLOU_ERR_STATE);
    if (!std::isfinite(minval)) return lfail(c, FLOU_ERR_ARG, "the limiter's minimum value must be finite");
    int r = ensure_weights(c);
    if (r) return r;
    c->limiter = kind;
    c->lim_min = minval;
    drop_step_graph(c);
    return FLOU_OK;
}

int32_t flou_limit(flou_ctx* c, double* Q, int32_t ptr_kind) {
    if (!c) return FLOU_ERR_ARG;
    if (c->limiter != FLOU_LIMITER_ZHANG_SHU) return lfail(c, FLOU_ERR_STATE, "no limiter is set (flou_set_limiter)");
    if (!Q) return lfail(c, FLOU_ERR_ARG, "null state pointer");
    size_t bytes = (size_t)c->ndofs * c->nv * sizeof(double);
    double* Qd = Q;
    int r;
    if (ptr_kind == FLOU_PTR_HOST) {
        if (!c->d_Qh && (r = lcuda(c, cudaMalloc((void**)&c->d_Qh, bytes), "staging buffer"))) return r;
        if ((r = lcuda(c, cudaMemcpyAsync(c->d_Qh, Q, bytes, cudaMemcpyHostToDevice, c->stream), "state upload")))
            return r;
        Qd = c->d_Qh;
    } else if (ptr_kind != FLOU_PTR_DEVICE) {
        return lfail(c, FLOU_ERR_ARG, "unknown pointer kind %d", ptr_kind);
    }
    if ((r = ctx_limit(c, c->stream, Qd))) return r;
    if (ptr_kind == FLOU_PTR_HOST &&
        (r = lcuda(c, cudaMemcpyAsync(Q, c->d_Qh, bytes, cudaMemcpyDeviceToHost, c->stream), "state download")))
        return r;
    return lcuda(c, cudaStreamSynchronize(c->stream), "limiter");
}

int32_t flou_monitor(flou_ctx* c, const double* Q, int32_t which, double* value, int32_t ptr_kind) {
    if (!c) return FLOU_ERR_ARG;
    if (!Q || !value) return lfail(c, FLOU_ERR_ARG, "null pointer");
    if (which != FLOU_MONITOR_KINETIC_ENERGY && which != FLOU_MONITOR_ENTROPY)
        return lfail(c, FLOU_ERR_ARG, "unknown monitor %d", which);
    if (!ready_for(c, "the monitors")) return (int)(c->cfg.equation != FLOU_EQ_EULER ? FLOU_ERR_UNSUPPORTED : FLOU_ERR_STATE);
    int r = ensure_monitor_buffers(c);
    if (r) return r;
    size_t bytes = (size_t)c->ndofs * c->nv * sizeof(double);
    const double* Qd = Q;
    if (ptr_kind == FLOU_PTR_HOST) {
        if (!c->d_Qh && (r = lcuda(c, cudaMalloc((void**)&c->d_Qh, bytes), "staging buffer"))) return r;
        if ((r = lcuda(c, cudaMemcpyAsync(c->d_Qh, Q, bytes, cudaMemcpyHostToDevice, c->stream), "state upload")))
            return r;
        Qd = c->d_Qh;
    } else if (ptr_kind != FLOU_PTR_DEVICE) {
        return lfail(c, FLOU_ERR_ARG, "unknown pointer kind %d", ptr_kind);
    }
    if ((r = lcuda(c, cudaMemsetAsync(c->d_moncount + 1, 0, sizeof(int32_t), c->stream), "monitor"))) return r;
    if ((r = launch_monitors(c, c->stream, Qd, which, c->d_monval, c->d_moncount + 1, 1))) return r;
    double v[2];
    if ((r = lcuda(c, cudaMemcpyAsync(v, c->d_monval, sizeof(v), cudaMemcpyDeviceToHost, c->stream), "monitor read")))
        return r;
    if ((r = lcuda(c, cudaStreamSynchronize(c->stream), "monitor"))) return r;
    *value = which == FLOU_MONITOR_KINETIC_ENERGY ? v[0] : v[1];
    return FLOU_OK;
}

int32_t flou_set_monitors(flou_ctx* c, int32_t mask, int32_t capacity) {
    if (!c) return FLOU_ERR_ARG;
    if (mask & ~3) return lfail(c, FLOU_ERR_ARG, "unknown monitor bits 0x%x", mask);
    if (mask && capacity < 1) return lfail(c, FLOU_ERR_ARG, "monitor capacity must be positive");
    if (mask) {
        if (!ready_for(c, "the monitors")) return (int)(c->cfg.equation != FLOU_EQ_EULER ? FLOU_ERR_UNSUPPORTED : FLOU_ERR_STATE);
        int r = ensure_monitor_buffers(c);
        if (r) return r;
        if (capacity != c->mon_cap) {
            if (c->d_mon) cudaFree(c->d_mon);
            c->d_mon = nullptr;
            c->mon_cap = 0;
            if ((r = lcuda(c, cudaMalloc((void**)&c->d_mon, 3 * (size_t)capacity * sizeof(double)), "monitor buffer")))
                return r;
            c->mon_cap = capacity;
        }
        if ((r = lcuda(c, cudaMemset(c->d_moncount, 0, sizeof(int32_t)), "monitor buffer"))) return r;
    }
    c->mon_mask = mask;
    drop_step_graph(c);
    return FLOU_OK;
}

int32_t flou_take_monitors(flou_ctx* c, double* out, int32_t max_steps, int32_t* nsteps) {
    return flou_take_monitors_timed(c, out, nullptr, max_steps, nsteps);
}

int32_t flou_take_monitors_timed(flou_ctx* c, double* out, double* times, int32_t max_steps, int32_t* nsteps) {
    if (!c) return FLOU_ERR_ARG;
    if (!nsteps) return lfail(c, FLOU_ERR_ARG, "null pointer");
    *nsteps = 0;
    if (!c->mon_mask || !c->d_moncount) return FLOU_OK;
    int32_t n = 0;
    int r;
    if ((r = lcuda(c, cudaStreamSynchronize(c->stream), "monitor read"))) return r;
    if ((r = lcuda(c, cudaMemcpy(&n, c->d_moncount, sizeof(n), cudaMemcpyDeviceToHost), "monitor read"))) return r;
    if (n > c->mon_cap) return lfail(c, FLOU_ERR_STATE, "%d steps recorded, capacity %d: values were lost", n, c->mon_cap);
    if (n > max_steps) return lfail(c, FLOU_ERR_ARG, "%d steps recorded, the output holds %d", n, max_steps);
    if (n && out && (r = lcuda(c, cudaMemcpy(out, c->d_mon, 2 * (size_t)n * sizeof(double), cudaMemcpyDeviceToHost),
                                "monitor read")))
        return r;
    if (n && times && (r = lcuda(c, cudaMemcpy(times, c->d_mon + 2 * (size_t)c->mon_cap, (size_t)n * sizeof(double),
                                              cudaMemcpyDeviceToHost), "monitor read")))
        return r;
    if ((r = lcuda(c, cudaMemset(c->d_moncount, 0, sizeof(int32_t)), "monitor reset"))) return r;
    *nsteps = n;
    return FLOU_OK;
}

}  // extern "C"
