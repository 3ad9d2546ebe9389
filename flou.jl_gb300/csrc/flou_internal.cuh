// flou_internal.cuh -- device-side building blocks of libflou_cuda.
//
// Data layout in HBM (kept identical to Flou's containers so a Julia caller passes its
// arrays as is):
//   state     Q[v * ndofs + e * n^d + i]        SoA, one contiguous column per variable,
//                                                element-contiguous, node i = x fastest
//   face flux Fn[v * nfacedofs + f * n^(d-1) + m] the master-side flux times the surface
//                                                Jacobian; the slave side reads -Fn
// Per-element Cartesian geometry is compressed on the host into 1/J and the diagonal of
// the metric Ja (PhysicalRegions.jl:370-408), per-face geometry into the surface Jacobian
// and the master's local face position (which fixes the frame, PhysicalRegions.jl:541-696).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "flou_cuda.h"

namespace flou {

constexpr int MAXN = 8;          // nodes per direction supported by the kernels
constexpr int MAXBC = 8;         // boundary conditions per context

__host__ __device__ constexpr int ipow(int b, int e) { return e == 0 ? 1 : b * ipow(b, e - 1); }

// Threads per block of the one-thread-per-face-node kernels: 256, halved (down to 32) while the
// grid would give fewer than 8 blocks per SM.  On small meshes (tens of thousands of face nodes)
// 256-thread blocks leave most SMs with one block and a few with two, and the kernel lasts two
// block times; smaller blocks spread the same work evenly.  The SM count is queried once per
// device (host code; no stream operation, so it is safe during stream capture after the first call).
inline int face_block_size(int64_t nthreads) {
    static int sms_of[64] = {0};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) dev = 0;
    int sms = __atomic_load_n(&sms_of[dev], __ATOMIC_RELAXED);
    if (sms <= 0) {
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0) sms = 152;
        __atomic_store_n(&sms_of[dev], sms, __ATOMIC_RELAXED);
    }
    int tb = 256;
    while (tb > 32 && nthreads < (int64_t)8 * sms * tb) tb >>= 1;
    return tb;
}

// ---------------------------------------------------------------------------------------
// Launch parameters (passed by value)
// ---------------------------------------------------------------------------------------
struct FaceParams {
    const double* Q;
    double* Fn;
    const int32_t* face_elem;    // nfaces x 2: (elem << 3) | local face position (0-based), -1 = boundary
    const double* faceJ;         // nfaces
    const int8_t* face_bc;       // nfaces: boundary index (0-based) or -1
    const double* l;             // l_l[n], l_r[n]
    const double* elem_c;        // optional per-element LxF dissipation scale (face: (c1 + c2)/2)
    int64_t ndofs, nfdofs;
    int32_t nfaces, n, npe, nfd;
    int32_t numflux, lxf_avg;
    double intensity, gamma;
    double adv[3];
    int32_t bc_kind[MAXBC];
    double bc_state[MAXBC][5];
    const double* bc_field;      // [NV][nfdofs]: FLOU_BC_STATE_FIELD states per face node
    // general (curvilinear / unstructured) geometry, read by the CURV kernels only
    const double* frames;        // [9][nfdofs]: n, t, b of every face node (master ordering)
    const double* faceJn;        // [nfdofs] surface Jacobian of every face node
    const uint8_t* orient;       // [nfaces] master2slave orientation
    int32_t* status;             // index-check reports (FLOU_CUDA_CHECKED builds)
};

struct ElemParams {
    const double* Q;             // stage input U
    const double* Q0;            // U^n (stage combinations)
    double* out;                 // dQ (mode 0) or the next stage state
    const double* Fn;            // face fluxes
    const int32_t* elem_face;    // nelem x 2d: (face << 1) | side (0 master, 1 slave)
    const double* elem_invJ;     // nelem
    const double* elem_Ja;       // nelem x d (diagonal of the metric)
    const double* ops;           // Ds[n*n], Dsharp[n*n], l_l[n], l_r[n], dg_l[n], dg_r[n]
    int64_t ndofs, nfdofs;
    int32_t nelem;
    int32_t mode;                // 0: out = dQ; 1: out = U + dt dQ; 2: out = a0 U^n + a1 (U + dt dQ);
                                 // 3: 2N-storage stage, k = a0 k + dt dQ (in aux), out = U + a1 k
    double dt, a0, a1;
    double* aux;                 // mode 3: the 2N-storage register k, read and rewritten per node
    const double* dtp;           // CFL stepping: dt lives in device memory (0: the run is over, skip)
    int32_t lift_ends;           // the lift ∂g acts on the end nodes only (else: every node of the line)
    int32_t diag_roundoff;       // the diagonal of D♯ is round-off (DGSEM on Gauss-Lobatto nodes)
    const double* subfr;         // CURV hybrid: [9][ns] n, t, b of each subcell interface
    const double* subJ;          //   and its surface Jacobian; point ((e·DIM + dir)·n^(d-1) + line)·(n+1) + s
    double gamma;
    double adv[3];
    int32_t* status;             // [0] flags, [1] lowest offending element (1-based)
    // HybridDivOperator (OpDivergence.jl:439-612, 781-801): subcell FV flux and blending
    const double* omega1;        // [n] 1D quadrature weights
    int32_t fvflux, fvavg;
    double fvintensity, blend;
    // general geometry (CURV kernels)
    const double* invJn;         // [ndofs] 1/J of every node
    const double* Jan;           // [DIM*DIM][ndofs]: metric Ja[k, d] at q = k + d*DIM (columns: dual basis)
    const uint8_t* orient;       // [nfaces] master2slave orientation
};

// master2slave of a face dof (StdSegment.jl:161-167, StdQuad.jl:161-181), 0-based, x fastest:
// the slave's face dof that holds the master's face dof m.
template <int DIM>
__host__ __device__ __forceinline__ int master2slave(int m, int o, int n) {
    if (DIM <= 1 || o == 0) return m;
    if (DIM == 2) return n - 1 - m;
    int m1 = m % n, m2 = m / n;
    switch (o) {
        case 1: return m2 + n * (n - 1 - m1);
        case 2: return (n - 1 - m1) + n * (n - 1 - m2);
        case 3: return (n - 1 - m2) + n * m1;
        case 4: return m2 + n * m1;
        case 5: return (n - 1 - m1) + n * m2;
        case 6: return (n - 1 - m2) + n * (n - 1 - m1);
        default: return m1 + n * (n - 1 - m2);
    }
}

// The orientation whose master2slave inverts o's (the two quarter turns of a quadrilateral
// face are each other's inverse; every other map is an involution).
template <int DIM>
__host__ __device__ __forceinline__ int inverse_orientation(int o) {
    return (DIM == 3 && (o == 1 || o == 3)) ? 4 - o : o;
}

// Local face positions follow the reference's face order: 2*dir (left) and 2*dir+1
// (right); frames of a face are those of its master position (PhysicalRegions.jl:541-696).
struct FrameTab { double n[3], t[3], b[3]; };

// Device-side index checks, compiled in with -DFLOU_CUDA_CHECKED (build.py --checked, the
// library libflou_cuda_checked.so): an index outside its array sets bit 2 of the status word
// (FLOU_ERR_INDEX on the host, with the lowest element involved) and the access is skipped.
// Nothing traps.  In the default build the checks compile to nothing.
#ifdef FLOU_CUDA_CHECKED
constexpr bool kChecked = true;
#else
constexpr bool kChecked = false;
#endif

__device__ __forceinline__ bool index_ok(int64_t i, int64_t n, int32_t* status, int64_t elem) {
    if (!kChecked || (i >= 0 && i < n)) return true;
    if (status) {
        atomicOr(status, 4);
        atomicMin(status + 1, (int32_t)(elem + 1));
    }
    return false;
}

__host__ __device__ inline FrameTab frame_of(int dim, int pos) {
    FrameTab F = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    if (dim == 1) {
        F.n[0] = (pos == 0) ? -1.0 : 1.0;
    } else if (dim == 2) {
        switch (pos) {
            case 0: F.n[0] = -1; F.t[1] = -1; break;
            case 1: F.n[0] = 1; F.t[1] = 1; break;
            case 2: F.n[1] = -1; F.t[0] = 1; break;
            default: F.n[1] = 1; F.t[0] = -1; break;
        }
    } else {
        switch (pos) {
            case 0: F.n[0] = -1; F.t[1] = -1; F.b[2] = 1; break;
            case 1: F.n[0] = 1; F.t[1] = 1; F.b[2] = 1; break;
            case 2: F.n[1] = -1; F.t[2] = -1; F.b[0] = 1; break;
            case 3: F.n[1] = 1; F.t[2] = 1; F.b[0] = 1; break;
            case 4: F.n[2] = -1; F.t[0] = -1; F.b[1] = 1; break;
            default: F.n[2] = 1; F.t[0] = 1; F.b[1] = 1; break;
        }
    }
    return F;
}

// Element-local node index of position `pos` on line `line` of direction `dir`
// (tpdofs: StdSegment.jl:143-146, StdQuad.jl:116-124, StdHex.jl:135-145).  The face-dof
// index of a face normal to `dir` is the line index.
template <int DIM>
__host__ __device__ inline int tp_node(int n, int dir, int line, int pos) {
    if (DIM == 1) return pos;
    if (DIM == 2) return dir == 0 ? pos + n * line : line + n * pos;
    int a = line % n, b = line / n;
    if (dir == 0) return pos + n * (a + n * b);
    if (dir == 1) return a + n * (pos + n * b);
    return a + n * (b + n * pos);
}

// Inverse: for element-local node i, its position along `dir` and its line index.
template <int DIM>
__host__ __device__ inline void tp_coords(int n, int i, int dir, int& pos, int& line) {
    if (DIM == 1) { pos = i; line = 0; return; }
    int x = i % n, y = (i / n) % n, z = i / (n * n);
    if (DIM == 2) {
        if (dir == 0) { pos = x; line = y; } else { pos = y; line = x; }
        return;
    }
    if (dir == 0) { pos = x; line = y + n * z; }
    else if (dir == 1) { pos = y; line = x + n * z; }
    else { pos = z; line = x + n * y; }
}

// ---------------------------------------------------------------------------------------
// Pointwise physics (src/FlouCommon/Euler.jl, src/FlouSpatial/Equations/Euler.jl)
// ---------------------------------------------------------------------------------------
// pressure = (γ-1)(ρe - |ρv|²/(2ρ)), Euler.jl:142-155
template <int DIM>
__device__ __forceinline__ double euler_pressure(const double* q, double g) {
    double s = q[1] * q[1];
    if (DIM > 1) s = s + q[2] * q[2];
    if (DIM > 2) s = s + q[3] * q[3];
    return (g - 1.0) * (q[DIM + 1] - s / (2.0 * q[0]));
}

// Face-frame physical normal flux of the Euler equations given conserved q and
// primitives (normal velocity un = q[1]/q[0], pressure p).
template <int DIM>
__device__ __forceinline__ void euler_normal_flux(const double* q, double un, double p, double* F) {
    F[0] = q[1];
    F[1] = q[1] * un + p;
    for (int k = 1; k < DIM; ++k) F[1 + k] = q[1 + k] * un;
    F[DIM + 1] = (q[DIM + 1] + p) * un;
}

// x < 0.01 for x >= 0 (or NaN, which fails like the floating-point test) as an integer
// comparison of the bit patterns, keeping the FP64 pipe for arithmetic.
__device__ __forceinline__ bool below_001(double x) {
    return __double_as_longlong(x) < 0x3F847AE147AE147BLL;   // the bits of 0.01
}

// 1/x for a normal x: the hardware's approximate reciprocal (rcp.approx.ftz.f64, on the MUFU
// unit) refined by one third-order step y(1 + e + e²), e = 1 - x y (the series of y/(1 - e)):
// three FMAs on the FP64 pipe instead of a correctly rounded division.  Measured on GB300 over
// 2^30 samples: the seed's relative error is below 2^-19.9, the refined value within 1 ulp of the
// correctly rounded 1/x (the step's remainder e³ is below 1e-18).
__device__ __forceinline__ double rcp_refined(double x) {
    double y;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
    double e = fma(-x, y, 1.0);
    return fma(y, fma(e, e, e), y);
}

// sqrt(x) for a normal x > 0: the hardware's approximate 1/√x (rsqrt.approx.ftz.f64, MUFU) gives
// s0 = x y; with e = 1 - s0 y = 1 - x y², √x = s0 (1 - e)^(-1/2), and the binomial series
// 1 + e/2 + 3e²/8 truncated after e² (remainder 5e³/16) gives one third-order step: four
// FP64 operations and a multiply instead of a correctly rounded square root.
__device__ __forceinline__ double sqrt_refined(double x) {
    double y;
    asm("rsqrt.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
    double s0 = x * y;
    double e = fma(-s0, y, 1.0);
    return fma(s0, e * fma(e, 0.375, 0.5), s0);
}

// 1/√x for a normal x > 0: rsqrt.approx.ftz.f64 refined by the same third-order step,
// y (1 + e/2 + 3e²/8) with e = 1 - x y².
__device__ __forceinline__ double rsqrt_refined(double x) {
    double y;
    asm("rsqrt.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
    double e = fma(-x * y, y, 1.0);
    return fma(y, e * fma(e, 0.375, 0.5), y);
}

// Logarithmic mean (src/FlouCommon/Utilities.jl:34-44) of a, b > 0 in sums and differences, given
// s = a + b and rs = 1/s (often from one reciprocal shared with a second mean):
//   f = (a - b)/s, u = f²;  u < 0.01: mean = s/(2F) with the reference's F = 1+u/3+u²/5+u³/7
//   (1/F from rcp_refined), else the log branch
//   mean = (a - b)/ln(a/b).  L = ln(a/b) comes along: from the log branch, or on the series
//   branch from 2f·atanh(f)/f summed to u⁸/17 (remainder below 1e-19 relative).
struct LogMean { double mean, inv, L; };

__device__ __forceinline__ LogMean logmean_sd(double a, double b, double s, double rs) {
    const double d = a - b, f = d * rs, u = f * f;
    LogMean m;
    if (below_001(u)) {
        double Fs = fma(u, fma(u, fma(u, 1.0 / 7.0, 0.2), 1.0 / 3.0), 1.0);
        m.mean = 0.5 * s * rcp_refined(Fs);
        m.inv = 2.0 * Fs * rs;
        double Fe = fma(u, 1.0 / 17.0, 1.0 / 15.0);
        Fe = fma(u, Fe, 1.0 / 13.0);
        Fe = fma(u, Fe, 1.0 / 11.0);
        Fe = fma(u, Fe, 1.0 / 9.0);
        Fe = fma(u, Fe, 1.0 / 7.0);
        Fe = fma(u, Fe, 0.2);
        Fe = fma(u, Fe, 1.0 / 3.0);
        Fe = fma(u, Fe, 1.0);
        m.L = 2.0 * f * Fe;
    } else {
        double L = log(a / b);
        m.mean = d / L;
        m.inv = L / d;
        m.L = L;
    }
    return m;
}

// The entropy-conserving and entropy-stable interface fluxes of src/FlouSpatial/Equations/Euler.jl
// in the face frame (momentum index 1 normal): ChandrasekharAverage (:167-226, 3D with the
// reference's wl² counted twice), LxF with either central flux (:138-165), ScalarDissipation
// (:228-301, 3D with the reference's zero momentum jump) and MatrixDissipation (:303-380).  One
// reciprocal per density and pressure, one shared by both logarithmic means; the entropy-variable
// jump takes its logarithms from the means, ln(p_l/p_r) = ln(ρ_l/ρ_r) - ln(β_l/β_r), so
// (s_r - s_l)/(γ-1) = L_ρ + L_β/(γ-1).  Same formulas as the reference up to rounding.
template <int DIM>
__device__ __forceinline__ void euler_face_flux_es(const double* ql, const double* qr, int kind, int avg,
                                                   double intensity, double g, double* F) {
    constexpr int NV = DIM + 2;
    const double rl = ql[0], rr = qr[0];
    const double irl = rcp_refined(rl), irr = rcp_refined(rr);
    double vl[3] = {0.0, 0.0, 0.0}, vr[3] = {0.0, 0.0, 0.0};
    double vl2 = 0.0, vr2 = 0.0;
#pragma unroll
    for (int k = 0; k < DIM; ++k) {
        vl[k] = ql[1 + k] * irl;
        vr[k] = qr[1 + k] * irr;
        vl2 = fma(vl[k], vl[k], vl2);
        vr2 = fma(vr[k], vr[k], vr2);
    }
    const double g1 = g - 1.0;
    const double ig1 = rcp_refined(g1);   // 1/(γ-1): multiplications instead of divisions below
    const double pl = g1 * fma(-0.5 * rl, vl2, ql[DIM + 1]), pr = g1 * fma(-0.5 * rr, vr2, qr[DIM + 1]);
    double vm[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) vm[k] = 0.5 * (vl[k] + vr[k]);
    double A[NV];
    const bool chandra = kind == FLOU_NF_CHANDRASHEKAR || avg == FLOU_NF_CHANDRASHEKAR;
    const bool needs_means = chandra || kind == FLOU_NF_SCALAR_DISSIPATION || kind == FLOU_NF_MATRIX_DISSIPATION;
    LogMean mr{0.0, 0.0, 0.0}, mb{0.0, 0.0, 0.0};
    double bl = 0.0, br = 0.0, phat = 0.0;
    if (needs_means) {
        const double ipl = rcp_refined(pl), ipr = rcp_refined(pr);
        bl = 0.5 * rl * ipl;
        br = 0.5 * rr * ipr;
        const double sr = rl + rr, sb = bl + br;
        const double R = rcp_refined(sr * sb);
        const double rsr = sb * R, rsb = sr * R;
        mr = logmean_sd(rl, rr, sr, rsr);
        mb = logmean_sd(bl, br, sb, rsb);
        phat = 0.5 * sr * rsb;   // (ρl + ρr)/(2(βl + βr))
    }
    if (chandra) {
        double s = vl2 + vr[0] * vr[0];
        if (DIM > 1) s = s + vr[1] * vr[1];
        if (DIM > 2) s = s + vl[2] * vl[2];
        double vv = vm[0] * vm[0];
        if (DIM > 1) vv = fma(vm[1], vm[1], vv);
        if (DIM > 2) vv = fma(vm[2], vm[2], vv);
        double h = fma(mb.inv, 0.5 * ig1, fma(-0.25, s, fma(phat, mr.inv, vv)));
        double m = mr.mean * vm[0];
        A[0] = m;
        A[1] = fma(m, vm[0], phat);
#pragma unroll
        for (int k = 1; k < DIM; ++k) A[1 + k] = m * vm[k];
        A[DIM + 1] = m * h;
    } else {   // StdAverage, Euler.jl:99-136
        A[0] = (ql[1] + qr[1]) * 0.5;
        A[1] = (fma(ql[1], vl[0], pl) + fma(qr[1], vr[0], pr)) * 0.5;
#pragma unroll
        for (int k = 1; k < DIM; ++k) A[1 + k] = fma(ql[1 + k], vl[0], qr[1 + k] * vr[0]) * 0.5;
        A[DIM + 1] = fma(ql[DIM + 1] + pl, vl[0], (qr[DIM + 1] + pr) * vr[0]) * 0.5;
    }
    if (kind == FLOU_NF_CHANDRASHEKAR || kind == FLOU_NF_STD_AVERAGE) {
#pragma unroll
        for (int k = 0; k < NV; ++k) F[k] = A[k];
        return;
    }
    if (kind == FLOU_NF_LXF || kind == FLOU_NF_SCALAR_DISSIPATION) {
        const double al = sqrt_refined(g * pl * irl), ar = sqrt_refined(g * pr * irr);
        const double lam = fmax(fabs(vl[0]) + al, fabs(vr[0]) + ar) * (0.5 * intensity);
        if (kind == FLOU_NF_LXF) {
#pragma unroll
            for (int k = 0; k < NV; ++k) F[k] = fma(lam, ql[k] - qr[k], A[k]);
            return;
        }
        double D[NV];
        D[0] = rr - rl;
        // the 3D branch takes the left momenta from Qr (Euler.jl:257): no momentum jump there
#pragma unroll
        for (int k = 0; k < DIM; ++k) D[1 + k] = (DIM == 3) ? 0.0 : qr[1 + k] - ql[1 + k];
        double c1 = mb.inv * ig1, c2 = 0.0;
#pragma unroll
        for (int k = 0; k < DIM; ++k) {
            c1 = fma(vl[k], vr[k], c1);
            c2 = fma(vm[k], vr[k] - vl[k], c2);
        }
        c2 = c2 + (pr * irr - pl * irl) * ig1;   // (1/βr - 1/βl)/(2(γ-1))
        D[DIM + 1] = fma(0.5 * c1, rr - rl, 0.5 * (rl + rr) * c2);
#pragma unroll
        for (int k = 0; k < NV; ++k) F[k] = fma(-lam, D[k], A[k]);
        return;
    }
    // MatrixDissipation: F = A + R Λ T Rᵀ (W_l - W_r)/2, evaluated as y = Rᵀ ΔW, z = Λ T y, R z
    double vv = vm[0] * vm[0];
#pragma unroll
    for (int k = 1; k < DIM; ++k) vv = fma(vm[k], vm[k], vv);
    const double v2 = fma(2.0, vv, -0.5 * (vl2 + vr2));
    const double a = sqrt_refined(g * phat * mr.inv);
    const double ig = rcp_refined(g);
    const double h = fma(0.5 * g * ig1, mb.inv, 0.5 * v2);
    double dW[NV];
    dW[0] = fma(mb.L, ig1, mr.L) - (vl2 * bl - vr2 * br);
#pragma unroll
    for (int k = 0; k < DIM; ++k) dW[1 + k] = 2.0 * (bl * vl[k] - br * vr[k]);
    dW[DIM + 1] = -2.0 * (bl - br);
    const double u = vm[0];
    double y[NV];
    double ye = fma(u, dW[1], dW[0]);
    y[0] = fma(-a, dW[1], ye);
    y[DIM + 1] = fma(a, dW[1], ye);
#pragma unroll
    for (int k = 1; k < DIM; ++k) {
        y[0] = fma(vm[k], dW[1 + k], y[0]);
        y[DIM + 1] = fma(vm[k], dW[1 + k], y[DIM + 1]);
        ye = fma(vm[k], dW[1 + k], ye);
        y[1 + k] = fma(vm[k], dW[DIM + 1], dW[1 + k]);
    }
    y[0] = fma(fma(-u, a, h), dW[DIM + 1], y[0]);
    y[DIM + 1] = fma(fma(u, a, h), dW[DIM + 1], y[DIM + 1]);
    y[1] = fma(0.5 * v2, dW[DIM + 1], ye);
    const double rho = mr.mean, ta = rho * (0.5 * ig);
    double z[NV];
    z[0] = fabs(u - a) * ta * y[0];
    z[1] = fabs(u) * (g1 * rho * ig) * y[1];
#pragma unroll
    for (int k = 1; k < DIM; ++k) z[1 + k] = fabs(u) * phat * y[1 + k];
    z[DIM + 1] = fabs(u + a) * ta * y[DIM + 1];
    const double zs = z[0] + z[1] + z[DIM + 1];
    double o[NV];
    o[0] = zs;
    o[1] = fma(u - a, z[0], fma(u, z[1], (u + a) * z[DIM + 1]));
    o[DIM + 1] = fma(fma(-u, a, h), z[0], fma(0.5 * v2, z[1], fma(u, a, h) * z[DIM + 1]));
#pragma unroll
    for (int k = 1; k < DIM; ++k) {
        o[1 + k] = fma(vm[k], zs, z[1 + k]);
        o[DIM + 1] = fma(vm[k], z[1 + k], o[DIM + 1]);
    }
    const double c = 0.5 * intensity;
#pragma unroll
    for (int k = 0; k < NV; ++k) F[k] = fma(c, o[k], A[k]);
}

// Signed axes of a Cartesian face frame (n, t, b) for a master at local position `pos`: the
// same frames as frame_of (PhysicalRegions.jl:541-696), whose rotations are signed
// permutations; rotating with them is exact.
struct FrameAxes { int ax[3]; bool neg[3]; };

template <int DIM>
__device__ __forceinline__ FrameAxes frame_axes(int pos) {
    // the table of PhysicalRegions.jl:568-696 in closed form (register arithmetic, no switch):
    // the normal is axis pos / 2, negative on the lower face; the tangents follow cyclically
    // (2D: t = ±e_other, negative when the normal is positive along y or negative along x)
    FrameAxes A = {{0, 0, 0}, {false, false, false}};
    const int dir = pos >> 1;
    const bool lower = (pos & 1) == 0;
    A.ax[0] = dir;
    A.neg[0] = lower;
    if (DIM == 2) {
        A.ax[1] = 1 - dir;
        A.neg[1] = lower != (dir == 1);
    } else if (DIM == 3) {
        A.ax[1] = dir == 2 ? 0 : dir + 1;
        A.ax[2] = dir == 0 ? 2 : dir - 1;
        A.neg[1] = lower;
    }
    return A;
}

__device__ __forceinline__ double flip(double x, bool neg) {
    return __longlong_as_double(__double_as_longlong(x) ^ (neg ? (long long)0x8000000000000000ULL : 0LL));
}

// Momentum components of a Cartesian face frame without runtime-indexed register arrays (which
// the compiler would place in local memory): to_face gives a[1 + r] = ±m[A.ax[r]], to_phys puts
// ±f[1 + r] back on axis A.ax[r]; the selects and sign flips run on the integer units.
template <int DIM>
__device__ __forceinline__ void cart_to_face(const double* q, const FrameAxes& A, double* a) {
#pragma unroll
    for (int r = 0; r < DIM; ++r) {
        double m = q[1];
#pragma unroll
        for (int k = 1; k < DIM; ++k) m = A.ax[r] == k ? q[1 + k] : m;
        a[1 + r] = flip(m, A.neg[r]);
    }
}

template <int DIM>
__device__ __forceinline__ void cart_to_phys(const double* f, const FrameAxes& A, double* q) {
#pragma unroll
    for (int k = 0; k < DIM; ++k) {
        double m = 0.0;
#pragma unroll
        for (int r = 0; r < DIM; ++r) m = A.ax[r] == k ? flip(f[1 + r], A.neg[r]) : m;
        q[1 + k] = m;
    }
}

// StdAverage / LxF(StdAverage) / HLL / HLLC in the face frame with one reciprocal of the
// density per side (u = m·(1/ρ), p = (γ-1)(ρe - ½|m|²/ρ)) and one shared reciprocal for the
// HLLC star state, reciprocals and sound speeds from rcp_refined / sqrt_refined; the
// reference's formulas (Euler.jl:99-165 and the HLL/HLLC of Toro 2009) up to rounding.
template <int DIM>
__device__ __forceinline__ void euler_face_flux_fast(const double* ql, const double* qr, int kind, double intensity,
                                                     double g, double* F) {
    constexpr int NV = DIM + 2;
    double irl = rcp_refined(ql[0]), irr = rcp_refined(qr[0]);
    double ul = ql[1] * irl, ur = qr[1] * irr;
    double sl2 = ql[1] * ql[1], sr2 = qr[1] * qr[1];
#pragma unroll
    for (int k = 1; k < DIM; ++k) { sl2 = fma(ql[1 + k], ql[1 + k], sl2); sr2 = fma(qr[1 + k], qr[1 + k], sr2); }
    double pl = (g - 1.0) * fma(-0.5 * sl2, irl, ql[DIM + 1]);
    double pr = (g - 1.0) * fma(-0.5 * sr2, irr, qr[DIM + 1]);
    if (kind == FLOU_NF_STD_AVERAGE || kind == FLOU_NF_LXF) {   // Euler.jl:99-165
        F[0] = (ql[1] + qr[1]) * 0.5;
        F[1] = (fma(ql[1], ul, pl) + fma(qr[1], ur, pr)) * 0.5;
#pragma unroll
        for (int k = 1; k < DIM; ++k) F[1 + k] = fma(ql[1 + k], ul, qr[1 + k] * ur) * 0.5;
        F[DIM + 1] = fma(ql[DIM + 1] + pl, ul, (qr[DIM + 1] + pr) * ur) * 0.5;
        if (kind == FLOU_NF_LXF) {
            double al = sqrt_refined(g * pl * irl), ar = sqrt_refined(g * pr * irr);
            double lam = fmax(fabs(ul) + al, fabs(ur) + ar) * (0.5 * intensity);
#pragma unroll
            for (int k = 0; k < NV; ++k) F[k] = fma(lam, ql[k] - qr[k], F[k]);
        }
        return;
    }
    double al = sqrt_refined(g * pl * irl), ar = sqrt_refined(g * pr * irr);
    double sl = fmin(ul - al, ur - ar), sr = fmax(ul + al, ur + ar);
    double Fl[NV], Fr[NV];
    euler_normal_flux<DIM>(ql, ul, pl, Fl);
    euler_normal_flux<DIM>(qr, ur, pr, Fr);
    if (sl >= 0.0) { for (int k = 0; k < NV; ++k) F[k] = Fl[k]; return; }
    if (sr <= 0.0) { for (int k = 0; k < NV; ++k) F[k] = Fr[k]; return; }
    if (kind == FLOU_NF_HLL) {
        double r = rcp_refined(sr - sl), slr = sl * sr;
        for (int k = 0; k < NV; ++k) F[k] = (fma(sr, Fl[k], -sl * Fr[k]) + slr * (qr[k] - ql[k])) * r;
        return;
    }
    double ml = ql[0] * (sl - ul), mr = qr[0] * (sr - ur);
    double ss = fma(ul, ml, (pr - pl) - ur * mr) * rcp_refined(ml - mr);
    bool left = ss >= 0.0;
    double qk[NV], Fk[NV];   // the star side's state and flux, selected per component (no local memory)
#pragma unroll
    for (int k = 0; k < NV; ++k) {
        qk[k] = left ? ql[k] : qr[k];
        Fk[k] = left ? Fl[k] : Fr[k];
    }
    double sk = left ? sl : sr, mk = left ? ml : mr, irk = left ? irl : irr, uk = left ? ul : ur,
           pk = left ? pl : pr;
    double R = rcp_refined((sk - ss) * mk);
    double coef = mk * mk * R;          // ρ_K (S_K - u_K)/(S_K - S*)
    double pm = pk * (sk - ss) * R;     // p_K / (ρ_K (S_K - u_K))
    double Us[NV];
    Us[0] = coef;
    Us[1] = coef * ss;
#pragma unroll
    for (int k = 1; k < DIM; ++k) Us[1 + k] = coef * (qk[1 + k] * irk);
    Us[DIM + 1] = coef * fma(ss - uk, ss + pm, qk[DIM + 1] * irk);
#pragma unroll
    for (int k = 0; k < NV; ++k) F[k] = fma(sk, Us[k] - qk[k], Fk[k]);
}

// numericalflux(Ql, Qr, n, eq, kind) in the face frame: the entropy-based fluxes through
// euler_face_flux_es, the others through euler_face_flux_fast.
template <int DIM>
__device__ __forceinline__ void euler_numflux(const double* ql, const double* qr, int kind, int avg,
                                              double intensity, double g, double* F) {
    if (kind == FLOU_NF_CHANDRASHEKAR || kind >= FLOU_NF_SCALAR_DISSIPATION ||
        (kind == FLOU_NF_LXF && avg == FLOU_NF_CHANDRASHEKAR))
        euler_face_flux_es<DIM>(ql, qr, kind, avg, intensity, g, F);
    else
        euler_face_flux_fast<DIM>(ql, qr, kind, intensity, g, F);
}

// ---------------------------------------------------------------------------------------
// Face kernel: traces (project2faces!, Interfaces.jl:51-109), boundary ghost states
// (applyBCs!, :25-49) and numerical fluxes times the surface Jacobian
// (interface_fluxes!, :111-136).  One thread per face node.
// ---------------------------------------------------------------------------------------
// rotate2face / rotate2phys (Euler.jl:16-64) with a general frame (n, t, b): the momentum's
// components along n, t, b, and back.
template <int DIM>
__device__ __forceinline__ void rotate_to_face(const double* q, const FrameTab& fr, double* a) {
    a[0] = q[0];
    a[DIM + 1] = q[DIM + 1];
    if (DIM == 1) { a[1] = q[1] * fr.n[0]; return; }
    if (DIM == 2) {
        a[1] = q[1] * fr.n[0] + q[2] * fr.n[1];
        a[2] = q[1] * fr.t[0] + q[2] * fr.t[1];
        return;
    }
    a[1] = q[1] * fr.n[0] + q[2] * fr.n[1] + q[3] * fr.n[2];
    a[2] = q[1] * fr.t[0] + q[2] * fr.t[1] + q[3] * fr.t[2];
    a[3] = q[1] * fr.b[0] + q[2] * fr.b[1] + q[3] * fr.b[2];
}

template <int DIM>
__device__ __forceinline__ void rotate_to_phys(const double* a, const FrameTab& fr, double* q) {
    q[0] = a[0];
    q[DIM + 1] = a[DIM + 1];
    if (DIM == 1) { q[1] = a[1] * fr.n[0]; return; }
    if (DIM == 2) {
        q[1] = a[1] * fr.n[0] + a[2] * fr.t[0];
        q[2] = a[1] * fr.n[1] + a[2] * fr.t[1];
        return;
    }
    q[1] = a[1] * fr.n[0] + a[2] * fr.t[0] + a[3] * fr.b[0];
    q[2] = a[1] * fr.n[1] + a[2] * fr.t[1] + a[3] * fr.b[1];
    q[3] = a[1] * fr.n[2] + a[2] * fr.t[2] + a[3] * fr.b[2];
}

// CURV: general geometry -- the slave trace at master2slave(m), the frame and surface Jacobian
// of this face node (Interfaces.jl:111-136 with PhysicalRegions.jl:797-971).
template <int DIM, int EQ, bool LGL, bool CURV = false>
__device__ __forceinline__ void face_node(const FaceParams& P, int64_t gid) {
    constexpr int NV = (EQ == FLOU_EQ_EULER) ? DIM + 2 : 1;
    if (gid >= (int64_t)P.nfaces * P.nfd) return;
    int f = (int)(gid / P.nfd), m = (int)(gid - (int64_t)f * P.nfd);
    int n = P.n;
    int32_t s0 = P.face_elem[2 * f], s1 = P.face_elem[2 * f + 1];
    if (kChecked) {
        const int64_t nel = P.ndofs / P.npe;
        bool ok = index_ok(s0 >> 3, nel, P.status, 0) && index_ok(s0 & 7, 2 * DIM, P.status, s0 >> 3);
        if (ok && s1 >= 0)
            ok = index_ok(s1 >> 3, nel, P.status, s0 >> 3) && index_ok(s1 & 7, 2 * DIM, P.status, s1 >> 3) &&
                 (!CURV || index_ok(master2slave<DIM>(m, P.orient[f], n), P.nfd, P.status, s1 >> 3));
        if (ok && s1 < 0) ok = index_ok(P.face_bc[f], MAXBC, P.status, s0 >> 3);
        if (!ok) return;
    }
    auto trace = [&](int32_t s, int mm, double* q) {
        int e = s >> 3, pos = s & 7, dir = pos >> 1, right = pos & 1;
        const double* Qe = P.Q + (int64_t)e * P.npe;
        if (LGL) {
            int node = tp_node<DIM>(n, dir, mm, right ? n - 1 : 0);
            if (!index_ok(node, P.npe, P.status, e)) node = 0;
#pragma unroll
            for (int k = 0; k < NV; ++k) q[k] = Qe[k * P.ndofs + node];
        } else {
            const double* lv = P.l + (right ? n : 0);
#pragma unroll
            for (int k = 0; k < NV; ++k) {
                double acc = 0.0;
                for (int p = 0; p < n; ++p) acc = acc + lv[p] * Qe[k * P.ndofs + tp_node<DIM>(n, dir, mm, p)];
                q[k] = acc;
            }
        }
    };
    double ql[NV], qr[NV];
    trace(s0, m, ql);
    FrameTab fr;
    if (CURV) {
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            fr.n[c] = P.frames[c * P.nfdofs + gid];
            fr.t[c] = P.frames[(3 + c) * P.nfdofs + gid];
            fr.b[c] = P.frames[(6 + c) * P.nfdofs + gid];
        }
    } else if (EQ != FLOU_EQ_EULER) {   // the Euler path rotates with frame_axes
        fr = frame_of(DIM, s0 & 7);
    }
    if (s1 >= 0) {
        trace(s1, CURV ? master2slave<DIM>(m, P.orient[f], n) : m, qr);
    } else {
        int b = P.face_bc[f];
        int kind = P.bc_kind[b];
        if (kind == FLOU_BC_INFLOW) {
#pragma unroll
            for (int k = 0; k < NV; ++k) qr[k] = P.bc_state[b][k];
        } else if (kind == FLOU_BC_STATE_FIELD) {
#pragma unroll
            for (int k = 0; k < NV; ++k) qr[k] = P.bc_field[k * P.nfdofs + gid];
        } else if (kind == FLOU_BC_SLIP && EQ == FLOU_EQ_EULER) {
            // EulerSlipBC (Euler.jl:88-94): rotate to the face frame, flip the normal momentum,
            // rotate back -- for a Cartesian frame, the momentum along the normal axis changes sign.
            if (CURV) {
                double a[NV];
                rotate_to_face<DIM>(ql, fr, a);
                a[1] = -a[1];
                rotate_to_phys<DIM>(a, fr, qr);
            } else {
                const int an = frame_axes<DIM>(s0 & 7).ax[0];
#pragma unroll
                for (int k = 0; k < NV; ++k) qr[k] = flip(ql[k], k >= 1 && k <= DIM && k - 1 == an);
            }
        } else {
#pragma unroll
            for (int k = 0; k < NV; ++k) qr[k] = ql[k];   // outflow
        }
    }
    double F[NV];
    double J = CURV ? P.faceJn[gid] : P.faceJ[f];
    double inten = P.intensity;
    if (P.elem_c) {
        int e1 = s0 >> 3, e2 = s1 >= 0 ? (s1 >> 3) : e1;
        inten = (P.elem_c[e1] + P.elem_c[e2]) * 0.5;
    }
    if (EQ == FLOU_EQ_EULER) {
        // rotate2face / rotate2phys (Euler.jl:16-64): signed permutations for a Cartesian frame
        FrameAxes A = frame_axes<DIM>(s0 & 7);
        double a[NV], b[NV];
        if (CURV) {
            rotate_to_face<DIM>(ql, fr, a);
            rotate_to_face<DIM>(qr, fr, b);
        } else {
            a[0] = ql[0]; b[0] = qr[0]; a[DIM + 1] = ql[DIM + 1]; b[DIM + 1] = qr[DIM + 1];
            cart_to_face<DIM>(ql, A, a);
            cart_to_face<DIM>(qr, A, b);
        }
        double Fr[NV];
        euler_numflux<DIM>(a, b, P.numflux, P.lxf_avg, inten, P.gamma, Fr);
        if (CURV) {
            rotate_to_phys<DIM>(Fr, fr, F);
        } else {
            F[0] = Fr[0];
            F[DIM + 1] = Fr[DIM + 1];
            cart_to_phys<DIM>(Fr, A, F);
        }
    } else if (EQ == FLOU_EQ_LINEAR_ADVECTION) {
        // LinearAdvection.jl:27-39
        double an = P.adv[0] * fr.n[0];
        if (DIM > 1) an = an + P.adv[1] * fr.n[1];
        if (DIM > 2) an = an + P.adv[2] * fr.n[2];
        F[0] = an * (ql[0] + qr[0]) / 2.0;
        if (P.numflux == FLOU_NF_LXF) F[0] = F[0] + fabs(an) * (ql[0] - qr[0]) / 2.0 * inten;
    } else {
        // Burgers.jl:27-38
        F[0] = (ql[0] * ql[0] + qr[0] * qr[0]) / 4.0 * fr.n[0];
        if (P.numflux == FLOU_NF_LXF) {
            double lam = fmax(fabs(ql[0]), fabs(qr[0]));
            F[0] = F[0] + lam * (ql[0] - qr[0]) / 2.0 * inten;
        }
    }
    int64_t o = (int64_t)f * P.nfd + m;
    if (!index_ok(o, P.nfdofs, P.status, s0 >> 3)) return;
#pragma unroll
    for (int k = 0; k < NV; ++k) P.Fn[k * P.nfdofs + o] = F[k] * J;
}

template <int DIM, int EQ, bool LGL, bool CURV = false>
__global__ void __launch_bounds__(256) face_kernel(FaceParams P) {
    face_node<DIM, EQ, LGL, CURV>(P, (int64_t)blockIdx.x * blockDim.x + threadIdx.x);
}

// ---------------------------------------------------------------------------------------
// Element kernels: volume term + surface lift + inverse mass + fused RK stage update.
// One block owns EPB consecutive elements, one thread per element node.
// ---------------------------------------------------------------------------------------
template <int DIM, int N, int TB = 256>
struct Shape {
    static constexpr int NPE = ipow(N, DIM);
    static constexpr int NFD = ipow(N, DIM - 1);
    static constexpr int EPB = (NPE >= TB) ? 1 : (TB / NPE);
    static constexpr int NN = EPB * NPE;
    static constexpr int BLOCK = ((NN + 31) / 32) * 32;
    static constexpr int NPAIR = N * (N - 1) / 2;
    static constexpr int NOPS = 2 * N * N + 4 * N;
};

__device__ __forceinline__ void raise_nonphysical(int32_t* status, int elem) {
    atomicOr(status, 1);
    atomicMin(status + 1, elem + 1);
}

// Surface lift (OpDivergence.jl:42-100) for node (pos along dir, line), then 1/J and the
// stage update.  Shared by both volume operators.
// CURV: a slave side reads the master's face dof that master2slave sends onto its own line
// index (the inverse orientation), and 1/J is taken per node.
// LIFT = false: the face fluxes already entered through the volume term (the hybrid operator on
// Gauss nodes, OpDivergence.jl:633-730), so only 1/J and the stage update remain.
template <int DIM, int N, int NV, bool LGL, bool CURV = false, bool LIFT = true>
__device__ __forceinline__ void surface_and_update(const ElemParams& P, const double* sops, int e, int i,
                                                   const double* q, double* dq) {
    const double* dgl = sops + 2 * N * N + 2 * N;
    const double* dgr = dgl + N;
#pragma unroll
    for (int dir = 0; dir < (LIFT ? DIM : 0); ++dir) {
        int pos, line;
        tp_coords<DIM>(N, i, dir, pos, line);
        int32_t pl = P.elem_face[e * 2 * DIM + 2 * dir], pr = P.elem_face[e * 2 * DIM + 2 * dir + 1];
        int linel = line, liner = line;
        if (CURV) {
            if (pl & 1) linel = master2slave<DIM>(line, inverse_orientation<DIM>(P.orient[pl >> 1]), N);
            if (pr & 1) liner = master2slave<DIM>(line, inverse_orientation<DIM>(P.orient[pr >> 1]), N);
        }
        int64_t ol = (int64_t)(pl >> 1) * ipow(N, DIM - 1) + linel;
        int64_t orr = (int64_t)(pr >> 1) * ipow(N, DIM - 1) + liner;
        if (kChecked && !(index_ok(linel, ipow(N, DIM - 1), P.status, e) && index_ok(liner, ipow(N, DIM - 1), P.status, e) &&
                          index_ok(ol, P.nfdofs, P.status, e) && index_ok(orr, P.nfdofs, P.status, e)))
            continue;
        double sl = (pl & 1) ? -1.0 : 1.0, sr = (pr & 1) ? -1.0 : 1.0;
        if (LGL && P.lift_ends) {
            // Only the two end nodes of a line take a face flux.  Where pos is the same for a whole
            // warp (a direction whose node stride is a multiple of the warp) the branches skip the
            // warp; elsewhere every thread would spend both branches' FP64 slots as predicated-off
            // instructions, so each thread selects its coefficient (zero inside the line) instead.
            constexpr int STRIDE = ipow(N, DIM - 1);   // the largest node stride, of the last direction
            const bool uniform = dir == DIM - 1 && STRIDE % 32 == 0 && ipow(N, DIM) % 32 == 0;
            if (uniform) {
                if (pos == 0) {
                    double c = dgl[0] * sl;
#pragma unroll
                    for (int k = 0; k < NV; ++k) dq[k] = dq[k] - c * __ldcg(P.Fn + k * P.nfdofs + ol);
                }
                if (pos == N - 1) {
                    double c = dgr[N - 1] * sr;
#pragma unroll
                    for (int k = 0; k < NV; ++k) dq[k] = dq[k] - c * __ldcg(P.Fn + k * P.nfdofs + orr);
                }
            } else {
                const bool atl = pos == 0;
                const double c0 = atl ? dgl[0] : dgr[N - 1], sg = atl ? sl : sr;
                const double c = (atl || pos == N - 1) ? c0 * sg : 0.0;
                const int64_t o = atl ? ol : orr;
#pragma unroll
                for (int k = 0; k < NV; ++k) dq[k] = fma(-c, __ldcg(P.Fn + k * P.nfdofs + o), dq[k]);
            }
        } else {
            double cl = dgl[pos] * sl, cr = dgr[pos] * sr;
#pragma unroll
            for (int k = 0; k < NV; ++k)
                dq[k] = dq[k] - (cl * __ldcg(P.Fn + k * P.nfdofs + ol) + cr * __ldcg(P.Fn + k * P.nfdofs + orr));
        }
    }
    int64_t g = (int64_t)e * ipow(N, DIM) + i;
    if (!(index_ok(e, P.nelem, P.status, e) && index_ok(g, P.ndofs, P.status, e))) return;
    double invJ = CURV ? P.invJn[g] : P.elem_invJ[e];
    const double dt = P.dtp ? *P.dtp : P.dt;
    const double c = dt * invJ;   // dt/J once per node: q + dt (dq/J) = q + c dq
    bool bad = false;
#pragma unroll
    for (int k = 0; k < NV; ++k) {
        double o;
        if (P.mode == 0) o = dq[k] * invJ;
        else if (P.mode == 1) o = fma(c, dq[k], q[k]);
        else if (P.mode == 2) o = fma(P.a0, P.Q0[k * P.ndofs + g], P.a1 * fma(c, dq[k], q[k]));
        else {
            // explicit FMAs, as in the other modes: every instantiation (the plain kernels, the
            // batched tiles) rounds alike
            double kk = c * dq[k];
            if (P.a0 != 0.0) kk = fma(P.a0, P.aux[k * P.ndofs + g], kk);   // first stage: k is not read
            P.aux[k * P.ndofs + g] = kk;
            o = fma(P.a1, kk, q[k]);
        }
        bad |= !isfinite(o);
        P.out[k * P.ndofs + g] = o;
    }
    if (bad) raise_nonphysical(P.status, e);
}

// Strong (== weak on LGL) divergence: dQ_line -= Ds * F̃_line per direction
// (OpDivergence.jl:109-160), F̃ = Ja_dd F_d (contravariant with a diagonal metric).
template <int DIM, int N, int EQ, bool LGL, int TB = 256, bool CURV = false>
__device__ __forceinline__ void strong_tile(const ElemParams& P, int e0, double* smem) {
    using S = Shape<DIM, N, TB>;
    constexpr int NV = (EQ == FLOU_EQ_EULER) ? DIM + 2 : 1;
    constexpr int NPE = S::NPE, NN = S::NN;
    double* sops = smem;
    double* sF = sops + S::NOPS;   // [DIM][NV][NN]
    const int tid = threadIdx.x;
    for (int t = tid; t < S::NOPS; t += blockDim.x) sops[t] = P.ops[t];
    const int el = tid / NPE, i = tid - el * NPE;
    const int e = e0 + el;
    const bool active = (tid < NN) && (e < P.nelem);
    double q[NV];
    if (active) {
        int64_t g = (int64_t)e * NPE + i;
#pragma unroll
        for (int k = 0; k < NV; ++k) q[k] = P.Q[k * P.ndofs + g];
        double F[NV];
        double v[DIM], p = 0.0;
        if (EQ == FLOU_EQ_EULER) {   // primitives once per node (volumeflux, Euler.jl:54-114)
            double ir = rcp_refined(q[0]), ke = 0.0;
#pragma unroll
            for (int k = 0; k < DIM; ++k) {
                v[k] = q[1 + k] * ir;
                ke = fma(q[1 + k], v[k], ke);
            }
            p = (P.gamma - 1.0) * fma(-0.5, ke, q[DIM + 1]);
            if (!(q[0] > 0.0 && p > 0.0)) raise_nonphysical(P.status, e);
        }
#pragma unroll
        for (int d = 0; d < DIM; ++d) {
            if constexpr (CURV) {   // contravariant flux Σ_k F_k Ja[k, d] (PhysicalRegions.jl:1006-1033)
                double a[DIM];
#pragma unroll
                for (int k = 0; k < DIM; ++k) a[k] = P.Jan[(k + d * DIM) * P.ndofs + g];
                if constexpr (EQ == FLOU_EQ_EULER) {
                    double mn = 0.0, vn = 0.0;
#pragma unroll
                    for (int k = 0; k < DIM; ++k) {
                        mn = fma(q[1 + k], a[k], mn);
                        vn = fma(v[k], a[k], vn);
                    }
                    F[0] = mn;
#pragma unroll
                    for (int k = 0; k < DIM; ++k) F[1 + k] = fma(q[1 + k], vn, p * a[k]);
                    F[DIM + 1] = (q[DIM + 1] + p) * vn;
                } else {
                    double an = 0.0;
#pragma unroll
                    for (int k = 0; k < DIM; ++k) an = fma(P.adv[k], a[k], an);
                    F[0] = an * q[0];
                }
#pragma unroll
                for (int k = 0; k < NV; ++k) sF[(d * NV + k) * NN + tid] = F[k];
                continue;
            }
            double Ja = P.elem_Ja[e * DIM + d];
            if (EQ == FLOU_EQ_EULER) {
                F[0] = q[1 + d];
#pragma unroll
                for (int k = 0; k < DIM; ++k) F[1 + k] = q[1 + d] * v[k];
                F[1 + d] = F[1 + d] + p;
                F[DIM + 1] = (q[DIM + 1] + p) * v[d];
            } else if (EQ == FLOU_EQ_LINEAR_ADVECTION) {
                F[0] = P.adv[d] * q[0];
            } else {
                F[0] = q[0] * q[0] / 2.0;
            }
#pragma unroll
            for (int k = 0; k < NV; ++k) sF[(d * NV + k) * NN + tid] = F[k] * Ja;
        }
    }
    __syncthreads();
    if (active) {
        const double* Ds = sops;
        double dq[NV];
#pragma unroll
        for (int k = 0; k < NV; ++k) dq[k] = 0.0;
#pragma unroll
        for (int dir = 0; dir < DIM; ++dir) {
            int pos, line;
            tp_coords<DIM>(N, i, dir, pos, line);
            const double* Fd = sF + dir * NV * NN + el * NPE;
#pragma unroll
            for (int c = 0; c < N; ++c) {
                int j = tp_node<DIM>(N, dir, line, c);
                double a = Ds[pos + c * N];
#pragma unroll
                for (int k = 0; k < NV; ++k) dq[k] = dq[k] - a * Fd[k * NN + j];
            }
        }
        surface_and_update<DIM, N, NV, LGL, CURV>(P, sops, e, i, q, dq);
    }
}

template <int DIM, int N, int EQ, bool LGL, bool CURV = false>
__global__ void __launch_bounds__(Shape<DIM, N>::BLOCK) elem_strong_kernel(ElemParams P) {
    extern __shared__ double smem[];
    if (P.dtp && *P.dtp == 0.0) return;   // CFL stepping past tfinal: the state stays as it is
    strong_tile<DIM, N, EQ, LGL, 256, CURV>(P, blockIdx.x * Shape<DIM, N>::EPB, smem);
}

// ---------------------------------------------------------------------------------------
// Split-form (flux-differencing) divergence, OpDivergence.jl:200-282:
//   dQ_i -= sum_j D♯_ij F♯(i, j), F♯(i, i) = F̃_i, F♯(i, j) = twopointflux(Q_i, Q_j).
// The two-point fluxes of a line are symmetric; each pair is evaluated once by one thread
// and kept in shared memory (the reference fills both triangle entries the same way).
// The residual is bound by the FP64 pipe, so every quantity that depends on one node only
// is computed once per node (pre-halved where the pair formulas average it) and the pair
// formulas share one reciprocal.
// ---------------------------------------------------------------------------------------
// Shared per-node arrays (length NN each) of the split form, by two-point flux:
//   Chandrashekar:  ρ, vh_k = v_k/2, β = ρ/(2p), v_k
//   Kennedy-Gruber: rh = ρ/2, vh_k = v_k/2, ph = p/2, eh = e/2 (e = ρe/ρ)
//   StdAverage:     v_k, p, then the conserved variables
//   scalar equations: u
template <int DIM, int EQ, int TP>
struct SplitLayout {
    static constexpr int NV = (EQ == FLOU_EQ_EULER) ? DIM + 2 : 1;
    static constexpr int NARR = (EQ != FLOU_EQ_EULER) ? 1
                                : (TP == FLOU_TP_STD_AVERAGE ? DIM + 1 + NV
                                                             : (TP == FLOU_TP_CHANDRASHEKAR ? 2 * DIM + 2 : DIM + 3));
};

// The pair kernels return a power-of-two multiple of F♯ (one scale for all variables, exact):
// 2 for the Chandrashekar flux, and on a general element a further 2 because the averaged
// metric column enters as Ja_a + Ja_b, the pair fluxes being linear in it.  The node phase
// divides the metric factor by the scale and multiplies the diagonal weight by it.
template <int EQ, int TP, bool CURV = false>
struct PairScale {
    static constexpr double value = ((EQ == FLOU_EQ_EULER && TP == FLOU_TP_CHANDRASHEKAR) ? 2.0 : 1.0) *
                                    (CURV ? 2.0 : 1.0);
};



// Chandrashekar two-point flux (Euler.jl:474-536) along direction d without the metric
// factor, times 2, with the logarithmic means of Utilities.jl:34-44 written in sums and
// differences:
//   u = ((a-b)/(a+b))²;  series branch (u < 0.01): mean = (a+b)/(2F), F = 1+u/3+u²/5+u³/7,
//   log branch: mean = (a-b)/ln(a/b).
// With sρ = ρ1+ρ2, sβ = β1+β2, one reciprocal R = 1/(sρ sβ) gives 1/sρ and 1/sβ; the averaged
// pressure is p̂ = sρ/(2 sβ), and with A = ρ̄/ρ_ln, B = β̄/β_ln (F itself on a series branch) the
// enthalpy is h = 1/(2(γ-1)β_ln) + p̂/ρ_ln + v1·v2/2 = (A + B/(γ-1))/sβ + v1·v2/2, the last term
// from the full velocity of one node and the halved one of the other.
// Both reciprocals (R and 1/F) come from rcp_refined.  c_g = 1/(γ-1).
// GEN: the flux along a general vector nv (the averaged metric column of a curvilinear element,
// Euler.jl:474-536 with n = (Ja1 + Ja2)/2) instead of the axis d.
template <int DIM, bool GEN = false>
__device__ __forceinline__ void chandrashekar_pair(const double* __restrict__ S, int NN, int i, int l, int d,
                                                   double c_g, double* F, const double* nv = nullptr) {
    const double* rho = S;
    const double* vh = S + NN;
    const double* beta = S + (1 + DIM) * NN;
    const double* vf = S + (2 + DIM) * NN;
    double r1 = rho[i], r2 = rho[l], b1 = beta[i], b2 = beta[l];
    double sr = r1 + r2, dr = r1 - r2;
    double sb = b1 + b2, db = b1 - b2;
    double R = rcp_refined(sr * sb);
    double rs = sb * R, rb = sr * R;           // 1/(ρ1+ρ2), 1/(β1+β2)
    double fr = dr * rs, fb = db * rb;
    double ur = fr * fr, ub = fb * fb;
    double rl2, A, B;                          // 2ρ_ln, ρ̄/ρ_ln, β̄/β_ln
    if (below_001(ur)) {
        A = fma(ur, fma(ur, fma(ur, 1.0 / 7.0, 0.2), 1.0 / 3.0), 1.0);
        rl2 = sr * rcp_refined(A);
    } else {
        double L = log(r1 / r2);
        rl2 = (2.0 * dr) / L;
        A = sr / rl2;
    }
    if (below_001(ub)) {
        B = fma(ub, fma(ub, fma(ub, 1.0 / 7.0, 0.2), 1.0 / 3.0), 1.0);
    } else {
        B = (0.5 * log(b1 / b2)) / fb;
    }
    double p2 = sr * rb;                       // 2p̂
    double va[DIM];
    double dot = 0.0;
#pragma unroll
    for (int k = 0; k < DIM; ++k) {
        va[k] = vh[k * NN + i] + vh[k * NN + l];
        dot = fma(vf[k * NN + i], vh[k * NN + l], dot);   // v1·v2/2
    }
    double h = fma(rb, fma(c_g, B, A), dot);
    if (GEN) {
        double vn = 0.0;
#pragma unroll
        for (int k = 0; k < DIM; ++k) vn = fma(va[k], nv[k], vn);
        double m = rl2 * vn;
        F[0] = m;
#pragma unroll
        for (int k = 0; k < DIM; ++k) F[1 + k] = fma(m, va[k], p2 * nv[k]);
        F[DIM + 1] = m * h;
        return;
    }
    double m = rl2 * va[d];
    F[0] = m;
#pragma unroll
    for (int k = 0; k < DIM; ++k) F[1 + k] = fma(m, va[k], k == d ? p2 : 0.0);
    F[DIM + 1] = m * h;
}

// The per-node quantities of SplitLayout for one state (q conserved, v velocity, p pressure,
// ir = 1/ρ), written at column `col` of arrays with stride `st`.
template <int DIM, int TP>
__device__ __forceinline__ void store_split_node(double* S, int st, int col, const double* q, const double* v,
                                                 double p, double ir) {
    if (TP == FLOU_TP_CHANDRASHEKAR) {
        S[col] = q[0];
#pragma unroll
        for (int k = 0; k < DIM; ++k) S[(1 + k) * st + col] = 0.5 * v[k];
        S[(1 + DIM) * st + col] = (0.5 * q[0]) * rcp_refined(p);
#pragma unroll
        for (int k = 0; k < DIM; ++k) S[(2 + DIM + k) * st + col] = v[k];
    } else if (TP == FLOU_TP_KENNEDY_GRUBER) {
        S[col] = 0.5 * q[0];
#pragma unroll
        for (int k = 0; k < DIM; ++k) S[(1 + k) * st + col] = 0.5 * v[k];
        S[(1 + DIM) * st + col] = 0.5 * p;
        S[(2 + DIM) * st + col] = 0.5 * (q[DIM + 1] * ir);
    } else {
#pragma unroll
        for (int k = 0; k < DIM; ++k) S[k * st + col] = v[k];
        S[DIM * st + col] = p;
#pragma unroll
        for (int k = 0; k < DIM + 2; ++k) S[(DIM + 1 + k) * st + col] = q[k];
    }
}

// GAUSS (Euler on a basis without boundary nodes, Cartesian): the entropy-projected coupling of
// OpDivergence.jl:301-437.  Per line, W is interpolated to both ends, Q̃ = entropy2cons(W̃), and
// each node adds ∂g_l (F♯(Q_i, Q̃_l) - l·F♯(·, Q̃_l)) - ∂g_r (F♯(Q_i, Q̃_r) - r·F♯(·, Q̃_r)) to
// the split volume term; the projected states sit behind the nodes in the per-node arrays and
// their 2N two-point fluxes per line behind the volume pairs.  With HYB (OpDivergence.jl:633-
// 780) the same terms enter the subcell fluxes, which start at the element's own face fluxes.
// HYB: the hybrid (telescopic) form of HybridDivOperator on LGL nodes (OpDivergence.jl:553-604):
// the split-form node sums give the high-order subcell fluxes by F̄_{p+1} = F̄_p + ω_p Σ_j D♯_pj F♯_pj
// (F̄ = 0 at both element ends; algebraically the reference's Σ_{l<p<=k} 2 ω_l D_lk F♯(l,k)), each
// blended with the subcell FV flux by δ = max((√(b²+c) - b)/√(b²+c), 1/2), b = ΔW·(F̄ - F̄_FV),
// and dQ_p += (F̄_p - F̄_{p+1})/ω_p.  Cartesian geometry (subcell frames along the axes).
template <int DIM, int N, int EQ, int TP, bool LGL, int TB = 256, bool CURV = false, bool HYB = false>
__device__ __forceinline__ void split_tile(const ElemParams& P, int e0, double* smem) {
    using S = Shape<DIM, N, TB>;
    using Lay = SplitLayout<DIM, EQ, TP>;
    constexpr int NV = Lay::NV;
    constexpr int NPE = S::NPE, NN = S::NN, NFD = S::NFD, NPAIR = S::NPAIR;
    constexpr int NPT = S::EPB * NFD * NPAIR;   // pairs per direction in the block
    constexpr bool EULER = (EQ == FLOU_EQ_EULER);
    constexpr bool GAUSS = !LGL && EULER;
    constexpr int NPROJ = GAUSS ? 2 * S::EPB * NFD : 0;       // projected states, 2 per line
    constexpr int SST = NN + NPROJ;                            // stride of the per-node arrays
    constexpr int NPTX = NPT + (GAUSS ? NPROJ * N : 0);        // + node x projected-state fluxes
    static_assert(!GAUSS || Lay::NARR >= NV, "the line reductions reuse the projected columns");
    double* sops = smem;
    double* sprim = sops + S::NOPS;                 // [Lay::NARR][SST]
    double* spair = sprim + Lay::NARR * SST;        // [NV][NPTX]
    double* sJa = spair + NV * NPTX;                // CURV: [DIM][SST] metric column of the direction
                                                    // (GAUSS: then n·Js of each line end's subcell interface)
    double* sW = sJa + (CURV ? DIM * SST : 0);      // HYB, GAUSS: [NV][NN] entropy variables
    double* sH = sW + ((HYB || GAUSS) ? NV * NN : 0);   // HYB: [NV][NN] the node's subcell increment
    // HYB: [NV][NN] blended flux at the node's left interface; written once the node phase has read
    // the pair fluxes, so it reuses their space when that is large enough
    constexpr bool FB_IN_PAIRS = NPTX >= NN;
    double* sFb = FB_IN_PAIRS ? spair : sH + (HYB ? NV * NN : 0);
    uint8_t* stab = (uint8_t*)(sH + (HYB ? (FB_IN_PAIRS ? 1 : 2) * NV * NN : 0));   // pair table: a, b
    const int tid = threadIdx.x;
    for (int t = tid; t < S::NOPS; t += blockDim.x) {
        double v = P.ops[t];
        // the diagonal of D♯ carries the pair scale (F♯(i, i) = F̃_i is not computed as a pair)
        if (t >= N * N && t < 2 * N * N && (t - N * N) % (N + 1) == 0) v = PairScale<EQ, TP, CURV>::value * v;
        sops[t] = v;
    }
    if (tid == 0) {
        int c = 0;
        for (int a = 0; a < N; ++a)
            for (int b = a + 1; b < N; ++b) { stab[2 * c] = (uint8_t)a; stab[2 * c + 1] = (uint8_t)b; ++c; }
    }
    const int el = tid / NPE, i = tid - el * NPE;
    const int e = e0 + el;
    const bool active = (tid < NN) && (e < P.nelem);
    const double g = P.gamma;
    double q[NV];
    double v[EULER ? DIM : 1];
    double p = 0.0, qe = 0.0;   // pressure, ρe + p
    if (active) {
        int64_t gi = (int64_t)e * NPE + i;
#pragma unroll
        for (int k = 0; k < NV; ++k) q[k] = P.Q[k * P.ndofs + gi];
        if (EULER) {
            double ir = rcp_refined(q[0]);
            double ke = 0.0;
#pragma unroll
            for (int k = 0; k < DIM; ++k) {
                v[k] = q[1 + k] * ir;
                ke = fma(q[1 + k], v[k], ke);
            }
            p = (g - 1.0) * fma(-0.5, ke, q[DIM + 1]);
            qe = q[DIM + 1] + p;
            if (!(q[0] > 0.0 && p > 0.0)) raise_nonphysical(P.status, e);
            if constexpr (HYB || GAUSS) {   // vars_cons2entropy, FlouCommon/Euler.jl:273-307
                double ip = rcp_refined(p);
                double sv = log(p) - g * log(q[0]);
                sW[tid] = (g - sv) * rcp_refined(g - 1.0) - ke * ip * 0.5;
#pragma unroll
                for (int k = 0; k < DIM; ++k) sW[(1 + k) * NN + tid] = q[1 + k] * ip;
                sW[(DIM + 1) * NN + tid] = -q[0] * ip;
            }
            if constexpr (EULER) store_split_node<DIM, TP>(sprim, SST, tid, q, v, p, ir);
        } else {
            sprim[tid] = q[0];
        }
    }
    __syncthreads();
    double dq[NV];
#pragma unroll
    for (int k = 0; k < NV; ++k) dq[k] = 0.0;
    const double* Dsh = sops + N * N;
    const double c_g = 1.0 / (g - 1.0);
#pragma unroll 1
    for (int dir = 0; dir < DIM; ++dir) {
        double fls[NV], frs[NV];   // GAUSS && HYB: this element's side values of its line's face fluxes
        if constexpr (GAUSS) {   // entropy-projected states at both ends of every line (OpDivergence.jl:405-409)
            for (int t = tid; t < NPROJ; t += blockDim.x) {
                int elp = t / (2 * NFD);
                if (e0 + elp >= P.nelem) continue;
                int rr = t - elp * 2 * NFD, line = rr >> 1, side = rr & 1;
                const double* lv = sops + 2 * N * N + side * N;
                double w[NV];
#pragma unroll
                for (int k = 0; k < NV; ++k) w[k] = 0.0;
                for (int pos = 0; pos < N; ++pos) {
                    int j = elp * NPE + tp_node<DIM>(N, dir, line, pos);
#pragma unroll
                    for (int k = 0; k < NV; ++k) w[k] = fma(lv[pos], sW[k * NN + j], w[k]);
                }
                // vars_entropy2prim, FlouCommon/Euler.jl:309-334, then vars_prim2cons
                double wl = w[DIM + 1], iwl = rcp_refined(wl);
                double vp[DIM], qp[NV], vv = 0.0;
#pragma unroll
                for (int k = 0; k < DIM; ++k) {
                    vp[k] = -w[1 + k] * iwl;
                    vv = fma(vp[k], vp[k], vv);
                }
                double sv = g - (g - 1.0) * (w[0] - wl * vv * 0.5);
                // ((-W_last)^γ e^s)^(1/(1-γ)) as one exponential
                const double ig1 = rcp_refined(g - 1.0);
                double pp = exp(-fma(g, log(-wl), sv) * ig1);
                double rho = -pp * wl;
                qp[0] = rho;
#pragma unroll
                for (int k = 0; k < DIM; ++k) qp[1 + k] = rho * vp[k];
                qp[DIM + 1] = fma(pp, ig1, 0.5 * rho * vv);
                if (!(rho > 0.0 && pp > 0.0)) raise_nonphysical(P.status, e0 + elp);
                store_split_node<DIM, TP>(sprim, SST, NN + t, qp, vp, pp, rcp_refined(rho));
                if constexpr (CURV) {   // the line end's subcell interface: n·Js (OpDivergence.jl:403-404)
                    const int64_t ns = (int64_t)P.nelem * DIM * NFD * (N + 1);
                    const int64_t si = (((int64_t)(e0 + elp) * DIM + dir) * NFD + line) * (N + 1) + (side ? N : 0);
                    const double js = P.subJ[si];
#pragma unroll
                    for (int k = 0; k < DIM; ++k) sJa[k * SST + NN + t] = P.subfr[k * ns + si] * js;
                }
            }
            __syncthreads();
        }
        if (CURV) {   // this direction's metric column Ja[:, dir] of every node of the block
            if (active) {
                int64_t g = (int64_t)e * NPE + i;
#pragma unroll
                for (int k = 0; k < DIM; ++k) sJa[k * SST + tid] = P.Jan[(k + dir * DIM) * P.ndofs + g];
            }
            __syncthreads();
        }
        // ---- pair phase: every symmetric two-point flux of the block, once (GAUSS: then every
        // node with both projected states of its line) ----
        for (int kp = tid; kp < NPTX; kp += blockDim.x) {
            int elp, ia, ib;
            if (kp < NPT) {
                elp = kp / (NFD * NPAIR);
                int r = kp - elp * (NFD * NPAIR);
                int line = r / NPAIR, pr = r - line * NPAIR;
                if (e0 + elp >= P.nelem) continue;
                int a = stab[2 * pr], b = stab[2 * pr + 1];
                ia = elp * NPE + tp_node<DIM>(N, dir, line, a);
                ib = elp * NPE + tp_node<DIM>(N, dir, line, b);
            } else {   // x = 2 (N (elp NFD + line) + pos) + side
                int x = kp - NPT, side = x & 1, rest = x >> 1;
                int pos = rest % N, ln = rest / N;
                elp = ln / NFD;
                if (e0 + elp >= P.nelem) continue;
                ia = elp * NPE + tp_node<DIM>(N, dir, ln - elp * NFD, pos);
                ib = NN + 2 * ln + side;
            }
            double F[NV];
            double nv[DIM];   // CURV: twice the averaged metric column, Ja_a + Ja_b (the pair scale)
            if (CURV) {
#pragma unroll
                for (int k = 0; k < DIM; ++k) nv[k] = sJa[k * SST + ia] + sJa[k * SST + ib];
            }
            if constexpr (CURV && EULER) {
                if (TP == FLOU_TP_CHANDRASHEKAR) {
                    chandrashekar_pair<DIM, true>(sprim, SST, ia, ib, dir, c_g, F, nv);
                } else if (TP == FLOU_TP_KENNEDY_GRUBER) {
                    const double* vh = sprim + SST;
                    double rho = sprim[ia] + sprim[ib];
                    double pm = sprim[(1 + DIM) * SST + ia] + sprim[(1 + DIM) * SST + ib];
                    double en = sprim[(2 + DIM) * SST + ia] + sprim[(2 + DIM) * SST + ib];
                    double vm[DIM], vn = 0.0;
#pragma unroll
                    for (int k = 0; k < DIM; ++k) {
                        vm[k] = vh[k * SST + ia] + vh[k * SST + ib];
                        vn = fma(vm[k], nv[k], vn);
                    }
                    double m = rho * vn;
                    F[0] = m;
#pragma unroll
                    for (int k = 0; k < DIM; ++k) F[1 + k] = fma(m, vm[k], pm * nv[k]);
                    F[DIM + 1] = fma(m, en, pm * vn);
                } else {   // StdAverage: the mean of the two contravariant fluxes
                    const double* sq = sprim + (DIM + 1) * SST;
                    double v1 = 0.0, v2 = 0.0, m1 = 0.0, m2 = 0.0;
#pragma unroll
                    for (int k = 0; k < DIM; ++k) {
                        v1 = fma(sprim[k * SST + ia], nv[k], v1);
                        v2 = fma(sprim[k * SST + ib], nv[k], v2);
                        m1 = fma(sq[(1 + k) * SST + ia], nv[k], m1);
                        m2 = fma(sq[(1 + k) * SST + ib], nv[k], m2);
                    }
                    double p1 = sprim[DIM * SST + ia], p2 = sprim[DIM * SST + ib];
                    F[0] = (m1 + m2) * 0.5;
#pragma unroll
                    for (int k = 0; k < DIM; ++k)
                        F[1 + k] = (fma(sq[(1 + k) * SST + ia], v1, p1 * nv[k]) + fma(sq[(1 + k) * SST + ib], v2, p2 * nv[k])) * 0.5;
                    F[DIM + 1] = ((sq[(DIM + 1) * SST + ia] + p1) * v1 + (sq[(DIM + 1) * SST + ib] + p2) * v2) * 0.5;
                }
            } else if constexpr (CURV) {   // linear advection (LinearAdvection.jl:44-47)
                double an = 0.0;
#pragma unroll
                for (int k = 0; k < DIM; ++k) an = fma(P.adv[k], nv[k], an);
                F[0] = an * (sprim[ia] + sprim[ib]) * 0.5;
            } else if (EULER) {
                if (TP == FLOU_TP_CHANDRASHEKAR) {
                    chandrashekar_pair<DIM>(sprim, SST, ia, ib, dir, c_g, F);
                } else if (TP == FLOU_TP_KENNEDY_GRUBER) {   // Kennedy & Gruber (2008)
                    const double* vh = sprim + SST;
                    double rho = sprim[ia] + sprim[ib];
                    double pm = sprim[(1 + DIM) * SST + ia] + sprim[(1 + DIM) * SST + ib];
                    double en = sprim[(2 + DIM) * SST + ia] + sprim[(2 + DIM) * SST + ib];
                    double vd = vh[dir * SST + ia] + vh[dir * SST + ib];
                    double m = rho * vd;
                    F[0] = m;
#pragma unroll
                    for (int k = 0; k < DIM; ++k) F[1 + k] = m * (vh[k * SST + ia] + vh[k * SST + ib]);
                    F[1 + dir] = F[1 + dir] + pm;
                    F[DIM + 1] = fma(m, en, pm * vd);
                } else {   // StdAverage two-point flux, Euler.jl:385-472
                    const double* sq = sprim + (DIM + 1) * SST;
                    double v1 = sprim[dir * SST + ia], v2 = sprim[dir * SST + ib];
                    double p1 = sprim[DIM * SST + ia], p2 = sprim[DIM * SST + ib];
                    F[0] = (sq[(1 + dir) * SST + ia] + sq[(1 + dir) * SST + ib]) * 0.5;
#pragma unroll
                    for (int k = 0; k < DIM; ++k) {
                        double m1 = sq[(1 + k) * SST + ia] * v1, m2 = sq[(1 + k) * SST + ib] * v2;
                        F[1 + k] = (k == dir) ? (((m1 + p1) + m2) + p2) * 0.5 : (m1 + m2) * 0.5;
                    }
                    F[DIM + 1] = ((sq[(DIM + 1) * SST + ia] + p1) * v1 + (sq[(DIM + 1) * SST + ib] + p2) * v2) * 0.5;
                }
            } else if (EQ == FLOU_EQ_LINEAR_ADVECTION) {
                F[0] = P.adv[dir] * (sprim[ia] + sprim[ib]) * 0.5;
            } else {
                F[0] = (sprim[ia] * sprim[ia] + sprim[ib] * sprim[ib]) * 0.25;
            }
#pragma unroll
            for (int k = 0; k < NV; ++k) spair[k * NPTX + kp] = F[k];
        }
        __syncthreads();
        if constexpr (GAUSS) {   // l·F♯(·, Q̃_l) and r·F♯(·, Q̃_r) once per line, into the projected columns
            for (int t = tid; t < NPROJ; t += blockDim.x) {
                int elp = t / (2 * NFD);
                if (e0 + elp >= P.nelem) continue;
                int rr = t - elp * 2 * NFD, side = rr & 1;
                const double* lv = sops + 2 * N * N + side * N;
                const int xb = NPT + 2 * N * (elp * NFD + (rr >> 1)) + side;
                double acc[NV];
#pragma unroll
                for (int k = 0; k < NV; ++k) acc[k] = 0.0;
#pragma unroll
                for (int j = 0; j < N; ++j) {
#pragma unroll
                    for (int k = 0; k < NV; ++k) acc[k] = fma(lv[j], spair[k * NPTX + xb + 2 * j], acc[k]);
                }
#pragma unroll
                for (int k = 0; k < NV; ++k) sprim[k * SST + NN + t] = acc[k];
            }
            __syncthreads();
        }
        // ---- node phase: dQ_i -= Ja_dd sum_j D♯_ij F♯(i, j) ----
        if (active) {
            int pos, line;
            tp_coords<DIM>(N, i, dir, pos, line);
            // F♯(i, i): the physical flux along dir (CURV: the contravariant flux).  Its weight D♯_ii
            // vanishes for an exact SBP operator, but the computed diagonal carries the round-off
            // that keeps the rows of D♯ summing to zero: dropping it loses discrete conservation
            // against a large constant pressure (the TGV's p0 = 1/(γM²)).
            // The diagonal of D♯ in shared memory already carries the pair scale.
            const double ad = Dsh[pos + pos * N];
            double acc[NV];
            if constexpr (CURV) {
                double an = 0.0, mn = 0.0, vn = 0.0;
#pragma unroll
                for (int k = 0; k < DIM; ++k) {
                    double a = sJa[k * SST + tid];
                    if constexpr (EULER) {
                        mn = fma(q[1 + k], a, mn);
                        vn = fma(v[k], a, vn);
                    } else {
                        an = fma(P.adv[k], a, an);
                    }
                }
                if constexpr (EULER) {
                    acc[0] = ad * mn;
#pragma unroll
                    for (int k = 0; k < DIM; ++k) acc[1 + k] = ad * fma(q[1 + k], vn, p * sJa[k * SST + tid]);
                    acc[DIM + 1] = ad * ((q[DIM + 1] + p) * vn);
                } else {
                    acc[0] = ad * (an * q[0]);
                }
            } else if constexpr (EULER) {
                // D♯_ii F̃_i = D♯_ii (m_d, m_d v + p e_d, (ρe + p) v_d) with the common factors
                // taken once (the pressure as a selected FMA addend, not a predicated update).
                // When D♯_ii is round-off (an SBP operator: DGSEM on Gauss-Lobatto nodes) the term
                // only completes the computed row sums of D♯ against the large fluxes, the pressure
                // and the enthalpy flux; the density and convective parts, D♯_ii m_d and
                // D♯_ii m_d v, are smaller than the pressure part by ρ|v|²/p, and with a round-off
                // weight they fall below the rounding of the terms kept, so they are left out.
                const double adp = ad * p;
                if (P.diag_roundoff) {
                    acc[0] = 0.0;
#pragma unroll
                    for (int k = 0; k < DIM; ++k) acc[1 + k] = k == dir ? adp : 0.0;
                } else {
                    const double aq = ad * q[1 + dir];
                    acc[0] = aq;
#pragma unroll
                    for (int k = 0; k < DIM; ++k) acc[1 + k] = fma(aq, v[k], k == dir ? adp : 0.0);
                }
                acc[DIM + 1] = (ad * qe) * v[dir];
            } else if constexpr (EQ == FLOU_EQ_LINEAR_ADVECTION) {
                acc[0] = ad * (P.adv[dir] * q[0]);
            } else {
                acc[0] = ad * (q[0] * q[0] / 2.0);
            }
            // the N-1 other nodes of the line, from pos+1 on cyclically: every iteration is a pair
            // (a loop over all j that skipped j = pos would still spend the FP64 issue slots of
            // the skipped iteration, as predicated-off instructions)
            int pbase = el * NFD * NPAIR + line * NPAIR;
#pragma unroll
            for (int r = 1; r < N; ++r) {
                const int j = pos + r < N ? pos + r : pos + r - N;
                const double a = Dsh[pos + j * N];
                int lo = j < pos ? j : pos, hi = j < pos ? pos : j;
                int pidx = pbase + lo * (2 * N - lo - 1) / 2 + (hi - lo - 1);
#pragma unroll
                for (int k = 0; k < NV; ++k) acc[k] = fma(a, spair[k * NPTX + pidx], acc[k]);
            }
            // CURV: the metric is in the fluxes; the pair scale comes off with it
            double Ja = (CURV ? 1.0 : P.elem_Ja[e * DIM + dir]) * (1.0 / PairScale<EQ, TP, CURV>::value);
            double Fl[NV], Fr[NV];   // GAUSS: F♯(Q_i, Q̃) - l·F♯(·, Q̃) at both ends (OpDivergence.jl:410-425)
            if constexpr (GAUSS) {
                const int xb = NPT + 2 * N * (el * NFD + line);
                const int cl = NN + 2 * (el * NFD + line);   // the line's reductions, left and right
#pragma unroll
                for (int k = 0; k < NV; ++k) {
                    Fl[k] = spair[k * NPTX + xb + 2 * pos] - sprim[k * SST + cl];
                    Fr[k] = spair[k * NPTX + xb + 2 * pos + 1] - sprim[k * SST + cl + 1];
                }
            }
            if constexpr (HYB) {
                double w = P.omega1[pos] * Ja;
                if constexpr (GAUSS) {   // F̄_{p+1} - F̄_p, OpDivergence.jl:747-751
                    const double* lvl = sops + 2 * N * N;
                    const double* lvr = lvl + N;
                    int32_t pl = P.elem_face[e * 2 * DIM + 2 * dir], pr = P.elem_face[e * 2 * DIM + 2 * dir + 1];
                    double sl = (pl & 1) ? -1.0 : 1.0, sr = (pr & 1) ? -1.0 : 1.0;
                    int linel = line, liner = line;   // CURV: a slave side reads through the orientation
                    if (CURV) {
                        if (pl & 1) linel = master2slave<DIM>(line, inverse_orientation<DIM>(P.orient[pl >> 1]), N);
                        if (pr & 1) liner = master2slave<DIM>(line, inverse_orientation<DIM>(P.orient[pr >> 1]), N);
                    }
                    int64_t ol = (int64_t)(pl >> 1) * NFD + linel, orr = (int64_t)(pr >> 1) * NFD + liner;
#pragma unroll
                    for (int k = 0; k < NV; ++k) {
                        fls[k] = sl * __ldcg(P.Fn + k * P.nfdofs + ol);
                        frs[k] = sr * __ldcg(P.Fn + k * P.nfdofs + orr);
                        sH[k * NN + tid] = w * acc[k] - lvl[pos] * fma(Ja, Fl[k], -fls[k]) +
                                           lvr[pos] * fma(Ja, Fr[k], frs[k]);
                    }
                } else {
#pragma unroll
                    for (int k = 0; k < NV; ++k) sH[k * NN + tid] = w * acc[k];
                }
            } else {
                if constexpr (GAUSS) {
                    const double* dgl = sops + 2 * N * N + 2 * N;
                    const double* dgr = dgl + N;
#pragma unroll
                    for (int k = 0; k < NV; ++k) acc[k] = acc[k] - (dgl[pos] * Fl[k] - dgr[pos] * Fr[k]);
                }
#pragma unroll
                for (int k = 0; k < NV; ++k) dq[k] = fma(-Ja, acc[k], dq[k]);
            }
        }
        if constexpr (HYB && EULER) {
            __syncthreads();
            if constexpr (!GAUSS) {
                // F̄_p = Σ_{r<p} increment_r: exclusive prefix sums along each line, in place, one
                // thread per line (the same order of additions as a sum from r = 0; a sum per node
                // would repeat the additions and diverge within warps on its trip count)
                for (int t = tid; t < S::EPB * NFD; t += blockDim.x) {
                    const int elp = t / NFD, ln = t - elp * NFD;
                    if (e0 + elp >= P.nelem) continue;
                    double run[NV];
#pragma unroll
                    for (int k = 0; k < NV; ++k) run[k] = 0.0;
                    for (int pp = 0; pp < N; ++pp) {
                        const int j = elp * NPE + tp_node<DIM>(N, dir, ln, pp);
#pragma unroll
                        for (int k = 0; k < NV; ++k) {
                            const double x = sH[k * NN + j];
                            sH[k * NN + j] = run[k];
                            run[k] += x;
                        }
                    }
                }
                __syncthreads();
            }
            // One thread per subcell interface (between positions pos-1 and pos, pos = 1..N-1), the
            // block's interfaces numbered consecutively: the threads beyond them (one in N) leave
            // whole warps idle instead of one lane in every warp.  The result goes to the slot of
            // the interface's right node.
            constexpr int NFV = S::EPB * NFD * (N - 1);
            for (int t = tid; t < NFV; t += blockDim.x) {
                const int elp = t / (NFD * (N - 1));
                const int rr = t - elp * (NFD * (N - 1));
                const int line = rr / (N - 1), pos = 1 + (rr - line * (N - 1));
                const int ef = e0 + elp;
                if (ef >= P.nelem) continue;
                const int jn = elp * NPE + tp_node<DIM>(N, dir, line, pos);
                const int il = elp * NPE + tp_node<DIM>(N, dir, line, pos - 1);
                double Fh[NV];
#pragma unroll
                for (int k = 0; k < NV; ++k) Fh[k] = GAUSS ? 0.0 : sH[k * NN + jn];
                // FV flux in the subcell interface's frame times its surface Jacobian
                // (PhysicalRegions.jl:68-300): the positive axis and Ja_dd on a Cartesian
                // element, the uploaded subgrid geometry on a general one
                double ql[NV], qr[NV], a[NV], b[NV], Fr[NV], Fv[NV];
                const int64_t gl = (int64_t)e0 * NPE + il, gr = (int64_t)e0 * NPE + jn;
#pragma unroll
                for (int k = 0; k < NV; ++k) {
                    ql[k] = P.Q[k * P.ndofs + gl];
                    qr[k] = P.Q[k * P.ndofs + gr];
                }
                if constexpr (CURV) {
                    const int64_t ns = (int64_t)P.nelem * DIM * NFD * (N + 1);
                    const int64_t si = (((int64_t)ef * DIM + dir) * NFD + line) * (N + 1) + pos;
                    FrameTab fr;
#pragma unroll
                    for (int r = 0; r < 3; ++r) {
                        fr.n[r] = P.subfr[r * ns + si];
                        fr.t[r] = P.subfr[(3 + r) * ns + si];
                        fr.b[r] = P.subfr[(6 + r) * ns + si];
                    }
                    rotate_to_face<DIM>(ql, fr, a);
                    rotate_to_face<DIM>(qr, fr, b);
                    euler_numflux<DIM>(a, b, P.fvflux, P.fvavg, P.fvintensity, g, Fr);
                    rotate_to_phys<DIM>(Fr, fr, Fv);
                    const double Js = P.subJ[si];
#pragma unroll
                    for (int k = 0; k < NV; ++k) Fv[k] = Fv[k] * Js;
                } else {
                    FrameAxes A = frame_axes<DIM>(2 * dir + 1);
                    a[0] = ql[0]; b[0] = qr[0]; a[DIM + 1] = ql[DIM + 1]; b[DIM + 1] = qr[DIM + 1];
                    cart_to_face<DIM>(ql, A, a);
                    cart_to_face<DIM>(qr, A, b);
                    euler_numflux<DIM>(a, b, P.fvflux, P.fvavg, P.fvintensity, g, Fr);
                    const double Js = P.elem_Ja[ef * DIM + dir];
                    Fv[0] = Fr[0] * Js;
                    Fv[DIM + 1] = Fr[DIM + 1] * Js;
                    cart_to_phys<DIM>(Fr, A, Fv);
#pragma unroll
                    for (int k = 0; k < DIM; ++k) Fv[1 + k] = Fv[1 + k] * Js;
                }
                if constexpr (GAUSS) {   // blended in the scan below
#pragma unroll
                    for (int k = 0; k < NV; ++k) sFb[k * NN + jn] = Fv[k];
                } else {
                    double bb = 0.0;
#pragma unroll
                    for (int k = 0; k < NV; ++k) bb = fma(sW[k * NN + jn] - sW[k * NN + il], Fh[k] - Fv[k], bb);
                    double dl = sqrt_refined(fma(bb, bb, P.blend));
                    dl = fmax((dl - bb) * rcp_refined(dl), 0.5);
#pragma unroll
                    for (int k = 0; k < NV; ++k) sFb[k * NN + jn] = fma(dl, Fh[k] - Fv[k], Fv[k]);
                }
            }
            __syncthreads();
            if constexpr (GAUSS) {
                // On Gauss nodes each subcell flux starts from the blended one before it
                // (OpDivergence.jl:741-769): F̄_1 = -Fn_left, F̄_{p+1} = blend(F̄_p + increment_p).
                // One thread per line runs the scan over the FV fluxes left in sFb.
                if (active) {
                    int pos, line;
                    tp_coords<DIM>(N, i, dir, pos, line);
                    if (pos == 0) {
                        double Fb[NV];
#pragma unroll
                        for (int k = 0; k < NV; ++k) Fb[k] = -fls[k];
                        int jp = tid;
                        for (int pp = 1; pp < N; ++pp) {
                            const int jn = el * NPE + tp_node<DIM>(N, dir, line, pp);
                            double bb = 0.0;
#pragma unroll
                            for (int k = 0; k < NV; ++k) {
                                Fb[k] += sH[k * NN + jp];
                                bb = fma(sW[k * NN + jn] - sW[k * NN + jp], Fb[k] - sFb[k * NN + jn], bb);
                            }
                            double dl = sqrt_refined(fma(bb, bb, P.blend));
                            dl = fmax((dl - bb) * rcp_refined(dl), 0.5);
#pragma unroll
                            for (int k = 0; k < NV; ++k) {
                                double fv = sFb[k * NN + jn];
                                Fb[k] = fma(dl, Fb[k] - fv, fv);
                                sFb[k * NN + jn] = Fb[k];
                            }
                            jp = jn;
                        }
                    }
                }
                __syncthreads();
            }
            if (active) {
                int pos, line;
                tp_coords<DIM>(N, i, dir, pos, line);
                double iw = rcp_refined(P.omega1[pos]);
                int jr = (pos < N - 1) ? el * NPE + tp_node<DIM>(N, dir, line, pos + 1) : -1;
#pragma unroll
                for (int k = 0; k < NV; ++k) {   // GAUSS: the element's face fluxes close both ends
                    double fl = pos > 0 ? sFb[k * NN + tid] : (GAUSS ? -fls[k] : 0.0);
                    double fr = jr >= 0 ? sFb[k * NN + jr] : (GAUSS ? frs[k] : 0.0);
                    dq[k] += (fl - fr) * iw;
                }
            }
        }
        __syncthreads();
    }
    if (active) surface_and_update<DIM, N, NV, LGL, CURV, !(GAUSS && HYB)>(P, sops, e, i, q, dq);
}

// Register cap of the plain 3D split-form kernels: resident blocks per SM = 64K / (BLOCK * cap).
// 64 registers (a few spilled words) measured 1.5% faster at p = 7 and 0.6% at p = 3 than the
// compiler's 101; the hybrid, Gauss-node and curvilinear variants keep their registers.
#ifndef FLOU_SPLIT_REGCAP
#define FLOU_SPLIT_REGCAP 64
#endif
template <int BLOCK, bool CAPPED>
constexpr int split_min_blocks() {
    return CAPPED && FLOU_SPLIT_REGCAP > 0 && 65536 / (BLOCK * FLOU_SPLIT_REGCAP) > 1
               ? 65536 / (BLOCK * FLOU_SPLIT_REGCAP) : 1;
}

template <int DIM, int N, int EQ, int TP, bool LGL, bool CURV = false, bool HYB = false>
__global__ void __launch_bounds__(Shape<DIM, N>::BLOCK,
                                  split_min_blocks<Shape<DIM, N>::BLOCK, DIM == 3 && LGL && !CURV && !HYB>())
    elem_split_kernel(ElemParams P) {
    extern __shared__ double smem[];
    if (P.dtp && *P.dtp == 0.0) return;   // CFL stepping past tfinal: the state stays as it is
    split_tile<DIM, N, EQ, TP, LGL, 256, CURV, HYB>(P, blockIdx.x * Shape<DIM, N>::EPB, smem);
}

template <int DIM, int N, int EQ, int VOL, int TP, int TB = 256, bool CURV = false, bool LGL = true>
constexpr size_t elem_smem_bytes() {
    using S = Shape<DIM, N, TB>;
    constexpr int NV = (EQ == FLOU_EQ_EULER) ? DIM + 2 : 1;
    if (VOL == FLOU_OP_STRONG) return sizeof(double) * (S::NOPS + DIM * NV * S::NN);
    constexpr int NARR = SplitLayout<DIM, EQ, TP>::NARR;
    constexpr int NPT = S::EPB * S::NFD * S::NPAIR;
    constexpr bool GAUSS = !LGL && EQ == FLOU_EQ_EULER;
    constexpr int NPROJ = GAUSS ? 2 * S::EPB * S::NFD : 0;
    constexpr bool HYB = VOL == FLOU_OP_HYBRID;
    constexpr int NPTX = NPT + NPROJ * N;
    return sizeof(double) * (S::NOPS + NARR * (S::NN + NPROJ) + NV * NPTX + (CURV ? DIM * (S::NN + NPROJ) : 0) +
                             (HYB ? (NPTX >= S::NN ? 2 : 3) * NV * S::NN : (GAUSS ? NV * S::NN : 0))) +
           2 * (S::NPAIR + 1);
}

// Launch one instantiation; the dynamic shared-memory opt-in is set once per kernel.
// With `prepare` set only the opt-in is made (it must precede stream capture).
template <int DIM, int N, int EQ, int VOL, int TP, bool LGL, bool CURV = false>
cudaError_t launch_elem_one(const ElemParams& P, cudaStream_t s, bool prepare) {
    using S = Shape<DIM, N>;
    constexpr size_t smem = elem_smem_bytes<DIM, N, EQ, VOL, TP, 256, CURV, LGL>();
    static_assert(smem <= 227 * 1024, "element tile exceeds the shared memory of one block");
    static bool attr_set = false;
    int grid = (P.nelem + S::EPB - 1) / S::EPB;
    auto k = (VOL == FLOU_OP_STRONG) ? (void (*)(ElemParams))elem_strong_kernel<DIM, N, EQ, LGL, CURV>
                                     : (void (*)(ElemParams))elem_split_kernel<DIM, N, EQ, TP, LGL, CURV,
                                                                               VOL == FLOU_OP_HYBRID>;
    if (!attr_set) {
        cudaError_t err = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (err != cudaSuccess) return err;
        attr_set = true;
    }
    if (prepare || grid == 0) return cudaSuccess;
    k<<<grid, S::BLOCK, smem, s>>>(P);
    return cudaGetLastError();
}

// All volume variants of one (dim, N, equation): strong (LGL or general basis) and split
// (LGL only, one kernel per two-point flux).
// VSEL >= 0 instantiates only that volume operator (one translation unit per operator).
template <int DIM, int N, int EQ, int VSEL = -1>
cudaError_t launch_elem_n(int vol, int tp, bool lgl, const ElemParams& P, cudaStream_t s, bool prep) {
    if (VSEL >= 0 && vol != VSEL) return cudaErrorInvalidValue;
    if (vol == FLOU_OP_STRONG) {
        if constexpr (VSEL < 0 || VSEL == FLOU_OP_STRONG)
            return lgl ? launch_elem_one<DIM, N, EQ, FLOU_OP_STRONG, 0, true>(P, s, prep)
                       : launch_elem_one<DIM, N, EQ, FLOU_OP_STRONG, 0, false>(P, s, prep);
        return cudaErrorInvalidValue;
    }
    if (!lgl) return cudaErrorInvalidValue;
    if (vol == FLOU_OP_HYBRID) {
        if constexpr (EQ == FLOU_EQ_EULER && (VSEL < 0 || VSEL == FLOU_OP_HYBRID)) {
            switch (tp) {
                case FLOU_TP_STD_AVERAGE:
                    return launch_elem_one<DIM, N, EQ, FLOU_OP_HYBRID, FLOU_TP_STD_AVERAGE, true>(P, s, prep);
                case FLOU_TP_CHANDRASHEKAR:
                    return launch_elem_one<DIM, N, EQ, FLOU_OP_HYBRID, FLOU_TP_CHANDRASHEKAR, true>(P, s, prep);
                case FLOU_TP_KENNEDY_GRUBER:
                    return launch_elem_one<DIM, N, EQ, FLOU_OP_HYBRID, FLOU_TP_KENNEDY_GRUBER, true>(P, s, prep);
                default: return cudaErrorInvalidValue;
            }
        }
        return cudaErrorInvalidValue;
    }
    if constexpr (VSEL < 0 || VSEL == FLOU_OP_SPLIT) {
        if (EQ != FLOU_EQ_EULER)
            return launch_elem_one<DIM, N, EQ, FLOU_OP_SPLIT, FLOU_TP_STD_AVERAGE, true>(P, s, prep);
        switch (tp) {
            case FLOU_TP_STD_AVERAGE:
                return launch_elem_one<DIM, N, EQ, FLOU_OP_SPLIT, FLOU_TP_STD_AVERAGE, true>(P, s, prep);
            case FLOU_TP_CHANDRASHEKAR:
                return launch_elem_one<DIM, N, EQ, FLOU_OP_SPLIT, FLOU_TP_CHANDRASHEKAR, true>(P, s, prep);
            case FLOU_TP_KENNEDY_GRUBER:
                return launch_elem_one<DIM, N, EQ, FLOU_OP_SPLIT, FLOU_TP_KENNEDY_GRUBER, true>(P, s, prep);
            default: return cudaErrorInvalidValue;
        }
    }
    return cudaErrorInvalidValue;
}

template <int DIM, int EQ, int VSEL = -1>
cudaError_t launch_elem_dim(int n, int vol, int tp, bool lgl, const ElemParams& P, cudaStream_t s, bool prep) {
    switch (n) {
        case 2: return launch_elem_n<DIM, 2, EQ, VSEL>(vol, tp, lgl, P, s, prep);
        case 3: return launch_elem_n<DIM, 3, EQ, VSEL>(vol, tp, lgl, P, s, prep);
        case 4: return launch_elem_n<DIM, 4, EQ, VSEL>(vol, tp, lgl, P, s, prep);
        case 5: return launch_elem_n<DIM, 5, EQ, VSEL>(vol, tp, lgl, P, s, prep);
        case 6: return launch_elem_n<DIM, 6, EQ, VSEL>(vol, tp, lgl, P, s, prep);
        case 7: return launch_elem_n<DIM, 7, EQ, VSEL>(vol, tp, lgl, P, s, prep);
        case 8: return launch_elem_n<DIM, 8, EQ, VSEL>(vol, tp, lgl, P, s, prep);
        default: return cudaErrorInvalidValue;
    }
}

// Gauss-node split and hybrid variants (Euler, Cartesian), one per two-point flux.
template <int DIM, int N, int VOL>
cudaError_t launch_elem_gauss_n(int tp, const ElemParams& P, cudaStream_t s, bool prep) {
    switch (tp) {
        case FLOU_TP_STD_AVERAGE:
            return launch_elem_one<DIM, N, FLOU_EQ_EULER, VOL, FLOU_TP_STD_AVERAGE, false>(P, s, prep);
        case FLOU_TP_CHANDRASHEKAR:
            return launch_elem_one<DIM, N, FLOU_EQ_EULER, VOL, FLOU_TP_CHANDRASHEKAR, false>(P, s, prep);
        case FLOU_TP_KENNEDY_GRUBER:
            return launch_elem_one<DIM, N, FLOU_EQ_EULER, VOL, FLOU_TP_KENNEDY_GRUBER, false>(P, s, prep);
        default: return cudaErrorInvalidValue;
    }
}

template <int DIM, int VOL>
cudaError_t launch_elem_gauss_dim(int n, int tp, const ElemParams& P, cudaStream_t s, bool prep) {
    switch (n) {
        case 2: return launch_elem_gauss_n<DIM, 2, VOL>(tp, P, s, prep);
        case 3: return launch_elem_gauss_n<DIM, 3, VOL>(tp, P, s, prep);
        case 4: return launch_elem_gauss_n<DIM, 4, VOL>(tp, P, s, prep);
        case 5: return launch_elem_gauss_n<DIM, 5, VOL>(tp, P, s, prep);
        case 6: return launch_elem_gauss_n<DIM, 6, VOL>(tp, P, s, prep);
        case 7: return launch_elem_gauss_n<DIM, 7, VOL>(tp, P, s, prep);
        case 8: return launch_elem_gauss_n<DIM, 8, VOL>(tp, P, s, prep);
        default: return cudaErrorInvalidValue;
    }
}

// Curvilinear variants (LGL only): strong form and split form per two-point flux.
// The hybrid operator on general elements (Euler), one per two-point flux.
template <int DIM, int N>
cudaError_t launch_elem_n_curv_hybrid(int tp, const ElemParams& P, cudaStream_t s, bool prep) {
    switch (tp) {
        case FLOU_TP_STD_AVERAGE:
            return launch_elem_one<DIM, N, FLOU_EQ_EULER, FLOU_OP_HYBRID, FLOU_TP_STD_AVERAGE, true, true>(P, s, prep);
        case FLOU_TP_CHANDRASHEKAR:
            return launch_elem_one<DIM, N, FLOU_EQ_EULER, FLOU_OP_HYBRID, FLOU_TP_CHANDRASHEKAR, true, true>(P, s, prep);
        case FLOU_TP_KENNEDY_GRUBER:
            return launch_elem_one<DIM, N, FLOU_EQ_EULER, FLOU_OP_HYBRID, FLOU_TP_KENNEDY_GRUBER, true, true>(P, s, prep);
        default: return cudaErrorInvalidValue;
    }
}

template <int DIM>
cudaError_t launch_elem_dim_curv_hybrid(int n, int tp, const ElemParams& P, cudaStream_t s, bool prep) {
    switch (n) {
        case 2: return launch_elem_n_curv_hybrid<DIM, 2>(tp, P, s, prep);
        case 3: return launch_elem_n_curv_hybrid<DIM, 3>(tp, P, s, prep);
        case 4: return launch_elem_n_curv_hybrid<DIM, 4>(tp, P, s, prep);
        case 5: return launch_elem_n_curv_hybrid<DIM, 5>(tp, P, s, prep);
        case 6: return launch_elem_n_curv_hybrid<DIM, 6>(tp, P, s, prep);
        case 7: return launch_elem_n_curv_hybrid<DIM, 7>(tp, P, s, prep);
        case 8: return launch_elem_n_curv_hybrid<DIM, 8>(tp, P, s, prep);
        default: return cudaErrorInvalidValue;
    }
}

// General elements on a basis without boundary nodes: the strong form (any equation on this
// path) and the entropy-projected split and hybrid forms (Euler), one per two-point flux.
template <int DIM, int N, int EQ>
cudaError_t launch_elem_n_curv_gauss(int vol, int tp, const ElemParams& P, cudaStream_t s, bool prep) {
    if (vol == FLOU_OP_STRONG) return launch_elem_one<DIM, N, EQ, FLOU_OP_STRONG, 0, false, true>(P, s, prep);
    if constexpr (EQ == FLOU_EQ_EULER) {
#define FLOU_CG(VOL)                                                                                            \
        switch (tp) {                                                                                           \
            case FLOU_TP_STD_AVERAGE:                                                                           \
                return launch_elem_one<DIM, N, EQ, VOL, FLOU_TP_STD_AVERAGE, false, true>(P, s, prep);          \
            case FLOU_TP_CHANDRASHEKAR:                                                                         \
                return launch_elem_one<DIM, N, EQ, VOL, FLOU_TP_CHANDRASHEKAR, false, true>(P, s, prep);        \
            case FLOU_TP_KENNEDY_GRUBER:                                                                        \
                return launch_elem_one<DIM, N, EQ, VOL, FLOU_TP_KENNEDY_GRUBER, false, true>(P, s, prep);       \
            default: return cudaErrorInvalidValue;                                                              \
        }
        if (vol == FLOU_OP_SPLIT) { FLOU_CG(FLOU_OP_SPLIT) }
        if (vol == FLOU_OP_HYBRID) { FLOU_CG(FLOU_OP_HYBRID) }
#undef FLOU_CG
    }
    return cudaErrorInvalidValue;
}

template <int DIM, int EQ>
cudaError_t launch_elem_dim_curv_gauss(int n, int vol, int tp, const ElemParams& P, cudaStream_t s, bool prep) {
    switch (n) {
        case 2: return launch_elem_n_curv_gauss<DIM, 2, EQ>(vol, tp, P, s, prep);
        case 3: return launch_elem_n_curv_gauss<DIM, 3, EQ>(vol, tp, P, s, prep);
        case 4: return launch_elem_n_curv_gauss<DIM, 4, EQ>(vol, tp, P, s, prep);
        case 5: return launch_elem_n_curv_gauss<DIM, 5, EQ>(vol, tp, P, s, prep);
        case 6: return launch_elem_n_curv_gauss<DIM, 6, EQ>(vol, tp, P, s, prep);
        case 7: return launch_elem_n_curv_gauss<DIM, 7, EQ>(vol, tp, P, s, prep);
        case 8: return launch_elem_n_curv_gauss<DIM, 8, EQ>(vol, tp, P, s, prep);
        default: return cudaErrorInvalidValue;
    }
}

template <int DIM, int N, int EQ>
cudaError_t launch_elem_n_curv(int vol, int tp, const ElemParams& P, cudaStream_t s, bool prep) {
    if (vol == FLOU_OP_STRONG) return launch_elem_one<DIM, N, EQ, FLOU_OP_STRONG, 0, true, true>(P, s, prep);
    if (vol != FLOU_OP_SPLIT) return cudaErrorInvalidValue;
    if (EQ != FLOU_EQ_EULER)
        return launch_elem_one<DIM, N, EQ, FLOU_OP_SPLIT, FLOU_TP_STD_AVERAGE, true, true>(P, s, prep);
    switch (tp) {
        case FLOU_TP_STD_AVERAGE:
            return launch_elem_one<DIM, N, EQ, FLOU_OP_SPLIT, FLOU_TP_STD_AVERAGE, true, true>(P, s, prep);
        case FLOU_TP_CHANDRASHEKAR:
            return launch_elem_one<DIM, N, EQ, FLOU_OP_SPLIT, FLOU_TP_CHANDRASHEKAR, true, true>(P, s, prep);
        case FLOU_TP_KENNEDY_GRUBER:
            return launch_elem_one<DIM, N, EQ, FLOU_OP_SPLIT, FLOU_TP_KENNEDY_GRUBER, true, true>(P, s, prep);
        default: return cudaErrorInvalidValue;
    }
}

template <int DIM, int EQ>
cudaError_t launch_elem_dim_curv(int n, int vol, int tp, const ElemParams& P, cudaStream_t s, bool prep) {
    switch (n) {
        case 2: return launch_elem_n_curv<DIM, 2, EQ>(vol, tp, P, s, prep);
        case 3: return launch_elem_n_curv<DIM, 3, EQ>(vol, tp, P, s, prep);
        case 4: return launch_elem_n_curv<DIM, 4, EQ>(vol, tp, P, s, prep);
        case 5: return launch_elem_n_curv<DIM, 5, EQ>(vol, tp, P, s, prep);
        case 6: return launch_elem_n_curv<DIM, 6, EQ>(vol, tp, P, s, prep);
        case 7: return launch_elem_n_curv<DIM, 7, EQ>(vol, tp, P, s, prep);
        case 8: return launch_elem_n_curv<DIM, 8, EQ>(vol, tp, P, s, prep);
        default: return cudaErrorInvalidValue;
    }
}

// Host-side dispatch: one function per translation unit.
struct ElemLaunch {
    int dim, eq, n, vol, tp;
    bool lgl;
    bool prepare;   // only set the kernel's shared-memory opt-in, launch nothing
    bool curv;      // general geometry (the CURV kernels)
};
cudaError_t launch_elem_curv2d(const ElemLaunch& L, const ElemParams& P, cudaStream_t s);
cudaError_t launch_elem_curv3d(const ElemLaunch& L, const ElemParams& P, cudaStream_t s);
cudaError_t launch_face_curv(int dim, int eq, bool lgl, const FaceParams& P, cudaStream_t s);
cudaError_t launch_elem_euler1d(const ElemLaunch& L, const ElemParams& P, cudaStream_t s);
cudaError_t launch_elem_euler2d(const ElemLaunch& L, const ElemParams& P, cudaStream_t s);
cudaError_t launch_elem_euler3d_strong(const ElemLaunch& L, const ElemParams& P, cudaStream_t s);
cudaError_t launch_elem_euler3d_split(const ElemLaunch& L, const ElemParams& P, cudaStream_t s);
cudaError_t launch_elem_euler3d_hybrid(const ElemLaunch& L, const ElemParams& P, cudaStream_t s);
cudaError_t launch_elem_scalar(const ElemLaunch& L, const ElemParams& P, cudaStream_t s);
cudaError_t launch_elem_gauss1d(const ElemLaunch& L, const ElemParams& P, cudaStream_t s);
cudaError_t launch_elem_curv_hybrid2d(const ElemLaunch& L, const ElemParams& P, cudaStream_t s);
cudaError_t launch_elem_curv_gauss2d(const ElemLaunch& L, const ElemParams& P, cudaStream_t s);
cudaError_t launch_elem_curv_gauss3d(const ElemLaunch& L, const ElemParams& P, cudaStream_t s);
cudaError_t launch_elem_curv_hybrid3d(const ElemLaunch& L, const ElemParams& P, cudaStream_t s);
cudaError_t launch_elem_gauss2d(const ElemLaunch& L, const ElemParams& P, cudaStream_t s);
cudaError_t launch_elem_gauss3d_split(const ElemLaunch& L, const ElemParams& P, cudaStream_t s);
cudaError_t launch_elem_gauss3d_hybrid(const ElemLaunch& L, const ElemParams& P, cudaStream_t s);
cudaError_t launch_face(int dim, int eq, bool lgl, const FaceParams& P, cudaStream_t s);
cudaError_t launch_elem(const ElemLaunch& L, const ElemParams& P, cudaStream_t s);

}  // namespace flou
