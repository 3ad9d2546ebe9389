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
    int64_t ndofs, nfdofs;
    int32_t nfaces, n, npe, nfd;
    int32_t numflux, lxf_avg;
    double intensity, gamma;
    double adv[3];
    int32_t bc_kind[MAXBC];
    double bc_state[MAXBC][5];
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
    int32_t mode;                // 0: out = dQ; 1: out = U + dt dQ; 2: out = a0 U^n + a1 (U + dt dQ)
    double dt, a0, a1;
    double gamma;
    double adv[3];
    int32_t* status;             // [0] flags, [1] lowest offending element (1-based)
};

// Local face positions follow the reference's face order: 2*dir (left) and 2*dir+1
// (right); frames of a face are those of its master position (PhysicalRegions.jl:541-696).
struct FrameTab { double n[3], t[3], b[3]; };

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

// logarithmic_mean (src/FlouCommon/Utilities.jl:34-44) with the series of Ismail & Roe
// when u = ((a-b)/(a+b))² < 0.01, otherwise log(a/b)/(2f) -- evaluated here as in the
// reference (the face path is not the bottleneck).
__device__ __forceinline__ double logmean_ref(double al, double ar) {
    double xi = al / ar;
    double f = (xi - 1.0) / (xi + 1.0);
    double u = f * f;
    double F;
    if (u < 0.01) F = ((1.0 + u / 3.0) + (u * u) / 5.0) + (u * u * u) / 7.0;
    else F = log(xi) / (2.0 * f);
    return (al + ar) / (2.0 * F);
}

template <int DIM>
__device__ __forceinline__ void euler_face_flux(const double* ql, const double* qr, int kind, int lxf_avg,
                                                double intensity, double g, double* F) {
    constexpr int NV = DIM + 2;
    double rl = ql[0], rr = qr[0];
    double ul = ql[1] / rl, ur = qr[1] / rr;
    double pl = euler_pressure<DIM>(ql, g), pr = euler_pressure<DIM>(qr, g);
    auto stdavg = [&](double* A) {   // Euler.jl:99-136
        A[0] = (ql[1] + qr[1]) / 2.0;
        A[1] = (((ql[1] * ul + pl) + qr[1] * ur) + pr) / 2.0;
        for (int k = 1; k < DIM; ++k) A[1 + k] = (ql[1 + k] * ul + qr[1 + k] * ur) / 2.0;
        A[DIM + 1] = ((ql[DIM + 1] + pl) * ul + (qr[DIM + 1] + pr) * ur) / 2.0;
    };
    auto chandra = [&](double* A) {   // Euler.jl:167-226 (3D keeps the reference's wl² term)
        double vl[3] = {ul, DIM > 1 ? ql[2] / rl : 0.0, DIM > 2 ? ql[3] / rl : 0.0};
        double vr[3] = {ur, DIM > 1 ? qr[2] / rr : 0.0, DIM > 2 ? qr[3] / rr : 0.0};
        double u = (vl[0] + vr[0]) / 2.0, v = (vl[1] + vr[1]) / 2.0, w = (vl[2] + vr[2]) / 2.0;
        double bl = rl / (2.0 * pl), br = rr / (2.0 * pr);
        double rho = logmean_ref(rl, rr);
        double p = (rl + rr) / (2.0 * (bl + br));
        double beta = logmean_ref(bl, br);
        double s = vl[0] * vl[0];
        if (DIM > 1) s = s + vl[1] * vl[1];
        if (DIM > 2) s = s + vl[2] * vl[2];
        s = s + vr[0] * vr[0];
        if (DIM > 1) s = s + vr[1] * vr[1];
        if (DIM > 2) s = s + vl[2] * vl[2];
        double h = (1.0 / ((2.0 * beta) * (g - 1.0)) - s / 4.0) + p / rho;
        h = h + u * u;
        if (DIM > 1) h = h + v * v;
        if (DIM > 2) h = h + w * w;
        A[0] = rho * u;
        A[1] = rho * (u * u) + p;
        if (DIM > 1) A[2] = rho * u * v;
        if (DIM > 2) A[3] = rho * u * w;
        A[DIM + 1] = rho * u * h;
    };
    if (kind == FLOU_NF_STD_AVERAGE) { stdavg(F); return; }
    if (kind == FLOU_NF_CHANDRASHEKAR) { chandra(F); return; }
    if (kind == FLOU_NF_LXF) {   // Euler.jl:138-165
        double A[NV];
        if (lxf_avg == FLOU_NF_CHANDRASHEKAR) chandra(A); else stdavg(A);
        double al = sqrt(g * pl / rl), ar = sqrt(g * pr / rr);
        double lam = fmax(fabs(ul) + al, fabs(ur) + ar);
        for (int k = 0; k < NV; ++k) F[k] = A[k] + lam * (ql[k] - qr[k]) / 2.0 * intensity;
        return;
    }
    // HLL / HLLC (Toro 2009, eqs. 10.21 and 10.37-10.39; Davis wave-speed estimates).
    double al = sqrt(g * pl / rl), ar = sqrt(g * pr / rr);
    double sl = fmin(ul - al, ur - ar), sr = fmax(ul + al, ur + ar);
    double Fl[NV], Fr[NV];
    euler_normal_flux<DIM>(ql, ul, pl, Fl);
    euler_normal_flux<DIM>(qr, ur, pr, Fr);
    if (sl >= 0.0) { for (int k = 0; k < NV; ++k) F[k] = Fl[k]; return; }
    if (sr <= 0.0) { for (int k = 0; k < NV; ++k) F[k] = Fr[k]; return; }
    if (kind == FLOU_NF_HLL) {
        for (int k = 0; k < NV; ++k) F[k] = ((sr * Fl[k] - sl * Fr[k]) + (sl * sr) * (qr[k] - ql[k])) / (sr - sl);
        return;
    }
    double ml = rl * (sl - ul), mr = rr * (sr - ur);
    double ss = ((pr - pl) + ul * ml - ur * mr) / (ml - mr);
    bool left = ss >= 0.0;
    const double* qk = left ? ql : qr;
    const double* Fk = left ? Fl : Fr;
    double sk = left ? sl : sr, mk = left ? ml : mr, rk = left ? rl : rr, uk = left ? ul : ur, pk = left ? pl : pr;
    double coef = mk / (sk - ss);
    double Us[NV];
    Us[0] = coef;
    Us[1] = coef * ss;
    for (int k = 1; k < DIM; ++k) Us[1 + k] = coef * (qk[1 + k] / rk);
    Us[DIM + 1] = coef * (qk[DIM + 1] / rk + (ss - uk) * (ss + pk / mk));
    for (int k = 0; k < NV; ++k) F[k] = Fk[k] + sk * (Us[k] - qk[k]);
}

// ---------------------------------------------------------------------------------------
// Face kernel: traces (project2faces!, Interfaces.jl:51-109), boundary ghost states
// (applyBCs!, :25-49) and numerical fluxes times the surface Jacobian
// (interface_fluxes!, :111-136).  One thread per face node.
// ---------------------------------------------------------------------------------------
template <int DIM, int EQ, bool LGL>
__global__ void __launch_bounds__(256) face_kernel(FaceParams P) {
    constexpr int NV = (EQ == FLOU_EQ_EULER) ? DIM + 2 : 1;
    int64_t gid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (gid >= (int64_t)P.nfaces * P.nfd) return;
    int f = (int)(gid / P.nfd), m = (int)(gid - (int64_t)f * P.nfd);
    int n = P.n;
    int32_t s0 = P.face_elem[2 * f], s1 = P.face_elem[2 * f + 1];
    auto trace = [&](int32_t s, double* q) {
        int e = s >> 3, pos = s & 7, dir = pos >> 1, right = pos & 1;
        const double* Qe = P.Q + (int64_t)e * P.npe;
        if (LGL) {
            int node = tp_node<DIM>(n, dir, m, right ? n - 1 : 0);
            for (int k = 0; k < NV; ++k) q[k] = Qe[k * P.ndofs + node];
        } else {
            const double* lv = P.l + (right ? n : 0);
            for (int k = 0; k < NV; ++k) {
                double acc = 0.0;
                for (int p = 0; p < n; ++p) acc = acc + lv[p] * Qe[k * P.ndofs + tp_node<DIM>(n, dir, m, p)];
                q[k] = acc;
            }
        }
    };
    double ql[NV], qr[NV];
    trace(s0, ql);
    FrameTab fr = frame_of(DIM, s0 & 7);
    if (s1 >= 0) {
        trace(s1, qr);
    } else {
        int b = P.face_bc[f];
        int kind = P.bc_kind[b];
        if (kind == FLOU_BC_INFLOW) {
            for (int k = 0; k < NV; ++k) qr[k] = P.bc_state[b][k];
        } else if (kind == FLOU_BC_SLIP && EQ == FLOU_EQ_EULER) {
            // EulerSlipBC: rotate to the face frame, flip the normal momentum, rotate back.
            double mn = ql[1] * fr.n[0], mt = ql[1] * fr.t[0], mb = ql[1] * fr.b[0];
            if (DIM > 1) { mn = mn + ql[2] * fr.n[1]; mt = mt + ql[2] * fr.t[1]; mb = mb + ql[2] * fr.b[1]; }
            if (DIM > 2) { mn = mn + ql[3] * fr.n[2]; mt = mt + ql[3] * fr.t[2]; mb = mb + ql[3] * fr.b[2]; }
            mn = -mn;
            for (int k = 0; k < NV; ++k) qr[k] = ql[k];
            qr[1] = mn * fr.n[0] + mt * fr.t[0] + (DIM > 2 ? mb * fr.b[0] : 0.0);
            if (DIM > 1) qr[2] = mn * fr.n[1] + mt * fr.t[1] + (DIM > 2 ? mb * fr.b[1] : 0.0);
            if (DIM > 2) qr[3] = mn * fr.n[2] + mt * fr.t[2] + mb * fr.b[2];
            if (DIM == 1) qr[1] = mn * fr.n[0];
        } else {
            for (int k = 0; k < NV; ++k) qr[k] = ql[k];   // outflow
        }
    }
    double F[NV];
    double J = P.faceJ[f];
    if (EQ == FLOU_EQ_EULER) {
        // rotate2face (Euler.jl:16-64)
        double a[NV], b[NV];
        a[0] = ql[0]; b[0] = qr[0]; a[DIM + 1] = ql[DIM + 1]; b[DIM + 1] = qr[DIM + 1];
        if (DIM == 1) { a[1] = ql[1] * fr.n[0]; b[1] = qr[1] * fr.n[0]; }
        if (DIM == 2) {
            a[1] = ql[1] * fr.n[0] + ql[2] * fr.n[1]; a[2] = ql[1] * fr.t[0] + ql[2] * fr.t[1];
            b[1] = qr[1] * fr.n[0] + qr[2] * fr.n[1]; b[2] = qr[1] * fr.t[0] + qr[2] * fr.t[1];
        }
        if (DIM == 3) {
            a[1] = ql[1] * fr.n[0] + ql[2] * fr.n[1] + ql[3] * fr.n[2];
            a[2] = ql[1] * fr.t[0] + ql[2] * fr.t[1] + ql[3] * fr.t[2];
            a[3] = ql[1] * fr.b[0] + ql[2] * fr.b[1] + ql[3] * fr.b[2];
            b[1] = qr[1] * fr.n[0] + qr[2] * fr.n[1] + qr[3] * fr.n[2];
            b[2] = qr[1] * fr.t[0] + qr[2] * fr.t[1] + qr[3] * fr.t[2];
            b[3] = qr[1] * fr.b[0] + qr[2] * fr.b[1] + qr[3] * fr.b[2];
        }
        double Fr[NV];
        euler_face_flux<DIM>(a, b, P.numflux, P.lxf_avg, P.intensity, P.gamma, Fr);
        // rotate2phys
        F[0] = Fr[0]; F[DIM + 1] = Fr[DIM + 1];
        if (DIM == 1) F[1] = Fr[1] * fr.n[0];
        if (DIM == 2) {
            F[1] = Fr[1] * fr.n[0] + Fr[2] * fr.t[0];
            F[2] = Fr[1] * fr.n[1] + Fr[2] * fr.t[1];
        }
        if (DIM == 3) {
            F[1] = Fr[1] * fr.n[0] + Fr[2] * fr.t[0] + Fr[3] * fr.b[0];
            F[2] = Fr[1] * fr.n[1] + Fr[2] * fr.t[1] + Fr[3] * fr.b[1];
            F[3] = Fr[1] * fr.n[2] + Fr[2] * fr.t[2] + Fr[3] * fr.b[2];
        }
    } else if (EQ == FLOU_EQ_LINEAR_ADVECTION) {
        // LinearAdvection.jl:27-39
        double an = P.adv[0] * fr.n[0];
        if (DIM > 1) an = an + P.adv[1] * fr.n[1];
        if (DIM > 2) an = an + P.adv[2] * fr.n[2];
        F[0] = an * (ql[0] + qr[0]) / 2.0;
        if (P.numflux == FLOU_NF_LXF) F[0] = F[0] + fabs(an) * (ql[0] - qr[0]) / 2.0 * P.intensity;
    } else {
        // Burgers.jl:27-38
        F[0] = (ql[0] * ql[0] + qr[0] * qr[0]) / 4.0 * fr.n[0];
        if (P.numflux == FLOU_NF_LXF) {
            double lam = fmax(fabs(ql[0]), fabs(qr[0]));
            F[0] = F[0] + lam * (ql[0] - qr[0]) / 2.0 * P.intensity;
        }
    }
    int64_t o = (int64_t)f * P.nfd + m;
    for (int k = 0; k < NV; ++k) P.Fn[k * P.nfdofs + o] = F[k] * J;
}

// ---------------------------------------------------------------------------------------
// Element kernels: volume term + surface lift + inverse mass + fused RK stage update.
// One block owns EPB consecutive elements, one thread per element node.
// ---------------------------------------------------------------------------------------
template <int DIM, int N>
struct Shape {
    static constexpr int NPE = ipow(N, DIM);
    static constexpr int NFD = ipow(N, DIM - 1);
    static constexpr int EPB = (NPE >= 256) ? 1 : (256 / NPE);
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
template <int DIM, int N, int NV, bool LGL>
__device__ __forceinline__ void surface_and_update(const ElemParams& P, const double* sops, int e, int i,
                                                   const double* q, double* dq) {
    const double* dgl = sops + 2 * N * N + 2 * N;
    const double* dgr = dgl + N;
#pragma unroll
    for (int dir = 0; dir < DIM; ++dir) {
        int pos, line;
        tp_coords<DIM>(N, i, dir, pos, line);
        int32_t pl = P.elem_face[e * 2 * DIM + 2 * dir], pr = P.elem_face[e * 2 * DIM + 2 * dir + 1];
        int64_t ol = (int64_t)(pl >> 1) * ipow(N, DIM - 1) + line;
        int64_t orr = (int64_t)(pr >> 1) * ipow(N, DIM - 1) + line;
        double sl = (pl & 1) ? -1.0 : 1.0, sr = (pr & 1) ? -1.0 : 1.0;
        if (LGL) {
            if (pos == 0) {
                double c = dgl[0] * sl;
#pragma unroll
                for (int k = 0; k < NV; ++k) dq[k] = dq[k] - c * P.Fn[k * P.nfdofs + ol];
            }
            if (pos == N - 1) {
                double c = dgr[N - 1] * sr;
#pragma unroll
                for (int k = 0; k < NV; ++k) dq[k] = dq[k] - c * P.Fn[k * P.nfdofs + orr];
            }
        } else {
            double cl = dgl[pos] * sl, cr = dgr[pos] * sr;
#pragma unroll
            for (int k = 0; k < NV; ++k)
                dq[k] = dq[k] - (cl * P.Fn[k * P.nfdofs + ol] + cr * P.Fn[k * P.nfdofs + orr]);
        }
    }
    double invJ = P.elem_invJ[e];
    int64_t g = (int64_t)e * ipow(N, DIM) + i;
    bool bad = false;
#pragma unroll
    for (int k = 0; k < NV; ++k) {
        double r = dq[k] * invJ;
        double o;
        if (P.mode == 0) o = r;
        else if (P.mode == 1) o = q[k] + P.dt * r;
        else o = P.a0 * P.Q0[k * P.ndofs + g] + P.a1 * (q[k] + P.dt * r);
        bad |= !isfinite(o);
        P.out[k * P.ndofs + g] = o;
    }
    if (bad) raise_nonphysical(P.status, e);
}

// Strong (== weak on LGL) divergence: dQ_line -= Ds * F̃_line per direction
// (OpDivergence.jl:109-160), F̃ = Ja_dd F_d (contravariant with a diagonal metric).
template <int DIM, int N, int EQ, bool LGL>
__global__ void __launch_bounds__(Shape<DIM, N>::BLOCK) elem_strong_kernel(ElemParams P) {
    using S = Shape<DIM, N>;
    constexpr int NV = (EQ == FLOU_EQ_EULER) ? DIM + 2 : 1;
    constexpr int NPE = S::NPE, NN = S::NN;
    extern __shared__ double smem[];
    double* sops = smem;
    double* sF = sops + S::NOPS;   // [DIM][NV][NN]
    const int tid = threadIdx.x;
    for (int t = tid; t < S::NOPS; t += blockDim.x) sops[t] = P.ops[t];
    const int e0 = blockIdx.x * S::EPB;
    const int el = tid / NPE, i = tid - el * NPE;
    const int e = e0 + el;
    const bool active = (tid < NN) && (e < P.nelem);
    double q[NV];
    if (active) {
        int64_t g = (int64_t)e * NPE + i;
#pragma unroll
        for (int k = 0; k < NV; ++k) q[k] = P.Q[k * P.ndofs + g];
        double F[NV];
#pragma unroll
        for (int d = 0; d < DIM; ++d) {
            double Ja = P.elem_Ja[e * DIM + d];
            if (EQ == FLOU_EQ_EULER) {
                double rho = q[0];
                double p = euler_pressure<DIM>(q, P.gamma);
                if (d == 0 && !(rho > 0.0 && p > 0.0)) raise_nonphysical(P.status, e);
                double vd = q[1 + d] / rho;
                F[0] = q[1 + d];
#pragma unroll
                for (int k = 0; k < DIM; ++k) F[1 + k] = q[1 + d] * (q[1 + k] / rho);
                F[1 + d] = F[1 + d] + p;
                F[DIM + 1] = (q[DIM + 1] + p) * vd;
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
    if (!active) return;
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
    surface_and_update<DIM, N, NV, LGL>(P, sops, e, i, q, dq);
}

// ---------------------------------------------------------------------------------------
// Split-form (flux-differencing) divergence, OpDivergence.jl:200-282:
//   dQ_i -= sum_j D♯_ij F♯(i, j), F♯(i, i) = F̃_i, F♯(i, j) = twopointflux(Q_i, Q_j).
// The two-point fluxes of a line are symmetric; each pair is evaluated once by one thread
// and kept in shared memory (the reference fills both triangle entries the same way).
// Per-node primitive quantities (velocities, pressure, β = ρ/2p and the logarithms of ρ
// and β) are computed once per node instead of once per pair.
// ---------------------------------------------------------------------------------------
struct PairPrims {   // primitive arrays in shared memory, each of length NN
    double *rho, *v[3], *p, *beta, *lrho, *lbeta, *vv, *e;
};

// Chandrashekar two-point flux (Euler.jl:474-536) along direction d without the metric
// factor.  The logarithmic means use the per-node logarithms:
//   series branch (u = ((a-b)/(a+b))² < 0.01): mean = (a+b)/(2F), F = 1+u/3+u²/5+u³/7
//   log branch:                               mean = (a-b)/(ln a - ln b)
// which is the reference's log(ξ)/(2f) form rewritten with ln ξ = ln a - ln b.
template <int DIM>
__device__ __forceinline__ void chandrashekar_pair(const PairPrims& S, int i, int l, int d, double g,
                                                   double* F) {
    double r1 = S.rho[i], r2 = S.rho[l];
    double b1 = S.beta[i], b2 = S.beta[l];
    double vavg[DIM];
#pragma unroll
    for (int k = 0; k < DIM; ++k) vavg[k] = (S.v[k][i] + S.v[k][l]) * 0.5;
    // ρ log-mean and its inverse
    double sr = r1 + r2, dr = r1 - r2;
    double rho_ln, inv_rho_ln;
    if (dr * dr < 0.01 * (sr * sr)) {
        double rs = 1.0 / sr;
        double f = dr * rs;
        double u = f * f;
        double Fs = ((1.0 + u * (1.0 / 3.0)) + (u * u) * 0.2) + (u * u * u) * (1.0 / 7.0);
        double iF = 1.0 / Fs;
        rho_ln = 0.5 * sr * iF;
        inv_rho_ln = 2.0 * Fs * rs;
    } else {
        double L = S.lrho[i] - S.lrho[l];
        rho_ln = dr / L;
        inv_rho_ln = L / dr;
    }
    // β log-mean (only its inverse is needed) and the pressure average
    double sb = b1 + b2, db = b1 - b2;
    double rb = 1.0 / sb;
    double inv_beta_ln;
    {
        double f = db * rb;
        double u = f * f;
        if (u < 0.01) {
            double Fs = ((1.0 + u * (1.0 / 3.0)) + (u * u) * 0.2) + (u * u * u) * (1.0 / 7.0);
            inv_beta_ln = 2.0 * Fs * rb;
        } else {
            inv_beta_ln = (S.lbeta[i] - S.lbeta[l]) / db;
        }
    }
    double p = 0.5 * sr * rb;
    double vv = 0.0;
#pragma unroll
    for (int k = 0; k < DIM; ++k) vv = vv + vavg[k] * vavg[k];
    double h = (inv_beta_ln * (0.5 / (g - 1.0)) - (S.vv[i] + S.vv[l]) * 0.25) + p * inv_rho_ln + vv;
    double m = rho_ln * vavg[d];
    F[0] = m;
#pragma unroll
    for (int k = 0; k < DIM; ++k) F[1 + k] = m * vavg[k];
    F[1 + d] = F[1 + d] + p;
    F[DIM + 1] = m * h;
}

template <int DIM, int N, int EQ, int TP, bool LGL>
__global__ void __launch_bounds__(Shape<DIM, N>::BLOCK) elem_split_kernel(ElemParams P) {
    using S = Shape<DIM, N>;
    constexpr int NV = (EQ == FLOU_EQ_EULER) ? DIM + 2 : 1;
    constexpr int NPE = S::NPE, NN = S::NN, NFD = S::NFD, NPAIR = S::NPAIR;
    constexpr int NPT = S::EPB * NFD * NPAIR;   // pairs per direction in the block
    constexpr bool EULER = (EQ == FLOU_EQ_EULER);
    // primitive arrays: rho, v[DIM], p, beta, lrho, lbeta, vv, e (+ conserved copies for
    // the StdAverage two-point flux)
    constexpr int NPRIM = EULER ? (DIM + 7 + (TP == FLOU_TP_STD_AVERAGE ? NV : 0)) : 1;
    extern __shared__ double smem[];
    double* sops = smem;
    double* sprim = sops + S::NOPS;
    double* spair = sprim + NPRIM * NN;   // [NV][NPT]
    uint8_t* stab = (uint8_t*)(spair + NV * NPT);   // pair table: a, b
    const int tid = threadIdx.x;
    for (int t = tid; t < S::NOPS; t += blockDim.x) sops[t] = P.ops[t];
    if (tid == 0) {
        int c = 0;
        for (int a = 0; a < N; ++a)
            for (int b = a + 1; b < N; ++b) { stab[2 * c] = (uint8_t)a; stab[2 * c + 1] = (uint8_t)b; ++c; }
    }
    PairPrims pp;
    if (EULER) {
        pp.rho = sprim;
        for (int k = 0; k < 3; ++k) pp.v[k] = sprim + (1 + (k < DIM ? k : 0)) * NN;
        pp.p = sprim + (1 + DIM) * NN;
        pp.beta = sprim + (2 + DIM) * NN;
        pp.lrho = sprim + (3 + DIM) * NN;
        pp.lbeta = sprim + (4 + DIM) * NN;
        pp.vv = sprim + (5 + DIM) * NN;
        pp.e = sprim + (6 + DIM) * NN;
    } else {
        pp.rho = sprim;
    }
    double* sq = sprim + (EULER ? (DIM + 7) : 0) * NN;   // conserved copies (StdAverage)
    const int e0 = blockIdx.x * S::EPB;
    const int el = tid / NPE, i = tid - el * NPE;
    const int e = e0 + el;
    const bool active = (tid < NN) && (e < P.nelem);
    const double g = P.gamma;
    double q[NV];
    if (active) {
        int64_t gi = (int64_t)e * NPE + i;
#pragma unroll
        for (int k = 0; k < NV; ++k) q[k] = P.Q[k * P.ndofs + gi];
        if (EULER) {
            double rho = q[0];
            double p = euler_pressure<DIM>(q, g);
            if (!(rho > 0.0 && p > 0.0)) raise_nonphysical(P.status, e);
            pp.rho[tid] = rho;
            double vv = 0.0;
#pragma unroll
            for (int k = 0; k < DIM; ++k) {
                double vk = q[1 + k] / rho;
                pp.v[k][tid] = vk;
                vv = (k == 0) ? vk * vk : vv + vk * vk;
            }
            pp.p[tid] = p;
            pp.vv[tid] = vv;
            if (TP == FLOU_TP_CHANDRASHEKAR) {
                double beta = rho / (2.0 * p);
                pp.beta[tid] = beta;
                pp.lrho[tid] = log(rho);
                pp.lbeta[tid] = log(beta);
            }
            if (TP == FLOU_TP_KENNEDY_GRUBER) pp.e[tid] = q[DIM + 1] / rho;
            if (TP == FLOU_TP_STD_AVERAGE)
#pragma unroll
                for (int k = 0; k < NV; ++k) sq[k * NN + tid] = q[k];
        } else {
            pp.rho[tid] = q[0];
        }
    }
    __syncthreads();
    double dq[NV];
#pragma unroll
    for (int k = 0; k < NV; ++k) dq[k] = 0.0;
    const double* Dsh = sops + N * N;
#pragma unroll 1
    for (int dir = 0; dir < DIM; ++dir) {
        // ---- pair phase: every symmetric two-point flux of the block, once ----
        for (int kp = tid; kp < NPT; kp += blockDim.x) {
            int elp = kp / (NFD * NPAIR);
            int r = kp - elp * (NFD * NPAIR);
            int line = r / NPAIR, pr = r - line * NPAIR;
            if (e0 + elp >= P.nelem) continue;
            int a = stab[2 * pr], b = stab[2 * pr + 1];
            int ia = elp * NPE + tp_node<DIM>(N, dir, line, a);
            int ib = elp * NPE + tp_node<DIM>(N, dir, line, b);
            double F[NV];
            if (EULER) {
                if (TP == FLOU_TP_CHANDRASHEKAR) {
                    chandrashekar_pair<DIM>(pp, ia, ib, dir, g, F);
                } else if (TP == FLOU_TP_KENNEDY_GRUBER) {
                    double rho = (pp.rho[ia] + pp.rho[ib]) * 0.5;
                    double vd = (pp.v[dir][ia] + pp.v[dir][ib]) * 0.5;
                    double p = (pp.p[ia] + pp.p[ib]) * 0.5;
                    double en = (pp.e[ia] + pp.e[ib]) * 0.5;
                    double m = rho * vd;
                    F[0] = m;
#pragma unroll
                    for (int k = 0; k < DIM; ++k) F[1 + k] = m * ((pp.v[k][ia] + pp.v[k][ib]) * 0.5);
                    F[1 + dir] = F[1 + dir] + p;
                    F[DIM + 1] = m * en + p * vd;
                } else {   // StdAverage two-point flux, Euler.jl:385-472
                    double v1 = pp.v[dir][ia], v2 = pp.v[dir][ib];
                    double p1 = pp.p[ia], p2 = pp.p[ib];
                    F[0] = (sq[(1 + dir) * NN + ia] + sq[(1 + dir) * NN + ib]) * 0.5;
#pragma unroll
                    for (int k = 0; k < DIM; ++k) {
                        double m1 = sq[(1 + k) * NN + ia] * v1, m2 = sq[(1 + k) * NN + ib] * v2;
                        F[1 + k] = (k == dir) ? (((m1 + p1) + m2) + p2) * 0.5 : (m1 + m2) * 0.5;
                    }
                    F[DIM + 1] = ((sq[(DIM + 1) * NN + ia] + p1) * v1 + (sq[(DIM + 1) * NN + ib] + p2) * v2) * 0.5;
                }
            } else if (EQ == FLOU_EQ_LINEAR_ADVECTION) {
                F[0] = P.adv[dir] * (pp.rho[ia] + pp.rho[ib]) * 0.5;
            } else {
                F[0] = (pp.rho[ia] * pp.rho[ia] + pp.rho[ib] * pp.rho[ib]) * 0.25;
            }
#pragma unroll
            for (int k = 0; k < NV; ++k) spair[k * NPT + kp] = F[k];
        }
        __syncthreads();
        // ---- node phase: dQ_i -= Ja_dd sum_j D♯_ij F♯(i, j) ----
        if (active) {
            int pos, line;
            tp_coords<DIM>(N, i, dir, pos, line);
            double Fd[NV];   // F♯(i, i): the physical flux along dir
            if (EULER) {
                double vd = pp.v[dir][tid], p = pp.p[tid];
                Fd[0] = q[1 + dir];
#pragma unroll
                for (int k = 0; k < DIM; ++k) Fd[1 + k] = q[1 + dir] * pp.v[k][tid];
                Fd[1 + dir] = Fd[1 + dir] + p;
                Fd[DIM + 1] = (q[DIM + 1] + p) * vd;
            } else if (EQ == FLOU_EQ_LINEAR_ADVECTION) {
                Fd[0] = P.adv[dir] * q[0];
            } else {
                Fd[0] = q[0] * q[0] / 2.0;
            }
            double acc[NV];
#pragma unroll
            for (int k = 0; k < NV; ++k) acc[k] = 0.0;
            int pbase = el * NFD * NPAIR + line * NPAIR;
#pragma unroll
            for (int j = 0; j < N; ++j) {
                double a = Dsh[pos + j * N];
                if (j == pos) {
#pragma unroll
                    for (int k = 0; k < NV; ++k) acc[k] = acc[k] + a * Fd[k];
                } else {
                    int lo = j < pos ? j : pos, hi = j < pos ? pos : j;
                    int pidx = pbase + lo * (2 * N - lo - 1) / 2 + (hi - lo - 1);
#pragma unroll
                    for (int k = 0; k < NV; ++k) acc[k] = acc[k] + a * spair[k * NPT + pidx];
                }
            }
            double Ja = P.elem_Ja[e * DIM + dir];
#pragma unroll
            for (int k = 0; k < NV; ++k) dq[k] = dq[k] - Ja * acc[k];
        }
        __syncthreads();
    }
    if (!active) return;
    surface_and_update<DIM, N, NV, LGL>(P, sops, e, i, q, dq);
}

template <int DIM, int N, int EQ, int VOL, int TP>
constexpr size_t elem_smem_bytes() {
    using S = Shape<DIM, N>;
    constexpr int NV = (EQ == FLOU_EQ_EULER) ? DIM + 2 : 1;
    if (VOL == FLOU_OP_STRONG) return sizeof(double) * (S::NOPS + DIM * NV * S::NN);
    constexpr int NPRIM = (EQ == FLOU_EQ_EULER) ? (DIM + 7 + (TP == FLOU_TP_STD_AVERAGE ? NV : 0)) : 1;
    constexpr int NPT = S::EPB * S::NFD * S::NPAIR;
    return sizeof(double) * (S::NOPS + NPRIM * S::NN + NV * NPT) + 2 * (S::NPAIR + 1);
}

// Launch one instantiation; the dynamic shared-memory opt-in is set once per kernel.
// With `prepare` set only the opt-in is made (it must precede stream capture).
template <int DIM, int N, int EQ, int VOL, int TP, bool LGL>
cudaError_t launch_elem_one(const ElemParams& P, cudaStream_t s, bool prepare) {
    using S = Shape<DIM, N>;
    constexpr size_t smem = elem_smem_bytes<DIM, N, EQ, VOL, TP>();
    static bool attr_set = false;
    int grid = (P.nelem + S::EPB - 1) / S::EPB;
    auto k = (VOL == FLOU_OP_STRONG) ? (void (*)(ElemParams))elem_strong_kernel<DIM, N, EQ, LGL>
                                     : (void (*)(ElemParams))elem_split_kernel<DIM, N, EQ, TP, LGL>;
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
template <int DIM, int N, int EQ>
cudaError_t launch_elem_n(int vol, int tp, bool lgl, const ElemParams& P, cudaStream_t s, bool prep) {
    if (vol == FLOU_OP_STRONG)
        return lgl ? launch_elem_one<DIM, N, EQ, FLOU_OP_STRONG, 0, true>(P, s, prep)
                   : launch_elem_one<DIM, N, EQ, FLOU_OP_STRONG, 0, false>(P, s, prep);
    if (!lgl) return cudaErrorInvalidValue;
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

template <int DIM, int EQ>
cudaError_t launch_elem_dim(int n, int vol, int tp, bool lgl, const ElemParams& P, cudaStream_t s, bool prep) {
    switch (n) {
        case 2: return launch_elem_n<DIM, 2, EQ>(vol, tp, lgl, P, s, prep);
        case 3: return launch_elem_n<DIM, 3, EQ>(vol, tp, lgl, P, s, prep);
        case 4: return launch_elem_n<DIM, 4, EQ>(vol, tp, lgl, P, s, prep);
        case 5: return launch_elem_n<DIM, 5, EQ>(vol, tp, lgl, P, s, prep);
        case 6: return launch_elem_n<DIM, 6, EQ>(vol, tp, lgl, P, s, prep);
        case 7: return launch_elem_n<DIM, 7, EQ>(vol, tp, lgl, P, s, prep);
        case 8: return launch_elem_n<DIM, 8, EQ>(vol, tp, lgl, P, s, prep);
        default: return cudaErrorInvalidValue;
    }
}

// Host-side dispatch: one function per translation unit.
struct ElemLaunch {
    int dim, eq, n, vol, tp;
    bool lgl;
    bool prepare;   // only set the kernel's shared-memory opt-in, launch nothing
};
cudaError_t launch_elem_euler1d(const ElemLaunch& L, const ElemParams& P, cudaStream_t s);
cudaError_t launch_elem_euler2d(const ElemLaunch& L, const ElemParams& P, cudaStream_t s);
cudaError_t launch_elem_euler3d_strong(const ElemLaunch& L, const ElemParams& P, cudaStream_t s);
cudaError_t launch_elem_euler3d_split(const ElemLaunch& L, const ElemParams& P, cudaStream_t s);
cudaError_t launch_elem_scalar(const ElemLaunch& L, const ElemParams& P, cudaStream_t s);
cudaError_t launch_face(int dim, int eq, bool lgl, const FaceParams& P, cudaStream_t s);
cudaError_t launch_elem(const ElemLaunch& L, const ElemParams& P, cudaStream_t s);

}  // namespace flou
