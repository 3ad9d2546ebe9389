// adjoint_kernels.cuh -- device side of the discrete adjoint: the parameter blocks, the VJPs of the
// fluxes (Euler.jl's and Toro's), the face and element VJP kernels and their launch templates.
// The translation units adjoint_face.cu, adjoint_elem.cu and adjoint_split{1d,2d,3d}.cu instantiate
// them (compiled in parallel); adjoint.cu holds the host side (stage adjoint, checkpoint schedule,
// reverse sweeps, C ABI) and calls them through the launchers declared at the end.
//
// discrete adjoint (vector-Jacobian products) of the residual and of the
// SSP-RK3 step for the Euler equations with the strong-form volume term and the LxF
// (Rusanov, StdAverage) interface flux on LGL nodes, and the checkpointed reverse sweep of
// a terminal functional.
//
// Residual (per element, node i):  dQ_i = (1/J) [ -Σ_d Ja_d Σ_j Ds(i,j) F_d(Q_j) - Σ_faces ∂g·(±Fn) ]
// (Hyperbolic.jl:31-69 with OpDivergence.jl:42-160, Interfaces.jl:111-136).  Its transpose,
// applied to a cotangent λ with w = λ/J:
//   volume:   Q̄_j -= Ja_d (∂F_d/∂Q)(Q_j)ᵀ Σ_i Ds(i,j) w_i           (transposed line contraction)
//   surface:  F̄(face node) = -∂g_1 w_1 + ∂g_2 w_2  (end nodes of side 1 / side 2)
//             then the face flux VJP scatters to the two traces and to the dissipation scale.
// SSP-RK3 step transpose (U1 = U0 + dt L0; U2 = 3/4 U0 + 1/4 (U1 + dt L1); U3 = 1/3 U0 + 2/3 (U2 + dt L2)):
//   (a) Ū2 = 2/3 Ū3 + VJP(U2; 2/3 dt Ū3),  B = 1/3 Ū3
//   (b) Ū1 = 1/4 Ū2 + VJP(U1; 1/4 dt Ū2),  B += 3/4 Ū2
//   (c) Ū0 = Ū1 + B + VJP(U0; dt Ū1)
// Split form (OpDivergence.jl:200-282 with the Chandrashekar flux of Euler.jl:474-536): the
// volume term -Ja_d Σ_j D♯(i,j) F♯(Q_i, Q_j) has, for a symmetric pair (a, b) of a line, the
// flux cotangent F̄ = -Ja_d (D♯(a,b) w_a + D♯(b,a) w_b); its VJP goes to the primitive
// variables (ρ, v, β = ρ/(2p)) of both nodes and from there to the conserved ones.  The
// LxF(Chandrashekar) interface flux differentiates the same pair flux (3D keeps the
// reference's mean of |v|² as written, Euler.jl:216).
// Non-smooth points follow Julia's Base (what ForwardDiff differentiates on the reference's
// CPU path): max(a, b) takes b unless b < a; d|u|/du = -1 if u has its sign bit set, else +1.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>

#include "flou_ctx.cuh"

namespace flou {

struct AdjFaceParams {
    int32_t* status;        // index-check reports (FLOU_CUDA_CHECKED builds)
    // general geometry (CURV kernels): per face node frame [9][nfdofs] and surface Jacobian,
    // per face orientation, per node 1/J
    const double* frames;
    const double* faceJn;
    const uint8_t* orient;
    const double* invJn;
    const double* U;        // state the residual is linearised at
    const double* Ain;      // adjoint input; λ = s_lam * Ain
    double s_lam;
    double* QbL;            // trace cotangent, side 1 [nv][nfdofs]
    double* QbR;            // trace cotangent, side 2 [nv][nfdofs]
    double* Ibar;           // cotangent of the face intensity [nfdofs]
    const int32_t* face_elem;
    const double* faceJ;
    const int8_t* face_bc;
    const double* invJ;
    const double* ops;      // to read ∂g_l[0], ∂g_r[n-1]
    const double* elem_c;
    double intensity, gamma;
    int64_t ndofs, nfdofs;
    int32_t nfaces, n, npe, nfd;
    int32_t bc_kind[MAXBC];
    // external states of FLOU_BC_INFLOW (per boundary) and FLOU_BC_STATE_FIELD ([nv][nfdofs]
    // per face node), in the physical frame; constants, so their cotangents are dropped
    double bc_state[MAXBC][5];
    const double* bc_field;
    double adv[3];          // linear advection velocity (scalar equations)
    int32_t lxf;            // scalar equations: LxF dissipation (else the central flux)
    // the hybrid operator on Gauss nodes: the face fluxes' cotangents come from the elements
    // ([2][nv][nfdofs], master and slave side), instead of the lift's transpose (nullable)
    const double* FbS;
};

struct AdjElemParams {
    int32_t* status;        // index-check reports (FLOU_CUDA_CHECKED builds)
    // general geometry (CURV kernels): per node 1/J and metric Ja[k][d] at (k + d DIM) * ndofs,
    // per face orientation
    const double* invJn;
    const double* Jan;
    const uint8_t* orient;
    const double* U;
    const double* Ain;
    double* Aout;           // alpha Ain + beta B + VJP
    double* B;              // accumulator: B = gamma_B B + delta_B Ain (when writeB)
    const double* QbL;
    const double* QbR;
    const double* Ibar;
    double* cbar;           // per element, accumulated (nullable)
    const int32_t* elem_face;
    const int32_t* face_elem;
    const double* invJ;
    const double* Ja;
    const double* ops;
    int64_t ndofs, nfdofs;
    int32_t nelem;
    double s_lam, alpha, beta, gamma_B, delta_B;
    int32_t readB, writeB;
    double gamma;
    // 2N-storage reverse stages: K = kA Ain + kB Aout per node (nullable; K may alias Ain, whose
    // other readers are done: the face kernel ran before, and a block reads only its own nodes)
    double* K;
    double kA, kB;
    // hybrid operator: 1D quadrature weights, the subcell FV flux (numflux_vjp kind) and its
    // intensity, the blending constant
    const double* omega1;
    int32_t fvkind, fvflux, fvavg;   // numflux_vjp kind; the forward's numflux and central part
    double fvintensity, blend;
    // general geometry, hybrid and Gauss-node forms: the subcell interfaces' frames [9][ns] and
    // surface Jacobians, at ((e DIM + dir) n^(d-1) + line)(n+1) + s
    const double* subfr;
    const double* subJ;
    double adv[3];          // linear advection velocity (scalar equations)
    // the hybrid operator on Gauss nodes (a stage in two element passes around the face VJP):
    // the forward face fluxes at U, the face-flux cotangents [2][nv][nfdofs] the first pass
    // writes, and its partial node cotangents (state-sized), which the second pass completes
    const double* FnU;
    double* FbS;
    double* Tq;
};

// q̄ += (∂F_d/∂q)ᵀ ḡ for the Euler flux along axis d, with v = m/ρ, p, H = (E+p)/ρ:
//   P̄ = ḡ_md + ḡ_E v_d,  s = Σ_k ḡ_mk v_k
//   q̄_ρ  += -v_d (s + ḡ_E H) + (γ-1) |v|²/2 P̄
//   q̄_mk += v_d ḡ_mk - (γ-1) v_k P̄ + [k = d] (ḡ_ρ + s + ḡ_E H)
//   q̄_E  += ḡ_E v_d + (γ-1) P̄
template <int DIM>
__device__ __forceinline__ void euler_flux_vjp(int d, const double* v, double vv, double H, double g1,
                                               const double* gb, double scale, double* qb) {
    double Pb = gb[1 + d] + gb[DIM + 1] * v[d];
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < DIM; ++k) s = fma(gb[1 + k], v[k], s);
    double t = s + gb[DIM + 1] * H;
    qb[0] += scale * (fma(0.5 * g1 * vv, Pb, -v[d] * t));
#pragma unroll
    for (int k = 0; k < DIM; ++k) {
        double r = fma(v[d], gb[1 + k], -g1 * v[k] * Pb);
        if (k == d) r += gb[0] + t;
        qb[1 + k] += scale * r;
    }
    qb[DIM + 1] += scale * fma(g1, Pb, gb[DIM + 1] * v[d]);
}

// The same for the flux along a general direction n (F_n = Σ_d n_d F_d, general geometry), with
// vn = v·n:  P̄ = Σ_k ḡ_mk n_k + ḡ_E vn,  q̄_ρ += -vn (s + ḡ_E H) + (γ-1)|v|²/2 P̄,
//   q̄_mk += vn ḡ_mk - (γ-1) v_k P̄ + n_k (ḡ_ρ + s + ḡ_E H),  q̄_E += ḡ_E vn + (γ-1) P̄.
template <int DIM>
__device__ __forceinline__ void euler_flux_vjp_n(const double* nrm, const double* v, double vv, double H, double g1,
                                                 const double* gb, double scale, double* qb) {
    double vn = 0.0, s = 0.0, Pb = 0.0;
#pragma unroll
    for (int k = 0; k < DIM; ++k) {
        vn = fma(v[k], nrm[k], vn);
        s = fma(gb[1 + k], v[k], s);
        Pb = fma(gb[1 + k], nrm[k], Pb);
    }
    Pb = fma(gb[DIM + 1], vn, Pb);
    double t = s + gb[DIM + 1] * H;
    qb[0] += scale * (fma(0.5 * g1 * vv, Pb, -vn * t));
#pragma unroll
    for (int k = 0; k < DIM; ++k) qb[1 + k] += scale * fma(nrm[k], gb[0] + t, fma(vn, gb[1 + k], -g1 * v[k] * Pb));
    qb[DIM + 1] += scale * fma(g1, Pb, gb[DIM + 1] * vn);
}

// Primitive quantities of one node with the reciprocals the VJPs reuse (1/ρ, 1/a), from the
// refined hardware reciprocals (within 1 ulp of the correctly rounded values).
struct Prim {
    double rho, v[3], vv, p, H, a, ir, ia;
};

template <int DIM, bool SOUND = true>
__device__ __forceinline__ Prim prim_of(const double* q, double g) {
    Prim P;
    P.rho = q[0];
    double ir = rcp_refined(q[0]), ke = 0.0, vv = 0.0;
    P.ir = ir;
#pragma unroll
    for (int k = 0; k < DIM; ++k) {
        P.v[k] = q[1 + k] * ir;
        ke = fma(q[1 + k], P.v[k], ke);
        vv = fma(P.v[k], P.v[k], vv);
    }
    P.vv = vv;
    P.p = (g - 1.0) * fma(-0.5, ke, q[DIM + 1]);
    P.H = (q[DIM + 1] + P.p) * ir;
    if (SOUND) {
        const double a2 = g * P.p * ir;
        P.ia = rsqrt_refined(a2);
        P.a = a2 * P.ia;
    } else {
        P.a = P.ia = 0.0;
    }
    return P;
}

// q̄ += κ ∇λ, λ = |u_n| + a (face frame, normal momentum first).
template <int DIM>
__device__ __forceinline__ void lambda_vjp(const Prim& P, double g, double kappa, double* qb) {
    double sg = signbit(P.v[0]) ? -1.0 : 1.0;
    double ir = P.ir;
    double ca = (0.5 * g * (g - 1.0)) * (P.ia * ir);   // ∂a/∂p · ∂p/∂E
    qb[0] += kappa * (-sg * P.v[0] * ir + ca * 0.5 * P.vv - P.a * 0.5 * ir);
#pragma unroll
    for (int k = 0; k < DIM; ++k) qb[1 + k] += kappa * ((k == 0 ? sg * ir : 0.0) - ca * P.v[k]);
    qb[DIM + 1] += kappa * ca;
}

// Cotangent of one node's primitive variables: (ρ, v, β) for the Chandrashekar flux, (ρ, v, p, e)
// for Kennedy-Gruber (b then holds p̄ and e the cotangent of the specific total energy E/ρ).
struct PrimBar {
    double r, v[3], b, e;
};

// Logarithmic mean (Utilities.jl:34-44) of a = 2 h1, b = 2 h2 given the half sum hs = (a+b)/2,
// the half difference hd = (a-b)/2 and r = 1/hs, with its partial derivatives:
//   f = (a-b)/(a+b), u = f²;  u < 0.01: L = (a+b)/(2F), F = 1+u/3+u²/5+u³/7, 1/L = F r,
//     ∂L/∂a = 1/(2F) - 2F'(u) f b/(F²(a+b)),  ∂L/∂b = 1/(2F) + 2F'(u) f a/(F²(a+b));
//   else L = (a-b)/ℓ, ℓ = ln(a/b):  ∂L/∂a = 1/ℓ - L/(ℓ a),  ∂L/∂b = L/(ℓ b) - 1/ℓ.
// 1/F takes two Newton steps from 1 - u/3 (relative error (4u²/45)^4 < 1e-20 for u < 0.01).
__device__ __forceinline__ void logmean_half(double h1, double h2, double hs, double hd, double r, double& L,
                                             double& iL, double& da, double& db) {
    double f = hd * r, u = f * f;
    if (u < 0.01) {
        double F = fma(u, fma(u, fma(u, 1.0 / 7.0, 0.2), 1.0 / 3.0), 1.0);
        double y = fma(-1.0 / 3.0, u, 1.0);
        y = y * fma(-F, y, 2.0);
        y = y * fma(-F, y, 2.0);
        L = hs * y;
        iL = F * r;
        double Fp2 = fma(u, fma(u, 6.0 / 7.0, 0.8), 2.0 / 3.0);   // 2 F'(u)
        double t = Fp2 * f * (y * y) * r;
        double hy = 0.5 * y;
        da = fma(-t, h2, hy);
        db = fma(t, h1, hy);
    } else {
        double l = log(h1 / h2), il = 1.0 / l;
        L = (2.0 * hd) * il;
        iL = l / (2.0 * hd);
        double c = 0.5 * L * il;
        da = il - c / h1;
        db = c / h2 - il;
    }
}

// VJP of the Chandrashekar pair flux along axis D (Euler.jl:474-536 as a function of the
// primitive variables), F = [m, m v̄ + p̂ e_D, m h] with
//   m = ρ̂ v̄_D, ρ̂ = ln-mean(ρ), β̂ = ln-mean(β), p̂ = (ρ1+ρ2)/(2(β1+β2)), v̄ = (v1+v2)/2,
//   h = 1/(2β̂(γ-1)) - S/4 + p̂/ρ̂ + |v̄|²,  S = |v1|² + |v2|²
// (WL2: S = |v1|² + |v2|² - v2_z² + v1_z², the 3D interface average of Euler.jl:216).
// Inputs are the halved node quantities rh = ρ/2, vh = v/2, bh = β/2, vq = |v|²/4; one
// reciprocal 1/(ρ̄ β̄) serves both means and the pressure average.  Cotangents are with
// respect to (ρ, v, β) of each side.
// D < 0: the flux along the general direction nrm (general geometry), m = ρ̂ v̄·n and p̂ n in the
// momentum flux.
template <int DIM, int D, bool WL2>
__device__ __forceinline__ void chandra_pair_vjp(double rh1, const double* vh1, double bh1, double vq1, double rh2,
                                                 const double* vh2, double bh2, double vq2, double cb,
                                                 const double* Fb, PrimBar& o1, PrimBar& o2,
                                                 const double* nrm = nullptr) {
    double hsr = rh1 + rh2, hdr = rh1 - rh2, hsb = bh1 + bh2, hdb = bh1 - bh2;
    double R = rcp_refined(hsr * hsb);
    double rs = hsb * R, rb = hsr * R;   // 1/hsr, 1/hsb
    double rho, irho, dra, drb, beta, ibeta, dba, dbb;
    logmean_half(rh1, rh2, hsr, hdr, rs, rho, irho, dra, drb);
    logmean_half(bh1, bh2, hsb, hdb, rb, beta, ibeta, dba, dbb);
    double p = 0.5 * hsr * rb;
    double va[DIM], vv = 0.0;
#pragma unroll
    for (int k = 0; k < DIM; ++k) {
        va[k] = vh1[k] + vh2[k];
        vv = fma(va[k], va[k], vv);
    }
    double S4 = vq1 + vq2;
    if (WL2 && DIM == 3) S4 = S4 + (vh1[2] * vh1[2] - vh2[2] * vh2[2]);
    double h = fma(cb, ibeta, -S4) + fma(p, irho, vv);
    double vd, fn;   // v̄ along the direction, and the normal component of the momentum cotangent
    if constexpr (D >= 0) {
        vd = va[D];
        fn = Fb[1 + D];
    } else {
        vd = 0.0;
        fn = 0.0;
#pragma unroll
        for (int k = 0; k < DIM; ++k) {
            vd = fma(va[k], nrm[k], vd);
            fn = fma(Fb[1 + k], nrm[k], fn);
        }
    }
    double m = rho * vd;
    double mb = fma(Fb[DIM + 1], h, Fb[0]);
#pragma unroll
    for (int k = 0; k < DIM; ++k) mb = fma(Fb[1 + k], va[k], mb);
    double hb = m * Fb[DIM + 1];
    double mh = 0.5 * m;
    double hvab[DIM];   // v̄̄/2: the cotangent of v̄, halved (v̄ = (v1 + v2)/2)
#pragma unroll
    for (int k = 0; k < DIM; ++k) hvab[k] = fma(mh, Fb[1 + k], hb * va[k]);
    if constexpr (D >= 0) {
        hvab[D] = fma(0.5 * mb, rho, hvab[D]);
    } else {
#pragma unroll
        for (int k = 0; k < DIM; ++k) hvab[k] = fma(0.5 * mb * rho, nrm[k], hvab[k]);
    }
    double pb = fma(hb, irho, fn);
    double rhob = fma(mb, vd, -hb * p * (irho * irho));
    double betab = -hb * cb * (ibeta * ibeta);
    double pr = 0.25 * pb * rb, pbb = -0.5 * pb * p * rb;
    o1.r = fma(rhob, dra, pr);
    o2.r = fma(rhob, drb, pr);
    o1.b = fma(betab, dba, pbb);
    o2.b = fma(betab, dbb, pbb);
#pragma unroll
    for (int k = 0; k < DIM; ++k) {
        o1.v[k] = fma(-hb, vh1[k], hvab[k]);
        o2.v[k] = fma(-hb, vh2[k], hvab[k]);
    }
    if (WL2 && DIM == 3) {
        o1.v[2] = fma(-hb, vh1[2], o1.v[2]);
        o2.v[2] = fma(hb, vh2[2], o2.v[2]);
    }
}

// q̄ += (∂(ρ, v, β)/∂q)ᵀ (ρ̄, v̄, β̄) with β = ρ/(2p):
//   ρ̄' = ρ̄ + β̄/(2p),  p̄ = -β̄ β/p,
//   q̄_ρ += ρ̄' - v·v̄/ρ + (γ-1)|v|²/2 p̄,  q̄_mk += v̄_k/ρ - (γ-1) v_k p̄,  q̄_E += (γ-1) p̄.
template <int DIM>
__device__ __forceinline__ void prim_to_cons_vjp(double rho, const double* v, double vv, double p, double g1,
                                                 const PrimBar& o, double* qb) {
    double ip = rcp_refined(p), ir = rcp_refined(rho);
    double rb = fma(0.5 * ip, o.b, o.r);
    double pb = -o.b * (0.5 * rho * ip) * ip * g1;   // (γ-1) p̄
    double vvb = 0.0;
#pragma unroll
    for (int k = 0; k < DIM; ++k) {
        vvb = fma(v[k], o.v[k], vvb);
        qb[1 + k] += fma(o.v[k], ir, -v[k] * pb);
    }
    qb[0] += fma(0.5 * vv, pb, fma(-vvb, ir, rb));
    qb[DIM + 1] += pb;
}

// VJP of the Kennedy-Gruber pair flux along axis D (Kennedy & Gruber 2008, as the forward kernel
// evaluates it), F = [m, m v̄ + p̄ e_D, m ē + p̄ v̄_D] with m = ρ̄ v̄_D and the arithmetic means
// ρ̄, v̄, p̄, ē (e = E/ρ).  Inputs are the halved node quantities (rh = ρ/2, vh = v/2, ph = p/2,
// eh = e/2), so each mean is a sum of two; both nodes receive half of each mean's cotangent.
// D < 0: along the general direction nrm, m = ρ̄ v̄·n, F = [m, m v̄ + p̄ n, m ē + p̄ v̄·n].
template <int DIM, int D>
__device__ __forceinline__ void kg_pair_vjp(double rh1, const double* vh1, double ph1, double eh1, double rh2,
                                            const double* vh2, double ph2, double eh2, const double* Fb,
                                            PrimBar& o1, PrimBar& o2, const double* nrm = nullptr) {
    const double rho = rh1 + rh2, pm = ph1 + ph2, en = eh1 + eh2;
    double vm[DIM];
#pragma unroll
    for (int k = 0; k < DIM; ++k) vm[k] = vh1[k] + vh2[k];
    double vd, fn;
    if constexpr (D >= 0) {
        vd = vm[D];
        fn = Fb[1 + D];
    } else {
        vd = 0.0;
        fn = 0.0;
#pragma unroll
        for (int k = 0; k < DIM; ++k) {
            vd = fma(vm[k], nrm[k], vd);
            fn = fma(Fb[1 + k], nrm[k], fn);
        }
    }
    const double m = rho * vd;
    double mb = fma(Fb[DIM + 1], en, Fb[0]);
#pragma unroll
    for (int k = 0; k < DIM; ++k) mb = fma(Fb[1 + k], vm[k], mb);
    o1.r = o2.r = 0.5 * mb * vd;
#pragma unroll
    for (int k = 0; k < DIM; ++k) o1.v[k] = 0.5 * Fb[1 + k] * m;
    if constexpr (D >= 0) {
        o1.v[D] = fma(0.5 * mb, rho, fma(0.5 * Fb[DIM + 1], pm, o1.v[D]));
    } else {
        const double cn = fma(0.5 * mb, rho, 0.5 * Fb[DIM + 1] * pm);   // the cotangent along n
#pragma unroll
        for (int k = 0; k < DIM; ++k) o1.v[k] = fma(cn, nrm[k], o1.v[k]);
    }
#pragma unroll
    for (int k = 0; k < DIM; ++k) o2.v[k] = o1.v[k];
    o1.b = o2.b = 0.5 * fma(Fb[DIM + 1], vd, fn);
    o1.e = o2.e = 0.5 * Fb[DIM + 1] * m;
}

// q̄ += (∂(ρ, v, p, e)/∂q)ᵀ (ρ̄, v̄, p̄, ē) with v = m/ρ, p = (γ-1)(E - ½|m|²/ρ), e = E/ρ:
//   q̄_ρ += ρ̄ - (v·v̄ + e ē)/ρ + (γ-1)|v|²/2 p̄,  q̄_mk += v̄_k/ρ - (γ-1) v_k p̄,
//   q̄_E += (γ-1) p̄ + ē/ρ.
template <int DIM>
__device__ __forceinline__ void kg_prim_to_cons_vjp(double rho, const double* v, double vv, double E, double g1,
                                                    const PrimBar& o, double* qb) {
    const double ir = rcp_refined(rho), e = E * ir, pb = g1 * o.b;
    double vvb = e * o.e;
#pragma unroll
    for (int k = 0; k < DIM; ++k) {
        vvb = fma(v[k], o.v[k], vvb);
        qb[1 + k] += fma(o.v[k], ir, -v[k] * pb);
    }
    qb[0] += fma(0.5 * vv, pb, fma(-vvb, ir, o.r));
    qb[DIM + 1] += fma(o.e, ir, pb);
}

// Cotangents of one side's primitive quantities in the face frame (normal velocity u, tangential
// velocities, pressure, sound speed), mapped to its conserved variables and added to qb:
//   p̄' = p̄ + ā γ/(2aρ)   (a = sqrt(γp/ρ)),
//   q̄_ρ += -ā a/(2ρ) - (ū u + Σ v̄_t v_t)/ρ + (γ-1)|v|²/2 p̄',
//   q̄_m1 += ū/ρ - (γ-1) u p̄',  q̄_mt += v̄_t/ρ - (γ-1) v_t p̄',  q̄_E += (γ-1) p̄'.
struct SideBar {
    double u, vt[2], p, a;
};

template <int DIM>
__device__ __forceinline__ void side_prim_vjp(const Prim& P, double g, const SideBar& b, double* qb) {
    const double g1 = g - 1.0, ir = P.ir;
    const double pb = fma(b.a * g, 0.5 * ir * P.ia, b.p);
    double vdot = b.u * P.v[0];
#pragma unroll
    for (int k = 1; k < DIM; ++k) vdot = fma(b.vt[k - 1], P.v[k], vdot);
    qb[0] += fma(0.5 * g1 * P.vv, pb, -(fma(b.a, 0.5 * P.a, vdot)) * ir);
    qb[1] += fma(b.u, ir, -g1 * P.v[0] * pb);
#pragma unroll
    for (int k = 1; k < DIM; ++k) qb[1 + k] += fma(b.vt[k - 1], ir, -g1 * P.v[k] * pb);
    qb[DIM + 1] += g1 * pb;
}

// VJP of the physical normal flux F = [m1, m1 u + p, m_t u, (E + p) u] (face frame) with the
// cotangent gb scaled by sc: the conserved variables it reads directly go to qb, u and p to b.
template <int DIM>
__device__ __forceinline__ void normal_flux_vjp(const double* q, const Prim& P, const double* gb, double sc,
                                                double* qb, SideBar& b) {
    const double u = P.v[0];
    double ub = gb[1] * q[1];
#pragma unroll
    for (int k = 1; k < DIM; ++k) {
        ub = fma(gb[1 + k], q[1 + k], ub);
        qb[1 + k] += sc * gb[1 + k] * u;
    }
    ub = fma(gb[DIM + 1], q[DIM + 1] + P.p, ub);
    qb[1] += sc * fma(gb[1], u, gb[0]);
    qb[DIM + 1] += sc * gb[DIM + 1] * u;
    b.u += sc * ub;
    b.p += sc * fma(gb[DIM + 1], u, gb[1]);
}

// VJP of the HLL (hllc = false) and HLLC interface fluxes in the face frame (no counterpart in
// Flou; Toro 2009, eqs. 10.21 and 10.37-10.39 with the Davis wave speeds S_L = min(u_L - a_L,
// u_R - a_R), S_R = max(u_L + a_L, u_R + a_R)).  a, b: the two states; fb: the flux cotangent;
// qa, qb: the states' cotangents (accumulated).  Branches and ties as the oracle's dual numbers
// take them: min(x, y) is y only when y < x, max(x, y) is x only when y < x, the supersonic
// cases when S_L >= 0 or S_R <= 0, the left star state when S* >= 0.
template <int DIM>
__device__ __forceinline__ void hll_family_vjp(bool hllc, const double* a, const double* b, const Prim& pa,
                                               const Prim& pb, double g, const double* fb, double* qa,
                                               double* qb) {
    constexpr int NV = DIM + 2;
    SideBar L = {}, R = {};
    const double ul = pa.v[0], ur = pb.v[0];
    const double sl1 = ul - pa.a, sl2 = ur - pb.a, sr1 = ul + pa.a, sr2 = ur + pb.a;
    const bool slR = sl2 < sl1, srL = sr2 < sr1;
    const double sl = slR ? sl2 : sl1, sr = srL ? sr1 : sr2;
    double slb = 0.0, srb = 0.0;
    if (sl >= 0.0) {
        normal_flux_vjp<DIM>(a, pa, fb, 1.0, qa, L);
    } else if (sr <= 0.0) {
        normal_flux_vjp<DIM>(b, pb, fb, 1.0, qb, R);
    } else if (!hllc) {
        double Fl[NV], Fr[NV];
        euler_normal_flux<DIM>(a, ul, pa.p, Fl);
        euler_normal_flux<DIM>(b, ur, pb.p, Fr);
        const double r = rcp_refined(sr - sl), slr = sl * sr * r;
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            const double dq = b[k] - a[k];
            const double F = (sr * Fl[k] - sl * Fr[k] + sl * sr * dq) * r;
            srb = fma(fb[k], (Fl[k] + sl * dq - F) * r, srb);
            slb = fma(fb[k], (F - Fr[k] + sr * dq) * r, slb);
            qb[k] += fb[k] * slr;
            qa[k] -= fb[k] * slr;
        }
        normal_flux_vjp<DIM>(a, pa, fb, sr * r, qa, L);
        normal_flux_vjp<DIM>(b, pb, fb, -sl * r, qb, R);
    } else {
        const double rl = pa.rho, rr = pb.rho;
        const double ml = rl * (sl - ul), mr = rr * (sr - ur);
        const double Dm = ml - mr;
        const double iDm = rcp_refined(Dm);
        const double ss = ((pb.p - pa.p) + ul * ml - ur * mr) * iDm;
        const bool left = ss >= 0.0;
        // the star side K, selected per component (no local memory); its cotangents are formed in
        // qkb / K and added to the side they belong to below
        double qk[NV], qkb[NV];
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            qk[k] = left ? a[k] : b[k];
            qkb[k] = 0.0;
        }
        Prim pk;
        pk.rho = left ? pa.rho : pb.rho;
        pk.p = left ? pa.p : pb.p;
        pk.ir = left ? pa.ir : pb.ir;
#pragma unroll
        for (int k = 0; k < DIM; ++k) pk.v[k] = left ? pa.v[k] : pb.v[k];
        SideBar K = {};
        const double sk = left ? sl : sr, mk = left ? ml : mr, uk = pk.v[0];
        const double isk = rcp_refined(sk - ss), coef = mk * isk, irk = pk.ir, imk = rcp_refined(mk);
        const double X = fma(ss - uk, ss + pk.p * imk, qk[DIM + 1] * irk);
        double Us[NV];
        Us[0] = coef;
        Us[1] = coef * ss;
#pragma unroll
        for (int k = 1; k < DIM; ++k) Us[1 + k] = coef * pk.v[k];
        Us[DIM + 1] = coef * X;
        double skb = 0.0;
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            skb = fma(fb[k], Us[k] - qk[k], skb);
            qkb[k] -= sk * fb[k];
        }
        normal_flux_vjp<DIM>(qk, pk, fb, 1.0, qkb, K);
        // Us̄ = sk fb
        double coefb = sk * fma(fb[1], ss, fma(fb[DIM + 1], X, fb[0]));
#pragma unroll
        for (int k = 1; k < DIM; ++k) {
            coefb = fma(sk * fb[1 + k], pk.v[k], coefb);
            K.vt[k - 1] += sk * fb[1 + k] * coef;
        }
        const double Xb = sk * fb[DIM + 1] * coef;
        double ssb = sk * fb[1] * coef + Xb * ((ss + pk.p * imk) + (ss - uk));
        qkb[DIM + 1] += Xb * irk;
        qkb[0] -= Xb * qk[DIM + 1] * irk * irk;
        K.u -= Xb * (ss + pk.p * imk);
        K.p += Xb * (ss - uk) * imk;
        double mkb = -Xb * (ss - uk) * pk.p * imk * imk;
        // coef = mk / (sk - ss)
        mkb = fma(coefb, isk, mkb);
        skb -= coefb * coef * isk;
        ssb = fma(coefb * coef, isk, ssb);
        // ss = N / Dm, N = (pr - pl) + ul ml - ur mr, Dm = ml - mr
        const double Nb = ssb * iDm, Dmb = -ssb * ss * iDm;
        // the star side's own cotangents go to the side it is
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            qa[k] += left ? qkb[k] : 0.0;
            qb[k] += left ? 0.0 : qkb[k];
        }
        L.u += left ? K.u : 0.0;
        R.u += left ? 0.0 : K.u;
        L.p += left ? K.p : 0.0;
        R.p += left ? 0.0 : K.p;
#pragma unroll
        for (int k = 0; k < DIM - 1; ++k) {
            L.vt[k] += left ? K.vt[k] : 0.0;
            R.vt[k] += left ? 0.0 : K.vt[k];
        }
        R.p += Nb;
        L.p -= Nb;
        L.u += Nb * ml;
        R.u -= Nb * mr;
        double mlb = fma(Nb, ul, Dmb), mrb = -fma(Nb, ur, Dmb);
        if (left) mlb += mkb;
        else mrb += mkb;
        if (left) slb += skb;
        else srb += skb;
        // ml = ρl (sl - ul), mr = ρr (sr - ur)
        qa[0] += mlb * (sl - ul);
        slb = fma(mlb, rl, slb);
        L.u -= mlb * rl;
        qb[0] += mrb * (sr - ur);
        srb = fma(mrb, rr, srb);
        R.u -= mrb * rr;
    }
    // S_L = min(u_L - a_L, u_R - a_R), S_R = max(u_L + a_L, u_R + a_R)
    const double slbL = slR ? 0.0 : slb, slbR = slR ? slb : 0.0;
    const double srbL = srL ? srb : 0.0, srbR = srL ? 0.0 : srb;
    L.u += slbL + srbL;
    L.a += srbL - slbL;
    R.u += slbR + srbR;
    R.a += srbR - slbR;
    side_prim_vjp<DIM>(pa, g, L, qa);
    side_prim_vjp<DIM>(pb, g, R, qb);
}

// The dissipation vector of ScalarDissipation (Euler.jl:228-301, as the forward face kernel forms
// it in the face frame), F = A - λ/2 · intensity · D with
//   D_ρ = ρ_r - ρ_l,  D_m = m_r - m_l (zero in 3D: the reference reads the left momenta from Q_r),
//   D_E = ½ c₁ (ρ_r - ρ_l) + ½ (ρ_l + ρ_r) c₂,
//   c₁ = 1/((γ-1) β_ln) + v_l·v_r,  c₂ = ½(|v_r|² - |v_l|²) + (p_r/ρ_r - p_l/ρ_l)/(γ-1),
// β = ρ/(2p), β_ln the logarithmic mean.  Returns D and adds Dbar·∂D/∂(a, b) to qa, qb (the
// direct conserved parts) and to L, R (the cotangents of the velocities and pressures).
template <int DIM>
__device__ __forceinline__ void sd_jump_vjp(const double* a, const double* b, const Prim& pa, const Prim& pb,
                                            double g, const double* Db, double* D, double* qa, double* qb,
                                            SideBar& L, SideBar& R) {
    constexpr int NV = DIM + 2;
    const double g1 = g - 1.0, ig1 = 1.0 / g1;
    const double ipl = rcp_refined(pa.p), ipr = rcp_refined(pb.p);
    const double bl = 0.5 * pa.rho * ipl, br = 0.5 * pb.rho * ipr;
    const double hs = 0.5 * (bl + br), hd = 0.5 * (bl - br);
    double Lb, iLb, dla, dlb;
    logmean_half(0.5 * bl, 0.5 * br, hs, hd, rcp_refined(hs), Lb, iLb, dla, dlb);
    double vlr = 0.0;
#pragma unroll
    for (int k = 0; k < DIM; ++k) vlr = fma(pa.v[k], pb.v[k], vlr);
    const double c1 = fma(ig1, iLb, vlr);
    const double c2 = fma(0.5, pb.vv - pa.vv, ig1 * (pb.p * pb.ir - pa.p * pa.ir));
    const double dr = pb.rho - pa.rho, sr = pa.rho + pb.rho;
    D[0] = dr;
#pragma unroll
    for (int k = 0; k < DIM; ++k) D[1 + k] = (DIM == 3) ? 0.0 : b[1 + k] - a[1 + k];
    D[DIM + 1] = fma(0.5 * c1, dr, 0.5 * sr * c2);
    // reverse
    qb[0] += Db[0];
    qa[0] -= Db[0];
    if (DIM != 3) {
#pragma unroll
        for (int k = 0; k < DIM; ++k) {
            qb[1 + k] += Db[1 + k];
            qa[1 + k] -= Db[1 + k];
        }
    }
    const double dE = Db[DIM + 1];
    const double c1b = 0.5 * dr * dE, c2b = 0.5 * sr * dE;
    qb[0] += 0.5 * (c1 + c2) * dE;
    qa[0] += 0.5 * (c2 - c1) * dE;
    // c1: 1/β_ln and v_l·v_r
    const double ib = -ig1 * c1b * iLb * iLb;   // cotangent of β_ln
    const double blb = ib * dla, brb = ib * dlb;
    // c2: ½(|v_r|² - |v_l|²) and (p/ρ) of both sides
    const double tr = c2b * ig1 * pb.ir, tl = c2b * ig1 * pa.ir;
    qb[0] -= tr * pb.p * pb.ir;
    qa[0] += tl * pa.p * pa.ir;
    R.p += tr;
    L.p -= tl;
    // β = ρ/(2p): ρ̄ += β̄/(2p), p̄ -= β̄ β/p
    qa[0] += 0.5 * blb * ipl;
    L.p -= blb * bl * ipl;
    qb[0] += 0.5 * brb * ipr;
    R.p -= brb * br * ipr;
    // velocities (face frame: component 0 normal, then the tangents)
    const double vlb0 = fma(c1b, pb.v[0], -c2b * pa.v[0]), vrb0 = fma(c1b, pa.v[0], c2b * pb.v[0]);
    L.u += vlb0;
    R.u += vrb0;
#pragma unroll
    for (int k = 1; k < DIM; ++k) {
        L.vt[k - 1] += fma(c1b, pb.v[k], -c2b * pa.v[k]);
        R.vt[k - 1] += fma(c1b, pa.v[k], c2b * pb.v[k]);
    }
    (void)NV;
}

// The matrix-dissipation part of MatrixDissipation (Euler.jl:303-380, in the factorised form the
// forward face kernel evaluates), F = A + ½ · intensity · o with o = R |Λ| T Rᵀ ΔW:
//   ΔW = (L_β/(γ-1) + L_ρ - (|v_l|² β_l - |v_r|² β_r), 2(β_l v_l - β_r v_r), -2(β_l - β_r)),
//   L_x = ln(x_l/x_r), β = ρ/(2p); at the averaged state (ρ_ln, v̄ = (v_l+v_r)/2, p̂, β_ln):
//   a² = γ p̂/ρ_ln, h = γ/(2(γ-1)β_ln) + ½ v2, v2 = 2|v̄|² - ½(|v_l|² + |v_r|²), u = v̄_1;
//   y = Rᵀ ΔW, z = |Λ| T y (|u ∓ a| ρ_ln/(2γ), |u| (γ-1) ρ_ln/γ, |u| p̂), o = R z.
// ob = ½ · intensity · (the flux cotangent).  Adds the cotangents of both sides' densities to
// qa[0], qb[0] and those of their velocities and pressures to L, R.  |x| differentiates as Base's
// abs on the dual numbers: -1 when the sign bit is set, else +1.
template <int DIM>
__device__ __forceinline__ void md_vjp(const Prim& pa, const Prim& pb, double g, const double* ob, double* qa,
                                       double* qb, SideBar& L, SideBar& R) {
    constexpr int NV = DIM + 2, E = DIM + 1;
    const double g1 = g - 1.0, ig1 = 1.0 / g1, ig = 1.0 / g;
    const double rl = pa.rho, rr = pb.rho, pl = pa.p, pr = pb.p;
    const double* vl = pa.v;
    const double* vr = pb.v;
    const double vl2 = pa.vv, vr2 = pb.vv;
    const double ipl = rcp_refined(pl), ipr = rcp_refined(pr);
    const double bl = 0.5 * rl * ipl, br = 0.5 * rr * ipr;
    const double sr = rl + rr, sb = bl + br;
    // logarithmic means with their derivatives (logmean_half takes halved values)
    double rho, irho, dra, drb, bet, ibet, dba, dbb;
    logmean_half(0.5 * rl, 0.5 * rr, 0.5 * sr, 0.5 * (rl - rr), rcp_refined(0.5 * sr), rho, irho, dra, drb);
    logmean_half(0.5 * bl, 0.5 * br, 0.5 * sb, 0.5 * (bl - br), rcp_refined(0.5 * sb), bet, ibet, dba, dbb);
    const double Lr = log(rl * pb.ir), Lb = log(bl * rcp_refined(br));
    const double isb = rcp_refined(sb), phat = 0.5 * sr * isb;
    double vm[3] = {0.0, 0.0, 0.0}, vv = 0.0;
#pragma unroll
    for (int k = 0; k < DIM; ++k) {
        vm[k] = 0.5 * (vl[k] + vr[k]);
        vv = fma(vm[k], vm[k], vv);
    }
    const double v2 = fma(2.0, vv, -0.5 * (vl2 + vr2));
    const double a2 = g * phat * irho, ia = rsqrt_refined(a2), a = a2 * ia;
    const double h = fma(0.5 * g * ig1, ibet, 0.5 * v2);
    double dW[NV];
    dW[0] = fma(Lb, ig1, Lr) - (vl2 * bl - vr2 * br);
#pragma unroll
    for (int k = 0; k < DIM; ++k) dW[1 + k] = 2.0 * (bl * vl[k] - br * vr[k]);
    dW[E] = -2.0 * (bl - br);
    const double u = vm[0];
    double S = fma(u, dW[1], dW[0]);
#pragma unroll
    for (int k = 1; k < DIM; ++k) S = fma(vm[k], dW[1 + k], S);
    double y[NV];
    y[0] = S - a * dW[1] + (h - u * a) * dW[E];
    y[E] = S + a * dW[1] + (h + u * a) * dW[E];
    y[1] = fma(0.5 * v2, dW[E], S);
#pragma unroll
    for (int k = 1; k < DIM; ++k) y[1 + k] = fma(vm[k], dW[E], dW[1 + k]);
    const double ta = rho * (0.5 * ig), c1 = g1 * rho * ig;
    const double um = u - a, up = u + a;
    const double sm = signbit(um) ? -1.0 : 1.0, sp = signbit(up) ? -1.0 : 1.0, su = signbit(u) ? -1.0 : 1.0;
    const double aum = fabs(um), aup = fabs(up), au = fabs(u);
    double z[NV];
    z[0] = aum * ta * y[0];
    z[1] = au * c1 * y[1];
#pragma unroll
    for (int k = 1; k < DIM; ++k) z[1 + k] = au * phat * y[1 + k];
    z[E] = aup * ta * y[E];
    const double zs = z[0] + z[1] + z[E];
    // reverse: o = R z
    double vmo = 0.0;   // Σ_{k≥1} v̄_k ō_{1+k}
#pragma unroll
    for (int k = 1; k < DIM; ++k) vmo = fma(vm[k], ob[1 + k], vmo);
    double zb[NV];
    zb[0] = ob[0] + um * ob[1] + (h - u * a) * ob[E] + vmo;
    zb[1] = ob[0] + u * ob[1] + 0.5 * v2 * ob[E] + vmo;
    zb[E] = ob[0] + up * ob[1] + (h + u * a) * ob[E] + vmo;
#pragma unroll
    for (int k = 1; k < DIM; ++k) zb[1 + k] = fma(vm[k], ob[E], ob[1 + k]);
    double vmb[3] = {0.0, 0.0, 0.0};
    double ab_ = ob[1] * (z[E] - z[0]) + ob[E] * u * (z[E] - z[0]);
    double hb = ob[E] * (z[0] + z[E]);
    double v2b = 0.5 * ob[E] * z[1];
    vmb[0] = ob[1] * zs + ob[E] * a * (z[E] - z[0]);
#pragma unroll
    for (int k = 1; k < DIM; ++k) vmb[k] = fma(ob[1 + k], zs, ob[E] * z[1 + k]);
    // z = |Λ| T y
    double yb[NV], tab = 0.0, rhob = 0.0, phb = 0.0;
    yb[0] = zb[0] * aum * ta;
    vmb[0] += zb[0] * sm * ta * y[0];
    ab_ -= zb[0] * sm * ta * y[0];
    tab += zb[0] * aum * y[0];
    yb[1] = zb[1] * au * c1;
    vmb[0] += zb[1] * su * c1 * y[1];
    rhob += zb[1] * au * g1 * ig * y[1];
#pragma unroll
    for (int k = 1; k < DIM; ++k) {
        yb[1 + k] = zb[1 + k] * au * phat;
        vmb[0] += zb[1 + k] * su * phat * y[1 + k];
        phb += zb[1 + k] * au * y[1 + k];
    }
    yb[E] = zb[E] * aup * ta;
    vmb[0] += zb[E] * sp * ta * y[E];
    ab_ += zb[E] * sp * ta * y[E];
    tab += zb[E] * aup * y[E];
    rhob += tab * 0.5 * ig;
    // y = Rᵀ ΔW
    const double Sb = yb[0] + yb[E] + yb[1];
    double dWb[NV];
    dWb[0] = Sb;
    dWb[1] = fma(u, Sb, a * (yb[E] - yb[0]));
    ab_ += dW[1] * (yb[E] - yb[0]) + u * dW[E] * (yb[E] - yb[0]);
    hb += dW[E] * (yb[0] + yb[E]);
    vmb[0] += dW[1] * Sb + a * dW[E] * (yb[E] - yb[0]);
    dWb[E] = (h - u * a) * yb[0] + (h + u * a) * yb[E] + 0.5 * v2 * yb[1];
    v2b += 0.5 * dW[E] * yb[1];
#pragma unroll
    for (int k = 1; k < DIM; ++k) {
        dWb[E] = fma(vm[k], yb[1 + k], dWb[E]);
        dWb[1 + k] = fma(vm[k], Sb, yb[1 + k]);
        vmb[k] += fma(dW[E], yb[1 + k], dW[1 + k] * Sb);
    }
    // h, a
    double ibetb = 0.5 * g * ig1 * hb;
    v2b += 0.5 * hb;
    phb += ab_ * g * irho * 0.5 * ia;
    double irhob = ab_ * g * phat * 0.5 * ia;
    // ΔW
    double Lbb = ig1 * dWb[0], Lrb = dWb[0];
    double vl2b = -dWb[0] * bl, vr2b = dWb[0] * br;
    double blb = -dWb[0] * vl2 - 2.0 * dWb[E], brb = dWb[0] * vr2 + 2.0 * dWb[E];
    double vlb[3] = {0.0, 0.0, 0.0}, vrb[3] = {0.0, 0.0, 0.0};
#pragma unroll
    for (int k = 0; k < DIM; ++k) {
        blb = fma(2.0 * dWb[1 + k], vl[k], blb);
        brb = fma(-2.0 * dWb[1 + k], vr[k], brb);
        vlb[k] = 2.0 * bl * dWb[1 + k];
        vrb[k] = -2.0 * br * dWb[1 + k];
    }
    // v2 = 2|v̄|² - ½(|v_l|² + |v_r|²), v̄ = (v_l + v_r)/2
    vl2b -= 0.5 * v2b;
    vr2b -= 0.5 * v2b;
#pragma unroll
    for (int k = 0; k < DIM; ++k) {
        const double m = vmb[k] + 4.0 * vm[k] * v2b;   // v̄_k cotangent incl. |v̄|²
        vlb[k] += fma(0.5, m, 2.0 * vl[k] * vl2b);
        vrb[k] += fma(0.5, m, 2.0 * vr[k] * vr2b);
    }
    // means: p̂ = ½ s_ρ/s_β, 1/ρ_ln, 1/β_ln, and the logarithms
    rhob -= irhob * irho * irho;
    const double betb = -ibetb * ibet * ibet;
    double rlb = fma(rhob, dra, 0.5 * phb * isb) + Lrb / rl;
    double rrb = fma(rhob, drb, 0.5 * phb * isb) - Lrb / rr;
    blb += fma(betb, dba, -phb * phat * isb) + Lbb / bl;
    brb += fma(betb, dbb, -phb * phat * isb) - Lbb / br;
    // β = ρ/(2p)
    rlb = fma(0.5 * ipl, blb, rlb);
    rrb = fma(0.5 * ipr, brb, rrb);
    L.p -= blb * bl * ipl;
    R.p -= brb * br * ipr;
    qa[0] += rlb;
    qb[0] += rrb;
    L.u += vlb[0];
    R.u += vrb[0];
#pragma unroll
    for (int k = 1; k < DIM; ++k) {
        L.vt[k - 1] += vlb[k];
        R.vt[k - 1] += vrb[k];
    }
}

// VJP of the numerical flux of kind KIND (adj_face_kernel's list) in the face frame: a, b the
// two states, fb the flux cotangent; ab, bbar receive the states' cotangents (overwritten).
// Returns the cotangent of the dissipation intensity (LxF only).
template <int DIM, int KIND>
__device__ __forceinline__ double numflux_vjp(const double* a, const double* b, double inten, double g,
                                              const double* fb, double* ab, double* bbar) {
    constexpr bool CHANDRA = KIND == 1 || KIND == 5 || KIND == 7;
    constexpr bool SD = KIND == 4 || KIND == 5;
    constexpr bool MD = KIND >= 6;
    constexpr int NV = DIM + 2;
    const double g1 = g - 1.0;
    Prim pa = prim_of<DIM>(a, g);
    const double* bb = b;
    Prim pb = prim_of<DIM>(bb, g);
    double Ib = 0.0;
    if (KIND == 2 || KIND == 3) {   // HLL / HLLC: no dissipation scale, so no intensity cotangent
#pragma unroll
        for (int k = 0; k < NV; ++k) ab[k] = bbar[k] = 0.0;
        hll_family_vjp<DIM>(KIND == 3, a, bb, pa, pb, g, fb, ab, bbar);
    } else {
    double ll = fabs(pa.v[0]) + pa.a, lr = fabs(pb.v[0]) + pb.a;
    bool left = lr < ll;   // Base.max(ll, lr)
    double lam = left ? ll : lr;
    double dot = 0.0;
    SideBar Ls = {}, Rs = {};
    if (MD) {   // F = A + ½ · intensity · R|Λ|TRᵀΔW: no wave-speed maximum
        double ob[NV];
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            ob[k] = 0.5 * inten * fb[k];
            ab[k] = bbar[k] = 0.0;
        }
        md_vjp<DIM>(pa, pb, g, ob, ab, bbar, Ls, Rs);
    } else if (SD) {   // F = A - λ/2 · intensity · D(a, b)
        double D[NV], Db[NV];
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            Db[k] = -0.5 * inten * lam * fb[k];
            ab[k] = bbar[k] = 0.0;
        }
        sd_jump_vjp<DIM>(a, bb, pa, pb, g, Db, D, ab, bbar, Ls, Rs);
#pragma unroll
        for (int k = 0; k < NV; ++k) dot = fma(-fb[k], D[k], dot);
    } else {    // F = A + λ/2 · intensity · (a - b)
#pragma unroll
        for (int k = 0; k < NV; ++k) dot = fma(fb[k], a[k] - bb[k], dot);
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            ab[k] = 0.5 * inten * lam * fb[k];
            bbar[k] = -ab[k];
        }
    }
    Ib = (SD || MD) ? 0.0 : 0.5 * lam * dot;   // the dissipation fluxes take no per-element scale
    if (CHANDRA) {   // LxF(ChandrasekharAverage): the pair flux of the two traces
        PrimBar o1, o2;
        double vh1[DIM], vh2[DIM];
#pragma unroll
        for (int k = 0; k < DIM; ++k) {
            vh1[k] = 0.5 * pa.v[k];
            vh2[k] = 0.5 * pb.v[k];
        }
        chandra_pair_vjp<DIM, 0, true>(0.5 * pa.rho, vh1, 0.25 * pa.rho * rcp_refined(pa.p), 0.25 * pa.vv,
                                       0.5 * pb.rho, vh2, 0.25 * pb.rho * rcp_refined(pb.p), 0.25 * pb.vv,
                                       0.5 / g1, fb, o1, o2);
        prim_to_cons_vjp<DIM>(pa.rho, pa.v, pa.vv, pa.p, g1, o1, ab);
        prim_to_cons_vjp<DIM>(pb.rho, pb.v, pb.vv, pb.p, g1, o2, bbar);
    } else {
        euler_flux_vjp<DIM>(0, pa.v, pa.vv, pa.H, g1, fb, 0.5, ab);
        euler_flux_vjp<DIM>(0, pb.v, pb.vv, pb.H, g1, fb, 0.5, bbar);
    }
    if (!MD) {
        double kappa = 0.5 * inten * dot;
        if (left) lambda_vjp<DIM>(pa, g, kappa, ab);
        else lambda_vjp<DIM>(pb, g, kappa, bbar);
    }
    if (SD || MD) {
        side_prim_vjp<DIM>(pa, g, Ls, ab);
        side_prim_vjp<DIM>(pb, g, Rs, bbar);
    }
    }
    return Ib;
}

// KIND: 0 LxF(StdAverage), 1 LxF(ChandrasekharAverage), 2 HLL, 3 HLLC,
// 4 ScalarDissipation(StdAverage), 5 ScalarDissipation(ChandrasekharAverage),
// 6 MatrixDissipation(StdAverage), 7 MatrixDissipation(ChandrasekharAverage).
// CURV: general geometry, the forward face kernel's CURV path transposed: the slave trace at
// master2slave(m, o), per-node 1/J on both sides, the face-node frame (n, t, b) and surface
// Jacobian (a = R q, F = J Rᵀ F_face: F̄_face = J R F̄, q̄ = Rᵀ ā).
// G: the forward's general trace path (the strong form without exact end-node injection, the
// split form on Gauss nodes): the traces are the interpolations Σ_p l[p] U_p along the line, and
// the lift reaches every node of it, so
// the flux cotangent gathers -Σ_p ∂g[p] w_p over the line (the element kernel scatters the trace
// cotangents back with l).
template <int DIM, int KIND, bool CURV = false, bool G = false>
__global__ void __launch_bounds__(256) adj_face_kernel(AdjFaceParams P) {
    constexpr int NV = DIM + 2;
    int64_t gid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (gid >= (int64_t)P.nfaces * P.nfd) return;
    int f = (int)(gid / P.nfd), m = (int)(gid - (int64_t)f * P.nfd);
    int n = P.n;
    int32_t s0 = P.face_elem[2 * f], s1 = P.face_elem[2 * f + 1];
    const double* dgl = P.ops + 2 * n * n + 2 * n;
    const double* dgr = dgl + n;
    auto endnode = [&](int32_t s, int mm, int64_t* g, double* dg) {
        int e = s >> 3, pos = s & 7, dir = pos >> 1, right = pos & 1;
        *g = (int64_t)e * P.npe + tp_node<DIM>(n, dir, mm, right ? n - 1 : 0);
        *dg = right ? dgr[n - 1] : dgl[0];
    };
    // G: the trace of side s (interpolated with l) and the lift transpose Σ_p ∂g[p] (w λ)_p
    auto line_sums = [&](int32_t s, int mm, double* q, double* fl) {
        int e = s >> 3, pos = s & 7, dir = pos >> 1, right = pos & 1;
        const double* lv = P.ops + 2 * n * n + (right ? n : 0);
        const double* dg = right ? dgr : dgl;
#pragma unroll
        for (int k = 0; k < DIM + 2; ++k) q[k] = fl[k] = 0.0;
        for (int p = 0; p < n; ++p) {
            const int64_t g = (int64_t)e * P.npe + tp_node<DIM>(n, dir, mm, p);
            const double wl = (CURV ? P.invJn[g] : P.invJ[e]) * P.s_lam * dg[p];
#pragma unroll
            for (int k = 0; k < DIM + 2; ++k) {
                q[k] = fma(lv[p], P.U[k * P.ndofs + g], q[k]);
                fl[k] = fma(wl, P.Ain[k * P.ndofs + g], fl[k]);
            }
        }
    };
    int64_t g1i = 0, g2i = 0;
    double dg1 = 0.0, dg2 = 0.0;
    if (kChecked && !(index_ok(s0 >> 3, P.ndofs / P.npe, P.status, 0) &&
                      (s1 < 0 || index_ok(s1 >> 3, P.ndofs / P.npe, P.status, s0 >> 3)) &&
                      (s1 >= 0 || index_ok(P.face_bc[f], MAXBC, P.status, s0 >> 3))))
        return;
    double qL[NV], qR[NV], Fb[NV];
    if constexpr (G) {
        double fl[NV];
        line_sums(s0, m, qL, fl);
#pragma unroll
        for (int k = 0; k < NV; ++k) Fb[k] = P.FbS ? P.FbS[k * P.nfdofs + gid] : -fl[k];
    } else {
        endnode(s0, m, &g1i, &dg1);
        double w1 = (CURV ? P.invJn[g1i] : P.invJ[s0 >> 3]) * P.s_lam;
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            qL[k] = P.U[k * P.ndofs + g1i];
            Fb[k] = -dg1 * (w1 * P.Ain[k * P.ndofs + g1i]);
        }
    }
    if (s1 >= 0) {
        const int mm = CURV ? master2slave<DIM>(m, P.orient[f], n) : m;
        if (CURV && !index_ok(mm, P.nfd, P.status, s1 >> 3)) return;
        if constexpr (G) {
            double fl[NV];
            line_sums(s1, mm, qR, fl);
#pragma unroll
            for (int k = 0; k < NV; ++k) Fb[k] += P.FbS ? P.FbS[(NV + k) * P.nfdofs + gid] : fl[k];
        } else {
            endnode(s1, mm, &g2i, &dg2);
            double w2 = (CURV ? P.invJn[g2i] : P.invJ[s1 >> 3]) * P.s_lam;
#pragma unroll
            for (int k = 0; k < NV; ++k) {
                qR[k] = P.U[k * P.ndofs + g2i];
                Fb[k] = fma(dg2, w2 * P.Ain[k * P.ndofs + g2i], Fb[k]);
            }
        }
    }
    FrameAxes A = frame_axes<DIM>(s0 & 7);
    FrameTab fr;
    if (CURV) {
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            fr.n[c] = P.frames[c * P.nfdofs + gid];
            fr.t[c] = P.frames[(3 + c) * P.nfdofs + gid];
            fr.b[c] = P.frames[(6 + c) * P.nfdofs + gid];
        }
    }
    double J = CURV ? P.faceJn[gid] : P.faceJ[f];
    // face frame: a = R qL, b = R qR (or the boundary state), F̄ = J R F̄_phys
    double a[NV], b[NV], fb[NV];
    a[0] = qL[0];
    a[DIM + 1] = qL[DIM + 1];
    fb[0] = J * Fb[0];
    fb[DIM + 1] = J * Fb[DIM + 1];
    {
        double t[NV];
        if (CURV) {
            rotate_to_face<DIM>(qL, fr, a);
            rotate_to_face<DIM>(Fb, fr, t);
        } else {
            cart_to_face<DIM>(qL, A, a);
            cart_to_face<DIM>(Fb, A, t);
        }
#pragma unroll
        for (int r = 0; r < DIM; ++r) fb[1 + r] = J * t[1 + r];
    }
    int bck = 0;
    if (s1 >= 0) {
        b[0] = qR[0];
        b[DIM + 1] = qR[DIM + 1];
        if (CURV) rotate_to_face<DIM>(qR, fr, b);
        else cart_to_face<DIM>(qR, A, b);
    } else {
        const int bi = P.face_bc[f];
        bck = P.bc_kind[bi];
        if (bck == FLOU_BC_INFLOW || bck == FLOU_BC_STATE_FIELD) {   // a fixed external state
            double qe[NV];
#pragma unroll
            for (int k = 0; k < NV; ++k)
                qe[k] = bck == FLOU_BC_INFLOW ? P.bc_state[bi][k] : P.bc_field[k * P.nfdofs + gid];
            b[0] = qe[0];
            b[DIM + 1] = qe[DIM + 1];
            if (CURV) rotate_to_face<DIM>(qe, fr, b);
            else cart_to_face<DIM>(qe, A, b);
        } else {
#pragma unroll
            for (int k = 0; k < NV; ++k) b[k] = a[k];   // outflow; slip flips the normal momentum
            if (bck == FLOU_BC_SLIP) b[1] = -a[1];
        }
    }
    double inten = P.intensity;
    if (P.elem_c) {
        int e1 = s0 >> 3, e2 = s1 >= 0 ? (s1 >> 3) : e1;
        inten = (P.elem_c[e1] + P.elem_c[e2]) * 0.5;
    }
    double ab[NV], bbar[NV];
    const double Ib = numflux_vjp<DIM, KIND>(a, b, inten, P.gamma, fb, ab, bbar);
    if (s1 < 0) {
        if (bck == FLOU_BC_OUTFLOW) {
#pragma unroll
            for (int k = 0; k < NV; ++k) ab[k] += bbar[k];
        } else if (bck == FLOU_BC_SLIP) {
#pragma unroll
            for (int k = 0; k < NV; ++k) ab[k] += (k == 1) ? -bbar[k] : bbar[k];
        }
    }
    // back to the physical frame (Rᵀ)
    double oL[NV], oR[NV];
    oL[0] = ab[0];
    oL[DIM + 1] = ab[DIM + 1];
    oR[0] = bbar[0];
    oR[DIM + 1] = bbar[DIM + 1];
    if (CURV) {
        rotate_to_phys<DIM>(ab, fr, oL);
        rotate_to_phys<DIM>(bbar, fr, oR);
    } else {
        cart_to_phys<DIM>(ab, A, oL);
        cart_to_phys<DIM>(bbar, A, oR);
    }
#pragma unroll
    for (int k = 0; k < NV; ++k) {
        P.QbL[k * P.nfdofs + gid] = oL[k];
        if (s1 >= 0) P.QbR[k * P.nfdofs + gid] = oR[k];
    }
    P.Ibar[gid] = Ib;
}

// Face-flux offset of the trace of line `line` of the face at local position fk of element e:
// a slave reads the master's face dof that master2slave sends onto its line (CURV), as the
// forward lift does.
template <int DIM, int N, bool CURV>
__device__ __forceinline__ int64_t trace_offset(const AdjElemParams& P, int e, int fk, int line) {
    const int32_t pk = P.elem_face[e * 2 * DIM + fk];
    int lm = line;
    if (CURV && (pk & 1)) lm = master2slave<DIM>(line, inverse_orientation<DIM>(P.orient[pk >> 1]), N);
    return (int64_t)(pk >> 1) * ipow(N, DIM - 1) + lm;
}

// CURV: general geometry: per-node 1/J, and the contravariant flux F̃_d = Σ_k Ja[k][d] F_k, whose
// transpose gathers the directions first, G̃_k = Σ_d Ja[k][d] G_d, then takes one flux VJP per k.
// G: a basis without exact end-node injection (the strong form on Gauss nodes): every node of a
// line takes l_l[pos] and l_r[pos] of the trace cotangents of the line's two faces.
template <int DIM, int N, bool CURV = false, bool G = false>
__global__ void __launch_bounds__(Shape<DIM, N>::BLOCK) adj_elem_kernel(AdjElemParams P) {
    using S = Shape<DIM, N>;
    constexpr int NV = DIM + 2, NPE = S::NPE, NN = S::NN, NFD = S::NFD;
    extern __shared__ double smem[];
    double* sops = smem;
    double* sw = sops + S::NOPS;   // [NV][NN]: w = λ / J
    const int tid = threadIdx.x;
    for (int t = tid; t < S::NOPS; t += blockDim.x) sops[t] = P.ops[t];
    const int e0 = blockIdx.x * S::EPB;
    const int el = tid / NPE, i = tid - el * NPE;
    const int e = e0 + el;
    const bool active = (tid < NN) && (e < P.nelem);
    int64_t gi = (int64_t)e * NPE + i;
    double ain[NV];
    if (active) {
        double w = (CURV ? P.invJn[gi] : P.invJ[e]) * P.s_lam;
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            ain[k] = P.Ain[k * P.ndofs + gi];
            sw[k * NN + tid] = w * ain[k];
        }
    }
    __syncthreads();
    if (!active) return;
    double q[NV];
#pragma unroll
    for (int k = 0; k < NV; ++k) q[k] = P.U[k * P.ndofs + gi];
    Prim pr = prim_of<DIM, false>(q, P.gamma);
    const double g1 = P.gamma - 1.0;
    double qb[NV];
#pragma unroll
    for (int k = 0; k < NV; ++k) qb[k] = 0.0;
    const double* Ds = sops;
    double Gt[CURV ? DIM : 1][NV];   // CURV: G̃_k = Σ_d Ja[k][d] G_d
#pragma unroll
    for (int k = 0; k < (CURV ? DIM : 1); ++k)
#pragma unroll
        for (int v = 0; v < NV; ++v) Gt[k][v] = 0.0;
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
        int pos, line;
        tp_coords<DIM>(N, i, d, pos, line);
        double Gd[NV];
#pragma unroll
        for (int k = 0; k < NV; ++k) Gd[k] = 0.0;
#pragma unroll
        for (int r = 0; r < N; ++r) {   // Σ_rows Ds(row, pos) w_row  (transpose)
            int j = el * NPE + tp_node<DIM>(N, d, line, r);
            double a = Ds[r + pos * N];
#pragma unroll
            for (int k = 0; k < NV; ++k) Gd[k] = fma(a, sw[k * NN + j], Gd[k]);
        }
        if constexpr (CURV) {
#pragma unroll
            for (int k = 0; k < DIM; ++k) {
                const double jkd = P.Jan[(k + d * DIM) * P.ndofs + gi];
#pragma unroll
                for (int v = 0; v < NV; ++v) Gt[k][v] = fma(jkd, Gd[v], Gt[k][v]);
            }
        } else {
            euler_flux_vjp<DIM>(d, pr.v, pr.vv, pr.H, g1, Gd, -P.Ja[e * DIM + d], qb);
        }
        // trace cotangents of the faces this node lies on (LGL: the end nodes)
        if constexpr (G) {
#pragma unroll
            for (int side = 0; side < 2; ++side) {
                const int fk = 2 * d + side;
                const int32_t pk = P.elem_face[e * 2 * DIM + fk];
                const double* src = (pk & 1) ? P.QbR : P.QbL;
                const double lw = sops[2 * N * N + side * N + pos];
                int64_t o = trace_offset<DIM, N, CURV>(P, e, fk, line);
                if (!index_ok(o, P.nfdofs, P.status, e)) continue;
#pragma unroll
                for (int k = 0; k < NV; ++k) qb[k] = fma(lw, __ldcg(src + k * P.nfdofs + o), qb[k]);
            }
        } else if (pos == 0 || pos == N - 1) {
            const int fk = 2 * d + (pos == 0 ? 0 : 1);
            const int32_t pk = P.elem_face[e * 2 * DIM + fk];
            const double* src = (pk & 1) ? P.QbR : P.QbL;
            int64_t o = trace_offset<DIM, N, CURV>(P, e, fk, line);
            if (!index_ok(o, P.nfdofs, P.status, e)) continue;
#pragma unroll
            for (int k = 0; k < NV; ++k) qb[k] += __ldcg(src + k * P.nfdofs + o);
        }
    }
    if constexpr (CURV) {
#pragma unroll
        for (int k = 0; k < DIM; ++k) euler_flux_vjp<DIM>(k, pr.v, pr.vv, pr.H, g1, Gt[k], -1.0, qb);
    }
#pragma unroll
    for (int k = 0; k < NV; ++k) {
        double o = fma(P.alpha, ain[k], qb[k]);
        if (P.readB) o = fma(P.beta, P.B[k * P.ndofs + gi], o);
        if (P.writeB) {
            double b = P.delta_B * ain[k];
            if (P.gamma_B != 0.0) b = fma(P.gamma_B, P.B[k * P.ndofs + gi], b);
            P.B[k * P.ndofs + gi] = b;
        }
        P.Aout[k * P.ndofs + gi] = o;
        if (P.K) P.K[k * P.ndofs + gi] = fma(P.kA, ain[k], P.kB * o);
    }
    if (P.cbar && i == 0) {   // intensity (c1 + c2)/2: each side gets half, a boundary face all
        double acc = 0.0;
        for (int fk = 0; fk < 2 * DIM; ++fk) {
            int32_t pk = P.elem_face[e * 2 * DIM + fk];
            int fc = pk >> 1;
            if (!index_ok((int64_t)fc * NFD + NFD - 1, P.nfdofs, P.status, e)) continue;
            double wgt = P.face_elem[2 * fc + 1] < 0 ? 1.0 : 0.5;
            for (int m = 0; m < NFD; ++m) acc = fma(wgt, __ldcg(P.Ibar + (int64_t)fc * NFD + m), acc);
        }
        P.cbar[e] += acc;
    }
}

template <int DIM, int N, bool CURV = false, bool G = false>
cudaError_t launch_adj_elem_n(const AdjElemParams& P, cudaStream_t s) {
    using S = Shape<DIM, N>;
    constexpr size_t smem = sizeof(double) * (S::NOPS + (DIM + 2) * S::NN);
    static std::once_flag once;
    static cudaError_t attr = cudaSuccess;
    std::call_once(once, [] {
        attr = cudaFuncSetAttribute(adj_elem_kernel<DIM, N, CURV, G>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)smem);
    });
    if (attr != cudaSuccess) return attr;
    int grid = (P.nelem + S::EPB - 1) / S::EPB;
    adj_elem_kernel<DIM, N, CURV, G><<<grid, S::BLOCK, smem, s>>>(P);
    return cudaGetLastError();
}

template <int DIM, bool CURV = false, bool G = false>
cudaError_t launch_adj_elem(int n, const AdjElemParams& P, cudaStream_t s) {
    switch (n) {
        case 2: return launch_adj_elem_n<DIM, 2, CURV, G>(P, s);
        case 3: return launch_adj_elem_n<DIM, 3, CURV, G>(P, s);
        case 4: return launch_adj_elem_n<DIM, 4, CURV, G>(P, s);
        case 5: return launch_adj_elem_n<DIM, 5, CURV, G>(P, s);
        case 6: return launch_adj_elem_n<DIM, 6, CURV, G>(P, s);
        case 7: return launch_adj_elem_n<DIM, 7, CURV, G>(P, s);
        case 8: return launch_adj_elem_n<DIM, 8, CURV, G>(P, s);
        default: return cudaErrorInvalidValue;
    }
}

// Split-form element adjoint.  Per direction, a pair phase evaluates every symmetric pair of
// the block's lines once and keeps the primitive cotangents of both nodes in shared memory;
// the node phase then sums its pairs, adds the diagonal term D♯(i,i) F(Q_i) (the physical flux;
// zero on interior LGL nodes) and the face traces, and finally maps (ρ̄, v̄, β̄) to the conserved
// variables.
template <int DIM, int N, int TP = FLOU_TP_CHANDRASHEKAR, bool G = false, bool H = false>
struct AdjSplitShape {
    using S = Shape<DIM, N>;
    static constexpr bool KG = TP == FLOU_TP_KENNEDY_GRUBER;
    static constexpr bool STD = TP == FLOU_TP_STD_AVERAGE;
    static constexpr int NV = DIM + 2;
    // per node: rh, vh, bh, vq (KG: rh, vh, ph, eh; StdAverage: H, v, |v|²)
    static constexpr int NARR = DIM + 3;
    // per side of a pair: ρ̄, v̄, β̄ (KG: ρ̄, v̄, p̄, ē; StdAverage: the conserved cotangent)
    static constexpr int NPB = KG ? DIM + 3 : DIM + 2;
    static constexpr int NPT = S::EPB * S::NFD * S::NPAIR;
    static constexpr int NSD = S::EPB * DIM * N * N;           // -Ja_d D♯ per element and direction
    // G (Gauss nodes): per line side the cotangent of its projected entropy variables, and per node
    // the cotangents of its two projected-state pair fluxes
    static constexpr int NPROJ = G ? 2 * S::EPB * S::NFD : 0;
    // H (hybrid operator): per node the subcell-flux values, then their cotangents; G and H (the
    // hybrid operator on Gauss nodes): also the projected-state flux differences of both line
    // sides per node, later the entropy-jump cotangents and the hand-over to the left neighbour
    static constexpr int NGX0 = (G ? NV * NPROJ + NPB * S::NN : 0) + (H ? NV * S::NN : 0) +
                                (G && H ? 2 * NV * S::NN : 0);
    static constexpr size_t FIXED =
        sizeof(double) * (S::NOPS + (size_t)NARR * S::NN + (size_t)NV * S::NN + NSD) + 2 * (S::NPAIR + 1);
    // The pair cotangents of a direction in CH chunks of its lines (one element per block): two
    // where all of them at once would not fit in shared memory (the 3D p=7 tiles of the
    // Gauss-node and Kennedy-Gruber hybrid forms), each chunk's pairs then its nodes.
    static constexpr int CH =
        (FIXED + sizeof(double) * (2 * (size_t)NPB * NPT + NGX0) > 227 * 1024 && S::EPB == 1 && S::NFD % 2 == 0) ? 2
                                                                                                              : 1;
    static constexpr int NPTC = NPT / CH;   // pairs of one chunk
    static constexpr size_t BASE = FIXED + sizeof(double) * 2 * (size_t)NPB * NPTC;
    // G, H: every node's entropy variables, evaluated once per block where the tile has room for
    // them (all but some 3D p=7 tiles); else each use evaluates them again
    static constexpr bool WC = (G || H) && BASE + sizeof(double) * ((size_t)NGX0 + (size_t)NV * S::NN) <= 227 * 1024;
    static constexpr int NGX = NGX0 + (WC ? NV * S::NN : 0);
    static constexpr size_t SMEM = BASE + sizeof(double) * (size_t)NGX;
    // two resident blocks where the register file allows 64K / (2 * BLOCK) >= 128 registers
    // (G, H: two where that still leaves 144 registers, else one, for the projection's registers)
    static constexpr int MINB = (!G && !H) ? ((S::BLOCK * 2 * 128 <= 65536) ? 2 : 1)
                                           : ((S::BLOCK * 2 * 144 <= 65536) ? 2 : 1);
};

// Per-node quantities the split adjoint keeps for a state q (p its pressure): Chandrashekar
// ρ/2, v/2, β/2, |v|²/4; Kennedy-Gruber ρ/2, v/2, p/2, e/2; StdAverage H, v, |v|².
template <int DIM, int TP>
__device__ __forceinline__ void split_node_values(const double* q, double p, double* o) {
    const double rho = q[0], ir = rcp_refined(rho);
    double v[DIM], vv = 0.0;
#pragma unroll
    for (int k = 0; k < DIM; ++k) {
        v[k] = q[1 + k] * ir;
        vv = fma(v[k], v[k], vv);
    }
    if constexpr (TP == FLOU_TP_STD_AVERAGE) {
        o[0] = (q[DIM + 1] + p) * ir;
#pragma unroll
        for (int k = 0; k < DIM; ++k) o[1 + k] = v[k];
        o[1 + DIM] = vv;
    } else {
        o[0] = 0.5 * rho;
#pragma unroll
        for (int k = 0; k < DIM; ++k) o[1 + k] = 0.5 * v[k];
        if constexpr (TP == FLOU_TP_KENNEDY_GRUBER) {
            o[1 + DIM] = 0.5 * p;
            o[2 + DIM] = 0.5 * (q[DIM + 1] * ir);
        } else {
            o[1 + DIM] = (0.25 * rho) * rcp_refined(p);
            o[2 + DIM] = 0.25 * vv;
        }
    }
}

// The two-point flux VJP of the split form along axis D for two nodes given by their
// split_node_values A and B: cotangents in the format the node phase sums (PrimBar; StdAverage:
// conserved).
// D < 0: along the general direction nrm (general geometry).
template <int DIM, int D, int TP>
__device__ __forceinline__ void split_pair_vjp(const double* A, const double* B, const double* Fb, double cb,
                                               double g1, PrimBar& o1, PrimBar& o2, const double* nrm = nullptr) {
    constexpr int NV = DIM + 2;
    if constexpr (TP == FLOU_TP_STD_AVERAGE) {
        double qa_[NV], qb_[NV];
#pragma unroll
        for (int k = 0; k < NV; ++k) qa_[k] = qb_[k] = 0.0;
        if constexpr (D >= 0) {
            euler_flux_vjp<DIM>(D, A + 1, A[1 + DIM], A[0], g1, Fb, 0.5, qa_);
            euler_flux_vjp<DIM>(D, B + 1, B[1 + DIM], B[0], g1, Fb, 0.5, qb_);
        } else {
            euler_flux_vjp_n<DIM>(nrm, A + 1, A[1 + DIM], A[0], g1, Fb, 0.5, qa_);
            euler_flux_vjp_n<DIM>(nrm, B + 1, B[1 + DIM], B[0], g1, Fb, 0.5, qb_);
        }
        o1.r = qa_[0];
        o2.r = qb_[0];
#pragma unroll
        for (int k = 0; k < DIM; ++k) {
            o1.v[k] = qa_[1 + k];
            o2.v[k] = qb_[1 + k];
        }
        o1.b = qa_[DIM + 1];
        o2.b = qb_[DIM + 1];
        o1.e = o2.e = 0.0;
    } else if constexpr (TP == FLOU_TP_KENNEDY_GRUBER) {
        kg_pair_vjp<DIM, D>(A[0], A + 1, A[1 + DIM], A[2 + DIM], B[0], B + 1, B[1 + DIM], B[2 + DIM], Fb, o1, o2,
                            nrm);
    } else {
        chandra_pair_vjp<DIM, D, false>(A[0], A + 1, A[1 + DIM], A[2 + DIM], B[0], B + 1, B[1 + DIM], B[2 + DIM], cb,
                                        Fb, o1, o2, nrm);
        o1.e = o2.e = 0.0;
    }
}

// Conserved cotangent of a state from the node-format cotangent o (split_node_values' format).
template <int DIM, int TP>
__device__ __forceinline__ void split_node_to_cons(const double* q, double p, double g1, const PrimBar& o,
                                                   double* qb) {
    if constexpr (TP == FLOU_TP_STD_AVERAGE) {
        qb[0] += o.r;
#pragma unroll
        for (int k = 0; k < DIM; ++k) qb[1 + k] += o.v[k];
        qb[DIM + 1] += o.b;
    } else {
        const double ir = rcp_refined(q[0]);
        double v[DIM], vv = 0.0;
#pragma unroll
        for (int k = 0; k < DIM; ++k) {
            v[k] = q[1 + k] * ir;
            vv = fma(v[k], v[k], vv);
        }
        if constexpr (TP == FLOU_TP_KENNEDY_GRUBER) kg_prim_to_cons_vjp<DIM>(q[0], v, vv, q[DIM + 1], g1, o, qb);
        else prim_to_cons_vjp<DIM>(q[0], v, vv, p, g1, o, qb);
    }
}

// Entropy variables W(q) = ((γ - s)/(γ-1) - ρ|v|²/(2p), ρv/p, -ρ/p), s = ln p - γ ln ρ
// (FlouCommon/Euler.jl:273-307), and the state of given entropy variables (Euler.jl:309-334).
template <int DIM>
__device__ __forceinline__ void entropy_of(const double* q, double g, double* w) {
    const double ir = rcp_refined(q[0]);
    double ke = 0.0;
#pragma unroll
    for (int k = 0; k < DIM; ++k) ke = fma(q[1 + k], q[1 + k] * ir, ke);
    const double p = (g - 1.0) * fma(-0.5, ke, q[DIM + 1]), ip = rcp_refined(p);
    const double sv = log(p) - g * log(q[0]);
    w[0] = (g - sv) * rcp_refined(g - 1.0) - ke * ip * 0.5;
#pragma unroll
    for (int k = 0; k < DIM; ++k) w[1 + k] = q[1 + k] * ip;
    w[DIM + 1] = -q[0] * ip;
}

template <int DIM>
__device__ __forceinline__ double state_of_entropy(const double* w, double g, double* q) {
    const double wl = w[DIM + 1], iwl = rcp_refined(wl), ig1 = rcp_refined(g - 1.0);
    double vp[DIM], vv = 0.0;
#pragma unroll
    for (int k = 0; k < DIM; ++k) {
        vp[k] = -w[1 + k] * iwl;
        vv = fma(vp[k], vp[k], vv);
    }
    const double sv = g - (g - 1.0) * (w[0] - wl * vv * 0.5);
    const double pp = exp(-fma(g, log(-wl), sv) * ig1);
    const double rho = -pp * wl;
    q[0] = rho;
#pragma unroll
    for (int k = 0; k < DIM; ++k) q[1 + k] = rho * vp[k];
    q[DIM + 1] = fma(pp, ig1, 0.5 * rho * vv);
    return pp;
}

// w̄ = (∂q/∂W)ᵀ q̄ = A₀ q̄, A₀ the symmetric Jacobian of the conserved variables with respect to
// the entropy variables: rows (ρ, ρv, E), (ρv_k, ρ v_k v + p e_k, ρH v_k), (E, ρH v, ρH² - γp²/((γ-1)ρ)).
template <int DIM>
__device__ __forceinline__ void entropy_jacobian_apply(const double* q, double p, double g, const double* qb,
                                                       double* wb) {
    const double rho = q[0], ir = rcp_refined(rho), E = q[DIM + 1], rH = E + p;
    double v[DIM], mq = 0.0;
#pragma unroll
    for (int k = 0; k < DIM; ++k) {
        v[k] = q[1 + k] * ir;
        mq = fma(q[1 + k], qb[1 + k], mq);   // ρ v·q̄_m
    }
    const double vm = mq * ir;               // v·q̄_m
    wb[0] = fma(rho, qb[0], fma(E, qb[DIM + 1], mq));
#pragma unroll
    for (int k = 0; k < DIM; ++k) wb[1 + k] = fma(q[1 + k], fma(rH * ir, qb[DIM + 1], qb[0] + vm), p * qb[1 + k]);
    const double eE = rH * rH * ir - g * p * p * ir * rcp_refined(g - 1.0);
    wb[DIM + 1] = fma(E, qb[0], fma(rH, vm, eE * qb[DIM + 1]));
}

// q̄ += (∂W/∂q)ᵀ w̄ for the entropy variables of q (pressure p):
//   p̄ = (-a/(γ-1) + (aρ|v|²/2 - ρ v·b + cρ)/p)/p   with w̄ = (a, b, c),
//   q̄_ρ += a(γ/((γ-1)ρ) + |v|²/(2p)) - c/p + (γ-1)|v|²/2 p̄,  q̄_m += (b - a v)/p - (γ-1) v p̄,
//   q̄_E += (γ-1) p̄.
template <int DIM>
__device__ __forceinline__ void entropy_vjp(const double* q, double p, double g, const double* wb, double* qb) {
    const double rho = q[0], ir = rcp_refined(rho), ip = rcp_refined(p), g1 = g - 1.0, ig1 = rcp_refined(g1);
    const double a = wb[0], c = wb[DIM + 1];
    double v[DIM], vv = 0.0, vb = 0.0;
#pragma unroll
    for (int k = 0; k < DIM; ++k) {
        v[k] = q[1 + k] * ir;
        vv = fma(v[k], v[k], vv);
        vb = fma(v[k], wb[1 + k], vb);
    }
    const double pb = fma(rho * ip, fma(0.5 * a, vv, c - vb), -a * ig1) * ip;
    qb[0] += fma(a, fma(g * ig1, ir, 0.5 * vv * ip), fma(0.5 * g1 * vv, pb, -c * ip));
#pragma unroll
    for (int k = 0; k < DIM; ++k) qb[1 + k] += fma(wb[1 + k] - a * v[k], ip, -g1 * v[k] * pb);
    qb[DIM + 1] += g1 * pb;
}

// G (Gauss nodes, Cartesian): the entropy-projected coupling of each line transposed.  The forward
// adds to node i the flux differences
//   Ja (∂g_l[i] (F♯(Q_i, Q̃_l) - Σ_j l_j F♯(Q_j, Q̃_l)) - ∂g_r[i] (F♯(Q_i, Q̃_r) - Σ_j r_j F♯(Q_j, Q̃_r)))
// with Q̃ = q(Σ_j l_j W(Q_j)).  With w = λ/J and T = Σ_i ∂g[i] w_i, the pair F♯(Q_j, Q̃) has the
// cotangent ±Ja (∂g[j] w_j - l_j T); its node-side cotangents go to snode, and its Q̃ side, summed
// over the line, is taken to the projected entropy variables (sWb), which the node phase spreads
// back with l.  One group of 8 lanes per line side (N <= 8), one lane per node: the sums over the
// line (W̃, T and the Q̃ cotangent) are butterfly shuffles within the group, which leave the same
// bits in every lane; each lane then takes its node's pair.  A node receives one cotangent from
// each side of its line, added into snode (zeroed first) in either order: two addends onto zero
// give the same sum.
// CURV: the pair of node j with a projected state is along n̄ = (Ja_j + n Js)/2, Ja_j the node's
// metric column of direction D and n Js the line end's subcell interface normal times its surface
// Jacobian (the forward's metric of the projected states); the metric is in the fluxes, so the
// cotangent carries ±1 instead of ±Ja.
// HG (the hybrid operator on Gauss nodes): sw holds the pair weights w' and ∂g[j] becomes
// l[j]/ω_j (the projected-state pairs enter the node increments through l).
template <int DIM, int N, int D, int TP, bool CURV = false, bool HG = false, bool WC = false>
__device__ __forceinline__ void adj_split_projection(const AdjElemParams& P, int e0, const double* sops,
                                                     const double* sprim, const double* sw, double* snode,
                                                     double* sWb, double cb, const double* sWn) {
    using S = Shape<DIM, N>;
    using A = AdjSplitShape<DIM, N, TP, true>;
    constexpr int NV = DIM + 2, NPE = S::NPE, NN = S::NN, NFD = S::NFD, NARR = A::NARR, NPB = A::NPB;
    constexpr int NPROJ = A::NPROJ;   // line sides of the block: the groups
    static_assert(N <= 8, "one lane per node of a line within a group of 8");
    const double g = P.gamma, g1 = g - 1.0;
    const double* lv = sops + 2 * N * N;   // l_l, then l_r
    const double* dgl = lv + 2 * N;        // ∂g_l, then ∂g_r
    for (int t = threadIdx.x; t < NPB * NN; t += blockDim.x) snode[t] = 0.0;
    __syncthreads();
    auto gsum = [](double v) {
#pragma unroll
        for (int o = 4; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        return v;
    };
    constexpr int TOTAL = ((NPROJ * 8 + 31) / 32) * 32;   // whole warps, so every shuffle has its partners
    for (int t = threadIdx.x; t < TOTAL; t += blockDim.x) {
        const int grp = t >> 3, pos = t & 7;
        const int elp = grp / (2 * NFD), rr = grp - elp * 2 * NFD, line = rr >> 1, sd = rr & 1;
        const bool on = grp < NPROJ && e0 + elp < P.nelem && pos < N;
        const int j = on ? elp * NPE + tp_node<DIM>(N, D, line, pos) : 0;
        double wt[NV], T[NV];
        if (on) {
            double wj[NV];
            if constexpr (WC) {
#pragma unroll
                for (int k = 0; k < NV; ++k) wj[k] = sWn[k * NN + j];
            } else {
                double q[NV];
#pragma unroll
                for (int k = 0; k < NV; ++k) q[k] = P.U[k * P.ndofs + (int64_t)e0 * NPE + j];
                entropy_of<DIM>(q, g, wj);
            }
            const double cf = HG ? lv[sd * N + pos] * rcp_refined(P.omega1[pos]) : dgl[sd * N + pos];
#pragma unroll
            for (int k = 0; k < NV; ++k) {
                wt[k] = lv[sd * N + pos] * wj[k];
                T[k] = cf * sw[k * NN + j];
            }
        } else {
#pragma unroll
            for (int k = 0; k < NV; ++k) wt[k] = T[k] = 0.0;
        }
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            wt[k] = gsum(wt[k]);
            T[k] = gsum(T[k]);
        }
        PrimBar o2;
        o2.r = o2.b = o2.e = 0.0;
#pragma unroll
        for (int k = 0; k < 3; ++k) o2.v[k] = 0.0;
        double qt[NV], pt = 1.0;
        const bool grp_on = grp < NPROJ && e0 + elp < P.nelem;
        if (grp_on) {
            pt = state_of_entropy<DIM>(wt, g, qt);
        } else {
#pragma unroll
            for (int k = 0; k < NV; ++k) qt[k] = k == 0 || k == DIM + 1 ? 1.0 : 0.0;
        }
        if (on) {
            double vt[NARR], vj[NARR], Fb[NV];
            split_node_values<DIM, TP>(qt, pt, vt);
#pragma unroll
            for (int k = 0; k < NARR; ++k) vj[k] = sprim[k * NN + j];
            const double Ja = CURV ? 1.0 : P.Ja[(e0 + elp) * DIM + D], sg = sd == 0 ? Ja : -Ja;
            const double lj = lv[sd * N + pos];
            const double dg = HG ? lj * rcp_refined(P.omega1[pos]) : dgl[sd * N + pos];
#pragma unroll
            for (int k = 0; k < NV; ++k) Fb[k] = sg * fma(dg, sw[k * NN + j], -lj * T[k]);
            PrimBar o1;
            if constexpr (CURV) {
                const int64_t ns = (int64_t)P.nelem * DIM * NFD * (N + 1);
                const int64_t si = (((int64_t)(e0 + elp) * DIM + D) * NFD + line) * (N + 1) + (sd ? N : 0);
                const int64_t gj = (int64_t)e0 * NPE + j;
                const double js = P.subJ[si];
                double nrm[DIM];
#pragma unroll
                for (int k = 0; k < DIM; ++k)
                    nrm[k] = 0.5 * fma(P.subfr[k * ns + si], js, P.Jan[(k + D * DIM) * P.ndofs + gj]);
                split_pair_vjp<DIM, -1, TP>(vj, vt, Fb, cb, g1, o1, o2, nrm);
            } else {
                split_pair_vjp<DIM, D, TP>(vj, vt, Fb, cb, g1, o1, o2);
            }
            atomicAdd(snode + j, o1.r);
#pragma unroll
            for (int k = 0; k < DIM; ++k) atomicAdd(snode + (1 + k) * NN + j, o1.v[k]);
            atomicAdd(snode + (1 + DIM) * NN + j, o1.b);
            if constexpr (NPB > DIM + 2) atomicAdd(snode + (2 + DIM) * NN + j, o1.e);
        }
        o2.r = gsum(o2.r);
        o2.b = gsum(o2.b);
        o2.e = gsum(o2.e);
#pragma unroll
        for (int k = 0; k < DIM; ++k) o2.v[k] = gsum(o2.v[k]);
        if (grp_on && pos == 0) {   // Q̃'s cotangent -> conserved -> entropy variables
            double qbt[NV], wbt[NV];
#pragma unroll
            for (int k = 0; k < NV; ++k) qbt[k] = 0.0;
            split_node_to_cons<DIM, TP>(qt, pt, g1, o2, qbt);
            entropy_jacobian_apply<DIM>(qt, pt, g, qbt, wbt);
#pragma unroll
            for (int k = 0; k < NV; ++k) sWb[k * NPROJ + grp] = wbt[k];
        }
    }
}

// The Euler flux along axis D of a conserved state.
template <int DIM, int D>
__device__ __forceinline__ void euler_flux_axis(const double* q, double g, double* F) {
    const double ir = rcp_refined(q[0]);
    double ke = 0.0;
#pragma unroll
    for (int k = 0; k < DIM; ++k) ke = fma(q[1 + k], q[1 + k] * ir, ke);
    const double p = (g - 1.0) * fma(-0.5, ke, q[DIM + 1]), vd = q[1 + D] * ir;
    F[0] = q[1 + D];
#pragma unroll
    for (int k = 0; k < DIM; ++k) F[1 + k] = fma(q[1 + k], vd, k == D ? p : 0.0);
    F[DIM + 1] = (q[DIM + 1] + p) * vd;
}

// The Euler flux along a general direction n: [ρ v·n, ρ v v·n + p n, (E+p) v·n].
template <int DIM>
__device__ __forceinline__ void euler_flux_n(const double* q, const double* n, double g, double* F) {
    const double ir = rcp_refined(q[0]);
    double ke = 0.0, mn = 0.0;
#pragma unroll
    for (int k = 0; k < DIM; ++k) {
        ke = fma(q[1 + k], q[1 + k] * ir, ke);
        mn = fma(q[1 + k], n[k], mn);
    }
    const double p = (g - 1.0) * fma(-0.5, ke, q[DIM + 1]), vn = mn * ir;
    F[0] = mn;
#pragma unroll
    for (int k = 0; k < DIM; ++k) F[1 + k] = fma(q[1 + k], vn, p * n[k]);
    F[DIM + 1] = (q[DIM + 1] + p) * vn;
}

// The split form's two-point flux along axis D (the forward of split_pair_vjp) from the nodes'
// split_node_values A, B; StdAverage takes the conserved states qa, qb.  D < 0: along the
// general direction nrm.
template <int DIM, int D, int TP>
__device__ __forceinline__ void split_pair_flux(const double* A, const double* B, const double* qa, const double* qb,
                                                double g, double* F, const double* nrm = nullptr) {
    constexpr int NV = DIM + 2;
    auto along = [&](const double* v) {   // v·(the direction)
        if constexpr (D >= 0) {
            return v[D];
        } else {
            double x = 0.0;
#pragma unroll
            for (int k = 0; k < DIM; ++k) x = fma(v[k], nrm[k], x);
            return x;
        }
    };
    auto dir = [&](int k) {   // the direction's component k
        if constexpr (D >= 0) return k == D ? 1.0 : 0.0;
        else return nrm[k];
    };
    if constexpr (TP == FLOU_TP_STD_AVERAGE) {
        double Fa[NV], Fc[NV];
        if constexpr (D >= 0) {
            euler_flux_axis<DIM, D>(qa, g, Fa);
            euler_flux_axis<DIM, D>(qb, g, Fc);
        } else {
            euler_flux_n<DIM>(qa, nrm, g, Fa);
            euler_flux_n<DIM>(qb, nrm, g, Fc);
        }
#pragma unroll
        for (int k = 0; k < NV; ++k) F[k] = 0.5 * (Fa[k] + Fc[k]);
    } else if constexpr (TP == FLOU_TP_KENNEDY_GRUBER) {
        const double rho = A[0] + B[0], pm = A[1 + DIM] + B[1 + DIM], en = A[2 + DIM] + B[2 + DIM];
        double vm[DIM];
#pragma unroll
        for (int k = 0; k < DIM; ++k) vm[k] = A[1 + k] + B[1 + k];
        const double vd = along(vm), m = rho * vd;
        F[0] = m;
#pragma unroll
        for (int k = 0; k < DIM; ++k) F[1 + k] = fma(m, vm[k], pm * dir(k));
        F[DIM + 1] = fma(m, en, pm * vd);
    } else {
        const double hsr = A[0] + B[0], hdr = A[0] - B[0], hsb = A[1 + DIM] + B[1 + DIM],
                     hdb = A[1 + DIM] - B[1 + DIM];
        const double R = rcp_refined(hsr * hsb), rs = hsb * R, rb = hsr * R;
        double rho, irho, beta, ibeta, d1, d2;
        logmean_half(A[0], B[0], hsr, hdr, rs, rho, irho, d1, d2);
        logmean_half(A[1 + DIM], B[1 + DIM], hsb, hdb, rb, beta, ibeta, d1, d2);
        const double p = 0.5 * hsr * rb;
        double va[DIM], vv = 0.0;
#pragma unroll
        for (int k = 0; k < DIM; ++k) {
            va[k] = A[1 + k] + B[1 + k];
            vv = fma(va[k], va[k], vv);
        }
        const double h = fma(0.5 * rcp_refined(g - 1.0), ibeta, -(A[2 + DIM] + B[2 + DIM])) + fma(p, irho, vv);
        const double m = rho * along(va);
        F[0] = m;
#pragma unroll
        for (int k = 0; k < DIM; ++k) F[1 + k] = fma(m, va[k], p * dir(k));
        F[DIM + 1] = m * h;
    }
}

// numflux_vjp for a kind known at run time (the hybrid operator's subcell FV flux).
template <int DIM>
__device__ __noinline__ void numflux_vjp_any(int kind, const double* a, const double* b, double inten, double g,
                                             const double* fb, double* ab, double* bbar) {
    switch (kind) {
        case 0: numflux_vjp<DIM, 0>(a, b, inten, g, fb, ab, bbar); break;
        case 1: numflux_vjp<DIM, 1>(a, b, inten, g, fb, ab, bbar); break;
        case 2: numflux_vjp<DIM, 2>(a, b, inten, g, fb, ab, bbar); break;
        case 3: numflux_vjp<DIM, 3>(a, b, inten, g, fb, ab, bbar); break;
        case 4: numflux_vjp<DIM, 4>(a, b, inten, g, fb, ab, bbar); break;
        case 5: numflux_vjp<DIM, 5>(a, b, inten, g, fb, ab, bbar); break;
        case 6: numflux_vjp<DIM, 6>(a, b, inten, g, fb, ab, bbar); break;
        default: numflux_vjp<DIM, 7>(a, b, inten, g, fb, ab, bbar); break;
    }
}

// One subcell interface of direction D (between positions pos-1 and pos of a line): the rotated
// states a, b and, on general geometry, the interface's uploaded frame and surface Jacobian
// (Cartesian: the positive axis and Ja_DD).
template <int DIM>
struct SubcellFace {
    double a[DIM + 2], b[DIM + 2];
    FrameTab fr;
    double Js;
};

// The interface's frame and the states in it.
template <int DIM, int N, int D, bool CURV>
__device__ __forceinline__ void subcell_face(const AdjElemParams& P, int e, int line, int pos, double Ja,
                                             const double* ql, const double* qr, SubcellFace<DIM>& sf) {
    constexpr int NFD = Shape<DIM, N>::NFD;
    sf.Js = Ja;
    if constexpr (CURV) {
        const int64_t ns = (int64_t)P.nelem * DIM * NFD * (N + 1);
        const int64_t si = (((int64_t)e * DIM + D) * NFD + line) * (N + 1) + pos;
#pragma unroll
        for (int r = 0; r < 3; ++r) {
            sf.fr.n[r] = P.subfr[r * ns + si];
            sf.fr.t[r] = P.subfr[(3 + r) * ns + si];
            sf.fr.b[r] = P.subfr[(6 + r) * ns + si];
        }
        sf.Js = P.subJ[si];
        rotate_to_face<DIM>(ql, sf.fr, sf.a);
        rotate_to_face<DIM>(qr, sf.fr, sf.b);
    } else {
        const FrameAxes Ax = frame_axes<DIM>(2 * D + 1);
        sf.a[0] = ql[0]; sf.b[0] = qr[0]; sf.a[DIM + 1] = ql[DIM + 1]; sf.b[DIM + 1] = qr[DIM + 1];
        cart_to_face<DIM>(ql, Ax, sf.a);
        cart_to_face<DIM>(qr, Ax, sf.b);
    }
}

// The subcell FV flux Fv = Js Fv(ql, qr) in physical components (PhysicalRegions.jl:68-300).
template <int DIM, int N, int D, bool CURV>
__device__ __forceinline__ void subcell_fv(const AdjElemParams& P, int e, int line, int pos, double Ja,
                                           const double* ql, const double* qr, SubcellFace<DIM>& sf, double* Fv) {
    constexpr int NV = DIM + 2;
    double Fr[NV];
    subcell_face<DIM, N, D, CURV>(P, e, line, pos, Ja, ql, qr, sf);
    euler_numflux<DIM>(sf.a, sf.b, P.fvflux, P.fvavg, P.fvintensity, P.gamma, Fr);
    if constexpr (CURV) {
        rotate_to_phys<DIM>(Fr, sf.fr, Fv);
#pragma unroll
        for (int k = 0; k < NV; ++k) Fv[k] *= sf.Js;
    } else {
        const FrameAxes Ax = frame_axes<DIM>(2 * D + 1);
        Fv[0] = Fr[0] * sf.Js;
        Fv[DIM + 1] = Fr[DIM + 1] * sf.Js;
        cart_to_phys<DIM>(Fr, Ax, Fv);
#pragma unroll
        for (int k = 0; k < DIM; ++k) Fv[1 + k] *= sf.Js;
    }
}

// The transpose of subcell_fv: the cotangent Fvb of Fv onto the two states (ol: the left one).
template <int DIM, int D, bool CURV>
__device__ __forceinline__ void subcell_fv_vjp(const AdjElemParams& P, const SubcellFace<DIM>& sf, const double* Fvb,
                                               double* ol, double* orr) {
    constexpr int NV = DIM + 2;
    const FrameAxes Ax = frame_axes<DIM>(2 * D + 1);
    double Frb[NV], ab[NV], bbr[NV], t[NV];
    if constexpr (CURV) {
        rotate_to_face<DIM>(Fvb, sf.fr, t);
#pragma unroll
        for (int k = 0; k < NV; ++k) Frb[k] = sf.Js * t[k];
    } else {
        Frb[0] = sf.Js * Fvb[0];
        Frb[DIM + 1] = sf.Js * Fvb[DIM + 1];
        cart_to_face<DIM>(Fvb, Ax, t);
#pragma unroll
        for (int k = 0; k < DIM; ++k) Frb[1 + k] = sf.Js * t[1 + k];
    }
    numflux_vjp_any<DIM>(P.fvkind, sf.a, sf.b, P.fvintensity, P.gamma, Frb, ab, bbr);
    if constexpr (CURV) {
        rotate_to_phys<DIM>(ab, sf.fr, ol);
        rotate_to_phys<DIM>(bbr, sf.fr, orr);
    } else {
        ol[0] = ab[0]; ol[DIM + 1] = ab[DIM + 1]; orr[0] = bbr[0]; orr[DIM + 1] = bbr[DIM + 1];
        cart_to_phys<DIM>(ab, Ax, ol);
        cart_to_phys<DIM>(bbr, Ax, orr);
    }
}

// The hybrid operators' forward pair fluxes F♯(Q_a, Q_b) of direction D, every pair of the block
// once, into spb as [NV][NPT] (CURV: along the averaged metric column).
template <int DIM, int N, int D, int TP, bool CURV>
__device__ __forceinline__ void hybrid_pair_fluxes(const AdjElemParams& P, int e0, const double* sprim, double* spb,
                                                   const uint8_t* stab) {
    using S = Shape<DIM, N>;
    using A = AdjSplitShape<DIM, N, TP>;
    constexpr int NV = DIM + 2, NPE = S::NPE, NN = S::NN, NFD = S::NFD, NPAIR = S::NPAIR, NARR = A::NARR;
    constexpr int NPT = A::NPT;
    const double g = P.gamma;
    const int tid = threadIdx.x;
    for (int kp = tid; kp < NPT; kp += blockDim.x) {
        const int elp = kp / (NFD * NPAIR);
        const int r = kp - elp * (NFD * NPAIR);
        const int line = r / NPAIR, pp = r - line * NPAIR;
        if (e0 + elp >= P.nelem) continue;
        const int ia = elp * NPE + tp_node<DIM>(N, D, line, stab[2 * pp]);
        const int ib = elp * NPE + tp_node<DIM>(N, D, line, stab[2 * pp + 1]);
        double Av[NARR], Bv[NARR], qa[NV], qc[NV], F[NV];
#pragma unroll
        for (int k = 0; k < NARR; ++k) {
            Av[k] = sprim[k * NN + ia];
            Bv[k] = sprim[k * NN + ib];
        }
        if constexpr (TP == FLOU_TP_STD_AVERAGE) {
#pragma unroll
            for (int k = 0; k < NV; ++k) {
                qa[k] = P.U[k * P.ndofs + (int64_t)e0 * NPE + ia];
                qc[k] = P.U[k * P.ndofs + (int64_t)e0 * NPE + ib];
            }
        }
        if constexpr (CURV) {
            const int64_t ga = (int64_t)e0 * NPE + ia, gb = (int64_t)e0 * NPE + ib;
            double nrm[DIM];
#pragma unroll
            for (int k = 0; k < DIM; ++k)
                nrm[k] = 0.5 * (P.Jan[(k + D * DIM) * P.ndofs + ga] + P.Jan[(k + D * DIM) * P.ndofs + gb]);
            split_pair_flux<DIM, -1, TP>(Av, Bv, qa, qc, g, F, nrm);
        } else {
            split_pair_flux<DIM, D, TP>(Av, Bv, qa, qc, g, F);
        }
#pragma unroll
        for (int k = 0; k < NV; ++k) spb[k * NPT + kp] = F[k];
    }
}

// Σ_j D♯_pj F♯_pj of node gi (position pos on its line) from the pair fluxes in spb, with the
// diagonal D♯_pp F(Q_p) (CURV: the node's contravariant flux).
template <int DIM, int N, int D, int TP, bool CURV>
__device__ __forceinline__ void hybrid_node_sum(const AdjElemParams& P, int64_t gi, int el, int pos, int line,
                                                const double* Dsh, const double* spb, double* acc) {
    using S = Shape<DIM, N>;
    constexpr int NV = DIM + 2, NFD = S::NFD, NPAIR = S::NPAIR;
    constexpr int NPT = AdjSplitShape<DIM, N, TP>::NPT;
    const double g = P.gamma;
    double q[NV];
#pragma unroll
    for (int k = 0; k < NV; ++k) q[k] = P.U[k * P.ndofs + gi];
    if constexpr (CURV) {
        double nrm[DIM];
#pragma unroll
        for (int k = 0; k < DIM; ++k) nrm[k] = P.Jan[(k + D * DIM) * P.ndofs + gi];
        euler_flux_n<DIM>(q, nrm, g, acc);
    } else {
        euler_flux_axis<DIM, D>(q, g, acc);
    }
    const double dii = Dsh[pos + pos * N];
#pragma unroll
    for (int k = 0; k < NV; ++k) acc[k] *= dii;
    const int pbase = el * NFD * NPAIR + line * NPAIR;
#pragma unroll
    for (int t = 1; t < N; ++t) {
        const int j = pos + t < N ? pos + t : pos + t - N;
        const int lo = j < pos ? j : pos, hi = j < pos ? pos : j;
        const int pidx = pbase + lo * (2 * N - lo - 1) / 2 + (hi - lo - 1);
        const double a = Dsh[pos + j * N];
#pragma unroll
        for (int k = 0; k < NV; ++k) acc[k] = fma(a, spb[k * NPT + pidx], acc[k]);
    }
}

// The pressure of a conserved state.
template <int DIM>
__device__ __forceinline__ double pressure_of(const double* q, double g) {
    double ke = 0.0;
#pragma unroll
    for (int k = 0; k < DIM; ++k) ke = fma(q[1 + k], q[1 + k], ke);
    return (g - 1.0) * fma(-0.5, ke * rcp_refined(q[0]), q[DIM + 1]);
}

// H (HybridDivOperator on Gauss-Lobatto nodes, Cartesian; OpDivergence.jl:553-604 with the
// blending of :781-801), one direction D.  Forward: the high-order subcell fluxes F̄_p =
// Σ_{r<p} ω_r Ja (Σ_j D♯_rj F♯_rj) (recomputed: pair fluxes, node sums, exclusive scan), the FV
// fluxes Fv_p = Ja Fv(Q_(p-1), Q_p) along the axis, b = (W_p - W_(p-1))·(F̄_p - Fv_p),
// δ = max(1 - b/√(b²+c), ½), F_p = Fv_p + δ (F̄_p - Fv_p), dQ_p += (F_p - F_(p+1))/ω_p (F_0 = F_N =
// 0).  Reverse, with w = λ/J: F̄b_p = w_p/ω_p - w_(p-1)/ω_(p-1); δ̄ = F̄b·(F̄ - Fv), b̄ = -δ̄ c/√(b²+c)³
// on the unclipped branch; the cotangent of F̄_p is δ F̄b + b̄ ΔW, that of Fv (1-δ) F̄b - b̄ ΔW (through
// the FV flux VJP to both nodes), ΔW's b̄ (F̄ - Fv) goes through W's VJP; the suffix sums of the F̄
// cotangents give each node's pair weight w'_r = -ω_r Σ_(p>r) F̄̄_p, left in sH for the split-form
// pair and node phases.  A node's contribution from the interface on its right is handed over in
// spb (free between the phases); the node's own goes to qb.
// CURV (general geometry): the pair fluxes along the averaged metric columns, the node's own
// column in the diagonal term, ω_p alone as the node-sum weight (the metric is in the fluxes), and
// each subcell interface's uploaded frame and surface Jacobian for the FV flux.
template <int DIM, int N, int D, int TP, bool CURV = false>
__device__ __forceinline__ void adj_hybrid_dir(const AdjElemParams& P, int e0, bool active, int el, int i,
                                               const double* sops, const double* sprim, const double* sw, double* sH,
                                               double* spb, const uint8_t* stab, const double* sWn, double* qb) {
    constexpr bool WC = AdjSplitShape<DIM, N, TP, false, true>::WC;
    using S = Shape<DIM, N>;
    constexpr int NV = DIM + 2, NPE = S::NPE, NN = S::NN, NFD = S::NFD;
    const double g = P.gamma;
    const double* Dsh = sops + N * N;
    const int tid = threadIdx.x;
    hybrid_pair_fluxes<DIM, N, D, TP, CURV>(P, e0, sprim, spb, stab);
    __syncthreads();
    const int e = e0 + el;
    int pos = 0, line = 0;
    tp_coords<DIM>(N, i, D, pos, line);
    const int64_t gi = (int64_t)e * NPE + i;
    const double Ja = active ? (CURV ? 1.0 : P.Ja[e * DIM + D]) : 0.0;
    if (active) {   // ω_p Ja Σ_j D♯_pj F♯_pj (with the diagonal D♯_pp F(Q_p))
        double acc[NV];
        hybrid_node_sum<DIM, N, D, TP, CURV>(P, gi, el, pos, line, Dsh, spb, acc);
        const double wq = P.omega1[pos] * Ja;
#pragma unroll
        for (int k = 0; k < NV; ++k) sH[k * NN + tid] = wq * acc[k];
    }
    __syncthreads();
    for (int t = tid; t < S::EPB * NFD; t += blockDim.x) {   // F̄_p: exclusive scan along each line
        const int elp = t / NFD, ln = t - elp * NFD;
        if (e0 + elp >= P.nelem) continue;
        double run[NV];
#pragma unroll
        for (int k = 0; k < NV; ++k) run[k] = 0.0;
        for (int pp = 0; pp < N; ++pp) {
            const int j = elp * NPE + tp_node<DIM>(N, D, ln, pp);
#pragma unroll
            for (int k = 0; k < NV; ++k) {
                const double x = sH[k * NN + j];
                sH[k * NN + j] = run[k];
                run[k] += x;
            }
        }
    }
    __syncthreads();
    if (active && pos > 0) {   // the subcell interface between pos-1 and pos
        const int il = el * NPE + tp_node<DIM>(N, D, line, pos - 1);
        const int64_t gl = (int64_t)e0 * NPE + il;
        double ql[NV], qr[NV], Fv[NV], wl[NV], wr[NV];
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            ql[k] = P.U[k * P.ndofs + gl];
            qr[k] = P.U[k * P.ndofs + gi];
        }
        SubcellFace<DIM> sf;
        subcell_fv<DIM, N, D, CURV>(P, e, line, pos, Ja, ql, qr, sf, Fv);
        if constexpr (WC) {
#pragma unroll
            for (int k = 0; k < NV; ++k) {
                wl[k] = sWn[k * NN + il];
                wr[k] = sWn[k * NN + tid];
            }
        } else {
            entropy_of<DIM>(ql, g, wl);
            entropy_of<DIM>(qr, g, wr);
        }
        double bb = 0.0, dW[NV], Fh[NV];
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            dW[k] = wr[k] - wl[k];
            Fh[k] = sH[k * NN + tid];
            bb = fma(dW[k], Fh[k] - Fv[k], bb);
        }
        const double dl = sqrt_refined(fma(bb, bb, P.blend)), idl = rcp_refined(dl);
        const double draw = (dl - bb) * idl;
        const bool free_ = 0.5 < draw;   // Base.max(draw, 0.5) takes draw only above 0.5
        const double dlt = free_ ? draw : 0.5;
        const double iwp = rcp_refined(P.omega1[pos]), iwm = rcp_refined(P.omega1[pos - 1]);
        double Fb[NV], db = 0.0;
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            Fb[k] = fma(sw[k * NN + tid], iwp, -sw[k * NN + il] * iwm);
            db = fma(Fb[k], Fh[k] - Fv[k], db);
        }
        const double bbar = free_ ? -db * P.blend * idl * idl * idl : 0.0;
        double Fvb[NV], wbar[NV];
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            sH[k * NN + tid] = fma(dlt, Fb[k], bbar * dW[k]);   // the cotangent of F̄_p
            Fvb[k] = fma(1.0 - dlt, Fb[k], -bbar * dW[k]);
            wbar[k] = bbar * (Fh[k] - Fv[k]);
        }
        double ol[NV], orr[NV];
        subcell_fv_vjp<DIM, D, CURV>(P, sf, Fvb, ol, orr);
        const double pr = pressure_of<DIM>(qr, g), plv = pressure_of<DIM>(ql, g);
#pragma unroll
        for (int k = 0; k < NV; ++k) qb[k] += orr[k];
        entropy_vjp<DIM>(qr, pr, g, wbar, qb);
#pragma unroll
        for (int k = 0; k < NV; ++k) wbar[k] = -wbar[k];
        entropy_vjp<DIM>(ql, plv, g, wbar, ol);
#pragma unroll
        for (int k = 0; k < NV; ++k) spb[k * NN + il] = ol[k];
    }
    __syncthreads();
    for (int t = tid; t < S::EPB * NFD; t += blockDim.x) {   // w'_r = -ω_r Σ_(p>r) F̄̄_p, in place
        const int elp = t / NFD, ln = t - elp * NFD;
        if (e0 + elp >= P.nelem) continue;
        double run[NV];
#pragma unroll
        for (int k = 0; k < NV; ++k) run[k] = 0.0;
        for (int pp = N - 1; pp >= 0; --pp) {
            const int j = elp * NPE + tp_node<DIM>(N, D, ln, pp);
            const double wq = -P.omega1[pp];
#pragma unroll
            for (int k = 0; k < NV; ++k) {
                const double x = pp > 0 ? sH[k * NN + j] : 0.0;
                sH[k * NN + j] = wq * run[k];
                run[k] += x;
            }
        }
    }
    if (active && pos < N - 1) {   // the cotangent from the interface on this node's right
#pragma unroll
        for (int k = 0; k < NV; ++k) qb[k] += spb[k * NN + tid];
    }
    __syncthreads();
}

// G and H (HybridDivOperator on Gauss nodes, OpDivergence.jl:633-780), one direction D, in the first
// of the stage's two element passes.  Forward (recomputed): per line the entropy-projected states
// Q̃_l, Q̃_r and every node's pair with them, Fl_i = F♯(Q_i, Q̃_l) - Σ_j l_l[j] F♯(Q_j, Q̃_l) (Fr
// alike), the element's side values of its line's face fluxes fls = ±Fn_left, frs = ±Fn_right, the
// node increments sH_i = ω_i Ja Σ_j D♯_ij F♯_ij - l_l[i] (Ja Fl_i - fls) + l_r[i] (Ja Fr_i + frs),
// the FV fluxes Fv_p (p = 1..N-1) and the blended scan F_0 = -fls, X_p = F_(p-1) + sH_(p-1),
// F_p = Fv_p + δ_p (X_p - Fv_p), δ_p from b_p = (W_p - W_(p-1))·(X_p - Fv_p); dQ_i += (F_i -
// F_(i+1))/ω_i with F_N = frs.  Reverse: one thread per line runs the scan backwards (the
// cotangent of F_p is w_p/ω_p - w_(p-1)/ω_(p-1) plus what X_(p+1) hands back), leaving per
// interface the cotangents of Fv_p and of the entropy jump, the pair weights w'_i = -ω_i s̄H_i in
// sH (s̄H_(N-1) = 0: the last increment closes on frs, not on the scan), and the cotangents of fls
// (-w_0/ω_0 - X̄_1 + Σ l_l s̄H) and of frs (-w_(N-1)/ω_(N-1) + Σ l_r s̄H), which the end nodes
// write to FbS for the face VJP.  The projected-state pairs take l_s[i] w'_i/ω_i as their
// coefficients in adj_split_projection.
// Shared memory: sF2 [2][NV][NN] (the projected pairs of both sides, then per interface Fv and
// X - Fv, then their cotangents), scl (the projection's [NV][NPROJ], free until it runs: the line
// reductions Σ_j l_s[j] F♯(Q_j, Q̃_s)), sdW (the projection's node array, zeroed when it runs:
// the entropy jumps, then the face-flux cotangents at the end nodes).
template <int DIM, int N, int D, int TP, bool CURV = false>
__device__ __forceinline__ void adj_hybrid_gauss_dir(const AdjElemParams& P, int e0, bool active, int el, int i,
                                                     const double* sops, const double* sprim, const double* sw,
                                                     double* sH, double* spb, const uint8_t* stab, double* sF2,
                                                     double* scl, double* sdW, const double* sWn, double* qb) {
    using S = Shape<DIM, N>;
    using A = AdjSplitShape<DIM, N, TP, true, true>;
    constexpr int NV = DIM + 2, NPE = S::NPE, NN = S::NN, NFD = S::NFD, NARR = A::NARR;
    constexpr int NPROJ = A::NPROJ;
    static_assert(N <= 8, "one lane per node of a line within a group of 8");
    const double g = P.gamma;
    const double* Dsh = sops + N * N;
    const double* lv = sops + 2 * N * N;   // l_l, then l_r
    const int tid = threadIdx.x;
    hybrid_pair_fluxes<DIM, N, D, TP, CURV>(P, e0, sprim, spb, stab);
    auto gsum = [](double v) {
#pragma unroll
        for (int o = 4; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        return v;
    };
    // the projected states and their pairs with every node of the line: one group of 8 lanes per
    // line side, one lane per node (the line sums are butterfly shuffles within the group)
    constexpr int TOTAL = ((NPROJ * 8 + 31) / 32) * 32;
    for (int t = tid; t < TOTAL; t += blockDim.x) {
        const int grp = t >> 3, pos = t & 7;
        const int elp = grp / (2 * NFD), rr = grp - elp * 2 * NFD, line = rr >> 1, sd = rr & 1;
        const bool grp_on = grp < NPROJ && e0 + elp < P.nelem;
        const bool on = grp_on && pos < N;
        const int j = on ? elp * NPE + tp_node<DIM>(N, D, line, pos) : 0;
        double q[NV], wt[NV];
        if (on) {
#pragma unroll
            for (int k = 0; k < NV; ++k) q[k] = P.U[k * P.ndofs + (int64_t)e0 * NPE + j];
            if constexpr (A::WC) {
#pragma unroll
                for (int k = 0; k < NV; ++k) wt[k] = sWn[k * NN + j];
            } else {
                entropy_of<DIM>(q, g, wt);
            }
#pragma unroll
            for (int k = 0; k < NV; ++k) wt[k] *= lv[sd * N + pos];
        } else {
#pragma unroll
            for (int k = 0; k < NV; ++k) wt[k] = 0.0;
        }
#pragma unroll
        for (int k = 0; k < NV; ++k) wt[k] = gsum(wt[k]);
        double qt[NV], pt = 1.0;
        if (grp_on) {
            pt = state_of_entropy<DIM>(wt, g, qt);
        } else {
#pragma unroll
            for (int k = 0; k < NV; ++k) qt[k] = k == 0 || k == DIM + 1 ? 1.0 : 0.0;
        }
        double cl[NV];
        if (on) {
            double vt[NARR], vj[NARR], F[NV];
            split_node_values<DIM, TP>(qt, pt, vt);
#pragma unroll
            for (int k = 0; k < NARR; ++k) vj[k] = sprim[k * NN + j];
            if constexpr (CURV) {
                const int64_t ns = (int64_t)P.nelem * DIM * NFD * (N + 1);
                const int64_t si = (((int64_t)(e0 + elp) * DIM + D) * NFD + line) * (N + 1) + (sd ? N : 0);
                const int64_t gj = (int64_t)e0 * NPE + j;
                const double js = P.subJ[si];
                double nrm[DIM];
#pragma unroll
                for (int k = 0; k < DIM; ++k)
                    nrm[k] = 0.5 * fma(P.subfr[k * ns + si], js, P.Jan[(k + D * DIM) * P.ndofs + gj]);
                split_pair_flux<DIM, -1, TP>(vj, vt, q, qt, g, F, nrm);
            } else {
                split_pair_flux<DIM, D, TP>(vj, vt, q, qt, g, F);
            }
#pragma unroll
            for (int k = 0; k < NV; ++k) {
                sF2[(sd * NV + k) * NN + j] = F[k];
                cl[k] = lv[sd * N + pos] * F[k];
            }
        } else {
#pragma unroll
            for (int k = 0; k < NV; ++k) cl[k] = 0.0;
        }
#pragma unroll
        for (int k = 0; k < NV; ++k) cl[k] = gsum(cl[k]);
        if (grp_on && pos == 0) {
#pragma unroll
            for (int k = 0; k < NV; ++k) scl[k * NPROJ + grp] = cl[k];
        }
    }
    __syncthreads();
    const int e = e0 + el;
    int pos = 0, line = 0;
    tp_coords<DIM>(N, i, D, pos, line);
    const int64_t gi = (int64_t)e * NPE + i;
    const double Ja = active ? (CURV ? 1.0 : P.Ja[e * DIM + D]) : 0.0;
    int32_t pl = 0, pr = 0;
    int64_t ofl = 0, ofr = 0;   // the face dofs of the line's two ends
    if (active) {
        pl = P.elem_face[e * 2 * DIM + 2 * D];
        pr = P.elem_face[e * 2 * DIM + 2 * D + 1];
        ofl = trace_offset<DIM, N, CURV>(P, e, 2 * D, line);
        ofr = trace_offset<DIM, N, CURV>(P, e, 2 * D + 1, line);
        if (!index_ok(ofl, P.nfdofs, P.status, e)) ofl = 0;
        if (!index_ok(ofr, P.nfdofs, P.status, e)) ofr = 0;
        const double sl = (pl & 1) ? -1.0 : 1.0, sr = (pr & 1) ? -1.0 : 1.0;
        double acc[NV];
        hybrid_node_sum<DIM, N, D, TP, CURV>(P, gi, el, pos, line, Dsh, spb, acc);
        const int c0 = 2 * (el * NFD + line);
        const double wq = P.omega1[pos] * Ja;
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            const double fls = sl * __ldcg(P.FnU + k * P.nfdofs + ofl);
            const double frs = sr * __ldcg(P.FnU + k * P.nfdofs + ofr);
            const double Fl = sF2[k * NN + tid] - scl[k * NPROJ + c0];
            const double Fr = sF2[(NV + k) * NN + tid] - scl[k * NPROJ + c0 + 1];
            sH[k * NN + tid] = wq * acc[k] - lv[pos] * fma(Ja, Fl, -fls) + lv[N + pos] * fma(Ja, Fr, frs);
            if (pos == 0) sF2[k * NN + tid] = -fls;   // F_0, read by the line's scan
        }
    }
    __syncthreads();   // the node phase has read sF2, whose interface slots the FV phase writes
    // the FV flux and the entropy jump of every subcell interface, one thread per interface (the
    // block's interfaces numbered consecutively: the spare threads are whole idle warps), into
    // the slot of the interface's right node
    constexpr int NFV = S::EPB * NFD * (N - 1);
    for (int t = tid; t < NFV; t += blockDim.x) {
        const int elp = t / (NFD * (N - 1));
        const int rr = t - elp * (NFD * (N - 1));
        const int ln = rr / (N - 1), ps = 1 + (rr - ln * (N - 1));
        const int ef = e0 + elp;
        if (ef >= P.nelem) continue;
        const int jn = elp * NPE + tp_node<DIM>(N, D, ln, ps);
        const int il = elp * NPE + tp_node<DIM>(N, D, ln, ps - 1);
        const int64_t gl = (int64_t)e0 * NPE + il, gr = (int64_t)e0 * NPE + jn;
        double ql[NV], qr[NV], Fv[NV];
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            ql[k] = P.U[k * P.ndofs + gl];
            qr[k] = P.U[k * P.ndofs + gr];
        }
        SubcellFace<DIM> sf;
        subcell_fv<DIM, N, D, CURV>(P, ef, ln, ps, CURV ? 1.0 : P.Ja[ef * DIM + D], ql, qr, sf, Fv);
        double wl[NV], wr[NV];
        if constexpr (A::WC) {
#pragma unroll
            for (int k = 0; k < NV; ++k) {
                wl[k] = sWn[k * NN + il];
                wr[k] = sWn[k * NN + jn];
            }
        } else {
            entropy_of<DIM>(ql, g, wl);
            entropy_of<DIM>(qr, g, wr);
        }
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            sF2[k * NN + jn] = Fv[k];
            sdW[k * NN + jn] = wr[k] - wl[k];
        }
    }
    __syncthreads();
    for (int t = tid; t < S::EPB * NFD; t += blockDim.x) {   // the scan, forward then reverse
        const int elp = t / NFD, ln = t - elp * NFD;
        if (e0 + elp >= P.nelem) continue;
        const int j0 = elp * NPE + tp_node<DIM>(N, D, ln, 0);
        double Fb[NV];
#pragma unroll
        for (int k = 0; k < NV; ++k) Fb[k] = sF2[k * NN + j0];
        int jp = j0;
        for (int pp = 1; pp < N; ++pp) {
            const int jn = elp * NPE + tp_node<DIM>(N, D, ln, pp);
            double d[NV], bb = 0.0;
#pragma unroll
            for (int k = 0; k < NV; ++k) {
                d[k] = (Fb[k] + sH[k * NN + jp]) - sF2[k * NN + jn];
                bb = fma(sdW[k * NN + jn], d[k], bb);
            }
            const double dl = sqrt_refined(fma(bb, bb, P.blend));
            const double dlt = fmax((dl - bb) * rcp_refined(dl), 0.5);
#pragma unroll
            for (int k = 0; k < NV; ++k) {
                Fb[k] = fma(dlt, d[k], sF2[k * NN + jn]);
                sF2[(NV + k) * NN + jn] = d[k];
            }
            jp = jn;
        }
        double carry[NV], sl_[NV], sr_[NV];
#pragma unroll
        for (int k = 0; k < NV; ++k) carry[k] = sl_[k] = sr_[k] = 0.0;
        int jn = jp;   // the line's last node
        for (int pp = N - 1; pp >= 1; --pp) {
            jp = elp * NPE + tp_node<DIM>(N, D, ln, pp - 1);
            const double iwp = rcp_refined(P.omega1[pp]), iwm = rcp_refined(P.omega1[pp - 1]);
            double Gb[NV], d[NV], dW[NV], bb = 0.0, db = 0.0;
#pragma unroll
            for (int k = 0; k < NV; ++k) {
                Gb[k] = fma(sw[k * NN + jn], iwp, -sw[k * NN + jp] * iwm) + carry[k];
                d[k] = sF2[(NV + k) * NN + jn];
                dW[k] = sdW[k * NN + jn];
                bb = fma(dW[k], d[k], bb);
                db = fma(Gb[k], d[k], db);
            }
            const double dl = sqrt_refined(fma(bb, bb, P.blend)), idl = rcp_refined(dl);
            const double draw = (dl - bb) * idl;
            const bool free_ = 0.5 < draw;   // Base.max(draw, 0.5) takes draw only above 0.5
            const double dlt = free_ ? draw : 0.5;
            const double bbar = free_ ? -db * P.blend * idl * idl * idl : 0.0;
            const double wm = P.omega1[pp - 1];
#pragma unroll
            for (int k = 0; k < NV; ++k) {
                const double xb = fma(dlt, Gb[k], bbar * dW[k]);   // the cotangent of X_pp
                sF2[k * NN + jn] = fma(1.0 - dlt, Gb[k], -bbar * dW[k]);
                sF2[(NV + k) * NN + jn] = bbar * d[k];
                sH[k * NN + jp] = -wm * xb;
                sl_[k] = fma(lv[pp - 1], xb, sl_[k]);
                sr_[k] = fma(lv[N + pp - 1], xb, sr_[k]);
                carry[k] = xb;
            }
            jn = jp;
        }
        const int jl = elp * NPE + tp_node<DIM>(N, D, ln, N - 1);
        const double iw0 = rcp_refined(P.omega1[0]), iwl = rcp_refined(P.omega1[N - 1]);
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            sH[k * NN + jl] = 0.0;
            sdW[k * NN + j0] = sl_[k] - fma(sw[k * NN + j0], iw0, carry[k]);
            sdW[k * NN + jl] = fma(-sw[k * NN + jl], iwl, sr_[k]);
        }
    }
    __syncthreads();
    if (active && pos > 0) {   // the FV flux and the entropy jump transposed
        const int il = el * NPE + tp_node<DIM>(N, D, line, pos - 1);
        const int64_t gl = (int64_t)e0 * NPE + il;
        double ql[NV], qr[NV], Fvb[NV], wbar[NV], ol[NV], orr[NV];
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            ql[k] = P.U[k * P.ndofs + gl];
            qr[k] = P.U[k * P.ndofs + gi];
            Fvb[k] = sF2[k * NN + tid];
            wbar[k] = sF2[(NV + k) * NN + tid];
        }
        SubcellFace<DIM> sf;
        subcell_face<DIM, N, D, CURV>(P, e, line, pos, Ja, ql, qr, sf);
        subcell_fv_vjp<DIM, D, CURV>(P, sf, Fvb, ol, orr);
        const double prr = pressure_of<DIM>(qr, g), plv = pressure_of<DIM>(ql, g);
#pragma unroll
        for (int k = 0; k < NV; ++k) qb[k] += orr[k];
        entropy_vjp<DIM>(qr, prr, g, wbar, qb);
#pragma unroll
        for (int k = 0; k < NV; ++k) wbar[k] = -wbar[k];
        entropy_vjp<DIM>(ql, plv, g, wbar, ol);
#pragma unroll
        for (int k = 0; k < NV; ++k) spb[k * NN + il] = ol[k];
    }
    if (active && (pos == 0 || pos == N - 1)) {   // the face-flux cotangents, by side of the face
        const bool left = pos == 0;
        const int32_t pk = left ? pl : pr;
        const int64_t o = left ? ofl : ofr;
        const double sg = (pk & 1) ? -1.0 : 1.0;
        double* dst = P.FbS + (int64_t)(pk & 1) * NV * P.nfdofs;
#pragma unroll
        for (int k = 0; k < NV; ++k) dst[k * P.nfdofs + o] = sg * sdW[k * NN + tid];
    }
    __syncthreads();
    if (active && pos < N - 1) {   // the cotangent from the interface on this node's right
#pragma unroll
        for (int k = 0; k < NV; ++k) qb[k] += spb[k * NN + tid];
    }
    __syncthreads();
}

// CURV: the pair flux along the averaged metric column n̄ = (Ja_a + Ja_b)/2 of direction D (the
// metric terms are in the flux; sJD then holds -D♯ alone).
template <int DIM, int N, int D, int TP, bool CURV = false, int CH = 1>
__device__ __forceinline__ void adj_split_pairs(const AdjElemParams& P, int e0, const double* sJD,
                                                const double* sprim, const double* sw, double* spb,
                                                const uint8_t* stab, double cb, int chunk = 0) {
    using S = Shape<DIM, N>;
    using A = AdjSplitShape<DIM, N, TP>;
    constexpr int NV = DIM + 2, NPE = S::NPE, NN = S::NN, NFD = S::NFD, NPAIR = S::NPAIR;
    constexpr int NPB = A::NPB, NPTC = A::NPT / CH;   // CH > 1: this chunk's pairs, spb holds them alone
    for (int kq = threadIdx.x; kq < NPTC; kq += blockDim.x) {
        const int kp = chunk * NPTC + kq;
        int elp = kp / (NFD * NPAIR);
        int r = kp - elp * (NFD * NPAIR);
        int line = r / NPAIR, pp = r - line * NPAIR;
        if (e0 + elp >= P.nelem) continue;
        int a = stab[2 * pp], b = stab[2 * pp + 1];
        int ia = elp * NPE + tp_node<DIM>(N, D, line, a);
        int ib = elp * NPE + tp_node<DIM>(N, D, line, b);
        const double* jd = sJD + (elp * DIM + D) * N * N;   // -Ja_D D♯(i, j) = jd[i + j N]
        double cab = jd[a + b * N], cba = jd[b + a * N];
        double Fb[NV];
#pragma unroll
        for (int k = 0; k < NV; ++k) Fb[k] = fma(cab, sw[k * NN + ia], cba * sw[k * NN + ib]);
        double v1[DIM], v2[DIM];
#pragma unroll
        for (int k = 0; k < DIM; ++k) {
            v1[k] = sprim[(1 + k) * NN + ia];
            v2[k] = sprim[(1 + k) * NN + ib];
        }
        constexpr int DD = CURV ? -1 : D;   // the flux direction: the axis, or nrm
        double nrm[DIM];
        if constexpr (CURV) {
            const int64_t ga = (int64_t)e0 * NPE + ia, gb = (int64_t)e0 * NPE + ib;
#pragma unroll
            for (int k = 0; k < DIM; ++k)
                nrm[k] = 0.5 * (P.Jan[(k + D * DIM) * P.ndofs + ga] + P.Jan[(k + D * DIM) * P.ndofs + gb]);
        }
        PrimBar o1, o2;
        if constexpr (A::STD) {   // F♯ = ½ (F(Q_a) + F(Q_b)): each node gets ½ J(Q)ᵀ F̄ in conserved variables
            const double g1 = P.gamma - 1.0;
            double qa_[NV], qb_[NV];
#pragma unroll
            for (int k = 0; k < NV; ++k) qa_[k] = qb_[k] = 0.0;
            if constexpr (CURV) {
                euler_flux_vjp_n<DIM>(nrm, v1, sprim[(1 + DIM) * NN + ia], sprim[ia], g1, Fb, 0.5, qa_);
                euler_flux_vjp_n<DIM>(nrm, v2, sprim[(1 + DIM) * NN + ib], sprim[ib], g1, Fb, 0.5, qb_);
            } else {
                euler_flux_vjp<DIM>(D, v1, sprim[(1 + DIM) * NN + ia], sprim[ia], g1, Fb, 0.5, qa_);
                euler_flux_vjp<DIM>(D, v2, sprim[(1 + DIM) * NN + ib], sprim[ib], g1, Fb, 0.5, qb_);
            }
            o1.r = qa_[0];
            o2.r = qb_[0];
#pragma unroll
            for (int k = 0; k < DIM; ++k) {
                o1.v[k] = qa_[1 + k];
                o2.v[k] = qb_[1 + k];
            }
            o1.b = qa_[DIM + 1];
            o2.b = qb_[DIM + 1];
        } else if constexpr (A::KG)
            kg_pair_vjp<DIM, DD>(sprim[ia], v1, sprim[(1 + DIM) * NN + ia], sprim[(2 + DIM) * NN + ia], sprim[ib], v2,
                                 sprim[(1 + DIM) * NN + ib], sprim[(2 + DIM) * NN + ib], Fb, o1, o2, nrm);
        else
            chandra_pair_vjp<DIM, DD, false>(sprim[ia], v1, sprim[(1 + DIM) * NN + ia], sprim[(2 + DIM) * NN + ia],
                                             sprim[ib], v2, sprim[(1 + DIM) * NN + ib], sprim[(2 + DIM) * NN + ib], cb,
                                             Fb, o1, o2, nrm);
        spb[kq] = o1.r;
        spb[NPB * NPTC + kq] = o2.r;
#pragma unroll
        for (int k = 0; k < DIM; ++k) {
            spb[(1 + k) * NPTC + kq] = o1.v[k];
            spb[(NPB + 1 + k) * NPTC + kq] = o2.v[k];
        }
        spb[(1 + DIM) * NPTC + kq] = o1.b;
        spb[(NPB + 1 + DIM) * NPTC + kq] = o2.b;
        if constexpr (A::KG) {
            spb[(2 + DIM) * NPTC + kq] = o1.e;
            spb[(NPB + 2 + DIM) * NPTC + kq] = o2.e;
        }
    }
}

// CURV: the diagonal term is the contravariant flux of node i (its own metric column), and a slave
// face reads its trace cotangent through the orientation.
// G: also the node's projected-state pair cotangents (snode), the spread of the projected
// entropy-variable cotangents (into wb), and the trace cotangents through l at every node (G and
// H: not yet known; the stage's second element pass adds them).
template <int DIM, int N, int D, int TP, bool CURV = false, bool G = false, bool H = false, int CH = 1>
__device__ __forceinline__ void adj_split_nodes(const AdjElemParams& P, int e, int el, int i, int64_t gi,
                                                const double* Dsh, const double* sw, const double* spb,
                                                const double* v, double rho, double p, double g1, double* qb,
                                                PrimBar& acc, const double* snode = nullptr,
                                                const double* sWb = nullptr, double* wb = nullptr, int chunk = 0) {
    using S = Shape<DIM, N>;
    using A = AdjSplitShape<DIM, N, TP, G>;
    constexpr int NV = DIM + 2, NN = S::NN, NFD = S::NFD, NPAIR = S::NPAIR;
    constexpr int NPB = A::NPB, NPTC = A::NPT / CH;
    int pos, line;
    tp_coords<DIM>(N, i, D, pos, line);
    if (CH > 1 && line / (NFD / CH) != chunk) return;   // the node's line is in another chunk
    const int tid = threadIdx.x;
    double dii = Dsh[pos + pos * N];
    if (dii != 0.0) {   // diagonal: F♯(i, i) = F(Q_i)
        double Gd[NV];
#pragma unroll
        for (int k = 0; k < NV; ++k) Gd[k] = dii * sw[k * NN + tid];
        double vv = 0.0;
#pragma unroll
        for (int k = 0; k < DIM; ++k) vv = fma(v[k], v[k], vv);
        double Hq = (P.U[(DIM + 1) * P.ndofs + gi] + p) * rcp_refined(rho);
        if constexpr (CURV) {
            double nrm[DIM];
#pragma unroll
            for (int k = 0; k < DIM; ++k) nrm[k] = P.Jan[(k + D * DIM) * P.ndofs + gi];
            euler_flux_vjp_n<DIM>(nrm, v, vv, Hq, g1, Gd, -1.0, qb);
        } else {
            euler_flux_vjp<DIM>(D, v, vv, Hq, g1, Gd, -P.Ja[e * DIM + D], qb);
        }
    }
    int pbase = el * NFD * NPAIR + line * NPAIR - chunk * NPTC;
    // the N-1 partners of pos, cyclically from pos + 1: every iteration is a pair (a skipped
    // j == pos would still take its FP64 issue slots as predicated-off instructions)
#pragma unroll
    for (int t = 1; t < N; ++t) {
        const int j = pos + t < N ? pos + t : pos + t - N;
        int lo = j < pos ? j : pos, hi = j < pos ? pos : j;
        int pidx = pbase + lo * (2 * N - lo - 1) / 2 + (hi - lo - 1);
        const double* src = spb + (pos == lo ? 0 : NPB * NPTC);
        acc.r += src[pidx];
#pragma unroll
        for (int k = 0; k < DIM; ++k) acc.v[k] += src[(1 + k) * NPTC + pidx];
        acc.b += src[(1 + DIM) * NPTC + pidx];
        if constexpr (A::KG) acc.e += src[(2 + DIM) * NPTC + pidx];
    }
    if constexpr (G) {
        const int tid = threadIdx.x;
        acc.r += snode[tid];
#pragma unroll
        for (int k = 0; k < DIM; ++k) acc.v[k] += snode[(1 + k) * NN + tid];
        acc.b += snode[(1 + DIM) * NN + tid];
        if constexpr (A::KG) acc.e += snode[(2 + DIM) * NN + tid];
        const double* lv = Dsh + N * N;   // l_l, l_r follow D♯
        const int c0 = 2 * (el * NFD + line);
#pragma unroll
        for (int k = 0; k < NV; ++k)
            wb[k] = fma(lv[pos], sWb[k * A::NPROJ + c0], fma(lv[N + pos], sWb[k * A::NPROJ + c0 + 1], wb[k]));
#pragma unroll
        for (int side = 0; side < (H ? 0 : 2); ++side) {
            const int fk = 2 * D + side;
            int32_t pk = P.elem_face[e * 2 * DIM + fk];
            const double* fsrc = (pk & 1) ? P.QbR : P.QbL;
            int64_t o = trace_offset<DIM, N, CURV>(P, e, fk, line);
            if (!index_ok(o, P.nfdofs, P.status, e)) continue;
#pragma unroll
            for (int k = 0; k < NV; ++k) qb[k] = fma(lv[side * N + pos], __ldcg(fsrc + k * P.nfdofs + o), qb[k]);
        }
    } else if (pos == 0 || pos == N - 1) {
        const int fk = 2 * D + (pos == 0 ? 0 : 1);
        int32_t pk = P.elem_face[e * 2 * DIM + fk];
        const double* fsrc = (pk & 1) ? P.QbR : P.QbL;
        int64_t o = trace_offset<DIM, N, CURV>(P, e, fk, line);
        if (index_ok(o, P.nfdofs, P.status, e)) {
#pragma unroll
            for (int k = 0; k < NV; ++k) qb[k] += __ldcg(fsrc + k * P.nfdofs + o);
        }
    }
}

// The adjoint stage combination at node gi with its transposed residual qb.
template <int DIM>
__device__ __forceinline__ void adj_node_epilogue(const AdjElemParams& P, int64_t gi, const double* qb) {
    constexpr int NV = DIM + 2;
    for (int k = 0; k < NV; ++k) {
        double ain = P.Ain[k * P.ndofs + gi];
        double o = fma(P.alpha, ain, qb[k]);
        if (P.readB) o = fma(P.beta, P.B[k * P.ndofs + gi], o);
        if (P.writeB) {
            double b = P.delta_B * ain;
            if (P.gamma_B != 0.0) b = fma(P.gamma_B, P.B[k * P.ndofs + gi], b);
            P.B[k * P.ndofs + gi] = b;
        }
        P.Aout[k * P.ndofs + gi] = o;
        if (P.K) P.K[k * P.ndofs + gi] = fma(P.kA, ain, P.kB * o);
    }
}

// cbar[e] += the element's share of its faces' intensity cotangents (interior faces half each).
template <int DIM, int N>
__device__ __forceinline__ void adj_elem_cbar(const AdjElemParams& P, int e) {
    using S = Shape<DIM, N>;
    double cacc = 0.0;
    for (int fk = 0; fk < 2 * DIM; ++fk) {
        int32_t pk = P.elem_face[e * 2 * DIM + fk];
        int fc = pk >> 1;
        if (!index_ok((int64_t)fc * S::NFD + S::NFD - 1, P.nfdofs, P.status, e)) continue;
        double wgt = P.face_elem[2 * fc + 1] < 0 ? 1.0 : 0.5;
        for (int m = 0; m < S::NFD; ++m) cacc = fma(wgt, __ldcg(P.Ibar + (int64_t)fc * S::NFD + m), cacc);
    }
    P.cbar[e] += cacc;
}

// H: the hybrid operator (adj_hybrid_dir gives the pair weights of each direction).
template <int DIM, int N, int TP, bool CURV = false, bool G = false, bool H = false>
__global__ void __launch_bounds__(Shape<DIM, N>::BLOCK, AdjSplitShape<DIM, N, TP, G, H>::MINB)
    adj_split_elem_kernel(AdjElemParams P) {
    using S = Shape<DIM, N>;
    using A = AdjSplitShape<DIM, N, TP, G, H>;
    constexpr int NV = DIM + 2, NPE = S::NPE, NN = S::NN;
    constexpr int NPB = A::NPB, NARR = A::NARR;
    extern __shared__ double smem[];
    double* sops = smem;
    double* sprim = sops + S::NOPS;   // [NARR][NN]: ρ/2, v/2, β/2, |v|²/4 (KG: ρ/2, v/2, p/2, (E/ρ)/2)
    double* sw = sprim + NARR * NN;   // [NV][NN]: w = λ / J
    double* spb = sw + NV * NN;       // [2][NPB][NPTC]: side-1 / side-2 cotangents of each pair (of a chunk)
    double* sJD = spb + 2 * NPB * A::NPTC;   // [EPB][DIM][N*N]: -Ja_d D♯
    double* sWb = sJD + A::NSD;          // G: [NV][NPROJ] projected entropy-variable cotangents
    double* snode = sWb + NV * A::NPROJ; // G: [NPB][NN] projected-state pair cotangents per node
    double* sHy = snode + (G ? NPB * NN : 0);   // H: [NV][NN] subcell fluxes, then the pair weights
    double* sF2 = sHy + (H ? NV * NN : 0);      // G and H: [2][NV][NN] (adj_hybrid_gauss_dir)
    double* sWn = sF2 + (G && H ? 2 * NV * NN : 0);   // A::WC: [NV][NN] the nodes' entropy variables
    uint8_t* stab = (uint8_t*)(sJD + A::NSD + A::NGX);
    const int tid = threadIdx.x;
    for (int t = tid; t < S::NOPS; t += blockDim.x) sops[t] = P.ops[t];
    for (int t = tid; t < A::NSD; t += blockDim.x) {
        int q = t / (N * N), ij = t - q * (N * N);
        int elq = q / DIM, d = q - elq * DIM;
        int eq_ = blockIdx.x * S::EPB + elq;
        sJD[t] = eq_ < P.nelem ? -(CURV ? 1.0 : P.Ja[eq_ * DIM + d]) * P.ops[N * N + ij] : 0.0;
    }
    if (tid == 0) {
        int c = 0;
        for (int a = 0; a < N; ++a)
            for (int b = a + 1; b < N; ++b) { stab[2 * c] = (uint8_t)a; stab[2 * c + 1] = (uint8_t)b; ++c; }
    }
    const int e0 = blockIdx.x * S::EPB;
    const int el = tid / NPE, i = tid - el * NPE;
    const int e = e0 + el;
    const bool active = (tid < NN) && (e < P.nelem);
    const int64_t gi = (int64_t)e * NPE + i;
    const double g = P.gamma, g1 = g - 1.0;
    double rho = 1.0, p = 1.0, v[DIM];
    if (active) {
        double w = (CURV ? P.invJn[gi] : P.invJ[e]) * P.s_lam;
        double q[NV];
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            sw[k * NN + tid] = w * P.Ain[k * P.ndofs + gi];
            q[k] = P.U[k * P.ndofs + gi];
        }
        rho = q[0];
        double ir = rcp_refined(rho), ke = 0.0, vv = 0.0;
#pragma unroll
        for (int k = 0; k < DIM; ++k) {
            v[k] = q[1 + k] * ir;
            ke = fma(q[1 + k], v[k], ke);
            vv = fma(v[k], v[k], vv);
        }
        p = g1 * fma(-0.5, ke, q[DIM + 1]);
        sprim[tid] = 0.5 * rho;
#pragma unroll
        for (int k = 0; k < DIM; ++k) sprim[(1 + k) * NN + tid] = 0.5 * v[k];
        if constexpr (A::STD) {
            sprim[tid] = (q[DIM + 1] + p) * ir;
#pragma unroll
            for (int k = 0; k < DIM; ++k) sprim[(1 + k) * NN + tid] = v[k];
            sprim[(1 + DIM) * NN + tid] = vv;
        } else if constexpr (A::KG) {
            sprim[(1 + DIM) * NN + tid] = 0.5 * p;
            sprim[(2 + DIM) * NN + tid] = 0.5 * (q[DIM + 1] * ir);
        } else {
            sprim[(1 + DIM) * NN + tid] = (0.25 * rho) * rcp_refined(p);
            sprim[(2 + DIM) * NN + tid] = 0.25 * vv;
        }
        if constexpr (A::WC) {
            double wn[NV];
            entropy_of<DIM>(q, g, wn);
#pragma unroll
            for (int k = 0; k < NV; ++k) sWn[k * NN + tid] = wn[k];
        }
    } else {
#pragma unroll
        for (int k = 0; k < DIM; ++k) v[k] = 0.0;
    }
    __syncthreads();
    const double* Dsh = sops + N * N;   // D♯(i, j) = Dsh[i + j N]
    const double cb = 0.5 / g1;
    double qb[NV];
    PrimBar acc;
    acc.r = 0.0;
    acc.b = 0.0;
    acc.e = 0.0;
#pragma unroll
    for (int k = 0; k < NV; ++k) qb[k] = 0.0;
#pragma unroll
    for (int k = 0; k < 3; ++k) acc.v[k] = 0.0;
    double wb[NV];   // G: cotangent of the node's entropy variables
#pragma unroll
    for (int k = 0; k < NV; ++k) wb[k] = 0.0;
    constexpr int D1 = DIM > 1 ? 1 : 0, D2 = DIM > 2 ? 2 : 0;
    const double* swd = H ? sHy : sw;   // the pair weights
#pragma unroll 1
    for (int dir = 0; dir < DIM; ++dir) {
        if constexpr (G && H) {
            if (dir == 0)
                adj_hybrid_gauss_dir<DIM, N, 0, TP, CURV>(P, e0, active, el, i, sops, sprim, sw, sHy, spb, stab, sF2,
                                                          sWb, snode, sWn, qb);
            else if (dir == 1)
                adj_hybrid_gauss_dir<DIM, N, D1, TP, CURV>(P, e0, active, el, i, sops, sprim, sw, sHy, spb, stab, sF2,
                                                           sWb, snode, sWn, qb);
            else
                adj_hybrid_gauss_dir<DIM, N, D2, TP, CURV>(P, e0, active, el, i, sops, sprim, sw, sHy, spb, stab, sF2,
                                                           sWb, snode, sWn, qb);
        } else if constexpr (H) {
            if (dir == 0)
                adj_hybrid_dir<DIM, N, 0, TP, CURV>(P, e0, active, el, i, sops, sprim, sw, sHy, spb, stab, sWn,
                                                    qb);
            else if (dir == 1)
                adj_hybrid_dir<DIM, N, D1, TP, CURV>(P, e0, active, el, i, sops, sprim, sw, sHy, spb, stab, sWn,
                                                     qb);
            else
                adj_hybrid_dir<DIM, N, D2, TP, CURV>(P, e0, active, el, i, sops, sprim, sw, sHy, spb, stab, sWn,
                                                     qb);
        }
        constexpr int CH = A::CH;
#pragma unroll 1
        for (int ch = 0; ch < CH; ++ch) {   // CH > 1: the lines in chunks, each its pairs then its nodes
            if (dir == 0) adj_split_pairs<DIM, N, 0, TP, CURV, CH>(P, e0, sJD, sprim, swd, spb, stab, cb, ch);
            else if (dir == 1) adj_split_pairs<DIM, N, D1, TP, CURV, CH>(P, e0, sJD, sprim, swd, spb, stab, cb, ch);
            else adj_split_pairs<DIM, N, D2, TP, CURV, CH>(P, e0, sJD, sprim, swd, spb, stab, cb, ch);
            if constexpr (G) {
                constexpr bool WC = A::WC;
                if (ch == 0) {
                    if (dir == 0)
                        adj_split_projection<DIM, N, 0, TP, CURV, H, WC>(P, e0, sops, sprim, swd, snode, sWb, cb, sWn);
                    else if (dir == 1)
                        adj_split_projection<DIM, N, D1, TP, CURV, H, WC>(P, e0, sops, sprim, swd, snode, sWb, cb,
                                                                         sWn);
                    else
                        adj_split_projection<DIM, N, D2, TP, CURV, H, WC>(P, e0, sops, sprim, swd, snode, sWb, cb,
                                                                         sWn);
                }
            }
            __syncthreads();
            if (active) {
                if (dir == 0)
                    adj_split_nodes<DIM, N, 0, TP, CURV, G, H, CH>(P, e, el, i, gi, Dsh, swd, spb, v, rho, p, g1, qb,
                                                                   acc, snode, sWb, wb, ch);
                else if (dir == 1)
                    adj_split_nodes<DIM, N, D1, TP, CURV, G, H, CH>(P, e, el, i, gi, Dsh, swd, spb, v, rho, p, g1, qb,
                                                                    acc, snode, sWb, wb, ch);
                else
                    adj_split_nodes<DIM, N, D2, TP, CURV, G, H, CH>(P, e, el, i, gi, Dsh, swd, spb, v, rho, p, g1, qb,
                                                                    acc, snode, sWb, wb, ch);
            }
            __syncthreads();
        }
    }
    if (!active) return;
    double vv = 0.0;
#pragma unroll
    for (int k = 0; k < DIM; ++k) vv = fma(v[k], v[k], vv);
    if constexpr (A::STD) {   // the pairs' cotangents are already conserved
        qb[0] += acc.r;
#pragma unroll
        for (int k = 0; k < DIM; ++k) qb[1 + k] += acc.v[k];
        qb[DIM + 1] += acc.b;
    } else if constexpr (A::KG) {
        kg_prim_to_cons_vjp<DIM>(rho, v, vv, P.U[(DIM + 1) * P.ndofs + gi], g1, acc, qb);
    } else {
        prim_to_cons_vjp<DIM>(rho, v, vv, p, g1, acc, qb);
    }
    if constexpr (G) {   // the projections' entropy variables of this node
        double q[NV];
#pragma unroll
        for (int k = 0; k < NV; ++k) q[k] = P.U[k * P.ndofs + gi];
        entropy_vjp<DIM>(q, p, g, wb, qb);
    }
    if constexpr (G && H) {   // the traces' cotangents follow the face VJP
#pragma unroll
        for (int k = 0; k < NV; ++k) P.Tq[k * P.ndofs + gi] = qb[k];
    } else {
        adj_node_epilogue<DIM>(P, gi, qb);
        if (P.cbar && i == 0) adj_elem_cbar<DIM, N>(P, e);
    }
}

template <int DIM, int N, int TP, bool CURV = false, bool G = false, bool H = false>
cudaError_t launch_adj_split_n(const AdjElemParams& P, cudaStream_t s) {
    using S = Shape<DIM, N>;
    constexpr size_t smem = AdjSplitShape<DIM, N, TP, G, H>::SMEM;
    if constexpr (smem > 227 * 1024) {   // G, H: the Kennedy-Gruber 3D p=7 tile (checked on the host first)
        return cudaErrorInvalidValue;
    } else {
    static std::once_flag once;
    static cudaError_t attr = cudaSuccess;
    std::call_once(once, [] {
        attr = cudaFuncSetAttribute(adj_split_elem_kernel<DIM, N, TP, CURV, G, H>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    });
    if (attr != cudaSuccess) return attr;
    int grid = (P.nelem + S::EPB - 1) / S::EPB;
    adj_split_elem_kernel<DIM, N, TP, CURV, G, H><<<grid, S::BLOCK, smem, s>>>(P);
    return cudaGetLastError();
    }
}

template <int DIM, int TP, bool CURV = false, bool G = false, bool H = false>
cudaError_t launch_adj_split_tp(int n, const AdjElemParams& P, cudaStream_t s) {
    switch (n) {
        case 2: return launch_adj_split_n<DIM, 2, TP, CURV, G, H>(P, s);
        case 3: return launch_adj_split_n<DIM, 3, TP, CURV, G, H>(P, s);
        case 4: return launch_adj_split_n<DIM, 4, TP, CURV, G, H>(P, s);
        case 5: return launch_adj_split_n<DIM, 5, TP, CURV, G, H>(P, s);
        case 6: return launch_adj_split_n<DIM, 6, TP, CURV, G, H>(P, s);
        case 7: return launch_adj_split_n<DIM, 7, TP, CURV, G, H>(P, s);
        case 8: return launch_adj_split_n<DIM, 8, TP, CURV, G, H>(P, s);
        default: return cudaErrorInvalidValue;
    }
}

// The split form's two-point flux: Chandrashekar, Kennedy-Gruber or StdAverage.
template <int DIM, bool CURV = false, bool G = false, bool H = false>
cudaError_t launch_adj_split(int n, int tp, const AdjElemParams& P, cudaStream_t s) {
    if (tp == FLOU_TP_KENNEDY_GRUBER) return launch_adj_split_tp<DIM, FLOU_TP_KENNEDY_GRUBER, CURV, G, H>(n, P, s);
    if (tp == FLOU_TP_STD_AVERAGE) return launch_adj_split_tp<DIM, FLOU_TP_STD_AVERAGE, CURV, G, H>(n, P, s);
    return launch_adj_split_tp<DIM, FLOU_TP_CHANDRASHEKAR, CURV, G, H>(n, P, s);
}

// Whether the split adjoint tile (G: Gauss nodes, H: the hybrid operator) fits in shared memory
// (with the pairs in two chunks of lines where all of them at once do not: every tile does).
template <int TP>
constexpr size_t adj_split_smem_3d8(bool G, bool H) {
    return G && H ? AdjSplitShape<3, 8, TP, true, true>::SMEM
                  : (G ? AdjSplitShape<3, 8, TP, true, false>::SMEM : AdjSplitShape<3, 8, TP, false, true>::SMEM);
}
inline bool adj_split_tile_fits(int dim, int n, int tp, bool gauss, bool hybrid) {
    if (!(dim == 3 && n == 8)) return true;
    const size_t smem = tp == FLOU_TP_KENNEDY_GRUBER ? adj_split_smem_3d8<FLOU_TP_KENNEDY_GRUBER>(gauss, hybrid)
                        : tp == FLOU_TP_STD_AVERAGE  ? adj_split_smem_3d8<FLOU_TP_STD_AVERAGE>(gauss, hybrid)
                                                     : adj_split_smem_3d8<FLOU_TP_CHANDRASHEKAR>(gauss, hybrid);
    return smem <= 227 * 1024;
}

// The second element pass of a hybrid stage on Gauss nodes: the first pass's partial node
// cotangents Tq, plus every node's l_l[pos] and l_r[pos] shares of its lines' trace cotangents
// (from the face VJP), then the stage combination and cbar.  One thread per node.
template <int DIM, int N, bool CURV = false>
__global__ void __launch_bounds__(256) adj_hybrid_gauss_finish_kernel(AdjElemParams P) {
    constexpr int NV = DIM + 2, NPE = Shape<DIM, N>::NPE;
    const int64_t gi = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (gi >= P.ndofs) return;
    const int e = (int)(gi / NPE), i = (int)(gi - (int64_t)e * NPE);
    const double* lv = P.ops + 2 * N * N;
    double qb[NV];
#pragma unroll
    for (int k = 0; k < NV; ++k) qb[k] = P.Tq[k * P.ndofs + gi];
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
        int pos, line;
        tp_coords<DIM>(N, i, d, pos, line);
#pragma unroll
        for (int side = 0; side < 2; ++side) {
            const int fk = 2 * d + side;
            const int32_t pk = P.elem_face[e * 2 * DIM + fk];
            const double* fsrc = (pk & 1) ? P.QbR : P.QbL;
            const int64_t o = trace_offset<DIM, N, CURV>(P, e, fk, line);
            if (!index_ok(o, P.nfdofs, P.status, e)) continue;
#pragma unroll
            for (int k = 0; k < NV; ++k) qb[k] = fma(lv[side * N + pos], __ldcg(fsrc + k * P.nfdofs + o), qb[k]);
        }
    }
    adj_node_epilogue<DIM>(P, gi, qb);
    if (P.cbar && i == 0) adj_elem_cbar<DIM, N>(P, e);
}

template <int DIM, bool CURV = false>
cudaError_t launch_adj_hybrid_gauss_finish_t(int n, const AdjElemParams& P, cudaStream_t s) {
    const int grid = (int)((P.ndofs + 255) / 256);
    switch (n) {
        case 2: adj_hybrid_gauss_finish_kernel<DIM, 2, CURV><<<grid, 256, 0, s>>>(P); break;
        case 3: adj_hybrid_gauss_finish_kernel<DIM, 3, CURV><<<grid, 256, 0, s>>>(P); break;
        case 4: adj_hybrid_gauss_finish_kernel<DIM, 4, CURV><<<grid, 256, 0, s>>>(P); break;
        case 5: adj_hybrid_gauss_finish_kernel<DIM, 5, CURV><<<grid, 256, 0, s>>>(P); break;
        case 6: adj_hybrid_gauss_finish_kernel<DIM, 6, CURV><<<grid, 256, 0, s>>>(P); break;
        case 7: adj_hybrid_gauss_finish_kernel<DIM, 7, CURV><<<grid, 256, 0, s>>>(P); break;
        case 8: adj_hybrid_gauss_finish_kernel<DIM, 8, CURV><<<grid, 256, 0, s>>>(P); break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

// ---- the scalar equations: linear advection (LinearAdvection.jl) and Burgers (Burgers.jl) ----
// Face VJP.  The flux is F = J (an (q_l + q_r)/2 + [LxF] |an| (q_l - q_r)/2 c) for linear
// advection (an = a·n), and F = J ((q_l² + q_r²)/4 n + [LxF] λ (q_l - q_r)/2 c) with
// λ = max(|q_l|, |q_r|) for Burgers (1D); the face normal n is the master side's.  Its cotangent
// comes from the lift as for the Euler face VJP (G: the interpolated traces and the full-line
// lift).  A fixed boundary state (Dirichlet, a state field) takes no cotangent; outflow passes
// the ghost's to the trace.  The intensity cotangent feeds dJ/dc.
// CURV (linear advection on general geometry): the slave trace through the orientation, per-node
// 1/J, the face node's normal and surface Jacobian.
template <int DIM, int EQ, bool G = false, bool CURV = false>
__global__ void __launch_bounds__(256) adj_face_scalar_kernel(AdjFaceParams P) {
    int64_t gid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (gid >= (int64_t)P.nfaces * P.nfd) return;
    const int f = (int)(gid / P.nfd), m = (int)(gid - (int64_t)f * P.nfd);
    const int n = P.n;
    const int32_t s0 = P.face_elem[2 * f], s1 = P.face_elem[2 * f + 1];
    if (kChecked && !(index_ok(s0 >> 3, P.ndofs / P.npe, P.status, 0) &&
                      (s1 < 0 || index_ok(s1 >> 3, P.ndofs / P.npe, P.status, s0 >> 3)) &&
                      (s1 >= 0 || index_ok(P.face_bc[f], MAXBC, P.status, s0 >> 3))))
        return;
    const double* lvb = P.ops + 2 * n * n;
    const double* dgl = lvb + 2 * n;
    const double* dgr = dgl + n;
    // the trace of side s and the lift transpose Σ ∂g (w λ) over its line (LGL: the end node)
    auto side = [&](int32_t s, int mm, double& q, double& fl) {
        const int e = s >> 3, pos = s & 7, dir = pos >> 1, right = pos & 1;
        if constexpr (G) {
            const double* lv = lvb + (right ? n : 0);
            const double* dg = right ? dgr : dgl;
            q = fl = 0.0;
            for (int p = 0; p < n; ++p) {
                const int64_t gg = (int64_t)e * P.npe + tp_node<DIM>(n, dir, mm, p);
                const double wj = (CURV ? P.invJn[gg] : P.invJ[e]) * P.s_lam;
                q = fma(lv[p], P.U[gg], q);
                fl = fma(wj * dg[p], P.Ain[gg], fl);
            }
        } else {
            const int64_t gg = (int64_t)e * P.npe + tp_node<DIM>(n, dir, mm, right ? n - 1 : 0);
            const double wj = (CURV ? P.invJn[gg] : P.invJ[e]) * P.s_lam;
            q = P.U[gg];
            fl = (right ? dgr[n - 1] : dgl[0]) * wj * P.Ain[gg];
        }
    };
    double ql, qr = 0.0, f1, f2 = 0.0;
    side(s0, m, ql, f1);
    double Fb = -f1;
    int bck = 0;
    if (s1 >= 0) {
        const int mm = CURV ? master2slave<DIM>(m, P.orient[f], n) : m;
        if (CURV && !index_ok(mm, P.nfd, P.status, s1 >> 3)) return;
        side(s1, mm, qr, f2);
        Fb += f2;
    } else {
        const int bi = P.face_bc[f];
        bck = P.bc_kind[bi];
        qr = bck == FLOU_BC_INFLOW ? P.bc_state[bi][0] : bck == FLOU_BC_STATE_FIELD ? P.bc_field[gid] : ql;
    }
    Fb *= CURV ? P.faceJn[gid] : P.faceJ[f];
    double inten = P.intensity;
    if (P.elem_c) {
        const int e1 = s0 >> 3, e2 = s1 >= 0 ? (s1 >> 3) : e1;
        inten = (P.elem_c[e1] + P.elem_c[e2]) * 0.5;
    }
    FrameTab fr = frame_of(DIM, s0 & 7);
    if constexpr (CURV) {
#pragma unroll
        for (int c = 0; c < 3; ++c) fr.n[c] = P.frames[c * P.nfdofs + gid];
    }
    double ab, bb, Ib = 0.0;
    if constexpr (EQ == FLOU_EQ_LINEAR_ADVECTION) {
        double an = P.adv[0] * fr.n[0];
        if (DIM > 1) an = an + P.adv[1] * fr.n[1];
        if (DIM > 2) an = an + P.adv[2] * fr.n[2];
        ab = bb = 0.5 * an * Fb;
        if (P.lxf) {
            const double d = 0.5 * fabs(an) * inten * Fb;
            ab += d;
            bb -= d;
            Ib = 0.5 * fabs(an) * (ql - qr) * Fb;
        }
    } else {   // Burgers
        ab = 0.5 * ql * fr.n[0] * Fb;
        bb = 0.5 * qr * fr.n[0] * Fb;
        if (P.lxf) {
            const double al = fabs(ql), ar = fabs(qr);
            const bool left = ar < al;   // Base.max(|q_l|, |q_r|)
            const double lam = left ? al : ar;
            const double d = 0.5 * lam * inten * Fb;
            ab += d;
            bb -= d;
            const double lb = 0.5 * (ql - qr) * inten * Fb;   // the cotangent of λ
            if (left) ab += lb * (signbit(ql) ? -1.0 : 1.0);
            else bb += lb * (signbit(qr) ? -1.0 : 1.0);
            Ib = 0.5 * lam * (ql - qr) * Fb;
        }
    }
    if (s1 < 0 && bck != FLOU_BC_INFLOW && bck != FLOU_BC_STATE_FIELD) ab += bb;   // the ghost is the trace
    P.QbL[gid] = ab;
    if (s1 >= 0) P.QbR[gid] = bb;
    P.Ibar[gid] = Ib;
}

// Element VJP of the scalar equations (Cartesian): per direction, with f'(u) = a_d (linear
// advection) or u (Burgers), the strong form F̃ = Ja f(u) gives ū += -Ja f'(u) Σ_r Ds(r, pos) w_r;
// the split form with the arithmetic-mean two-point flux F♯ = (f(u_i) + f(u_j))/2 gives
// ū_i += -Ja f'(u_i) (½ Σ_(j≠i) (D♯_ij w_i + D♯_ji w_j) + D♯_ii w_i).  Then the trace cotangents
// (G: through l at every node), the stage combination and dJ/dc as for the Euler kernels.
// CURV (linear advection on general geometry): per-node 1/J; the strong form's flux derivative is
// the contravariant a·Ja_d of the node, the split form's pair (i, j) runs along a·(Ja_i + Ja_j)/2
// and its diagonal along a·Ja_i, and the slave traces are read through the orientation.
template <int DIM, int N, int EQ, bool SPLIT, bool G = false, bool CURV = false>
__global__ void __launch_bounds__(Shape<DIM, N>::BLOCK) adj_elem_scalar_kernel(AdjElemParams P) {
    using S = Shape<DIM, N>;
    constexpr int NPE = S::NPE, NN = S::NN, NFD = S::NFD;
    extern __shared__ double smem[];
    double* sops = smem;
    double* sw = sops + S::NOPS;
    const int tid = threadIdx.x;
    for (int t = tid; t < S::NOPS; t += blockDim.x) sops[t] = P.ops[t];
    const int e0 = blockIdx.x * S::EPB;
    const int el = tid / NPE, i = tid - el * NPE;
    const int e = e0 + el;
    const bool active = (tid < NN) && (e < P.nelem);
    const int64_t gi = (int64_t)e * NPE + i;
    double ain = 0.0;
    if (active) {
        ain = P.Ain[gi];
        sw[tid] = (CURV ? P.invJn[gi] : P.invJ[e]) * P.s_lam * ain;
    }
    __syncthreads();
    if (!active) return;
    const double u = P.U[gi];
    const double* Ds = sops;
    const double* Dsh = sops + N * N;
    const double* lv = sops + 2 * N * N;
    double qb = 0.0;
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
        int pos, line;
        tp_coords<DIM>(N, i, d, pos, line);
        auto a_dot_Ja = [&](int64_t g) {   // a·Ja[:, d] of node g
            double x = 0.0;
#pragma unroll
            for (int k = 0; k < DIM; ++k) x = fma(P.adv[k], P.Jan[(k + d * DIM) * P.ndofs + g], x);
            return x;
        };
        if constexpr (CURV && SPLIT) {
            const double wi = sw[tid], ai = a_dot_Ja(gi);
            double acc = 0.0;
#pragma unroll
            for (int r = 0; r < N; ++r) {
                if (r == pos) continue;
                const int j = el * NPE + tp_node<DIM>(N, d, line, r);
                const double aij = 0.5 * (ai + a_dot_Ja((int64_t)e0 * NPE + j));
                acc = fma(aij, fma(Dsh[pos + r * N], wi, Dsh[r + pos * N] * sw[j]), acc);
            }
            qb -= fma(Dsh[pos + pos * N] * ai, wi, 0.5 * acc);
        } else {
            double Gs = 0.0;
            if constexpr (SPLIT) {
                const double wi = sw[tid];
                double acc = 0.0;
#pragma unroll
                for (int r = 0; r < N; ++r) {
                    if (r == pos) continue;
                    const int j = el * NPE + tp_node<DIM>(N, d, line, r);
                    acc = fma(Dsh[pos + r * N], wi, fma(Dsh[r + pos * N], sw[j], acc));
                }
                Gs = fma(Dsh[pos + pos * N], wi, 0.5 * acc);
            } else {
#pragma unroll
                for (int r = 0; r < N; ++r) Gs = fma(Ds[r + pos * N], sw[el * NPE + tp_node<DIM>(N, d, line, r)], Gs);
            }
            double fp;
            if constexpr (CURV) fp = a_dot_Ja(gi);
            else fp = (EQ == FLOU_EQ_LINEAR_ADVECTION ? P.adv[d] : u) * P.Ja[e * DIM + d];
            qb = fma(-fp, Gs, qb);
        }
#pragma unroll
        for (int sd = 0; sd < 2; ++sd) {
            if (!G && pos != (sd ? N - 1 : 0)) continue;
            const int fk = 2 * d + sd;
            const int32_t pk = P.elem_face[e * 2 * DIM + fk];
            const double* src = (pk & 1) ? P.QbR : P.QbL;
            const int64_t o = trace_offset<DIM, N, CURV>(P, e, fk, line);
            if (!index_ok(o, P.nfdofs, P.status, e)) continue;
            qb = fma(G ? lv[sd * N + pos] : 1.0, __ldcg(src + o), qb);
        }
    }
    double o = fma(P.alpha, ain, qb);
    if (P.readB) o = fma(P.beta, P.B[gi], o);
    if (P.writeB) {
        double b = P.delta_B * ain;
        if (P.gamma_B != 0.0) b = fma(P.gamma_B, P.B[gi], b);
        P.B[gi] = b;
    }
    P.Aout[gi] = o;
    if (P.K) P.K[gi] = fma(P.kA, ain, P.kB * o);
    if (P.cbar && i == 0) {   // intensity (c1 + c2)/2: each side gets half, a boundary face all
        double acc = 0.0;
        for (int fk = 0; fk < 2 * DIM; ++fk) {
            const int fc = P.elem_face[e * 2 * DIM + fk] >> 1;
            if (!index_ok((int64_t)fc * NFD + NFD - 1, P.nfdofs, P.status, e)) continue;
            const double wgt = P.face_elem[2 * fc + 1] < 0 ? 1.0 : 0.5;
            for (int mm = 0; mm < NFD; ++mm) acc = fma(wgt, __ldcg(P.Ibar + (int64_t)fc * NFD + mm), acc);
        }
        P.cbar[e] += acc;
    }
}

// Scalar equations: eq FLOU_EQ_LINEAR_ADVECTION (1D-3D; general geometry in 2D and 3D) or
// FLOU_EQ_BURGERS (1D).
cudaError_t launch_adj_scalar(int dim, int eq, int n, bool split, bool gauss, bool curv, int grid, int tb,
                              const AdjFaceParams& F, const AdjElemParams& P, cudaStream_t s);

// Launchers, one translation unit each (explicit instantiations of the templates above).
// curv: the general-geometry kernels (2D and 3D); gauss: the interpolated traces and full-line
// lift of a basis without exact end-node injection (strong form).
cudaError_t launch_adj_face(int dim, int kind, bool curv, bool gauss, int grid, int tb, const AdjFaceParams& F,
                            cudaStream_t s);
cudaError_t launch_adj_elem_dim(int dim, int n, bool curv, bool gauss, const AdjElemParams& P, cudaStream_t s);
// The hybrid operator on Gauss nodes: the first element pass (before the face VJP) and the second.
cudaError_t launch_adj_hybrid_gauss(int dim, int n, int tp, bool curv, const AdjElemParams& P, cudaStream_t s);
cudaError_t launch_adj_hybrid_gauss_finish(int dim, int n, bool curv, const AdjElemParams& P, cudaStream_t s);
// gauss: the split form on a basis without boundary nodes (the entropy-projected coupling);
// hybrid: the hybrid operator on Gauss-Lobatto nodes (curv: general geometry in both)
cudaError_t launch_adj_split_dim(int dim, int n, int tp, bool curv, bool gauss, bool hybrid, const AdjElemParams& P,
                                 cudaStream_t s);

}  // namespace flou
