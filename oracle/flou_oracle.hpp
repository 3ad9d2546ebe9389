// flou_oracle.hpp -- TEST INFRASTRUCTURE ONLY.
//
// CPU restatement of Flou.jl's DGSEM residual `rhs!` and its set-up (Cartesian mesh
// connectivity with periodic stitching, Lagrange operators, Cartesian geometry), plus the
// Shu-Osher SSP-RK3 integrator and the CFL time step.  The CUDA library is compared against
// it; nothing in the product links, imports or runs it.
// Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may load it.
//
// Parity status of this oracle (pinning):
//   * Pinned against the reference's own known-answer tests that do not depend on
//     third-party integrator coefficients: the Advection1D / Advection2D period property
//     (test/tests.jl:16-88, test/runtests.jl:23-32), re-run with SSP-RK3 at the same dt.
//   * The Sod golden min/max (test/runtests.jl:35-39) needs OrdinaryDiffEq's ORK256
//     tableau, which is not in this container: not reproduced.
//   * No reference test pins a single residual value; the residual is pinned by
//     restating the reference loops line by line (file:line cited at each function) and by
//     the invariants in tests/ (freestream, conservation, entropy conservation,
//     convergence order).
//
// Every loop below keeps the reference's evaluation order (accumulation order, operand
// order) so that, compiled with -ffp-contract=off, it reproduces the reference's
// floating-point arithmetic up to library differences (log/sqrt) and the reference's
// use of Polynomials.fit for the operator matrices (built here in long double).
#pragma once

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

namespace oracle {

// ============================================================================
// Mesh: src/FlouCommon/CartesianMesh.jl + src/FlouCommon/Mesh.jl
// Indices are 1-based like the reference (0 = "no element").
// ============================================================================
struct Mesh {
    int dim = 0;
    int nx[3] = {1, 1, 1};
    double start[3] = {0, 0, 0}, finish[3] = {0, 0, 0}, dx[3] = {1, 1, 1};
    std::vector<std::array<double, 3>> nodes;
    int nvert_e = 0, nvert_f = 0, nfpe = 0;   // vertices per element/face, faces per element
    std::vector<int> e_nodeinds, e_faceinds, e_facepos;   // nelem * (nvert_e | nfpe)
    std::vector<int> f_nodeinds;                          // nfaces * nvert_f
    std::vector<int> f_eleminds, f_elempos;               // nfaces * 2
    std::vector<uint8_t> f_orient;
    std::vector<int> intfaces;
    std::vector<std::vector<int>> bdfaces;
    std::map<int, int> bdmap;                              // boundary id -> boundary index
    std::vector<std::pair<int, int>> periodic;

    int nelem() const { return (int)e_facepos.size() / nfpe; }
    int nfaces() const { return (int)f_orient.size(); }
    int& faceind(int e, int k) { return e_faceinds[(e - 1) * nfpe + (k - 1)]; }
    int& facepos(int e, int k) { return e_facepos[(e - 1) * nfpe + (k - 1)]; }
    int& elemind(int f, int s) { return f_eleminds[(f - 1) * 2 + (s - 1)]; }
    int& elempos(int f, int s) { return f_elempos[(f - 1) * 2 + (s - 1)]; }
};

// CartesianMesh ctor, src/FlouCommon/CartesianMesh.jl:38-97; element connectivity :152-236;
// face connectivity :238-500.
inline Mesh cartesian_mesh(int dim, const double* start, const double* finish, const int* n) {
    Mesh m;
    m.dim = dim;
    for (int d = 0; d < dim; ++d) {
        if (!(start[d] < finish[d])) throw std::invalid_argument("start must be < finish");
        m.nx[d] = n[d];
        m.start[d] = start[d];
        m.finish[d] = finish[d];
        m.dx[d] = (finish[d] - start[d]) / n[d];   // RT.(finish .- start) ./ nxyz
    }
    m.nvert_e = 1 << dim;
    m.nvert_f = 1 << (dim - 1);
    m.nfpe = 2 * dim;
    // Nodes: range.(start, finish, n+1) in column-major product order.
    auto rng = [&](int d, int i) {   // Julia range(a, b, length=k)[i] for i in 0..k-1
        int k = m.nx[d];
        // StepRangeLen evaluation: a + i*(b-a)/(k) computed with extended precision by
        // Julia; the coordinates only feed initial data, never the residual arithmetic.
        return start[d] + (finish[d] - start[d]) * ((double)i / (double)k);
    };
    int np[3] = {m.nx[0] + 1, dim > 1 ? m.nx[1] + 1 : 1, dim > 2 ? m.nx[2] + 1 : 1};
    for (int k = 0; k < np[2]; ++k)
        for (int j = 0; j < np[1]; ++j)
            for (int i = 0; i < np[0]; ++i)
                m.nodes.push_back({rng(0, i), dim > 1 ? rng(1, j) : 0.0, dim > 2 ? rng(2, k) : 0.0});

    if (dim == 1) {
        int nx = m.nx[0];
        for (int ie = 1; ie <= nx; ++ie) {
            m.e_nodeinds.insert(m.e_nodeinds.end(), {ie, ie + 1});
            m.e_faceinds.insert(m.e_faceinds.end(), {ie, ie + 1});
            m.e_facepos.insert(m.e_facepos.end(), {ie == 1 ? 1 : 2, 1});
        }
        int nf = nx + 1;
        m.bdfaces.assign(2, {});
        for (int f = 1; f <= nf; ++f) {
            if (f == 1) {
                m.bdfaces[0].push_back(f);
                m.f_eleminds.insert(m.f_eleminds.end(), {1, 0});
                m.f_elempos.insert(m.f_elempos.end(), {1, 0});
            } else if (f == nf) {
                m.bdfaces[1].push_back(f);
                m.f_eleminds.insert(m.f_eleminds.end(), {nx, 0});
                m.f_elempos.insert(m.f_elempos.end(), {2, 0});
            } else {
                m.intfaces.push_back(f);
                m.f_eleminds.insert(m.f_eleminds.end(), {f - 1, f});
                m.f_elempos.insert(m.f_elempos.end(), {2, 1});
            }
            m.f_nodeinds.push_back(f);
            m.f_orient.push_back(0);
        }
    } else if (dim == 2) {
        int nx = m.nx[0], ny = m.nx[1], npx = nx + 1, npy = ny + 1;
        for (int j = 1; j <= ny; ++j)
            for (int i = 1; i <= nx; ++i) {
                m.e_nodeinds.insert(m.e_nodeinds.end(),
                                    {(j - 1) * npx + i, (j - 1) * npx + i + 1,
                                     (j - 1) * npx + i + 1 + npx, (j - 1) * npx + i + npx});
                m.e_faceinds.insert(m.e_faceinds.end(),
                                    {(j - 1) * npx + i, (j - 1) * npx + i + 1,
                                     npx * ny + (j - 1) * nx + i, npx * ny + (j - 1) * nx + i + nx});
                m.e_facepos.insert(m.e_facepos.end(), {i == 1 ? 1 : 2, 1, j == 1 ? 1 : 2, 1});
            }
        int nf = npx * ny + npy * nx;
        m.f_eleminds.assign(2 * nf, 0);
        m.f_elempos.assign(2 * nf, 0);
        m.f_nodeinds.assign(2 * nf, 0);
        m.f_orient.assign(nf, 0);
        m.bdfaces.assign(4, {});
        auto setf = [&](int f, int e1, int e2, int p1, int p2, int n1, int n2) {
            m.elemind(f, 1) = e1; m.elemind(f, 2) = e2;
            m.elempos(f, 1) = p1; m.elempos(f, 2) = p2;
            m.f_nodeinds[(f - 1) * 2] = n1; m.f_nodeinds[(f - 1) * 2 + 1] = n2;
        };
        for (int j = 1; j <= ny; ++j)
            for (int i = 1; i <= npx; ++i) {   // vertical faces
                int f = (j - 1) * npx + i;
                int n1 = (j - 1) * npx + i, n2 = (j - 1) * npx + i + npx;
                if (i == 1) { m.bdfaces[0].push_back(f); setf(f, (j - 1) * nx + 1, 0, 1, 0, n1, n2); }
                else if (i == npx) { m.bdfaces[1].push_back(f); setf(f, (j - 1) * nx + nx, 0, 2, 0, n1, n2); }
                else { m.intfaces.push_back(f); setf(f, (j - 1) * nx + i - 1, (j - 1) * nx + i, 2, 1, n1, n2); }
            }
        for (int j = 1; j <= npy; ++j)
            for (int i = 1; i <= nx; ++i) {    // horizontal faces
                int f = npx * ny + (j - 1) * nx + i;
                int n1 = (j - 1) * npx + i, n2 = (j - 1) * npx + i + 1;
                if (j == 1) { m.bdfaces[2].push_back(f); setf(f, i, 0, 3, 0, n1, n2); }
                else if (j == npy) { m.bdfaces[3].push_back(f); setf(f, (ny - 1) * nx + i, 0, 4, 0, n1, n2); }
                else { m.intfaces.push_back(f); setf(f, (j - 2) * nx + i, (j - 2) * nx + i + nx, 4, 3, n1, n2); }
            }
    } else {
        int nx = m.nx[0], ny = m.nx[1], nz = m.nx[2];
        int npx = nx + 1, npy = ny + 1, npz = nz + 1;
        for (int k = 1; k <= nz; ++k)
            for (int j = 1; j <= ny; ++j)
                for (int i = 1; i <= nx; ++i) {
                    int b = (k - 1) * npx * npy + (j - 1) * npx + i;
                    m.e_nodeinds.insert(m.e_nodeinds.end(),
                                        {b, b + 1, b + 1 + npx, b + npx, npx * npy + b, npx * npy + b + 1,
                                         npx * npy + b + 1 + npx, npx * npy + b + npx});
                    m.e_faceinds.insert(
                        m.e_faceinds.end(),
                        {(k - 1) * npx * ny + (j - 1) * npx + i, (k - 1) * npx * ny + (j - 1) * npx + i + 1,
                         npx * ny * nz + (k - 1) * nx * npy + (j - 1) * nx + i,
                         npx * ny * nz + (k - 1) * nx * npy + (j - 1) * nx + i + nx,
                         npx * ny * nz + nx * npy * nz + (k - 1) * nx * ny + (j - 1) * nx + i,
                         npx * ny * nz + nx * npy * nz + (k - 1) * nx * ny + (j - 1) * nx + i + nx * ny});
                    m.e_facepos.insert(m.e_facepos.end(),
                                       {i == 1 ? 1 : 2, 1, j == 1 ? 1 : 2, 1, k == 1 ? 1 : 2, 1});
                }
        int nf = npx * ny * nz + npy * nx * nz + npz * nx * ny;
        m.f_eleminds.assign(2 * nf, 0);
        m.f_elempos.assign(2 * nf, 0);
        m.f_nodeinds.assign(4 * nf, 0);
        m.f_orient.assign(nf, 0);
        m.bdfaces.assign(6, {});
        auto setf = [&](int f, int e1, int e2, int p1, int p2, std::array<int, 4> nn) {
            m.elemind(f, 1) = e1; m.elemind(f, 2) = e2;
            m.elempos(f, 1) = p1; m.elempos(f, 2) = p2;
            for (int q = 0; q < 4; ++q) m.f_nodeinds[(f - 1) * 4 + q] = nn[q];
        };
        for (int k = 1; k <= nz; ++k)
            for (int j = 1; j <= ny; ++j)
                for (int i = 1; i <= npx; ++i) {   // X faces
                    int f = (k - 1) * npx * ny + (j - 1) * npx + i;
                    int b = (k - 1) * npx * npy + (j - 1) * npx + i;
                    std::array<int, 4> nn = {b, b + npx, npx * npy + b + npx, npx * npy + b};
                    int eb = (k - 1) * nx * ny + (j - 1) * nx;
                    if (i == 1) { m.bdfaces[0].push_back(f); setf(f, eb + 1, 0, 1, 0, nn); }
                    else if (i == npx) { m.bdfaces[1].push_back(f); setf(f, eb + nx, 0, 2, 0, nn); }
                    else { m.intfaces.push_back(f); setf(f, eb + i - 1, eb + i, 2, 1, nn); }
                }
        for (int k = 1; k <= nz; ++k)
            for (int j = 1; j <= npy; ++j)
                for (int i = 1; i <= nx; ++i) {    // Y faces
                    int f = npx * ny * nz + (k - 1) * nx * npy + (j - 1) * nx + i;
                    int b = (k - 1) * npx * npy + (j - 1) * npx + i;
                    std::array<int, 4> nn = {b, b + 1, npx * npy + b + 1, npx * npy + b};
                    if (j == 1) { m.bdfaces[2].push_back(f); setf(f, (k - 1) * nx * ny + i, 0, 3, 0, nn); }
                    else if (j == npy) {
                        m.bdfaces[3].push_back(f);
                        setf(f, (k - 1) * nx * ny + (ny - 1) * nx + i, 0, 4, 0, nn);
                    } else {
                        m.intfaces.push_back(f);
                        setf(f, (k - 1) * nx * ny + (j - 2) * nx + i, (k - 1) * nx * ny + (j - 2) * nx + i + nx, 4, 3, nn);
                    }
                }
        for (int k = 1; k <= npz; ++k)
            for (int j = 1; j <= ny; ++j)
                for (int i = 1; i <= nx; ++i) {    // Z faces
                    int f = npx * ny * nz + npy * nx * nz + (k - 1) * nx * ny + (j - 1) * nx + i;
                    int b = (k - 1) * npx * npy + (j - 1) * npx + i;
                    std::array<int, 4> nn = {b, b + 1, npx + b + 1, npx + b};
                    if (k == 1) { m.bdfaces[4].push_back(f); setf(f, (j - 1) * nx + i, 0, 5, 0, nn); }
                    else if (k == npz) { m.bdfaces[5].push_back(f); setf(f, (nz - 1) * nx * ny + (j - 1) * nx + i, 0, 6, 0, nn); }
                    else {
                        m.intfaces.push_back(f);
                        setf(f, (k - 2) * nx * ny + (j - 1) * nx + i, (k - 2) * nx * ny + (j - 1) * nx + i + nx * ny, 6, 5, nn);
                    }
                }
    }
    for (int b = 1; b <= 2 * dim; ++b) m.bdmap[b] = b;
    return m;
}

// apply_periodicBCs! (CartesianMesh.jl:127-150) -> _apply_periodicBCs! (Mesh.jl:236-322).
// `pairs` holds boundary ids (bd1, bd2) with bd1 odd and bd2 = bd1 + 1.  The reference
// iterates a Dict; the result does not depend on the iteration order (faces are sorted
// and renumbered at the end), so ascending bd1 is used.
inline void apply_periodic(Mesh& m, std::vector<std::pair<int, int>> pairs) {
    for (auto& p : pairs) {
        int nb = (int)m.bdfaces.size();
        if (!(1 <= p.first && p.first <= nb && 1 <= p.second && p.second <= nb))
            throw std::invalid_argument("boundary ids out of range");
        if (!(p.second % 2 == 0 && p.first + 1 == p.second))
            throw std::invalid_argument("boundaries cannot be made periodic");
    }
    std::sort(pairs.begin(), pairs.end());
    std::vector<int> faces2del;
    for (auto& p : pairs) {
        int bd1 = p.first, bd2 = p.second;
        if (!m.bdmap.count(bd1) || !m.bdmap.count(bd2))
            throw std::invalid_argument("boundaries cannot be periodic");
        int b1 = m.bdmap[bd1], b2 = m.bdmap[bd2];
        const auto& l1 = m.bdfaces[b1 - 1];
        const auto& l2 = m.bdfaces[b2 - 1];
        for (size_t q = 0; q < std::min(l1.size(), l2.size()); ++q) {   // Mesh.jl:249-259
            int if1 = l1[q], if2 = l2[q];
            int elmind = m.elemind(if2, 1), elmpos = m.elempos(if2, 1);
            m.elemind(if1, 2) = elmind;
            m.elempos(if1, 2) = elmpos;
            m.faceind(elmind, elmpos) = if1;
            m.facepos(elmind, elmpos) = 2;
        }
        m.intfaces.insert(m.intfaces.end(), l1.begin(), l1.end());    // :262
        faces2del.insert(faces2del.end(), l2.begin(), l2.end());      // :263
        m.bdfaces.erase(m.bdfaces.begin() + (b2 - 1));                // :264 (deleteat! b1=>b2)
        m.bdfaces.erase(m.bdfaces.begin() + (b1 - 1));
        m.bdmap.erase(bd1);                                            // :267-276
        m.bdmap.erase(bd2);
        for (auto& kv : m.bdmap) {
            if (kv.second > b2) kv.second -= 1;
            if (kv.second > b1) kv.second -= 1;
        }
        m.periodic.push_back({bd1, bd2});
    }
    std::sort(m.intfaces.begin(), m.intfaces.end());                 // :281-302
    std::sort(faces2del.begin(), faces2del.end());
    auto shift = [&](int x) {
        auto it = std::upper_bound(faces2del.begin(), faces2del.end(), x);   // findfirst(>(x))
        int delta = (it == faces2del.end()) ? (int)faces2del.size() : (int)(it - faces2del.begin());
        return x - delta;
    };
    for (auto& f : m.intfaces) f = shift(f);
    for (auto& l : m.bdfaces)
        for (auto& f : l) f = shift(f);
    // deleteat!(mesh.faces, faces2del), Mesh.jl:152-185: drop each deleted face.
    for (size_t ipos = 0; ipos < faces2del.size(); ++ipos) {
        int f = faces2del[ipos] - (int)ipos;   // i[ipos] - (ipos - 1) with 1-based ipos
        m.f_nodeinds.erase(m.f_nodeinds.begin() + (f - 1) * m.nvert_f, m.f_nodeinds.begin() + f * m.nvert_f);
        m.f_eleminds.erase(m.f_eleminds.begin() + (f - 1) * 2, m.f_eleminds.begin() + f * 2);
        m.f_elempos.erase(m.f_elempos.begin() + (f - 1) * 2, m.f_elempos.begin() + f * 2);
        m.f_orient.erase(m.f_orient.begin() + (f - 1));
    }
    for (int f = 1; f <= m.nfaces(); ++f) {                          // :308-320
        m.faceind(m.elemind(f, 1), m.elempos(f, 1)) = f;
        if (m.elemind(f, 2) != 0) m.faceind(m.elemind(f, 2), m.elempos(f, 2)) = f;
    }
}

// ============================================================================
// Standard-region operators: ApproximationBases.jl:68-91,135-186; Reconstruction.jl:125-134;
// StdSegment.jl:51-89.  Built in long double through the monomial (Vandermonde) form the
// reference uses (Polynomials.fit, derivative, integrate).
// ============================================================================
typedef long double LD;

inline LD legendre(int n, LD x, LD* dp) {
    LD p0 = 1, p1 = x, dp0 = 0, dp1 = 1;
    if (n == 0) { if (dp) *dp = 0; return 1; }
    for (int k = 2; k <= n; ++k) {
        LD p2 = ((2 * k - 1) * x * p1 - (k - 1) * p0) / k;
        LD dp2 = dp0 + (2 * k - 1) * p1;
        p0 = p1; p1 = p2; dp0 = dp1; dp1 = dp2;
    }
    if (dp) *dp = dp1;
    return p1;
}

// Gauss-Lobatto (gausslobatto) and Gauss-Legendre (gausslegendre) nodes, ascending.
inline std::vector<LD> nodes_lobatto(int n) {
    std::vector<LD> x(n);
    const LD pi = 3.141592653589793238462643383279502884L;
    if (n == 1) { x[0] = 0; return x; }
    x[0] = -1; x[n - 1] = 1;
    for (int i = 1; i < n - 1; ++i) {
        // roots of P'_{n-1}; Chebyshev-Gauss-Lobatto initial guess, Newton on P'_{n-1}.
        LD z = -std::cos(pi * i / (n - 1));
        for (int it = 0; it < 100; ++it) {
            // f = P'_{n-1}(z); f' = P''_{n-1} = (2 z P' - m(m+1) P) / (1 - z^2)
            LD dp, p = legendre(n - 1, z, &dp);
            LD m = n - 1;
            LD d2p = (2 * z * dp - m * (m + 1) * p) / (1 - z * z);
            LD dz = dp / d2p;
            z -= dz;
            if (std::fabs(dz) < 1e-30L) break;
        }
        x[i] = z;
    }
    std::sort(x.begin(), x.end());
    return x;
}

inline std::vector<LD> nodes_legendre(int n) {
    std::vector<LD> x(n);
    const LD pi = 3.141592653589793238462643383279502884L;
    for (int i = 0; i < n; ++i) {
        LD z = -std::cos(pi * (i + 0.75L) / (n + 0.5L));
        for (int it = 0; it < 100; ++it) {
            LD dp, p = legendre(n, z, &dp);
            LD dz = p / dp;
            z -= dz;
            if (std::fabs(dz) < 1e-30L) break;
        }
        x[i] = z;
    }
    std::sort(x.begin(), x.end());
    return x;
}

struct StdOps {
    int n = 0;
    bool lobatto = true;
    std::vector<double> xi, omega, D, Ds, Dsharp, ll, lr, dgl, dgr;   // matrices column-major n x n
};

// Lagrange basis in monomial coefficients: C[k + j*n] = coefficient of x^k in l_j
// (Polynomials.fit(ξ, e_j), ApproximationBases.jl:154-165), via Gaussian elimination with
// partial pivoting on the Vandermonde system.
inline std::vector<LD> monomial_basis(const std::vector<LD>& xi) {
    int n = (int)xi.size();
    std::vector<LD> C(n * n, 0);
    for (int j = 0; j < n; ++j) {
        std::vector<LD> A(n * n), b(n, 0);
        for (int r = 0; r < n; ++r) {
            LD p = 1;
            for (int c = 0; c < n; ++c) { A[r * n + c] = p; p *= xi[r]; }
        }
        b[j] = 1;
        for (int c = 0; c < n; ++c) {
            int piv = c;
            for (int r = c + 1; r < n; ++r)
                if (std::fabs(A[r * n + c]) > std::fabs(A[piv * n + c])) piv = r;
            if (piv != c) {
                for (int q = 0; q < n; ++q) std::swap(A[c * n + q], A[piv * n + q]);
                std::swap(b[c], b[piv]);
            }
            for (int r = c + 1; r < n; ++r) {
                LD f = A[r * n + c] / A[c * n + c];
                for (int q = c; q < n; ++q) A[r * n + q] -= f * A[c * n + q];
                b[r] -= f * b[c];
            }
        }
        for (int r = n - 1; r >= 0; --r) {
            LD s = b[r];
            for (int q = r + 1; q < n; ++q) s -= A[r * n + q] * C[q + j * n];
            C[r + j * n] = s / A[r * n + r];
        }
    }
    return C;
}

inline StdOps std_operators(int n, bool lobatto) {
    StdOps s;
    s.n = n;
    s.lobatto = lobatto;
    std::vector<LD> xi = lobatto ? nodes_lobatto(n) : nodes_legendre(n);
    std::vector<LD> C = monomial_basis(xi);
    auto eval = [&](int j, LD x) { LD v = 0, p = 1; for (int k = 0; k < n; ++k) { v += C[k + j * n] * p; p *= x; } return v; };
    auto deval = [&](int j, LD x) { LD v = 0, p = 1; for (int k = 1; k < n; ++k) { v += k * C[k + j * n] * p; p *= x; } return v; };
    std::vector<LD> w(n), Dl(n * n), L(n), R(n);
    for (int j = 0; j < n; ++j) {                 // _weights_from_basis, :179-186
        // int(1) - int(-1) of sum_k c_k x^k = sum over even k of 2 c_k / (k + 1)
        LD v = 0;
        for (int k = 0; k < n; k += 2) v += 2 * C[k + j * n] / (k + 1);
        w[j] = v;
    }
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) Dl[i + j * n] = deval(j, xi[i]);   // derivative_matrix, :89-91
    for (int j = 0; j < n; ++j) { L[j] = eval(j, -1); R[j] = eval(j, 1); }   // interp_matrix at -1, +1
    // DGSEMrec (Reconstruction.jl:125-134) gives (-l_l/ω, +l_r/ω); StdSegment.jl:85 flips the
    // first sign: ∂g = (l_l/ω, l_r/ω).  B = ∂g_r l_rᵀ - ∂g_l l_lᵀ; Ds = D - B; D♯ = 2D - B.
    s.xi.resize(n); s.omega.resize(n); s.ll.resize(n); s.lr.resize(n); s.dgl.resize(n); s.dgr.resize(n);
    s.D.resize(n * n); s.Ds.resize(n * n); s.Dsharp.resize(n * n);
    for (int j = 0; j < n; ++j) {
        s.xi[j] = (double)xi[j];
        s.omega[j] = (double)w[j];
        s.ll[j] = (double)L[j];
        s.lr[j] = (double)R[j];
        s.dgl[j] = (double)(L[j] / w[j]);
        s.dgr[j] = (double)(R[j] / w[j]);
    }
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) {
            LD B = (R[i] / w[i]) * R[j] - (L[i] / w[i]) * L[j];
            s.D[i + j * n] = (double)Dl[i + j * n];
            s.Ds[i + j * n] = (double)(Dl[i + j * n] - B);
            s.Dsharp[i + j * n] = (double)(2 * Dl[i + j * n] - B);
        }
    return s;
}

// ============================================================================
// Equations and fluxes
// ============================================================================
enum EqKind { EQ_ADVECTION = 0, EQ_BURGERS = 1, EQ_EULER = 2 };
enum VolOp { OP_STRONG = 0, OP_SPLIT = 1, OP_HYBRID = 2 };
enum TwoPoint { TP_STDAVG = 0, TP_CHANDRASHEKAR = 1, TP_KENNEDY_GRUBER = 2 };
enum NumFlux {
    NF_STDAVG = 0, NF_LXF = 1, NF_CHANDRASHEKAR = 2, NF_HLL = 3, NF_HLLC = 4,
    NF_SCALAR_DISSIPATION = 5, NF_MATRIX_DISSIPATION = 6
};
enum BcKind { BC_NONE = 0, BC_OUTFLOW = 1, BC_INFLOW = 2, BC_SLIP = 3, BC_STATE_FIELD = 4 };

struct Config {
    int dim = 2, nv = 4, eq = EQ_EULER;
    double gamma = 1.4;
    double a[3] = {0, 0, 0};
    int volop = OP_STRONG, tpflux = TP_STDAVG, numflux = NF_LXF, lxf_avg = NF_STDAVG;
    double intensity = 1.0;
    // HybridDivOperator (OpDivergence.jl:439-472): subcell FV flux and blending constant
    int fvflux = NF_LXF, fvavg = NF_STDAVG;
    double fvintensity = 1.0, blend = 0.0;
};

template <class T> using Vec = std::array<T, 5>;

template <class T> inline T sq(const T& x) { return x * x; }

// logarithmic_mean, src/FlouCommon/Utilities.jl:34-44
template <class T> inline T logarithmic_mean(const T& al, const T& ar) {
    using std::log;
    T xi = al / ar;
    T f = (xi - 1.0) / (xi + 1.0);
    T u = f * f;
    T F;
    if (u < 0.01) F = ((1.0 + u / 3.0) + (u * u) / 5.0) + (u * u * u) / 7.0;
    else F = log(xi) / (2.0 * f);
    return (al + ar) / (2.0 * F);
}

// pressure, src/FlouCommon/Euler.jl:142-155:  (γ-1)(ρe - |ρv|²/2ρ)
template <class T> inline T pressure(const Vec<T>& Q, int dim, double g) {
    T k;
    if (dim == 1) k = sq(Q[1]) / (2.0 * Q[0]);
    else if (dim == 2) k = (sq(Q[1]) + sq(Q[2])) / (2.0 * Q[0]);
    else k = (sq(Q[1]) + sq(Q[2]) + sq(Q[3])) / (2.0 * Q[0]);
    return (g - 1.0) * (Q[dim + 1] - k);
}

// vars_cons2prim, Euler.jl:237-253: (ρ, u[, v, w], p)
template <class T> inline Vec<T> cons2prim(const Vec<T>& Q, int dim, double g) {
    Vec<T> P{};
    P[0] = Q[0];
    for (int d = 0; d < dim; ++d) P[1 + d] = Q[1 + d] / Q[0];
    P[dim + 1] = pressure(Q, dim, g);
    return P;
}

template <class T> inline T soundvelocity(const T& rho, const T& p, double g) {
    using std::sqrt;
    return sqrt(g * p / rho);   // soundvelocity_sqr = γ p / ρ, Euler.jl:225-235
}

// volumeflux, Euler.jl:54-114 (physical flux in direction d), LinearAdvection.jl:42-44,
// Burgers.jl:31-33.
template <class T> inline Vec<T> volumeflux(const Vec<T>& Q, int d, const Config& c) {
    Vec<T> F{};
    if (c.eq == EQ_ADVECTION) { F[0] = c.a[d] * Q[0]; return F; }
    if (c.eq == EQ_BURGERS) { F[0] = sq(Q[0]) / 2.0; return F; }
    int dim = c.dim;
    T vel[3];
    for (int k = 0; k < dim; ++k) vel[k] = Q[1 + k] / Q[0];
    T p = pressure(Q, dim, c.gamma);
    F[0] = Q[1 + d];
    for (int k = 0; k < dim; ++k) {
        F[1 + k] = Q[1 + d] * vel[k];
        if (k == d) F[1 + k] = F[1 + k] + p;
    }
    F[dim + 1] = (Q[dim + 1] + p) * vel[d];
    return F;
}

// Per-node reference frame (PhysicalRegions.jl:19-23) with normal n, tangents t, b.
struct Frame { double n[3], t[3], b[3]; };

// rotate2face / rotate2phys, src/FlouSpatial/Equations/Euler.jl:16-64
template <class T> inline Vec<T> rotate2face(const Vec<T>& Q, const Frame& fr, const Config& c) {
    if (c.eq != EQ_EULER) return Q;
    Vec<T> R = Q;
    if (c.dim == 1) { R[1] = Q[1] * fr.n[0]; }
    else if (c.dim == 2) {
        R[1] = Q[1] * fr.n[0] + Q[2] * fr.n[1];
        R[2] = Q[1] * fr.t[0] + Q[2] * fr.t[1];
    } else {
        R[1] = Q[1] * fr.n[0] + Q[2] * fr.n[1] + Q[3] * fr.n[2];
        R[2] = Q[1] * fr.t[0] + Q[2] * fr.t[1] + Q[3] * fr.t[2];
        R[3] = Q[1] * fr.b[0] + Q[2] * fr.b[1] + Q[3] * fr.b[2];
    }
    return R;
}

template <class T> inline Vec<T> rotate2phys(const Vec<T>& Q, const Frame& fr, const Config& c) {
    if (c.eq != EQ_EULER) return Q;
    Vec<T> R = Q;
    if (c.dim == 1) { R[1] = Q[1] * fr.n[0]; }
    else if (c.dim == 2) {
        R[1] = Q[1] * fr.n[0] + Q[2] * fr.t[0];
        R[2] = Q[1] * fr.n[1] + Q[2] * fr.t[1];
    } else {
        R[1] = Q[1] * fr.n[0] + Q[2] * fr.t[0] + Q[3] * fr.b[0];
        R[2] = Q[1] * fr.n[1] + Q[2] * fr.t[1] + Q[3] * fr.b[1];
        R[3] = Q[1] * fr.n[2] + Q[2] * fr.t[2] + Q[3] * fr.b[2];
    }
    return R;
}

// Euler StdAverage numerical flux (face frame), Euler.jl:99-136
template <class T> inline Vec<T> euler_stdavg(const Vec<T>& Ql, const Vec<T>& Qr, int dim, double g) {
    Vec<T> Pl = cons2prim(Ql, dim, g), Pr = cons2prim(Qr, dim, g);
    T ul = Pl[1], ur = Pr[1], pl = Pl[dim + 1], pr = Pr[dim + 1];
    Vec<T> F{};
    F[0] = (Ql[1] + Qr[1]) / 2.0;
    F[1] = (((Ql[1] * ul + pl) + Qr[1] * ur) + pr) / 2.0;
    for (int k = 1; k < dim; ++k) F[1 + k] = (Ql[1 + k] * ul + Qr[1 + k] * ur) / 2.0;
    F[dim + 1] = ((Ql[dim + 1] + pl) * ul + (Qr[dim + 1] + pr) * ur) / 2.0;
    return F;
}

// Euler Chandrashekar numerical flux (face frame), Euler.jl:167-226.  The 3D branch
// reproduces the reference's `+ wl^2` in place of `wr^2` (Euler.jl:216).
template <class T> inline Vec<T> euler_chandrashekar(const Vec<T>& Ql, const Vec<T>& Qr, int dim, double g) {
    Vec<T> Pl = cons2prim(Ql, dim, g), Pr = cons2prim(Qr, dim, g);
    T rl = Pl[0], rr = Pr[0], pl = Pl[dim + 1], pr = Pr[dim + 1];
    T u = (Pl[1] + Pr[1]) / 2.0;
    T v = dim > 1 ? (Pl[2] + Pr[2]) / 2.0 : T(0.0);
    T w = dim > 2 ? (Pl[3] + Pr[3]) / 2.0 : T(0.0);
    T bl = rl / (2.0 * pl), br = rr / (2.0 * pr);
    T rho = logarithmic_mean(rl, rr);
    T p = (rl + rr) / (2.0 * (bl + br));
    T beta = logarithmic_mean(bl, br);
    Vec<T> F{};
    T h;
    if (dim == 1) {
        h = ((1.0 / ((2.0 * beta) * (g - 1.0)) - (sq(Pl[1]) + sq(Pr[1])) / 4.0) + p / rho) + sq(u);
        F[0] = rho * u; F[1] = rho * sq(u) + p; F[2] = rho * u * h;
    } else if (dim == 2) {
        h = (((1.0 / ((2.0 * beta) * (g - 1.0)) - (((sq(Pl[1]) + sq(Pl[2])) + sq(Pr[1])) + sq(Pr[2])) / 4.0) + p / rho) + sq(u)) + sq(v);
        F[0] = rho * u; F[1] = rho * sq(u) + p; F[2] = rho * u * v; F[3] = rho * u * h;
    } else {
        T s = ((((sq(Pl[1]) + sq(Pl[2])) + sq(Pl[3])) + sq(Pr[1])) + sq(Pr[2])) + sq(Pl[3]);
        h = ((((1.0 / ((2.0 * beta) * (g - 1.0)) - s / 4.0) + p / rho) + sq(u)) + sq(v)) + sq(w);
        F[0] = rho * u; F[1] = rho * sq(u) + p; F[2] = rho * u * v; F[3] = rho * u * w; F[4] = rho * u * h;
    }
    return F;
}

// Wave-speed estimates for HLL/HLLC (no counterpart in Flou): Davis estimates
// S_L = min(u_L - a_L, u_R - a_R), S_R = max(u_L + a_L, u_R + a_R) (Toro, ch. 10.5).
template <class T> inline Vec<T> euler_face_physflux(const Vec<T>& Q, const Vec<T>& P, int dim) {
    // physical flux along the face normal in the face frame (momentum index 1 is normal)
    Vec<T> F{};
    T un = P[1], p = P[dim + 1];
    F[0] = Q[1];
    F[1] = Q[1] * un + p;
    for (int k = 1; k < dim; ++k) F[1 + k] = Q[1 + k] * un;
    F[dim + 1] = (Q[dim + 1] + p) * un;
    return F;
}

// HLL (Harten, Lax, van Leer 1983; Toro eq. 10.21) in the face frame.
template <class T> inline Vec<T> euler_hll(const Vec<T>& Ql, const Vec<T>& Qr, int dim, double g) {
    using std::min; using std::max;
    Vec<T> Pl = cons2prim(Ql, dim, g), Pr = cons2prim(Qr, dim, g);
    T al = soundvelocity(Pl[0], Pl[dim + 1], g), ar = soundvelocity(Pr[0], Pr[dim + 1], g);
    T sl = min(Pl[1] - al, Pr[1] - ar), sr = max(Pl[1] + al, Pr[1] + ar);
    Vec<T> Fl = euler_face_physflux(Ql, Pl, dim), Fr = euler_face_physflux(Qr, Pr, dim);
    Vec<T> F{};
    int nv = dim + 2;
    if (sl >= 0.0) return Fl;
    if (sr <= 0.0) return Fr;
    for (int k = 0; k < nv; ++k) F[k] = ((sr * Fl[k] - sl * Fr[k]) + (sl * sr) * (Qr[k] - Ql[k])) / (sr - sl);
    return F;
}

// HLLC (Toro, Spruce, Speares 1994; Toro eqs. 10.37-10.39) in the face frame.
template <class T> inline Vec<T> euler_hllc(const Vec<T>& Ql, const Vec<T>& Qr, int dim, double g) {
    using std::min; using std::max;
    Vec<T> Pl = cons2prim(Ql, dim, g), Pr = cons2prim(Qr, dim, g);
    T rl = Pl[0], rr = Pr[0], ul = Pl[1], ur = Pr[1], pl = Pl[dim + 1], pr = Pr[dim + 1];
    T al = soundvelocity(rl, pl, g), ar = soundvelocity(rr, pr, g);
    T sl = min(ul - al, ur - ar), sr = max(ul + al, ur + ar);
    Vec<T> Fl = euler_face_physflux(Ql, Pl, dim), Fr = euler_face_physflux(Qr, Pr, dim);
    if (sl >= 0.0) return Fl;
    if (sr <= 0.0) return Fr;
    T ml = rl * (sl - ul), mr = rr * (sr - ur);
    T ss = ((pr - pl) + ul * ml - ur * mr) / (ml - mr);
    int nv = dim + 2;
    const Vec<T>& Qk = (ss >= 0.0) ? Ql : Qr;
    const Vec<T>& Pk = (ss >= 0.0) ? Pl : Pr;
    const Vec<T>& Fk = (ss >= 0.0) ? Fl : Fr;
    T sk = (ss >= 0.0) ? sl : sr;
    T mk = (ss >= 0.0) ? ml : mr;
    T coef = mk / (sk - ss);   // ρ_K (S_K - u_K)/(S_K - S*)
    Vec<T> Us{};
    Us[0] = coef;
    Us[1] = coef * ss;
    for (int k = 1; k < dim; ++k) Us[1 + k] = coef * Pk[1 + k];
    Us[dim + 1] = coef * (Qk[dim + 1] / Pk[0] + (ss - Pk[1]) * (ss + Pk[dim + 1] / mk));
    Vec<T> F{};
    for (int k = 0; k < nv; ++k) F[k] = Fk[k] + sk * (Us[k] - Qk[k]);
    return F;
}

// Entropy variables, src/FlouCommon/Euler.jl:273-307 (s = log(p) - γ log(ρ), :202-206).
template <class T> inline Vec<T> cons2entropy(const Vec<T>& Q, int dim, double g) {
    using std::log;
    T rho = Q[0];
    T p = pressure(Q, dim, g);
    T s = log(p) - g * log(rho);
    T m2 = sq(Q[1]);
    for (int k = 1; k < dim; ++k) m2 = m2 + sq(Q[1 + k]);
    Vec<T> W{};
    W[0] = (g - s) / (g - 1.0) - m2 / rho / (2.0 * p);
    for (int k = 0; k < dim; ++k) W[1 + k] = Q[1 + k] / p;
    W[dim + 1] = -rho / p;
    return W;
}

// vars_entropy2cons = vars_prim2cons ∘ vars_entropy2prim, src/FlouCommon/Euler.jl:309-339.
template <class T> inline Vec<T> entropy2cons(const Vec<T>& W, int dim, double g) {
    using std::exp; using std::pow;
    T wl = W[dim + 1];
    T u[3], u2 = T(0.0);
    for (int k = 0; k < dim; ++k) {
        u[k] = -W[1 + k] / wl;
        u2 = u2 + sq(u[k]);
    }
    T s = g - (g - 1.0) * (W[0] - wl * u2 / 2.0);
    T p = pow(pow(-wl, g) * exp(s), 1.0 / (1.0 - g));
    T rho = -p * wl;
    Vec<T> Q{};
    Q[0] = rho;
    for (int k = 0; k < dim; ++k) Q[1 + k] = rho * u[k];
    Q[dim + 1] = p / (g - 1.0) + rho * u2 / 2.0;
    return Q;
}

template <class T> inline Vec<T> euler_average(const Vec<T>& Ql, const Vec<T>& Qr, int dim, double g, int avg) {
    return avg == NF_CHANDRASHEKAR ? euler_chandrashekar(Ql, Qr, dim, g) : euler_stdavg(Ql, Qr, dim, g);
}

// ScalarDissipation, src/FlouSpatial/Equations/Euler.jl:228-301.  The 3D branch reads the left
// momenta from Qr (Euler.jl:257), so its momentum jumps vanish; kept as written.
template <class T>
inline Vec<T> euler_scalar_dissipation(const Vec<T>& Ql, const Vec<T>& Qr, int dim, double g, int avg,
                                       const T& intensity) {
    using std::fabs; using std::max;
    Vec<T> Pl = cons2prim(Ql, dim, g), Pr = cons2prim(Qr, dim, g);
    T rl = Pl[0], rr = Pr[0], pl = Pl[dim + 1], pr = Pr[dim + 1];
    T ml[3], mr[3], vm[3];
    for (int k = 0; k < dim; ++k) {
        mr[k] = Qr[1 + k];
        ml[k] = (dim == 3) ? Qr[1 + k] : Ql[1 + k];
        vm[k] = (Pl[1 + k] + Pr[1 + k]) / 2.0;
    }
    T rho = (rl + rr) / 2.0;
    T bl = rl / (2.0 * pl), br = rr / (2.0 * pr);
    T beta = logarithmic_mean(bl, br);
    T al = soundvelocity(rl, pl, g), ar = soundvelocity(rr, pr, g);
    Vec<T> Fn = euler_average(Ql, Qr, dim, g, avg);
    T lam = max(fabs(Pl[1]) + al, fabs(Pr[1]) + ar);
    Vec<T> D{};
    D[0] = rr - rl;
    for (int k = 0; k < dim; ++k) D[1 + k] = mr[k] - ml[k];
    T c1 = 1.0 / beta / (g - 1.0);
    for (int k = 0; k < dim; ++k) c1 = c1 + Pl[1 + k] * Pr[1 + k];
    T c2 = vm[0] * (Pr[1] - Pl[1]);
    for (int k = 1; k < dim; ++k) c2 = c2 + vm[k] * (Pr[1 + k] - Pl[1 + k]);
    c2 = c2 + (1.0 / br - 1.0 / bl) / (2.0 * (g - 1.0));
    D[dim + 1] = c1 * (rr - rl) / 2.0 + rho * c2;
    Vec<T> F{};
    for (int k = 0; k < dim + 2; ++k) F[k] = Fn[k] - lam / 2.0 * D[k] * intensity;
    return F;
}

// MatrixDissipation, src/FlouSpatial/Equations/Euler.jl:303-380:
// F = Fn + R Λ T Rᵀ (W_l - W_r)/2 · intensity, the matrix product formed first as written.
template <class T>
inline Vec<T> euler_matrix_dissipation(const Vec<T>& Ql, const Vec<T>& Qr, int dim, double g, int avg,
                                       const T& intensity) {
    using std::fabs;
    Vec<T> Pl = cons2prim(Ql, dim, g), Pr = cons2prim(Qr, dim, g);
    T rl = Pl[0], rr = Pr[0], pl = Pl[dim + 1], pr = Pr[dim + 1];
    T vm[3], v2;
    for (int k = 0; k < dim; ++k) vm[k] = (Pl[1 + k] + Pr[1 + k]) / 2.0;
    if (dim == 1) v2 = 2.0 * sq(vm[0]) - (sq(Pl[1]) + sq(Pr[1])) / 2.0;
    else if (dim == 2)
        v2 = 2.0 * (sq(vm[0]) + sq(vm[1])) - (((sq(Pl[1]) + sq(Pl[2])) + sq(Pr[1])) + sq(Pr[2])) / 2.0;
    else
        v2 = 2.0 * ((sq(vm[0]) + sq(vm[1])) + sq(vm[2])) -
             (((((sq(Pl[1]) + sq(Pl[2])) + sq(Pl[3])) + sq(Pr[1])) + sq(Pr[2])) + sq(Pr[3])) / 2.0;
    T bl = rl / (2.0 * pl), br = rr / (2.0 * pr);
    T rho = logarithmic_mean(rl, rr);
    T p = (rl + rr) / (2.0 * (bl + br));
    T beta = logarithmic_mean(bl, br);
    T a = soundvelocity(rho, p, g);
    T h = g / (2.0 * beta) / (g - 1.0) + v2 / 2.0;
    Vec<T> Fn = euler_average(Ql, Qr, dim, g, avg);
    Vec<T> Wl = cons2entropy(Ql, dim, g), Wr = cons2entropy(Qr, dim, g);
    int nv = dim + 2;
    T u = vm[0];
    // R (column j = wave j), Λ and T as in the reference
    T R[5][5], Lam[5], Td[5];
    for (int i = 0; i < 5; ++i)
        for (int j = 0; j < 5; ++j) R[i][j] = T(0.0);
    R[0][0] = T(1.0); R[1][0] = u - a;
    R[0][1] = T(1.0); R[1][1] = u;
    R[0][nv - 1] = T(1.0); R[1][nv - 1] = u + a;
    for (int k = 1; k < dim; ++k) {
        R[1 + k][0] = vm[k]; R[1 + k][1] = vm[k]; R[1 + k][nv - 1] = vm[k];
        R[1 + k][1 + k] = T(1.0);
        R[nv - 1][1 + k] = vm[k];
    }
    R[nv - 1][0] = h - u * a;
    R[nv - 1][1] = v2 / 2.0;
    R[nv - 1][nv - 1] = h + u * a;
    Lam[0] = fabs(u - a); Lam[nv - 1] = fabs(u + a);
    for (int k = 1; k < nv - 1; ++k) Lam[k] = fabs(u);
    Td[0] = rho / (2.0 * g); Td[nv - 1] = rho / (2.0 * g);
    Td[1] = (g - 1.0) * rho / g;
    for (int k = 2; k < nv - 1; ++k) Td[k] = p;
    T M[5][5];
    for (int i = 0; i < nv; ++i)
        for (int k = 0; k < nv; ++k) {
            T acc = T(0.0);
            for (int j = 0; j < nv; ++j) acc = acc + ((R[i][j] * Lam[j]) * Td[j]) * R[k][j];
            M[i][k] = acc;
        }
    Vec<T> F{};
    for (int i = 0; i < nv; ++i) {
        T acc = T(0.0);
        for (int k = 0; k < nv; ++k) acc = acc + M[i][k] * (Wl[k] - Wr[k]);
        F[i] = Fn[i] + acc / 2.0 * intensity;
    }
    return F;
}

// numericalflux dispatch.  Ql/Qr are in the face frame (rotated), n is the physical
// normal (used by the scalar equations).  Interfaces.jl:111-136; Euler.jl:99-226;
// LinearAdvection.jl:27-39; Burgers.jl:27-38.
template <class T>
inline Vec<T> numericalflux(const Vec<T>& Ql, const Vec<T>& Qr, const double* n, const Config& c, int kind,
                           const T& intensity) {
    Vec<T> F{};
    if (c.eq == EQ_ADVECTION) {
        double an = 0;   // dot(eq.a, n)
        for (int d = 0; d < c.dim; ++d) an = an + c.a[d] * n[d];
        F[0] = an * (Ql[0] + Qr[0]) / 2.0;
        if (kind == NF_LXF) F[0] = F[0] + std::fabs(an) * (Ql[0] - Qr[0]) / 2.0 * intensity;
        return F;
    }
    if (c.eq == EQ_BURGERS) {
        using std::fabs; using std::max;
        F[0] = (sq(Ql[0]) + sq(Qr[0])) / 4.0 * n[0];
        if (kind == NF_LXF) {
            T lam = max(fabs(Ql[0]), fabs(Qr[0]));
            F[0] = F[0] + lam * (Ql[0] - Qr[0]) / 2.0 * intensity;
        }
        return F;
    }
    int dim = c.dim, nv = dim + 2;
    switch (kind) {
        case NF_STDAVG: return euler_stdavg(Ql, Qr, dim, c.gamma);
        case NF_CHANDRASHEKAR: return euler_chandrashekar(Ql, Qr, dim, c.gamma);
        case NF_HLL: return euler_hll(Ql, Qr, dim, c.gamma);
        case NF_HLLC: return euler_hllc(Ql, Qr, dim, c.gamma);
        case NF_SCALAR_DISSIPATION: return euler_scalar_dissipation(Ql, Qr, dim, c.gamma, c.lxf_avg, intensity);
        case NF_MATRIX_DISSIPATION: return euler_matrix_dissipation(Ql, Qr, dim, c.gamma, c.lxf_avg, intensity);
        default: break;
    }
    // LxF (Euler.jl:138-165)
    using std::fabs; using std::max;
    Vec<T> Fa = (c.lxf_avg == NF_CHANDRASHEKAR) ? euler_chandrashekar(Ql, Qr, dim, c.gamma)
                                                : euler_stdavg(Ql, Qr, dim, c.gamma);
    Vec<T> Pl = cons2prim(Ql, dim, c.gamma), Pr = cons2prim(Qr, dim, c.gamma);
    T al = soundvelocity(Pl[0], Pl[dim + 1], c.gamma);
    T ar = soundvelocity(Pr[0], Pr[dim + 1], c.gamma);
    T lam = max(fabs(Pl[1]) + al, fabs(Pr[1]) + ar);
    for (int k = 0; k < nv; ++k) F[k] = Fa[k] + lam * (Ql[k] - Qr[k]) / 2.0 * intensity;
    return F;
}

template <class T>
inline Vec<T> numericalflux(const Vec<T>& Ql, const Vec<T>& Qr, const double* n, const Config& c, int kind) {
    return numericalflux(Ql, Qr, n, c, kind, T(c.intensity));
}

// twopointflux (contravariant, direction column of the metric averaged):
// Euler StdAverage Euler.jl:385-472; Chandrashekar :474-536; LinearAdvection.jl:44-47;
// Burgers.jl:43-45.  Kennedy-Gruber (Kennedy & Gruber 2008) has no Flou counterpart.
template <class T>
inline Vec<T> twopointflux(const Vec<T>& Q1, const Vec<T>& Q2, const double* Ja1, const double* Ja2,
                           const Config& c) {
    Vec<T> F{};
    int dim = c.dim;
    double n[3] = {0, 0, 0};
    for (int d = 0; d < dim; ++d) n[d] = (Ja1[d] + Ja2[d]) / 2.0;
    if (c.eq == EQ_ADVECTION) return numericalflux(Q1, Q2, n, c, NF_STDAVG);
    if (c.eq == EQ_BURGERS) return numericalflux(Q1, Q2, n, c, NF_STDAVG);
    double g = c.gamma;
    Vec<T> P1 = cons2prim(Q1, dim, g), P2 = cons2prim(Q2, dim, g);
    int nv = dim + 2;
    if (c.tpflux == TP_STDAVG) {
        T p1 = P1[dim + 1], p2 = P2[dim + 1];
        for (int k = 0; k < nv; ++k) F[k] = T(0.0);
        // f_k[d] averaged physical flux component, then dot with n in order d = 1..dim
        for (int d = 0; d < dim; ++d) {
            Vec<T> f{};
            f[0] = (Q1[1 + d] + Q2[1 + d]) / 2.0;
            for (int k = 0; k < dim; ++k) {
                if (k == d) f[1 + k] = (((Q1[1 + k] * P1[1 + d] + p1) + Q2[1 + k] * P2[1 + d]) + p2) / 2.0;
                else f[1 + k] = (Q1[1 + k] * P1[1 + d] + Q2[1 + k] * P2[1 + d]) / 2.0;
            }
            f[dim + 1] = ((Q1[dim + 1] + p1) * P1[1 + d] + (Q2[dim + 1] + p2) * P2[1 + d]) / 2.0;
            for (int k = 0; k < nv; ++k) F[k] = (d == 0) ? f[k] * n[0] : F[k] + f[k] * n[d];
        }
        return F;
    }
    if (c.tpflux == TP_KENNEDY_GRUBER) {
        T rho = (P1[0] + P2[0]) / 2.0;
        T vel[3]{};
        for (int k = 0; k < dim; ++k) vel[k] = (P1[1 + k] + P2[1 + k]) / 2.0;
        T p = (P1[dim + 1] + P2[dim + 1]) / 2.0;
        T e = (Q1[dim + 1] / P1[0] + Q2[dim + 1] / P2[0]) / 2.0;
        T vn = vel[0] * n[0];
        for (int k = 1; k < dim; ++k) vn = vn + vel[k] * n[k];
        T mdot = rho * vn;
        F[0] = mdot;
        for (int k = 0; k < dim; ++k) F[1 + k] = mdot * vel[k] + p * n[k];
        F[dim + 1] = mdot * e + p * vn;
        return F;
    }
    // Chandrashekar
    T r1 = P1[0], r2 = P2[0], p1 = P1[dim + 1], p2 = P2[dim + 1];
    T vel[3];
    for (int k = 0; k < dim; ++k) vel[k] = (P1[1 + k] + P2[1 + k]) / 2.0;
    T b1 = r1 / (2.0 * p1), b2 = r2 / (2.0 * p2);
    T rho = logarithmic_mean(r1, r2);
    T p = (r1 + r2) / (2.0 * (b1 + b2));
    T beta = logarithmic_mean(b1, b2);
    T s = sq(P1[1]);
    for (int k = 1; k < dim; ++k) s = s + sq(P1[1 + k]);
    for (int k = 0; k < dim; ++k) s = s + sq(P2[1 + k]);
    T h = (1.0 / ((2.0 * beta) * (g - 1.0)) - s / 4.0) + p / rho;
    for (int k = 0; k < dim; ++k) h = h + sq(vel[k]);
    // component j along direction d: (ρ v_d)(...)*n[d], summed over d in order
    for (int d = 0; d < dim; ++d) {
        Vec<T> f{};
        f[0] = rho * vel[d];
        for (int k = 0; k < dim; ++k) {
            if (k == d) f[1 + k] = rho * sq(vel[k]) + p;
            else f[1 + k] = (k < d) ? rho * vel[k] * vel[d] : rho * vel[d] * vel[k];
        }
        f[dim + 1] = rho * vel[d] * h;
        for (int k = 0; k < nv; ++k) F[k] = (d == 0) ? f[k] * n[0] : F[k] + f[k] * n[d];
    }
    return F;
}

// ============================================================================
// Discretization + residual
// ============================================================================
struct Bc { int kind = BC_NONE; double state[5] = {0, 0, 0, 0, 0}; };

struct Disc {
    Config cfg;
    int n = 0, npe = 0, nfd = 0, nelem = 0, nfaces = 0;
    // operators (n x n column-major)
    std::vector<double> Ds, Dsharp, ll, lr, dgl, dgr;
    std::vector<double> D, omega1d;       // derivative matrix, 1D weights (HybridDivOperator)
    bool lobatto = true;                  // hasboundaries(basis): l_l, l_r pick the end nodes
    // subcell-interface geometry of general elements (geometry.subgrids, PhysicalRegions.jl:180-300):
    // point ((e·dim + d)·nfd + line)·(n+1) + s; empty on Cartesian meshes (the axes)
    std::vector<Frame> subframes;
    std::vector<double> subjac;
    // GenericBC external states per boundary face node, 5 per node (BC_STATE_FIELD boundaries)
    std::vector<double> bcfield;
    // connectivity (1-based, like the reference)
    std::vector<int> faceinds, facepos;   // nelem * 2dim
    std::vector<int> eleminds, elempos;   // nfaces * 2
    std::vector<uint8_t> orient;
    std::vector<int> bdid;                // nfaces: boundary index (1-based) or 0
    std::vector<Bc> bcs;                  // per boundary index
    // geometry
    std::vector<double> J;                // ndofs
    std::vector<double> Ja;               // ndofs * dim * dim (column-major per node)
    std::vector<Frame> frames;            // nfaces * nfd
    std::vector<double> faceJ;            // nfaces * nfd
    long ndofs() const { return (long)nelem * npe; }
    long nfdofs() const { return (long)nfaces * nfd; }
};

// tpdofs (StdSegment.jl:143-146, StdQuad.jl:116-124, StdHex.jl:135-145): node index (0-based,
// element-local) of position `pos` on line `line` of direction `dir`.  The face-dof index of
// a face in direction `dir` equals the line index.
inline int tp_node(int dim, int n, int dir, int line, int pos) {
    if (dim == 1) return pos;
    if (dim == 2) return dir == 0 ? pos + n * line : line + n * pos;
    int a = line % n, b = line / n;
    if (dir == 0) return pos + n * a + n * n * b;
    if (dir == 1) return a + n * pos + n * n * b;
    return a + n * b + n * n * pos;
}

// master2slave (StdQuad.jl:161-181, StdSegment.jl:161-167) for face dof i (0-based).
inline int master2slave(int i, int orient, int dim, int n) {
    if (orient == 0 || dim == 1) return i;
    if (dim == 2) return orient == 0 ? i : n - 1 - i;
    int m1 = i % n, m2 = i / n;   // cartesiandofs: (m[1], m[2]) with m[1] fastest
    auto li = [&](int a, int b) { return a + n * b; };
    switch (orient) {
        case 1: return li(m2, n - 1 - m1);
        case 2: return li(n - 1 - m1, n - 1 - m2);
        case 3: return li(n - 1 - m2, m1);
        case 4: return li(m2, m1);
        case 5: return li(n - 1 - m1, m2);
        case 6: return li(n - 1 - m2, n - 1 - m1);
        default: return li(m1, n - 1 - m2);
    }
}

template <class T> struct Workspace {
    std::vector<T> Qf[2], Fn[2];
};

template <class T> inline Vec<T> getv(const T* A, long stride, long idx, int nv) {
    Vec<T> v{};
    for (int k = 0; k < nv; ++k) v[k] = A[k * stride + idx];
    return v;
}
template <class T> inline void setv(T* A, long stride, long idx, const Vec<T>& v, int nv) {
    for (int k = 0; k < nv; ++k) A[k * stride + idx] = v[k];
}

// EulerSlipBC, Euler.jl:88-94; EulerOutflowBC :82-86; EulerInflowBC :69-80.
template <class T> inline Vec<T> apply_bc(const Bc& bc, const Vec<T>& Qin, const Frame& fr, const Config& c) {
    Vec<T> Q{};
    switch (bc.kind) {
        case BC_OUTFLOW: return Qin;
        case BC_INFLOW: for (int k = 0; k < c.nv; ++k) Q[k] = T(bc.state[k]); return Q;
        case BC_SLIP: {
            Vec<T> Qn = rotate2face(Qin, fr, c);
            Qn[1] = -Qn[1];
            return rotate2phys(Qn, fr, c);
        }
        default: throw std::runtime_error("boundary face without a boundary condition");
    }
}

// rhs!, src/FlouSpatial/Equations/Hyperbolic.jl:31-69 (steps C1-C8, in order).
// `celem` (optional): per-element scale c_e of the LxF dissipation; a face uses
// intensity = (c_1 + c_2)/2 of its two elements (c_1 on boundary faces).  c = 1 is LxF(., 1.0).
// Frame of the subgrid interfaces of a Cartesian element along `dir` (PhysicalRegions.jl:68-148):
// the positive axis, completed like the face frames of the reference.
inline Frame subgrid_frame(int dim, int dir) {
    Frame fr{};
    if (dim == 1) { fr.n[0] = 1; }
    else if (dim == 2) {
        if (dir == 0) { fr.n[0] = 1; fr.t[1] = 1; } else { fr.n[1] = 1; fr.t[0] = -1; }
    } else {
        if (dir == 0) { fr.n[0] = 1; fr.t[1] = 1; fr.b[2] = 1; }
        else if (dir == 1) { fr.n[1] = 1; fr.t[2] = 1; fr.b[0] = 1; }
        else { fr.n[2] = 1; fr.t[0] = 1; fr.b[1] = 1; }
    }
    return fr;
}

// _hybrid_compute_delta, OpDivergence.jl:781-801 (Fisher's indicator, limited at 0.5)
template <class T> inline T hybrid_delta(const T& b, double c) {
    using std::sqrt; using std::max;
    T dl = sqrt(b * b + c);
    dl = (dl - b) / dl;
    return max(dl, T(0.5));
}

// _flux_splitdiv_nb_tensorproduct!, OpDivergence.jl:382-427, on one line of direction `dir`:
// Fl[ii], Fr[ii] for the line's nodes from the entropy-projected boundary states, with the
// line's interface fluxes Fnl, Fnr (this element's sides).  Cartesian subgrid: nl = nr = the
// positive axis times Js.
template <class T>
void splitdiv_nb_line(const Disc& g, const T* Q, long base, int dir, int line, const std::vector<Vec<T>>& W,
                      const Vec<T>& Fnl, const Vec<T>& Fnr, std::vector<Vec<T>>& Fl, std::vector<Vec<T>>& Fr) {
    const Config& c = g.cfg;
    const int dim = c.dim, n = g.n, nv = c.nv;
    const long nd = g.ndofs();
    // nl = frames[dir][i1].n Js[dir][i1], nr likewise at the last subcell interface (OpDivergence.jl:
    // 403-404): the positive axis and Ja_dd on a Cartesian element, the subgrid data on a general one
    Frame fr = subgrid_frame(dim, dir);
    double Js = g.Ja[base * dim * dim + dir + dir * dim];
    double nl[3], nr[3];
    for (int k = 0; k < 3; ++k) { nl[k] = fr.n[k] * Js; nr[k] = fr.n[k] * Js; }
    if (!g.subjac.empty()) {
        long sb = (((base / g.npe) * dim + dir) * g.nfd + line) * (n + 1);
        for (int k = 0; k < 3; ++k) {
            nl[k] = g.subframes[sb].n[k] * g.subjac[sb];
            nr[k] = g.subframes[sb + n].n[k] * g.subjac[sb + n];
        }
    }
    Vec<T> Wl{}, Wr{};
    for (int ii = 0; ii < n; ++ii) {
        int i = tp_node(dim, n, dir, line, ii);
        for (int q = 0; q < nv; ++q) {
            Wl[q] = Wl[q] + g.ll[ii] * W[i][q];
            Wr[q] = Wr[q] + g.lr[ii] * W[i][q];
        }
    }
    Vec<T> Ql = entropy2cons(Wl, dim, c.gamma), Qr = entropy2cons(Wr, dim, c.gamma);
    for (int ii = 0; ii < n; ++ii) {
        int i = tp_node(dim, n, dir, line, ii);
        Vec<T> Qi = getv(Q, nd, base + i, nv);
        const double* Jai = &g.Ja[(base + i) * dim * dim + dir * dim];
        Fl[ii] = twopointflux(Qi, Ql, Jai, nl, c);
        Fr[ii] = twopointflux(Qi, Qr, Jai, nr, c);
    }
    Vec<T> lF{}, rF{};
    for (int ii = 0; ii < n; ++ii)
        for (int q = 0; q < nv; ++q) {
            lF[q] = lF[q] + g.ll[ii] * Fl[ii][q];
            rF[q] = rF[q] + g.lr[ii] * Fr[ii][q];
        }
    for (int ii = 0; ii < n; ++ii)
        for (int q = 0; q < nv; ++q) {
            Fl[ii][q] = Fl[ii][q] - (lF[q] + Fnl[q]);
            Fr[ii][q] = Fr[ii][q] - (rF[q] - Fnr[q]);
        }
}

template <class T> void rhs(const Disc& g, T* dQ, const T* Q, double time, Workspace<T>& ws,
                            const T* celem = nullptr) {
    (void)time;
    const Config& c = g.cfg;
    const int dim = c.dim, n = g.n, nv = c.nv, npe = g.npe, nfd = g.nfd;
    const long nd = g.ndofs(), nf = g.nfdofs();
    for (int s = 0; s < 2; ++s) { ws.Qf[s].assign(nv * nf, T(0.0)); ws.Fn[s].assign(nv * nf, T(0.0)); }

    // 1. fill!(dQ, 0), :45
    for (long i = 0; i < nv * nd; ++i) dQ[i] = T(0.0);

    // 2. project2faces!, Interfaces.jl:51-109
#pragma omp parallel for schedule(static)
    for (int e = 0; e < g.nelem; ++e) {
        for (int dir = 0; dir < dim; ++dir) {
            int fl = g.faceinds[e * 2 * dim + 2 * dir] - 1, sl = g.facepos[e * 2 * dim + 2 * dir] - 1;
            int fr = g.faceinds[e * 2 * dim + 2 * dir + 1] - 1, sr = g.facepos[e * 2 * dim + 2 * dir + 1] - 1;
            T* Ql = ws.Qf[sl].data();
            T* Qr = ws.Qf[sr].data();
            for (int line = 0; line < nfd; ++line) {
                for (int k = 0; k < nv; ++k) {
                    T a = T(0.0), b = T(0.0);
                    for (int pos = 0; pos < n; ++pos) {
                        T q = Q[k * nd + (long)e * npe + tp_node(dim, n, dir, line, pos)];
                        a = a + g.ll[pos] * q;
                    }
                    for (int pos = 0; pos < n; ++pos) {
                        T q = Q[k * nd + (long)e * npe + tp_node(dim, n, dir, line, pos)];
                        b = b + g.lr[pos] * q;
                    }
                    Ql[k * nf + (long)fl * nfd + line] = a;
                    Qr[k * nf + (long)fr * nfd + line] = b;
                }
            }
        }
    }

    // 3. volume_contribution!, Hyperbolic.jl:71-77 -> OpDivergence.jl:109-160 / 200-282
#pragma omp parallel for schedule(static)
    for (int e = 0; e < g.nelem; ++e) {
        long base = (long)e * npe;
        // _volumeflux!: F̃[i, d] = contravariant(volumeflux(Q_i), Ja_i, d)
        std::vector<Vec<T>> Ft(npe * dim);
        for (int i = 0; i < npe; ++i) {
            Vec<T> Qi = getv(Q, nd, base + i, nv);
            const double* M = &g.Ja[(base + i) * dim * dim];
            std::array<Vec<T>, 3> F;
            for (int d = 0; d < dim; ++d) F[d] = volumeflux(Qi, d, c);
            for (int d = 0; d < dim; ++d) {
                Vec<T> r{};
                for (int k = 0; k < nv; ++k) {
                    T acc = F[0][k] * M[0 + d * dim];
                    for (int q = 1; q < dim; ++q) acc = acc + F[q][k] * M[q + d * dim];
                    r[k] = acc;
                }
                Ft[i * dim + d] = r;
            }
        }
        if (c.volop == OP_HYBRID && !g.lobatto) {
            // Gauss nodes: "everything as a surface contribution" (OpDivergence.jl:485-490)
        } else if (c.volop == OP_HYBRID) {
            // _vol_hybrid_tensorproduct!, OpDivergence.jl:553-604, with the Cartesian subgrid of
            // PhysicalRegions.jl:68-148 (frames along the positive axes, Js the face Jacobian)
            using std::sqrt; using std::max;
            std::vector<Vec<T>> W(npe);
            for (int i = 0; i < npe; ++i) W[i] = cons2entropy(getv(Q, nd, base + i, nv), dim, c.gamma);
            Config fv = c;
            fv.lxf_avg = c.fvavg;
            std::vector<Vec<T>> Fb(n + 1);
            for (int dir = 0; dir < dim; ++dir) {
                Frame fr = subgrid_frame(dim, dir);
                double Js = g.Ja[base * dim * dim + dir + dir * dim];
                for (int line = 0; line < nfd; ++line) {
                    long sbase = (((long)e * dim + dir) * nfd + line) * (n + 1);
                    for (int ii = 0; ii <= n; ++ii) Fb[ii] = Vec<T>{};
                    for (int ii = 1; ii < n; ++ii) {
                        for (int ik = ii; ik < n; ++ik) {
                            int k = tp_node(dim, n, dir, line, ik);
                            for (int il = 0; il < ii; ++il) {
                                int l = tp_node(dim, n, dir, line, il);
                                Vec<T> Ft = twopointflux(getv(Q, nd, base + l, nv), getv(Q, nd, base + k, nv),
                                                         &g.Ja[(base + l) * dim * dim + dir * dim],
                                                         &g.Ja[(base + k) * dim * dim + dir * dim], c);
                                double coef = (2.0 * g.omega1d[il]) * g.D[il + ik * n];
                                for (int q = 0; q < nv; ++q) Fb[ii][q] = Fb[ii][q] + coef * Ft[q];
                            }
                        }
                        int i = tp_node(dim, n, dir, line, ii), il = tp_node(dim, n, dir, line, ii - 1);
                        const bool gen = !g.subjac.empty();   // frames[dir][is], Js[dir][is] of the element
                        const Frame& sf = gen ? g.subframes[sbase + ii] : fr;
                        double sJ = gen ? g.subjac[sbase + ii] : Js;
                        Vec<T> Qln = rotate2face(getv(Q, nd, base + il, nv), sf, c);
                        Vec<T> Qrn = rotate2face(getv(Q, nd, base + i, nv), sf, c);
                        Vec<T> Fn = numericalflux(Qln, Qrn, sf.n, fv, c.fvflux, T(c.fvintensity));
                        Vec<T> Fv = rotate2phys(Fn, sf, c);
                        for (int q = 0; q < nv; ++q) Fv[q] = Fv[q] * sJ;
                        T bb = T(0.0);
                        for (int q = 0; q < nv; ++q) bb = bb + (W[i][q] - W[il][q]) * (Fb[ii][q] - Fv[q]);
                        T dl = hybrid_delta(bb, c.blend);
                        for (int q = 0; q < nv; ++q) Fb[ii][q] = (1.0 - dl) * Fv[q] + dl * Fb[ii][q];
                    }
                    for (int ii = 0; ii < n; ++ii) {
                        int i = tp_node(dim, n, dir, line, ii);
                        for (int q = 0; q < nv; ++q) {
                            T& y = dQ[q * nd + base + i];
                            y = y + (Fb[ii][q] - Fb[ii + 1][q]) / g.omega1d[ii];
                        }
                    }
                }
            }
        } else if (c.volop == OP_STRONG) {
            for (int dir = 0; dir < dim; ++dir)
                for (int line = 0; line < nfd; ++line)
                    for (int col = 0; col < n; ++col) {   // mul!(y, Ds, x, -1, 1): y[i] += Ds[i,k]*(-x[k])
                        int nk = tp_node(dim, n, dir, line, col);
                        for (int row = 0; row < n; ++row) {
                            int ni = tp_node(dim, n, dir, line, row);
                            double a = g.Ds[row + col * n];
                            for (int k = 0; k < nv; ++k) {
                                T& y = dQ[k * nd + base + ni];
                                y = y + a * (-Ft[nk * dim + dir][k]);
                            }
                        }
                    }
        } else {
            std::vector<Vec<T>> Fs(n * npe);   // F♯.dofs[ii, node]
            for (int dir = 0; dir < dim; ++dir) {
                // _flux_splitdiv_tensorproduct!, OpDivergence.jl:248-271
                for (int line = 0; line < nfd; ++line)
                    for (int ii = 0; ii < n; ++ii) {
                        int i = tp_node(dim, n, dir, line, ii);
                        Fs[ii + n * i] = Ft[i * dim + dir];
                        Vec<T> Qi = getv(Q, nd, base + i, nv);
                        const double* Jai = &g.Ja[(base + i) * dim * dim + dir * dim];
                        for (int il = ii + 1; il < n; ++il) {
                            int l = tp_node(dim, n, dir, line, il);
                            Vec<T> Ql = getv(Q, nd, base + l, nv);
                            const double* Jal = &g.Ja[(base + l) * dim * dim + dir * dim];
                            Vec<T> F = twopointflux(Qi, Ql, Jai, Jal, c);
                            Fs[il + n * i] = F;
                            Fs[ii + n * l] = F;
                        }
                    }
                // _vol_splitdiv_tensorproduct!, :273-282
                for (int line = 0; line < nfd; ++line)
                    for (int ij = 0; ij < n; ++ij) {
                        int j = tp_node(dim, n, dir, line, ij);
                        for (int ii = 0; ii < n; ++ii) {
                            int i = tp_node(dim, n, dir, line, ii);
                            double a = g.Dsharp[ii + ij * n];
                            for (int k = 0; k < nv; ++k) {
                                T& y = dQ[k * nd + base + i];
                                y = y - a * Fs[ii + n * j][k];
                            }
                        }
                    }
            }
        }
    }

    // 4. applyBCs!, Interfaces.jl:25-49
    for (int f = 0; f < g.nfaces; ++f) {
        if (g.bdid[f] == 0) continue;
        const Bc& bc = g.bcs[g.bdid[f] - 1];
        for (int m = 0; m < nfd; ++m) {
            long idx = (long)f * nfd + m;
            Vec<T> Qin = getv(ws.Qf[0].data(), nf, idx, nv);
            if (bc.kind == BC_STATE_FIELD) {   // GenericBC: Qext(x) at this face node
                Vec<T> Qe{};
                for (int k = 0; k < nv; ++k) Qe[k] = T(g.bcfield.at(5 * idx + k));
                setv(ws.Qf[1].data(), nf, idx, Qe, nv);
                continue;
            }
            setv(ws.Qf[1].data(), nf, idx, apply_bc(bc, Qin, g.frames[idx], c), nv);
        }
    }

    // 5. interface_fluxes!, Interfaces.jl:111-136
#pragma omp parallel for schedule(static)
    for (int f = 0; f < g.nfaces; ++f) {
        for (int i = 0; i < nfd; ++i) {
            int j = master2slave(i, g.orient[f], dim, n);
            long ii = (long)f * nfd + i, jj = (long)f * nfd + j;
            const Frame& fr = g.frames[ii];
            Vec<T> Qln = rotate2face(getv(ws.Qf[0].data(), nf, ii, nv), fr, c);
            Vec<T> Qrn = rotate2face(getv(ws.Qf[1].data(), nf, jj, nv), fr, c);
            T inten = T(c.intensity);
            if (celem) {
                int e1 = g.eleminds[2 * f] - 1, e2 = g.eleminds[2 * f + 1] - 1;
                inten = (celem[e1] + celem[e2 >= 0 ? e2 : e1]) * 0.5;
            }
            Vec<T> Fni = numericalflux(Qln, Qrn, fr.n, c, c.numflux, inten);
            Vec<T> F = rotate2phys(Fni, fr, c);
            for (int k = 0; k < nv; ++k) {
                F[k] = F[k] * g.faceJ[ii];
                ws.Fn[0][k * nf + ii] = F[k];
                ws.Fn[1][k * nf + jj] = -F[k];
            }
        }
    }

    // 6. surface_contribution! -> _reconstruction_tensorproduct!, OpDivergence.jl:42-100, or on
    // Gauss nodes the entropy-projected split form (:284-437) / hybrid form (:614-780)
#pragma omp parallel for schedule(static)
    for (int e = 0; e < g.nelem; ++e) {
        long base = (long)e * npe;
        if (!g.lobatto && (c.volop == OP_SPLIT || c.volop == OP_HYBRID)) {
            std::vector<Vec<T>> W(npe), Fl(n), Fr(n), Fs(n * npe), Fb(n + 1);
            for (int i = 0; i < npe; ++i) W[i] = cons2entropy(getv(Q, nd, base + i, nv), dim, c.gamma);
            Config fv = c;
            fv.lxf_avg = c.fvavg;
            for (int dir = 0; dir < dim; ++dir) {
                int fl = g.faceinds[e * 2 * dim + 2 * dir] - 1, sl = g.facepos[e * 2 * dim + 2 * dir] - 1;
                int fr = g.faceinds[e * 2 * dim + 2 * dir + 1] - 1, sr = g.facepos[e * 2 * dim + 2 * dir + 1] - 1;
                if (c.volop == OP_HYBRID) {   // _flux_splitdiv_tensorproduct!: F♯ of every line
                    for (int line = 0; line < nfd; ++line)
                        for (int ii = 0; ii < n; ++ii) {
                            int i = tp_node(dim, n, dir, line, ii);
                            Vec<T> Qi = getv(Q, nd, base + i, nv);
                            const double* Jai = &g.Ja[(base + i) * dim * dim + dir * dim];
                            std::array<Vec<T>, 3> F;
                            for (int d = 0; d < dim; ++d) F[d] = volumeflux(Qi, d, c);
                            Vec<T> Ft{};
                            for (int k = 0; k < nv; ++k) {
                                T acc = F[0][k] * Jai[0];
                                for (int q = 1; q < dim; ++q) acc = acc + F[q][k] * Jai[q];
                                Ft[k] = acc;
                            }
                            Fs[ii + n * i] = Ft;
                            for (int il = ii + 1; il < n; ++il) {
                                int l = tp_node(dim, n, dir, line, il);
                                const double* Jal = &g.Ja[(base + l) * dim * dim + dir * dim];
                                Vec<T> F2 = twopointflux(Qi, getv(Q, nd, base + l, nv), Jai, Jal, c);
                                Fs[il + n * i] = F2;
                                Fs[ii + n * l] = F2;
                            }
                        }
                }
                Frame sfr = subgrid_frame(dim, dir);
                double Js = g.Ja[base * dim * dim + dir + dir * dim];
                for (int line = 0; line < nfd; ++line) {
                    Vec<T> Fnl = getv(ws.Fn[sl].data(), nf, (long)fl * nfd + line, nv);
                    Vec<T> Fnr = getv(ws.Fn[sr].data(), nf, (long)fr * nfd + line, nv);
                    splitdiv_nb_line(g, Q, base, dir, line, W, Fnl, Fnr, Fl, Fr);
                    if (c.volop == OP_SPLIT) {   // _surf_splitdiv_nb_tensorproduct!, :429-437
                        for (int ii = 0; ii < n; ++ii) {
                            int i = tp_node(dim, n, dir, line, ii);
                            for (int k = 0; k < nv; ++k) {
                                T& y = dQ[k * nd + base + i];
                                y = y + (g.dgl[ii] * Fl[ii][k] - g.dgr[ii] * Fr[ii][k]);
                            }
                        }
                        continue;
                    }
                    // _surf_hybrid_nb_tensorproduct!, :732-779
                    for (int k = 0; k < nv; ++k) { Fb[0][k] = -Fnl[k]; Fb[n][k] = Fnr[k]; }
                    for (int ii = 0; ii < n - 1; ++ii) {
                        int i = tp_node(dim, n, dir, line, ii), ir = tp_node(dim, n, dir, line, ii + 1);
                        Vec<T> sum{};
                        for (int j = 0; j < n; ++j)
                            for (int k = 0; k < nv; ++k) sum[k] = sum[k] + g.Dsharp[ii + j * n] * Fs[j + n * i][k];
                        for (int k = 0; k < nv; ++k)
                            Fb[ii + 1][k] = Fb[ii][k] + sum[k] * g.omega1d[ii] - g.ll[ii] * Fl[ii][k] +
                                            g.lr[ii] * Fr[ii][k];
                        const bool gen = !g.subjac.empty();   // frames[dir][sinds[ii+1]] of the element
                        long sidx = (((long)e * dim + dir) * nfd + line) * (n + 1) + ii + 1;
                        const Frame& f2 = gen ? g.subframes[sidx] : sfr;
                        double J2 = gen ? g.subjac[sidx] : Js;
                        Vec<T> Qln = rotate2face(getv(Q, nd, base + i, nv), f2, c);
                        Vec<T> Qrn = rotate2face(getv(Q, nd, base + ir, nv), f2, c);
                        Vec<T> Fv = rotate2phys(numericalflux(Qln, Qrn, f2.n, fv, c.fvflux, T(c.fvintensity)), f2, c);
                        for (int k = 0; k < nv; ++k) Fv[k] = Fv[k] * J2;
                        T bb = T(0.0);
                        for (int k = 0; k < nv; ++k) bb = bb + (W[ir][k] - W[i][k]) * (Fb[ii + 1][k] - Fv[k]);
                        T dl = hybrid_delta(bb, c.blend);
                        for (int k = 0; k < nv; ++k) Fb[ii + 1][k] = (1.0 - dl) * Fv[k] + dl * Fb[ii + 1][k];
                    }
                    for (int ii = 0; ii < n; ++ii) {
                        int i = tp_node(dim, n, dir, line, ii);
                        for (int k = 0; k < nv; ++k) {
                            T& y = dQ[k * nd + base + i];
                            y = y + (Fb[ii][k] - Fb[ii + 1][k]) / g.omega1d[ii];
                        }
                    }
                }
            }
            continue;
        }
        for (int dir = 0; dir < dim; ++dir) {
            int fl = g.faceinds[e * 2 * dim + 2 * dir] - 1, sl = g.facepos[e * 2 * dim + 2 * dir] - 1;
            int fr = g.faceinds[e * 2 * dim + 2 * dir + 1] - 1, sr = g.facepos[e * 2 * dim + 2 * dir + 1] - 1;
            for (int line = 0; line < nfd; ++line)
                for (int ii = 0; ii < n; ++ii) {
                    int i = tp_node(dim, n, dir, line, ii);
                    for (int k = 0; k < nv; ++k) {
                        T fli = ws.Fn[sl][k * nf + (long)fl * nfd + line];
                        T fri = ws.Fn[sr][k * nf + (long)fr * nfd + line];
                        T& y = dQ[k * nd + base + i];
                        y = y - (g.dgl[ii] * fli + g.dgr[ii] * fri);
                    }
                }
        }
    }

    // 7. apply_massmatrix!, MultielementDiscontinuous.jl:132-137 (Diagonal(J) blocks)
#pragma omp parallel for schedule(static)
    for (long i = 0; i < nd; ++i)
        for (int k = 0; k < nv; ++k) dQ[k * nd + i] = dQ[k * nd + i] / g.J[i];
    // 8. apply_sourceterm!: no source term on this path (a no-op closure, :75-79).
}

// Shu-Osher SSP-RK3 (Shu & Osher 1988), the method behind OrdinaryDiffEq's SSPRK33:
//   U1 = U0 + dt L(U0); U2 = 3/4 U0 + 1/4 (U1 + dt L(U1)); U3 = 1/3 U0 + 2/3 (U2 + dt L(U2)).
template <class T> void ssprk3_step(const Disc& g, T* Q, double dt, double t, Workspace<T>& ws,
                                    std::vector<T>& U, std::vector<T>& L, const T* celem = nullptr) {
    long N = g.ndofs() * g.cfg.nv;
    U.resize(N);
    L.resize(N);
    rhs(g, L.data(), Q, t, ws, celem);
#pragma omp parallel for schedule(static)
    for (long i = 0; i < N; ++i) U[i] = Q[i] + dt * L[i];
    rhs(g, L.data(), U.data(), t + dt, ws, celem);
#pragma omp parallel for schedule(static)
    for (long i = 0; i < N; ++i) U[i] = 0.75 * Q[i] + 0.25 * (U[i] + dt * L[i]);
    rhs(g, L.data(), U.data(), t + 0.5 * dt, ws, celem);
#pragma omp parallel for schedule(static)
    for (long i = 0; i < N; ++i) Q[i] = (1.0 / 3.0) * Q[i] + (2.0 / 3.0) * (U[i] + dt * L[i]);
}

// Zhang–Shu positivity limiter as written in src/FlouSpatial/Equations/Euler.jl:611-654, per
// element: Q̄ = Σ Jω Q / vol (vol = Σ Jω, PhysicalRegions.jl:366-407); density scaled toward ρ̄
// with θ = |(ρ̄ - m)/(ρ̄ - ρ_min)|, m = min(minval, ρ̄), when θ <= 1; then the pressure of the
// density-limited nodes gives p̄ = Σ Jω p / vol and θ = |(p̄ - m)/(p̄ - p_min)|, m = min(minval,
// p̄), and when θ <= 1 every variable is scaled toward the mean Q̄ taken before the density
// step.  `omega` holds the tensor-product quadrature weights per element node.
// T = Dual: forward-mode derivatives through the means, the minima (the first minimal node, as
// Julia's min keeps), the absolute values and the θ <= 1 branches.
template <class T>
void zhang_shu(const Disc& g, T* Q, double minval, const std::vector<double>& omega) {
    using std::min; using std::fabs;
    const Config& c = g.cfg;
    long nd = g.ndofs();
    int nv = c.nv, npe = g.npe;
    std::vector<double> Jw(npe);
    std::vector<T> p(npe);
    for (int e = 0; e < g.nelem; ++e) {
        long b = (long)e * npe;
        double vol = 0.0;
        for (int i = 0; i < npe; ++i) {
            Jw[i] = g.J[b + i] * omega[i];
            vol = vol + Jw[i];
        }
        Vec<T> Qm{};
        for (int k = 0; k < nv; ++k) {
            T acc = T(0.0);
            for (int i = 0; i < npe; ++i) acc = acc + Jw[i] * Q[k * nd + b + i];
            Qm[k] = acc / vol;
        }
        T m = min(T(minval), Qm[0]);
        T rmin = T(INFINITY);
        for (int i = 0; i < npe; ++i) rmin = min(rmin, Q[b + i]);
        T th = fabs((Qm[0] - m) / (Qm[0] - rmin));
        if (th <= 1.0)
            for (int i = 0; i < npe; ++i) Q[b + i] = th * (Q[b + i] - Qm[0]) + Qm[0];
        T ps = T(0.0), pmin = T(INFINITY);
        for (int i = 0; i < npe; ++i) {
            p[i] = pressure(getv(Q, nd, b + i, nv), c.dim, c.gamma);
            ps = ps + Jw[i] * p[i];
            pmin = min(pmin, p[i]);
        }
        T pbar = ps / vol;
        m = min(T(minval), pbar);
        th = fabs((pbar - m) / (pbar - pmin));
        if (th <= 1.0)
            for (int i = 0; i < npe; ++i)
                for (int k = 0; k < nv; ++k) Q[k * nd + b + i] = th * (Q[k * nd + b + i] - Qm[k]) + Qm[k];
    }
}

// Integral monitors, src/FlouSpatial/Equations/Euler.jl:560-590: Σ_e Jω'·f(Q) with f the kinetic
// energy |ρv|²/(2ρ) (which = 1, Euler.jl:162-175 in FlouCommon) or the mathematical entropy
// -ρ s/(γ-1), s = log p - γ log ρ (which = 2, FlouCommon/Euler.jl:202-217).
inline double monitor(const Disc& g, const double* Q, int which, const std::vector<double>& omega) {
    const Config& c = g.cfg;
    long nd = g.ndofs();
    double total = 0.0;
    for (int e = 0; e < g.nelem; ++e) {
        long b = (long)e * g.npe;
        double se = 0.0;
        for (int i = 0; i < g.npe; ++i) {
            Vec<double> q = getv(Q, nd, b + i, c.nv);
            double f;
            if (which == 1) {
                double m2 = sq(q[1]);
                for (int k = 1; k < c.dim; ++k) m2 = m2 + sq(q[1 + k]);
                f = m2 / (2.0 * q[0]);
            } else {
                double pr = pressure(q, c.dim, c.gamma);
                double sv = std::log(pr) - c.gamma * std::log(q[0]);
                f = -q[0] * sv / (c.gamma - 1.0);
            }
            se = se + (g.J[b + i] * omega[i]) * f;
        }
        total = total + se;
    }
    return total;
}

// SSP-RK3 with the limiter as OrdinaryDiffEq's stage_limiter! (FlouTime.jl:136-148): applied
// to U1, U2 and the new state.
template <class T>
void ssprk3_step_limited(const Disc& g, T* Q, double dt, double t, Workspace<T>& ws, std::vector<T>& U,
                         std::vector<T>& L, double minval, const std::vector<double>& omega,
                         const T* celem = nullptr) {
    long N = g.ndofs() * g.cfg.nv;
    U.resize(N);
    L.resize(N);
    rhs(g, L.data(), Q, t, ws, celem);
    for (long i = 0; i < N; ++i) U[i] = Q[i] + dt * L[i];
    zhang_shu(g, U.data(), minval, omega);
    rhs(g, L.data(), U.data(), t + dt, ws, celem);
    for (long i = 0; i < N; ++i) U[i] = 0.75 * Q[i] + 0.25 * (U[i] + dt * L[i]);
    zhang_shu(g, U.data(), minval, omega);
    rhs(g, L.data(), U.data(), t + 0.5 * dt, ws, celem);
    for (long i = 0; i < N; ++i) Q[i] = (1.0 / 3.0) * Q[i] + (2.0 / 3.0) * (U[i] + dt * L[i]);
    zhang_shu(g, Q, minval, omega);
}

// Williamson (1980) 2N-storage Runge-Kutta, the form of OrdinaryDiffEq 6.49.1's LowStorageRK2N
// methods (ORK256, CarpenterKennedy2N54) with williamson_condition = false, which the reference's
// tests and examples step with (test/tests.jl:19,56,93,139; examples/src/3D_Euler.jl:77):
//   k = dt L(u); u = u + B_1 k;   for i = 2..s: k = A_i k + dt L(u, t + c_i dt); u = u + B_i k.
// The stage limiter, when `omega` is given, acts on u after every stage.
// T = Dual: forward-mode derivatives, with the per-element dissipation scales celem.
template <class T>
void lsrk2n_step(const Disc& g, T* Q, double dt, double t, Workspace<T>& ws, std::vector<T>& K, std::vector<T>& L,
                 int s, const double* A, const double* B, const double* c, double minval = 0.0,
                 const std::vector<double>* omega = nullptr, const T* celem = nullptr) {
    long N = g.ndofs() * g.cfg.nv;
    K.resize(N);
    L.resize(N);
    for (int st = 0; st < s; ++st) {
        rhs(g, L.data(), Q, t + c[st] * dt, ws, celem);
        if (st == 0) {
#pragma omp parallel for schedule(static)
            for (long i = 0; i < N; ++i) K[i] = dt * L[i];
        } else {
#pragma omp parallel for schedule(static)
            for (long i = 0; i < N; ++i) K[i] = A[st] * K[i] + dt * L[i];
        }
#pragma omp parallel for schedule(static)
        for (long i = 0; i < N; ++i) Q[i] = Q[i] + B[st] * K[i];
        if (omega) zhang_shu(g, Q, minval, *omega);
    }
}

// get_max_dt, MultielementDiscontinuous.jl:162-178 with the pointwise estimates of
// src/FlouCommon/Euler.jl:116-135, LinearAdvection.jl:46-48, Burgers.jl:35-37 (no abs, as
// in the reference).  `omega` holds the tensor-product quadrature weights per element node.
inline double get_max_dt(const Disc& g, const double* Q, double cfl, const std::vector<double>& omega) {
    const Config& c = g.cfg;
    double dt = INFINITY;
    long nd = g.ndofs();
    for (int e = 0; e < g.nelem; ++e) {
        double vol = 0.0;
        for (int i = 0; i < g.npe; ++i) vol += g.J[(long)e * g.npe + i] * omega[i];
        double dx = vol / g.npe;
        dx = c.dim == 1 ? dx : (c.dim == 2 ? std::sqrt(dx) : std::cbrt(dx));
        for (int i = 0; i < g.npe; ++i) {
            long idx = (long)e * g.npe + i;
            double v;
            if (c.eq == EQ_ADVECTION) {
                double an = 0;
                for (int d = 0; d < c.dim; ++d) an += c.a[d] * c.a[d];
                v = cfl * dx / std::sqrt(an);
            } else if (c.eq == EQ_BURGERS) {
                v = cfl * dx / Q[idx];
            } else {
                Vec<double> q = getv(Q, nd, idx, c.nv);
                double p = pressure(q, c.dim, c.gamma);
                double a = std::sqrt(c.gamma * p / q[0]);
                double s = 0;
                for (int d = 0; d < c.dim; ++d) s += sq(q[1 + d] / q[0]);
                double speed = c.dim == 1 ? std::fabs(q[1] / q[0]) : std::sqrt(s);
                v = cfl * dx / (speed + a);
            }
            dt = std::min(dt, v);
        }
    }
    return dt;
}

}  // namespace oracle
