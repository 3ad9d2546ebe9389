// oracle_capi.cpp -- TEST INFRASTRUCTURE ONLY: C entry points over flou_oracle.hpp so the
// Python tests can drive the CPU restatement of Flou.jl through ctypes.  Not part of the
// product; the CUDA library never links or calls it.
#include <omp.h>

#include <cstdio>

#include "flou_oracle.hpp"

using namespace oracle;

// ---------------------------------------------------------------------------------------
// Counting scalar: every + - * is one flop, divisions / sqrt / log tallied separately.
// Used to measure the algorithmic operation count of the reference's residual.
// ---------------------------------------------------------------------------------------
struct OpCount { long long add = 0, mul = 0, div = 0, sqrt = 0, log = 0, cmp = 0; };
static OpCount g_count;

struct CD {
    double v = 0;
    CD() = default;
    CD(double x) : v(x) {}
};
static inline CD operator+(CD a, CD b) { g_count.add++; return CD(a.v + b.v); }
static inline CD operator-(CD a, CD b) { g_count.add++; return CD(a.v - b.v); }
static inline CD operator*(CD a, CD b) { g_count.mul++; return CD(a.v * b.v); }
static inline CD operator/(CD a, CD b) { g_count.div++; return CD(a.v / b.v); }
static inline CD operator-(CD a) { return CD(-a.v); }
static inline CD operator+(CD a, double b) { return a + CD(b); }
static inline CD operator-(CD a, double b) { return a - CD(b); }
static inline CD operator*(CD a, double b) { return a * CD(b); }
static inline CD operator/(CD a, double b) { return a / CD(b); }
static inline CD operator+(double a, CD b) { return CD(a) + b; }
static inline CD operator-(double a, CD b) { return CD(a) - b; }
static inline CD operator*(double a, CD b) { return CD(a) * b; }
static inline CD operator/(double a, CD b) { return CD(a) / b; }
static inline bool operator<(CD a, CD b) { g_count.cmp++; return a.v < b.v; }
static inline bool operator<(CD a, double b) { g_count.cmp++; return a.v < b; }
static inline bool operator>=(CD a, double b) { g_count.cmp++; return a.v >= b; }
static inline bool operator<=(CD a, double b) { g_count.cmp++; return a.v <= b; }
static inline CD sqrt(CD a) { g_count.sqrt++; return CD(std::sqrt(a.v)); }
static inline CD log(CD a) { g_count.log++; return CD(std::log(a.v)); }
static inline CD fabs(CD a) { return CD(std::fabs(a.v)); }
static inline CD exp(CD a) { g_count.log++; return CD(std::exp(a.v)); }
static inline CD pow(CD a, double b) { g_count.log++; return CD(std::pow(a.v, b)); }
namespace std {
static inline CD min(CD a, CD b) { g_count.cmp++; return a.v < b.v ? a : b; }
static inline CD max(CD a, CD b) { g_count.cmp++; return a.v < b.v ? b : a; }
}  // namespace std

// ---------------------------------------------------------------------------------------
// Forward-mode dual number (value, directional derivative): the derivative checks of the
// adjoint run the oracle with it, the role ForwardDiff plays on the reference's CPU path.
// Non-smooth points follow Base's conventions: max(a, b) = b unless b < a, abs' = sign with
// abs'(+0) = 1.
// ---------------------------------------------------------------------------------------
struct Dual {
    double v = 0, d = 0;
    Dual() = default;
    Dual(double x) : v(x), d(0) {}
    Dual(double x, double dx) : v(x), d(dx) {}
};
static inline Dual operator+(Dual a, Dual b) { return Dual(a.v + b.v, a.d + b.d); }
static inline Dual operator-(Dual a, Dual b) { return Dual(a.v - b.v, a.d - b.d); }
static inline Dual operator*(Dual a, Dual b) { return Dual(a.v * b.v, a.d * b.v + a.v * b.d); }
static inline Dual operator/(Dual a, Dual b) { return Dual(a.v / b.v, (a.d * b.v - a.v * b.d) / (b.v * b.v)); }
static inline Dual operator-(Dual a) { return Dual(-a.v, -a.d); }
static inline Dual operator+(Dual a, double b) { return Dual(a.v + b, a.d); }
static inline Dual operator-(Dual a, double b) { return Dual(a.v - b, a.d); }
static inline Dual operator*(Dual a, double b) { return Dual(a.v * b, a.d * b); }
static inline Dual operator/(Dual a, double b) { return Dual(a.v / b, a.d / b); }
static inline Dual operator+(double a, Dual b) { return Dual(a + b.v, b.d); }
static inline Dual operator-(double a, Dual b) { return Dual(a - b.v, -b.d); }
static inline Dual operator*(double a, Dual b) { return Dual(a * b.v, a * b.d); }
static inline Dual operator/(double a, Dual b) { return Dual(a / b.v, -a * b.d / (b.v * b.v)); }
static inline bool operator<(Dual a, Dual b) { return a.v < b.v; }
static inline bool operator<(Dual a, double b) { return a.v < b; }
static inline bool operator>=(Dual a, double b) { return a.v >= b; }
static inline bool operator<=(Dual a, double b) { return a.v <= b; }
static inline Dual sqrt(Dual a) { double s = std::sqrt(a.v); return Dual(s, a.d / (2.0 * s)); }
static inline Dual log(Dual a) { return Dual(std::log(a.v), a.d / a.v); }
static inline Dual fabs(Dual a) { return std::signbit(a.v) ? -a : a; }
static inline Dual exp(Dual a) { double e = std::exp(a.v); return Dual(e, e * a.d); }
static inline Dual pow(Dual a, double b) { double p = std::pow(a.v, b); return Dual(p, b * std::pow(a.v, b - 1.0) * a.d); }
namespace std {
static inline Dual min(Dual a, Dual b) { return b.v < a.v ? b : a; }
static inline Dual max(Dual a, Dual b) { return b.v < a.v ? a : b; }
}  // namespace std

extern "C" {

void oracle_set_threads(int n) { omp_set_num_threads(n > 0 ? n : 1); }
int oracle_max_threads() { return omp_get_max_threads(); }

// ------------------------------- mesh ------------------------------------------------
void* oracle_mesh_new(int dim, const double* start, const double* finish, const int* n, int nperiodic,
                      const int* pairs) {
    try {
        Mesh* m = new Mesh(cartesian_mesh(dim, start, finish, n));
        std::vector<std::pair<int, int>> p;
        for (int i = 0; i < nperiodic; ++i) p.push_back({pairs[2 * i], pairs[2 * i + 1]});
        if (nperiodic) apply_periodic(*m, p);
        return m;
    } catch (std::exception& e) {
        std::fprintf(stderr, "oracle_mesh_new: %s\n", e.what());
        return nullptr;
    }
}
void oracle_mesh_free(void* h) { delete (Mesh*)h; }
void oracle_mesh_sizes(void* h, int* nelem, int* nfaces, int* nint, int* nbd_lists) {
    Mesh* m = (Mesh*)h;
    *nelem = m->nelem();
    *nfaces = m->nfaces();
    *nint = (int)m->intfaces.size();
    *nbd_lists = (int)m->bdfaces.size();
}
// Connectivity in the reference's own 1-based form, plus bdid[f] = boundary index (1-based)
// for boundary faces, 0 otherwise, and bdindex_of_id[id-1] = bdmap[id] (0 when periodic).
void oracle_mesh_get(void* h, int* faceinds, int* facepos, int* eleminds, int* elempos, unsigned char* orient,
                     int* bdid, int* intfaces, int* bdindex_of_id) {
    Mesh* m = (Mesh*)h;
    std::copy(m->e_faceinds.begin(), m->e_faceinds.end(), faceinds);
    std::copy(m->e_facepos.begin(), m->e_facepos.end(), facepos);
    std::copy(m->f_eleminds.begin(), m->f_eleminds.end(), eleminds);
    std::copy(m->f_elempos.begin(), m->f_elempos.end(), elempos);
    std::copy(m->f_orient.begin(), m->f_orient.end(), orient);
    std::copy(m->intfaces.begin(), m->intfaces.end(), intfaces);
    for (int f = 0; f < m->nfaces(); ++f) bdid[f] = 0;
    for (size_t b = 0; b < m->bdfaces.size(); ++b)
        for (int f : m->bdfaces[b]) bdid[f - 1] = (int)b + 1;
    for (int id = 1; id <= 2 * m->dim; ++id) bdindex_of_id[id - 1] = m->bdmap.count(id) ? m->bdmap[id] : 0;
}

// Cartesian geometry (PhysicalRegions.jl:370-408 elements, :541-696 faces, Mesh.jl:364-487
// coordinates).  Outputs per node: J, Ja (dim x dim column-major), coords (3 per node);
// per face node: frames (n, t, b; 3 x 3 doubles), faceJ.
void oracle_geometry(void* h, int n, const double* xi, double* J, double* Ja, double* coords, double* frames,
                     double* faceJ) {
    Mesh* m = (Mesh*)h;
    int dim = m->dim;
    int npe = 1, nfd = 1;
    for (int d = 0; d < dim; ++d) npe *= n;
    for (int d = 0; d < dim - 1; ++d) nfd *= n;
    const double* dx = m->dx;
    double jac = dim == 1 ? dx[0] / 2 : (dim == 2 ? (dx[0] * dx[1]) / 4 : (dx[0] * dx[1] * dx[2]) / 8);
    double M[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    if (dim == 1) M[0] = 1.0;
    else if (dim == 2) { M[0] = dx[1] / 2; M[3] = dx[0] / 2; }
    else { M[0] = dx[1] * dx[2] / 4; M[4] = dx[0] * dx[2] / 4; M[8] = dx[0] * dx[1] / 4; }
    for (int e = 0; e < m->nelem(); ++e) {
        const int* nodes = &m->e_nodeinds[e * m->nvert_e];
        for (int i = 0; i < npe; ++i) {
            long g = (long)e * npe + i;
            J[g] = jac;
            for (int q = 0; q < dim * dim; ++q) Ja[g * dim * dim + q] = M[q];
            int ix = i % n, iy = (i / n) % n, iz = i / (n * n);
            double r[3] = {(xi[ix] + 1) / 2, dim > 1 ? (xi[iy] + 1) / 2 : 0.0, dim > 2 ? (xi[iz] + 1) / 2 : 0.0};
            for (int c = 0; c < 3; ++c) {
                auto X = [&](int v) { return m->nodes[nodes[v] - 1][c]; };
                double x;
                if (dim == 1) x = X(0) * (1 - r[0]) + X(1) * r[0];
                else if (dim == 2)
                    x = X(0) * (1 - r[0]) * (1 - r[1]) + X(1) * r[0] * (1 - r[1]) + X(2) * r[0] * r[1] +
                        X(3) * (1 - r[0]) * r[1];
                else
                    x = X(0) * (1 - r[0]) * (1 - r[1]) * (1 - r[2]) + X(1) * r[0] * (1 - r[1]) * (1 - r[2]) +
                        X(2) * r[0] * r[1] * (1 - r[2]) + X(3) * (1 - r[0]) * r[1] * (1 - r[2]) +
                        X(4) * (1 - r[0]) * (1 - r[1]) * r[2] + X(5) * r[0] * (1 - r[1]) * r[2] +
                        X(6) * r[0] * r[1] * r[2] + X(7) * (1 - r[0]) * r[1] * r[2];
                coords[g * 3 + c] = c < dim ? x : 0.0;
            }
        }
    }
    for (int f = 0; f < m->nfaces(); ++f) {
        int pos = m->elempos(f + 1, 1);
        double fr[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};   // n, t, b
        double fj = 1.0;
        auto set = [&](std::array<double, 3> nn, std::array<double, 3> tt, std::array<double, 3> bb) {
            for (int q = 0; q < 3; ++q) { fr[q] = nn[q]; fr[3 + q] = tt[q]; fr[6 + q] = bb[q]; }
        };
        if (dim == 1) {
            set({pos == 1 ? -1.0 : 1.0, 0, 0}, {0, 0, 0}, {0, 0, 0});
        } else if (dim == 2) {
            if (pos == 1) { fj = dx[1] / 2; set({-1, 0, 0}, {0, -1, 0}, {0, 0, 0}); }
            else if (pos == 2) { fj = dx[1] / 2; set({1, 0, 0}, {0, 1, 0}, {0, 0, 0}); }
            else if (pos == 3) { fj = dx[0] / 2; set({0, -1, 0}, {1, 0, 0}, {0, 0, 0}); }
            else { fj = dx[0] / 2; set({0, 1, 0}, {-1, 0, 0}, {0, 0, 0}); }
        } else {
            if (pos == 1) { fj = dx[1] * dx[2] / 4; set({-1, 0, 0}, {0, -1, 0}, {0, 0, 1}); }
            else if (pos == 2) { fj = dx[1] * dx[2] / 4; set({1, 0, 0}, {0, 1, 0}, {0, 0, 1}); }
            else if (pos == 3) { fj = dx[0] * dx[2] / 4; set({0, -1, 0}, {0, 0, -1}, {1, 0, 0}); }
            else if (pos == 4) { fj = dx[0] * dx[2] / 4; set({0, 1, 0}, {0, 0, 1}, {1, 0, 0}); }
            else if (pos == 5) { fj = dx[0] * dx[1] / 4; set({0, 0, -1}, {-1, 0, 0}, {0, 1, 0}); }
            else { fj = dx[0] * dx[1] / 4; set({0, 0, 1}, {1, 0, 0}, {0, 1, 0}); }
        }
        for (int q = 0; q < nfd; ++q) {
            long idx = (long)f * nfd + q;
            for (int c = 0; c < 9; ++c) frames[idx * 9 + c] = fr[c];
            faceJ[idx] = fj;
        }
    }
}

// ------------------------------- operators -------------------------------------------
void oracle_std_operators(int n, int lobatto, double* xi, double* omega, double* D, double* Ds, double* Dsharp,
                          double* ll, double* lr, double* dgl, double* dgr) {
    StdOps s = std_operators(n, lobatto != 0);
    std::copy(s.xi.begin(), s.xi.end(), xi);
    std::copy(s.omega.begin(), s.omega.end(), omega);
    std::copy(s.D.begin(), s.D.end(), D);
    std::copy(s.Ds.begin(), s.Ds.end(), Ds);
    std::copy(s.Dsharp.begin(), s.Dsharp.end(), Dsharp);
    std::copy(s.ll.begin(), s.ll.end(), ll);
    std::copy(s.lr.begin(), s.lr.end(), lr);
    std::copy(s.dgl.begin(), s.dgl.end(), dgl);
    std::copy(s.dgr.begin(), s.dgr.end(), dgr);
}

// ------------------------------- discretization --------------------------------------
struct Handle {
    Disc g;
    Workspace<double> ws;
    std::vector<double> U, L;
};

void* oracle_disc_new(int dim, int eq, double gamma, const double* adv, int volop, int tpflux, int numflux,
                      int lxf_avg, double intensity, int n, const double* Ds, const double* Dsharp, const double* ll,
                      const double* lr, const double* dgl, const double* dgr, int nelem, int nfaces,
                      const int* faceinds, const int* facepos, const int* eleminds, const int* elempos,
                      const unsigned char* orient, const int* bdid, int nbcs, const int* bc_kinds,
                      const double* bc_states, const double* J, const double* Ja, const double* frames,
                      const double* faceJ) {
    Handle* h = new Handle();
    Disc& g = h->g;
    Config& c = g.cfg;
    c.dim = dim;
    c.eq = eq;
    c.nv = eq == EQ_EULER ? dim + 2 : 1;
    c.gamma = gamma;
    for (int d = 0; d < 3; ++d) c.a[d] = adv ? adv[d] : 0.0;
    c.volop = volop;
    c.tpflux = tpflux;
    c.numflux = numflux;
    c.lxf_avg = lxf_avg;
    c.intensity = intensity;
    g.n = n;
    g.npe = 1;
    g.nfd = 1;
    for (int d = 0; d < dim; ++d) g.npe *= n;
    for (int d = 0; d < dim - 1; ++d) g.nfd *= n;
    g.nelem = nelem;
    g.nfaces = nfaces;
    g.Ds.assign(Ds, Ds + n * n);
    g.Dsharp.assign(Dsharp, Dsharp + n * n);
    g.ll.assign(ll, ll + n);
    g.lr.assign(lr, lr + n);
    g.dgl.assign(dgl, dgl + n);
    g.dgr.assign(dgr, dgr + n);
    // hasboundaries(basis): the end-node interpolation to round-off (operators fitted like the
    // reference's carry ~1e-16 in the entries that vanish on Gauss-Lobatto nodes)
    g.lobatto = std::fabs(ll[0] - 1.0) < 1e-10 && std::fabs(lr[n - 1] - 1.0) < 1e-10;
    for (int i = 0; i < n; ++i) {
        if (i != 0 && std::fabs(ll[i]) > 1e-10) g.lobatto = false;
        if (i != n - 1 && std::fabs(lr[i]) > 1e-10) g.lobatto = false;
    }
    g.faceinds.assign(faceinds, faceinds + nelem * 2 * dim);
    g.facepos.assign(facepos, facepos + nelem * 2 * dim);
    g.eleminds.assign(eleminds, eleminds + nfaces * 2);
    g.elempos.assign(elempos, elempos + nfaces * 2);
    g.orient.assign(orient, orient + nfaces);
    g.bdid.assign(bdid, bdid + nfaces);
    g.bcs.resize(nbcs);
    for (int b = 0; b < nbcs; ++b) {
        g.bcs[b].kind = bc_kinds[b];
        for (int k = 0; k < 5; ++k) g.bcs[b].state[k] = bc_states[b * 5 + k];
    }
    long nd = g.ndofs(), nf = g.nfdofs();
    g.J.assign(J, J + nd);
    g.Ja.assign(Ja, Ja + nd * dim * dim);
    g.frames.resize(nf);
    for (long i = 0; i < nf; ++i)
        for (int q = 0; q < 3; ++q) {
            g.frames[i].n[q] = frames[i * 9 + q];
            g.frames[i].t[q] = frames[i * 9 + 3 + q];
            g.frames[i].b[q] = frames[i * 9 + 6 + q];
        }
    g.faceJ.assign(faceJ, faceJ + nf);
    return h;
}

void oracle_disc_free(void* h) { delete (Handle*)h; }

int oracle_rhs(void* hp, double* dQ, const double* Q, double t) {
    Handle* h = (Handle*)hp;
    try {
        rhs(h->g, dQ, Q, t, h->ws);
    } catch (std::exception& e) {
        std::fprintf(stderr, "oracle_rhs: %s\n", e.what());
        return 1;
    }
    return 0;
}

int oracle_ssprk3(void* hp, double* Q, double dt, int nsteps, double t0) {
    Handle* h = (Handle*)hp;
    try {
        for (int s = 0; s < nsteps; ++s) ssprk3_step(h->g, Q, dt, t0 + s * dt, h->ws, h->U, h->L);
    } catch (std::exception& e) {
        std::fprintf(stderr, "oracle_ssprk3: %s\n", e.what());
        return 1;
    }
    return 0;
}

// `nsteps` steps of a 2N-storage Runge-Kutta method with `nstages` stages (A[0] unused); with
// omega_tp set, the Zhang-Shu limiter with `minval` after every stage.
int oracle_lsrk2n(void* hp, double* Q, double dt, int nsteps, double t0, int nstages, const double* A,
                  const double* B, const double* c, double minval, const double* omega_tp) {
    Handle* h = (Handle*)hp;
    std::vector<double> w;
    if (omega_tp) w.assign(omega_tp, omega_tp + h->g.npe);
    try {
        for (int s = 0; s < nsteps; ++s)
            lsrk2n_step(h->g, Q, dt, t0 + s * dt, h->ws, h->U, h->L, nstages, A, B, c, minval,
                        omega_tp ? &w : nullptr);
    } catch (std::exception& e) {
        std::fprintf(stderr, "oracle_lsrk2n: %s\n", e.what());
        return 1;
    }
    return 0;
}

// HybridDivOperator parameters: the subcell FV flux (kind, its central flux, intensity), the
// blending constant, the 1D weights and the derivative matrix (n x n, column-major).
void oracle_set_hybrid(void* hp, int fvflux, int fvavg, double fvintensity, double blend, const double* omega1d,
                       const double* D) {
    Handle* h = (Handle*)hp;
    Config& c = h->g.cfg;
    c.fvflux = fvflux;
    c.fvavg = fvavg;
    c.fvintensity = fvintensity;
    c.blend = blend;
    int n = h->g.n;
    h->g.omega1d.assign(omega1d, omega1d + n);
    h->g.D.assign(D, D + (size_t)n * n);
}

// Subcell-interface frames (9 doubles per point) and surface Jacobians of general elements, in
// the layout of flou_set_subgrid.
void oracle_set_subgrid(void* hp, const double* frames, const double* jac) {
    Handle* h = (Handle*)hp;
    Disc& g = h->g;
    size_t ns = (size_t)g.nelem * g.cfg.dim * g.nfd * (g.n + 1);
    g.subframes.resize(ns);
    g.subjac.assign(jac, jac + ns);
    for (size_t i = 0; i < ns; ++i)
        for (int q = 0; q < 3; ++q) {
            g.subframes[i].n[q] = frames[9 * i + q];
            g.subframes[i].t[q] = frames[9 * i + 3 + q];
            g.subframes[i].b[q] = frames[9 * i + 6 + q];
        }
}

// External states of the BC_STATE_FIELD boundaries, 5 per face node (flou_set_bc_field's layout).
void oracle_set_bc_field(void* hp, const double* states) {
    Handle* h = (Handle*)hp;
    h->g.bcfield.assign(states, states + 5 * (size_t)h->g.nfdofs());
}

void oracle_limit(void* hp, double* Q, double minval, const double* omega_tp) {
    Handle* h = (Handle*)hp;
    std::vector<double> w(omega_tp, omega_tp + h->g.npe);
    zhang_shu(h->g, Q, minval, w);
}

double oracle_monitor(void* hp, const double* Q, int which, const double* omega_tp) {
    Handle* h = (Handle*)hp;
    std::vector<double> w(omega_tp, omega_tp + h->g.npe);
    return monitor(h->g, Q, which, w);
}

int oracle_ssprk3_limited(void* hp, double* Q, double dt, int nsteps, double t0, double minval,
                          const double* omega_tp) {
    Handle* h = (Handle*)hp;
    std::vector<double> w(omega_tp, omega_tp + h->g.npe);
    try {
        for (int s = 0; s < nsteps; ++s)
            ssprk3_step_limited(h->g, Q, dt, t0 + s * dt, h->ws, h->U, h->L, minval, w);
    } catch (std::exception& e) {
        std::fprintf(stderr, "oracle_ssprk3_limited: %s\n", e.what());
        return 1;
    }
    return 0;
}

double oracle_max_dt(void* hp, const double* Q, double cfl, const double* omega_tp) {
    Handle* h = (Handle*)hp;
    std::vector<double> w(omega_tp, omega_tp + h->g.npe);
    return get_max_dt(h->g, Q, cfl, w);
}

// Directional derivative of one residual: rhs(Q + ε dQ, c + ε dc) -> (R, dR).  c may be null
// (then the configured LxF intensity, no derivative).
void oracle_rhs_jvp(void* hp, const double* Q, const double* dQ, const double* c, const double* dc, double* R,
                    double* dR) {
    Handle* h = (Handle*)hp;
    long N = h->g.ndofs() * h->g.cfg.nv;
    std::vector<Dual> q(N), r(N), ce;
    for (long i = 0; i < N; ++i) q[i] = Dual(Q[i], dQ ? dQ[i] : 0.0);
    if (c) {
        ce.resize(h->g.nelem);
        for (int e = 0; e < h->g.nelem; ++e) ce[e] = Dual(c[e], dc ? dc[e] : 0.0);
    }
    Workspace<Dual> ws;
    rhs(h->g, r.data(), q.data(), 0.0, ws, c ? ce.data() : nullptr);
    for (long i = 0; i < N; ++i) { R[i] = r[i].v; dR[i] = r[i].d; }
}

// Terminal functional J = 1/2 Σ_i w_i (ρ_i(T) - ρt_i)² after `nsteps` SSP-RK3 steps from Q0 with
// dissipation scales c, and its directional derivative along (dQ0, dc).
void oracle_solve_jvp(void* hp, const double* Q0, const double* dQ0, const double* c, const double* dc, double dt,
                      int nsteps, const double* rho_t, const double* w, double* J, double* dJ) {
    Handle* h = (Handle*)hp;
    long nd = h->g.ndofs(), N = nd * h->g.cfg.nv;
    std::vector<Dual> q(N), ce, U, L;
    for (long i = 0; i < N; ++i) q[i] = Dual(Q0[i], dQ0 ? dQ0[i] : 0.0);
    if (c) {
        ce.resize(h->g.nelem);
        for (int e = 0; e < h->g.nelem; ++e) ce[e] = Dual(c[e], dc ? dc[e] : 0.0);
    }
    Workspace<Dual> ws;
    for (int s = 0; s < nsteps; ++s) ssprk3_step(h->g, q.data(), dt, s * dt, ws, U, L, c ? ce.data() : nullptr);
    Dual acc(0.0);
    for (long i = 0; i < nd; ++i) {
        Dual r = q[i] - rho_t[i];
        acc = acc + (0.5 * w[i]) * (r * r);
    }
    *J = acc.v;
    *dJ = acc.d;
}

// The same for nsteps steps of a 2N-storage method (nstages, A, B, c as oracle_lsrk2n; nstages = 0:
// SSP-RK3), with the Zhang-Shu stage limiter when omega_tp is given.
void oracle_solve_jvp_lsrk(void* hp, const double* Q0, const double* dQ0, const double* c, const double* dc,
                           double dt, int nsteps, const double* rho_t, const double* w, int nstages, const double* A,
                           const double* B, const double* cst, double* J, double* dJ, double minval = 0.0,
                           const double* omega_tp = nullptr) {
    Handle* h = (Handle*)hp;
    long nd = h->g.ndofs(), N = nd * h->g.cfg.nv;
    std::vector<Dual> q(N), ce, K, L;
    for (long i = 0; i < N; ++i) q[i] = Dual(Q0[i], dQ0 ? dQ0[i] : 0.0);
    if (c) {
        ce.resize(h->g.nelem);
        for (int e = 0; e < h->g.nelem; ++e) ce[e] = Dual(c[e], dc ? dc[e] : 0.0);
    }
    Workspace<Dual> ws;
    std::vector<double> om;
    if (omega_tp) om.assign(omega_tp, omega_tp + h->g.npe);
    for (int s = 0; s < nsteps; ++s) {
        if (nstages == 0 && omega_tp)
            ssprk3_step_limited(h->g, q.data(), dt, s * dt, ws, K, L, minval, om, c ? ce.data() : nullptr);
        else if (nstages == 0)
            ssprk3_step(h->g, q.data(), dt, s * dt, ws, K, L, c ? ce.data() : nullptr);
        else
            lsrk2n_step(h->g, q.data(), dt, s * dt, ws, K, L, nstages, A, B, cst, minval, omega_tp ? &om : nullptr,
                        c ? ce.data() : nullptr);
    }
    Dual acc(0.0);
    for (long i = 0; i < nd; ++i) {
        Dual r = q[i] - rho_t[i];
        acc = acc + (0.5 * w[i]) * (r * r);
    }
    *J = acc.v;
    *dJ = acc.d;
}

// Operation count of one residual evaluation (single thread).  out = {add, mul, div, sqrt,
// log, cmp}.
void oracle_count_rhs(void* hp, const double* Q, double t, long long* out) {
    Handle* h = (Handle*)hp;
    int nt = omp_get_max_threads();
    omp_set_num_threads(1);
    long N = h->g.ndofs() * h->g.cfg.nv;
    std::vector<CD> q(N), dq(N);
    for (long i = 0; i < N; ++i) q[i] = CD(Q[i]);
    Workspace<CD> ws;
    g_count = OpCount();
    rhs(h->g, dq.data(), q.data(), t, ws);
    out[0] = g_count.add; out[1] = g_count.mul; out[2] = g_count.div;
    out[3] = g_count.sqrt; out[4] = g_count.log; out[5] = g_count.cmp;
    omp_set_num_threads(nt);
}

}  // extern "C"
