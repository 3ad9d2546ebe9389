"""The oracle against the reference's own known-answer tests and the invariants of the
scheme.  Pins: the golden values of the Sod tube and the 2D normal shock (test/runtests.jl:34-45,
rtol 1e-7: split form and hybrid operator with MatrixDissipation, GenericBC, ORK256); the
Advection1D / Advection2D period property (test/tests.jl:16-88, test/runtests.jl:23-32:
u(T) ≈ u(0), rtol 1e-3) with ORK256 at the reference's dt; freestream preservation; discrete
conservation; entropy conservation of the split form with entropy-conserving fluxes; the
convergence order of examples/src/Convergence.jl."""
import numpy as np
import pytest

import flou_cuda as F
import oracle_ref
import reference_problems as RP
from cases import build, oracle_for, smooth_euler_state

ORK = F.ORK256()


def _norm_close(a, b, rtol):   # Julia's isapprox for arrays: norm(a-b) <= rtol*max(norm(a), norm(b))
    return np.linalg.norm(a - b) <= rtol * max(np.linalg.norm(a), np.linalg.norm(b))


def _oracle_disc(disc, lobatto):
    """Oracle fed with the operators built by its own (reference) construction."""
    a = disc.abi_arrays()
    o = oracle_ref.operators(disc.std.n, lobatto)
    for k in ("D", "Ds", "Dsharp", "omega", "l_l", "l_r", "dg_l", "dg_r"):
        a[k] = o[k]
    return oracle_for(disc, a)


def test_advection1d_period():
    """Advection1D: GL n=5, 20 elements on [0,1], a=2, LxF(StdAverage,1), dt=1e-3, t=0.5."""
    eq = F.LinearAdvection(2.0)
    disc = build(1, 5, (20,), eq, F.StrongDivOperator(F.LxF(F.StdAverage(), 1.0)), basis="GL",
                 box=((0.0,), (1.0,)))
    Q0 = np.asfortranarray(F.initial.gaussian_bump(disc.coords, (0.5,), (0.1,), 1.0)[:, None])
    o = _oracle_disc(disc, lobatto=False)
    Q = o.lsrk2n(Q0, 1e-3, 500, ORK.A, ORK.B, ORK.c)
    assert _norm_close(Q, Q0, 1e-3)
    assert not np.allclose(o.lsrk2n(Q0, 1e-3, 250, ORK.A, ORK.B, ORK.c), Q0, rtol=1e-3)   # it did move
    assert _norm_close(o.ssprk3(Q0, 1e-3, 500), Q0, 1e-3)   # and so does SSP-RK3 at that dt


def test_advection2d_period():
    """Advection2D: GL n=5, 20x10 elements on [0,1.5]x[0,2], a=(3,4), dt=1e-3, t=0.5."""
    eq = F.LinearAdvection(3.0, 4.0)
    disc = build(2, 5, (20, 10), eq, F.StrongDivOperator(F.LxF(F.StdAverage(), 1.0)), basis="GL",
                 box=((0.0, 0.0), (1.5, 2.0)))
    Q0 = np.asfortranarray(F.initial.gaussian_bump(disc.coords[:, :2], (0.75, 1.0), (0.2, 0.2), 1.0)[:, None])
    o = _oracle_disc(disc, lobatto=False)
    Q = o.lsrk2n(Q0, 1e-3, 500, ORK.A, ORK.B, ORK.c)
    assert _norm_close(Q, Q0, 1e-3)


def test_sod_tube_golden():
    """SodTube1D (test/tests.jl:90-134) hits the reference's golden min / max (rtol 1e-7)."""
    disc, Q0, dt, tf = RP.sod_tube()
    o = _oracle_disc(disc, lobatto=True)
    Q = o.lsrk2n(Q0, dt, int(round(tf / dt)), ORK.A, ORK.B, ORK.c)
    assert RP.isclose(Q.min(), RP.SOD_MIN, 1e-7), Q.min()
    assert RP.isclose(Q.max(), RP.SOD_MAX, 1e-7), Q.max()


def test_shockwave2d_golden():
    """Shockwave2D (test/tests.jl:136-181), the hybrid operator, hits the reference's golden
    maximum (rtol 1e-7) and its minimum test (rtol 1: a round-off y-momentum of either sign
    passes when it is negative, as the reference's is)."""
    disc, Q0, dt, tf = RP.shockwave_2d()
    o = _oracle_disc(disc, lobatto=True)
    Q = o.lsrk2n(Q0, dt, int(round(tf / dt)), ORK.A, ORK.B, ORK.c)
    assert RP.isclose(Q.max(), RP.SHOCK_MAX, 1e-7), Q.max()
    assert RP.isclose(Q.min(), RP.SHOCK_MIN, 1.0), Q.min()


def test_low_storage_tableaux_orders():
    """ORK256 is second order and CarpenterKennedy2N54 fourth order: the order conditions of
    the Butcher tableau equivalent to each 2N-storage form (ORK256's five-digit coefficients
    meet b·c = 1/2 to 6e-7)."""
    def butcher(m):
        s = len(m.B)
        alpha, beta = np.zeros((s, s)), np.zeros((s + 1, s))
        for i in range(s):
            alpha[i] = (m.A[i] * alpha[i - 1] if i else 0.0) + np.eye(s)[i]
            beta[i + 1] = beta[i] + m.B[i] * alpha[i]
        return beta[:s], beta[s]
    a, b = butcher(F.ORK256())
    c = a.sum(1)
    assert abs(b.sum() - 1) < 1e-15 and abs(b @ c - 0.5) < 1e-6
    assert np.allclose(c, F.ORK256().c, atol=1e-15)
    a, b = butcher(F.CarpenterKennedy2N54())
    c = a.sum(1)
    conds = [(b.sum(), 1), (b @ c, 1 / 2), (b @ c ** 2, 1 / 3), (b @ a @ c, 1 / 6), (b @ c ** 3, 1 / 4),
             (b @ (c * (a @ c)), 1 / 8), (b @ a @ c ** 2, 1 / 12), (b @ a @ a @ c, 1 / 24)]
    for got, want in conds:
        assert abs(got - want) < 1e-14


@pytest.mark.parametrize("dim,n,vol", [(1, 5, "strong"), (2, 4, "strong"), (2, 5, "split"), (3, 3, "split"),
                                       (3, 4, "strong")])
def test_freestream_and_conservation(dim, n, vol):
    eq = F.EulerEquation(dim, 1.4)
    if vol == "strong":
        op = F.StrongDivOperator(F.LxF(F.StdAverage(), 1.0))
    else:
        op = F.SplitDivOperator(F.ChandrasekharAverage(), F.HLLC())
    disc = build(dim, n, (3,) * dim, eq, op)
    o = oracle_for(disc)
    P = np.zeros((disc.ndofs, dim + 2))
    P[:, 0], P[:, 1:1 + dim], P[:, -1] = 1.3, 0.4, 2.0
    Qf = np.asfortranarray(eq.vars_prim2cons(P))
    assert np.max(np.abs(o.rhs(Qf))) < 1e-12
    Q = smooth_euler_state(disc, seed=1)
    dQ = o.rhs(Q)
    w = np.tile(disc.std.omega, disc.mesh.nelements) * disc.J
    for v in range(dim + 2):
        assert abs(w @ dQ[:, v]) < 1e-12 * np.sum(w * np.abs(dQ[:, v]))


def test_entropy_conservation_split_form():
    """Split form with Chandrashekar volume and interface fluxes conserves entropy (2D)."""
    eq = F.EulerEquation(2, 1.4)
    disc = build(2, 5, (3, 3), eq, F.SplitDivOperator(F.ChandrasekharAverage(), F.ChandrasekharAverage()))
    o = oracle_for(disc)
    Q = smooth_euler_state(disc, seed=3, amp=0.2)
    dQ = o.rhs(Q)
    g = eq.gamma
    p = eq.pressure(Q)
    s = np.log(p) - g * np.log(Q[:, 0])
    W = np.stack([(g - s) / (g - 1) - (Q[:, 1] ** 2 + Q[:, 2] ** 2) / Q[:, 0] / (2 * p), Q[:, 1] / p, Q[:, 2] / p,
                  -Q[:, 0] / p], axis=1)
    w = np.tile(disc.std.omega, disc.mesh.nelements) * disc.J
    dS = w @ np.sum(W * dQ, axis=1)
    scale = w @ np.sum(np.abs(W * dQ), axis=1)
    # exact up to the truncated log-mean series (relative error <= u^4/9 for u < 0.01)
    assert abs(dS) < 1e-10 * scale


def test_convergence_order():
    """1D Euler, smooth solution 2 + sin(π(x - t)) with u = p = 1 (examples/src/Convergence.jl),
    LGL p=3, split form with LxF(Chandrashekar): the error falls like h^(p+1)."""
    eq = F.EulerEquation(1, 1.4)
    errs = []
    for ne in (8, 16):
        disc = build(1, 4, (ne,), eq, F.SplitDivOperator(F.LxF(F.ChandrasekharAverage(), 1.0)))
        x = disc.coords[:, 0]
        sol = lambda t: np.asfortranarray(eq.vars_prim2cons(np.stack([2 + np.sin(np.pi * (x - t)),
                                                                      np.ones_like(x), np.ones_like(x)], 1)))
        o = oracle_for(disc)
        dt, T = 1e-3, 0.2
        Q = o.ssprk3(sol(0.0), dt, int(round(T / dt)))
        errs.append(np.sqrt(np.mean((Q - sol(T)) ** 2)))
    rate = np.log2(errs[0] / errs[1])
    assert rate > 3.3, (errs, rate)


def test_oracle_max_dt_formula():
    eq = F.EulerEquation(2, 1.4)
    disc = build(2, 5, (4, 4), eq, F.StrongDivOperator(F.LxF(F.StdAverage(), 1.0)),
                 box=((-5.0, -5.0), (5.0, 5.0)))
    Q = np.asfortranarray(F.initial.isentropic_vortex(eq, disc.coords, (0.3, -0.2), period=(10, 10)))
    o = oracle_for(disc)
    dt = o.max_dt(Q, 0.5, disc.std.omega)
    P = eq.vars_cons2prim(Q)
    c = np.sqrt(1.4 * P[:, 3] / P[:, 0])
    ref = np.min(0.5 * np.sqrt(2.5 ** 2 / 25) / (np.hypot(P[:, 1], P[:, 2]) + c))
    assert abs(dt - ref) < 1e-14 * ref


def _entropy_rate(disc, Q, dQ):
    """Σ_i J ω W(Q_i)·dQ_i: the semi-discrete rate of the total mathematical entropy."""
    eq = disc.equation
    d = disc.mesh.dim
    g = eq.gamma
    p = eq.pressure(Q)
    s = np.log(p) - g * np.log(Q[:, 0])
    m2 = np.sum(Q[:, 1:1 + d] ** 2, axis=1)
    W = np.concatenate([((g - s) / (g - 1) - m2 / Q[:, 0] / (2 * p))[:, None], Q[:, 1:1 + d] / p[:, None],
                        (-Q[:, 0] / p)[:, None]], axis=1)
    w = np.tile(disc.std.omega, disc.mesh.nelements) * disc.J
    return w @ np.sum(W * dQ, axis=1), w @ np.sum(np.abs(W * dQ), axis=1)


@pytest.mark.parametrize("flux,dim", [("matrix", 1), ("matrix", 2), ("matrix", 3), ("scalar", 1), ("scalar", 2)])
def test_dissipative_fluxes_are_entropy_stable(flux, dim):
    """Split form with the Chandrashekar volume flux and ScalarDissipation / MatrixDissipation of
    the Chandrashekar average at the interfaces: the entropy can only decrease (Euler.jl:228-380),
    and it does decrease when the traces jump.  (The 3D ScalarDissipation of the reference takes
    the left momenta from the right state, Euler.jl:257, so its sign is not guaranteed there.)"""
    eq = F.EulerEquation(dim, 1.4)
    nf = (F.MatrixDissipation if flux == "matrix" else F.ScalarDissipation)(F.ChandrasekharAverage(), 1.0)
    disc = build(dim, 4, (3,) * dim, eq, F.SplitDivOperator(F.ChandrasekharAverage(), nf))
    o = oracle_for(disc)
    Q = smooth_euler_state(disc, seed=5, amp=0.3)
    dS0, scale0 = _entropy_rate(disc, Q, o.rhs(Q))   # LGL traces of a pointwise state do not jump
    assert abs(dS0) < 1e-10 * scale0
    # element-wise jumps: a different constant offset of the primitive variables per element
    rng = np.random.default_rng(11)
    P = eq.vars_cons2prim(Q)
    npe = disc.std.n ** dim
    P += np.repeat(0.05 * rng.standard_normal((disc.mesh.nelements, dim + 2)), npe, axis=0)
    Qj = np.asfortranarray(eq.vars_prim2cons(P))
    dS, scale = _entropy_rate(disc, Qj, o.rhs(Qj))
    assert dS < -1e-6 * scale, (dS, scale)
    # freestream preservation and conservation
    P = np.zeros((disc.ndofs, dim + 2))
    P[:, 0], P[:, 1:1 + dim], P[:, -1] = 1.3, 0.4, 2.0
    assert np.max(np.abs(o.rhs(np.asfortranarray(eq.vars_prim2cons(P))))) < 1e-12
    dQ = o.rhs(Q)
    w = np.tile(disc.std.omega, disc.mesh.nelements) * disc.J
    for v in range(dim + 2):
        assert abs(w @ dQ[:, v]) < 1e-12 * np.sum(w * np.abs(dQ[:, v]))


def test_dissipative_fluxes_reduce_to_the_average_without_jumps():
    """With continuous traces (a state that is one smooth polynomial across elements), the
    dissipation terms vanish: ScalarDissipation and MatrixDissipation give the average flux."""
    eq = F.EulerEquation(2, 1.4)
    base = build(2, 4, (3, 3), eq, F.SplitDivOperator(F.ChandrasekharAverage(), F.ChandrasekharAverage()),
                 periodic=(), bcs={"1": F.EulerOutflowBC(), "2": F.EulerOutflowBC(), "3": F.EulerOutflowBC(),
                                   "4": F.EulerOutflowBC()})
    X = base.coords
    P = np.stack([1.2 + 0.1 * X[:, 0], 0.3 + 0.05 * X[:, 1], -0.2 + 0.02 * X[:, 0], 2.0 + 0.1 * X[:, 1]], axis=1)
    Q = np.asfortranarray(eq.vars_prim2cons(P))
    R0 = oracle_for(base).rhs(Q)
    for nf in (F.MatrixDissipation(F.ChandrasekharAverage(), 1.0), F.ScalarDissipation(F.ChandrasekharAverage(), 1.0)):
        d = build(2, 4, (3, 3), eq, F.SplitDivOperator(F.ChandrasekharAverage(), nf), periodic=(),
                  bcs={"1": F.EulerOutflowBC(), "2": F.EulerOutflowBC(), "3": F.EulerOutflowBC(),
                       "4": F.EulerOutflowBC()})
        R = oracle_for(d).rhs(Q)
        assert np.max(np.abs(R - R0)) < 1e-12 * np.max(np.abs(R0))


def _dipped_state(disc, seed, rho_dip=0.02, p_dip=0.03):
    """Smooth state with a density dip in one element and a pressure dip in another."""
    eq = disc.equation
    P = eq.vars_cons2prim(smooth_euler_state(disc, seed=seed, amp=0.2))
    npe = disc.std.n ** disc.mesh.dim
    ne = disc.mesh.nelements
    P[1 * npe + npe // 2, 0] = rho_dip
    P[(ne - 1) * npe + 1, -1] = p_dip
    return np.asfortranarray(eq.vars_prim2cons(P))


@pytest.mark.parametrize("dim", [1, 2, 3])
def test_zhang_shu_limiter_properties(dim):
    """Euler.jl:611-654: element means are kept, the density is raised to min(minval, ρ̄), and
    elements already above the thresholds are untouched bit for bit."""
    eq = F.EulerEquation(dim, 1.4)
    disc = build(dim, 4, (3,) * dim, eq, F.StrongDivOperator(F.LxF(F.StdAverage(), 1.0)))
    o = oracle_for(disc)
    Q = _dipped_state(disc, seed=4)
    minval = 0.1
    Ql = o.limit(Q, minval, disc.std.omega)
    npe = disc.std.n ** dim
    w = disc.std.omega
    J = disc.J
    changed = 0
    for e in range(disc.mesh.nelements):
        sl = slice(e * npe, (e + 1) * npe)
        jw = J[sl] * w
        m0 = jw @ Q[sl]
        m1 = jw @ Ql[sl]
        assert np.allclose(m1, m0, rtol=1e-13, atol=1e-15 * np.max(np.abs(m0)))
        rbar = m0[0] / jw.sum()
        assert Ql[sl, 0].min() >= min(minval, rbar) * (1 - 1e-13)
        p = eq.pressure(Q[sl])
        if Q[sl, 0].min() > minval and p.min() > minval:
            assert np.array_equal(Ql[sl], Q[sl])
        else:
            changed += 1
    assert changed == 2


def test_monitors_and_limited_steps_are_consistent():
    """The kinetic-energy monitor of the oracle equals the quadrature of |ρv|²/2ρ, and limited
    steps keep the density above the minimum."""
    eq = F.EulerEquation(2, 1.4)
    disc = build(2, 4, (4, 4), eq, F.SplitDivOperator(F.LxF(F.ChandrasekharAverage(), 1.0)))
    o = oracle_for(disc)
    Q = _dipped_state(disc, seed=8)
    w = np.tile(disc.std.omega, disc.mesh.nelements) * disc.J
    ke = w @ (np.sum(Q[:, 1:3] ** 2, axis=1) / (2 * Q[:, 0]))
    assert abs(o.monitor(Q, 1, disc.std.omega) - ke) < 1e-12 * abs(ke)
    dt = 0.2 * o.max_dt(Q, 1.0, disc.std.omega)
    Qs = o.ssprk3_limited(Q, dt, 4, 0.05, disc.std.omega)
    assert Qs[:, 0].min() > 0.0


@pytest.mark.parametrize("dim", [1, 2, 3])
def test_hybrid_operator_properties(dim):
    """HybridDivOperator (OpDivergence.jl:442-604): with δ -> 1 (huge blending constant) the
    telescopic subcell form is the split form (Fisher & Carpenter's equivalence); with blending it
    stays conservative and freestream-preserving."""
    eq = F.EulerEquation(dim, 1.4)
    nf = F.LxF(F.ChandrasekharAverage(), 1.0)
    hy = build(dim, 4, (3,) * dim, eq, F.HybridDivOperator(F.ChandrasekharAverage(), nf, 1e30))
    sp = build(dim, 4, (3,) * dim, eq, F.SplitDivOperator(F.ChandrasekharAverage(), nf))
    Q = smooth_euler_state(hy, seed=3, amp=0.2)
    Rh, Rs = oracle_for(hy).rhs(Q), oracle_for(sp).rhs(Q)
    assert np.max(np.abs(Rh - Rs)) < 1e-13 * np.max(np.abs(Rs))
    bl = build(dim, 4, (3,) * dim, eq, F.HybridDivOperator(F.ChandrasekharAverage(), nf, 1e-3))
    o = oracle_for(bl)
    R = o.rhs(Q)
    assert np.max(np.abs(R - Rs)) > 1e-3 * np.max(np.abs(Rs))   # the blending acts
    w = np.tile(bl.std.omega, bl.mesh.nelements) * bl.J
    for v in range(dim + 2):
        assert abs(w @ R[:, v]) < 1e-12 * np.sum(w * np.abs(R[:, v]))
    P = np.zeros((bl.ndofs, dim + 2))
    P[:, 0], P[:, 1:1 + dim], P[:, -1] = 1.3, 0.4, 2.0
    assert np.max(np.abs(o.rhs(np.asfortranarray(eq.vars_prim2cons(P))))) < 1e-12


@pytest.mark.parametrize("dim", [1, 2, 3])
def test_gauss_node_split_and_hybrid_properties(dim):
    """The Gauss-node branches (OpDivergence.jl:301-437, 614-780): entropy-projected boundary
    states couple the split volume term to the faces.  Conservative and freestream-preserving;
    the hybrid form with δ -> 1 equals the Gauss split form (the subcell fluxes telescope to the
    face fluxes by the SBP property of the Gauss operators); with blending it stays conservative."""
    eq = F.EulerEquation(dim, 1.4)
    nf = F.LxF(F.ChandrasekharAverage(), 1.0)
    sp = build(dim, 4, (3,) * dim, eq, F.SplitDivOperator(F.ChandrasekharAverage(), nf), basis="GL")
    hy = build(dim, 4, (3,) * dim, eq, F.HybridDivOperator(F.ChandrasekharAverage(), nf, 1e30), basis="GL")
    bl = build(dim, 4, (3,) * dim, eq, F.HybridDivOperator(F.ChandrasekharAverage(), F.HLLC(), nf, 1e-2),
               basis="GL")
    Q = smooth_euler_state(sp, seed=5, amp=0.2)
    w = np.tile(sp.std.omega, sp.mesh.nelements) * sp.J
    P = np.zeros((sp.ndofs, dim + 2))
    P[:, 0], P[:, 1:1 + dim], P[:, -1] = 1.3, 0.4, 2.0
    Qc = np.asfortranarray(eq.vars_prim2cons(P))
    Rs = oracle_for(sp).rhs(Q)
    Rh = oracle_for(hy).rhs(Q)
    assert np.max(np.abs(Rh - Rs)) < 1e-12 * np.max(np.abs(Rs))
    for d in (sp, bl):
        o = oracle_for(d)
        R = o.rhs(Q)
        for v in range(dim + 2):
            assert abs(w @ R[:, v]) < 1e-12 * np.sum(w * np.abs(R[:, v]))
        assert np.max(np.abs(o.rhs(Qc))) < 1e-12
    assert np.max(np.abs(oracle_for(bl).rhs(Q) - Rs)) > 1e-3 * np.max(np.abs(Rs))   # the blending acts


def test_gauss_node_split_convergence():
    """examples/src/Convergence.jl runs SplitDivOperator(LxF(ChandrasekharAverage(), 1)) on Gauss
    nodes too: the density wave ρ = 2 + sin(π(x - t)), u = p = 1 on [-1, 1] converges at the
    design order p + 1 = 4 (CarpenterKennedy2N54, dt small enough not to pollute it)."""
    eq = F.EulerEquation(1, 1.4)
    ck = F.CarpenterKennedy2N54()
    errs = []
    for ne in (8, 16):
        d = build(1, 4, (ne,), eq, F.SplitDivOperator(F.LxF(F.ChandrasekharAverage(), 1.0)), basis="GL")
        x = d.coords[:, 0]
        exact = lambda t: eq.vars_prim2cons(np.column_stack([2 + np.sin(np.pi * (x - t)), np.ones_like(x),
                                                            np.ones_like(x)]))
        tf, nsteps = 0.2, 40 * ne // 8
        Q = oracle_for(d).lsrk2n(np.asfortranarray(exact(0.0)), tf / nsteps, nsteps, ck.A, ck.B, ck.c)
        errs.append(np.sqrt(np.mean((Q - exact(tf)) ** 2)))
    order = np.log2(errs[0] / errs[1])
    assert order > 3.5, (errs, order)


@pytest.mark.parametrize("dim", [2, 3])
def test_generic_bc_with_a_varying_state(dim):
    """GenericBC(Qext) whose state varies along the boundary (FlouSpatial.jl:80-91), uploaded per
    face node: a shear flow ρ(y, z), u = const, v = w = 0, p = const is a steady solution, so with
    its own profile imposed at the inflow and outflow the residual is round-off; a profile
    mapped to the wrong face nodes would not be."""
    eq = F.EulerEquation(dim, 1.4)

    def prim(x):
        rho = 1.0 + 0.3 * np.sin(2 * np.pi * x[1]) * (np.cos(2 * np.pi * x[2]) if dim == 3 else 1.0)
        P = np.zeros(dim + 2)
        P[0], P[1], P[-1] = rho, 0.4, 1.0
        return eq.vars_prim2cons(P)

    qext = lambda _q, x, _f, _t, _e: prim(x)
    bcs = {"1": F.GenericBC(qext), "2": F.GenericBC(qext)}
    disc = build(dim, 4, (3,) * dim, eq, F.SplitDivOperator(F.LxF(F.ChandrasekharAverage(), 1.0)),
                 periodic=tuple(range(1, dim)), bcs=bcs, box=((0.0,) * dim, (1.0,) * dim))
    assert isinstance(disc.bcs[0], F.equations.StateFieldBC)
    Q = np.asfortranarray(np.array([prim(x) for x in disc.coords[:, :dim]]))
    R = oracle_for(disc).rhs(Q)
    assert np.max(np.abs(R)) < 1e-11, np.max(np.abs(R))
    a = disc.abi_arrays()
    nfd = disc.std.n ** (dim - 1)
    wrong = a["bc_field"].copy()
    for f in disc.bcs[0].states:   # the same states on the wrong nodes of each face
        wrong[f * nfd:(f + 1) * nfd] = wrong[f * nfd:(f + 1) * nfd][::-1]
    a["bc_field"] = wrong
    assert np.max(np.abs(oracle_for(disc, a).rhs(Q))) > 1e-3
