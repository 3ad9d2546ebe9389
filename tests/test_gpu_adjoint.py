"""Discrete adjoint: residual VJP and checkpointed gradient of a terminal functional.

Checked against forward-mode dual numbers run through the oracle (the role ForwardDiff plays
on the reference's CPU path): <VJP(λ), δ> must equal <λ, JVP(δ)>, and <∇J, δ> must equal the
directional derivative of J; also against central finite differences (h = 1e-6).
"""
import numpy as np
import pytest

import flou_cuda as F
from cases import build, oracle_for, smooth_euler_state

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _dev(a):
    return torch.from_numpy(np.ascontiguousarray(np.asarray(a).T if np.asarray(a).ndim == 2 else a)).cuda()


def _host(t):
    x = t.cpu().numpy()
    return np.asfortranarray(x.T) if x.ndim == 2 else x


def _lxf():
    return F.StrongDivOperator(F.LxF(F.StdAverage(), 1.0))


def _split(face_avg="chandra"):
    avg = F.ChandrasekharAverage() if face_avg == "chandra" else F.StdAverage()
    return F.SplitDivOperator(F.ChandrasekharAverage(), F.LxF(avg, 1.0))


# HLL, HLLC and ScalarDissipation carry no per-element dissipation scale: their contexts take no
# flou_set_dissipation and no dJ/dc
HLL_FAMILY = ("split_hllc", "strong_hll", "strong_hllc", "split_sd", "strong_sd", "split_md", "strong_md")


def _with_c(disc, op, c):
    """Sets the dissipation scale where the flux has one; returns the scale the oracle is given."""
    if op in HLL_FAMILY:
        return np.ones_like(c)
    disc.ctx.set_dissipation(c)
    return c


OPERATORS = {"strong": _lxf, "split": _split, "split_stdface": lambda: _split("std"),
             # the headline configuration's pair: Chandrashekar split form with the HLLC interface flux
             "split_hllc": lambda: F.SplitDivOperator(F.ChandrasekharAverage(), F.HLLC()),
             "strong_hll": lambda: F.StrongDivOperator(F.HLL()),
             "strong_hllc": lambda: F.StrongDivOperator(F.HLLC()),
             "split_kg": lambda: F.SplitDivOperator(F.KennedyGruberAverage(), F.LxF(F.StdAverage(), 1.0)),
             "split_sd": lambda: F.SplitDivOperator(F.ChandrasekharAverage(),
                                                    F.ScalarDissipation(F.ChandrasekharAverage(), 1.0)),
             "strong_sd": lambda: F.StrongDivOperator(F.ScalarDissipation(F.StdAverage(), 1.0)),
             "split_md": lambda: F.SplitDivOperator(F.MatrixDissipation(F.ChandrasekharAverage(), 1.0)),
             "split_std": lambda: F.SplitDivOperator(F.LxF(F.StdAverage(), 1.0)),
             "strong_md": lambda: F.StrongDivOperator(F.MatrixDissipation(F.StdAverage(), 1.0))}


CASES = [
    dict(dim=2, n=5, ne=(3, 3), periodic=True, bcs=None),
    dict(dim=2, n=4, ne=(3, 4), periodic=(), bcs={"1": "slip", "2": "slip", "3": "out", "4": "slip"}),
    dict(dim=1, n=6, ne=(5,), periodic=True, bcs=None),
    dict(dim=3, n=4, ne=(2, 2, 3), periodic=True, bcs=None),
    dict(dim=3, n=3, ne=(2, 2, 2), periodic=(2,), bcs={"1": "slip", "2": "out", "3": "slip", "4": "slip"}),
]


def _disc(case, op="strong"):
    eq = F.EulerEquation(case["dim"], 1.4)
    bcs = None
    if case["bcs"]:
        bcs = {k: (F.EulerSlipBC() if v == "slip" else F.EulerOutflowBC()) for k, v in case["bcs"].items()}
    d = build(case["dim"], case["n"], case["ne"], eq, OPERATORS[op](), periodic=case["periodic"], bcs=bcs)
    return d


@pytest.mark.parametrize("op", ["strong", "split", "split_stdface", "split_hllc", "strong_hll", "strong_hllc",
                                "split_kg", "split_sd", "strong_sd", "split_md", "strong_md", "split_std"])
@pytest.mark.parametrize("case", CASES, ids=lambda c: "%dd_n%d" % (c["dim"], c["n"]))
def test_rhs_vjp_dot_product(case, op):
    disc = _disc(case, op)
    rng = np.random.default_rng(7)
    Q = smooth_euler_state(disc, seed=11)
    if case["bcs"]:
        P = disc.equation.vars_cons2prim(Q)
        P[:, 1:1 + case["dim"]] *= 0.2   # gentle flow towards the walls
        Q = np.asfortranarray(disc.equation.vars_prim2cons(P))
    c = 1.0 + 0.3 * rng.random(disc.mesh.nelements)
    lam = rng.standard_normal(Q.shape)
    dQ = rng.standard_normal(Q.shape)
    dc = rng.standard_normal(c.shape)
    c = _with_c(disc, op, c)
    hll = op in HLL_FAMILY
    if hll:
        dc = 0.0 * dc
    Qbar = torch.empty(Q.shape[::-1], dtype=torch.float64, device="cuda")
    cbar = None if hll else torch.empty(disc.mesh.nelements, dtype=torch.float64, device="cuda")
    disc.ctx.rhs_vjp(Qbar, cbar, _dev(Q), _dev(lam))
    lhs = np.sum(_host(Qbar) * dQ) + (0.0 if hll else np.sum(cbar.cpu().numpy() * dc))
    R, dR = oracle_for(disc).rhs_jvp(Q, dQ, c, dc)
    rhs = np.sum(lam * dR)
    scale = np.sum(np.abs(lam * dR))
    assert abs(lhs - rhs) <= 1e-12 * scale, (lhs, rhs, scale)
    # the forward with c matches the oracle's residual too
    dQg = disc.new_state()
    disc.ctx.rhs(dQg, Q)
    assert np.max(np.abs(dQg - R)) <= 1e-12 * np.max(np.abs(R))


@pytest.mark.parametrize("op", ["strong_hll", "strong_hllc", "split_hllc"])
@pytest.mark.parametrize("dim", [2, 3])
def test_hll_family_vjp_through_every_branch(dim, op):
    """HLL and HLLC with a flow that is supersonic in both directions in places (S_L >= 0 and
    S_R <= 0) and subsonic elsewhere (both signs of the contact speed S*): every branch of the
    flux is differentiated, against the oracle's dual numbers."""
    disc = build(dim, 4, (4,) + (2,) * (dim - 1), F.EulerEquation(dim, 1.4), OPERATORS[op]())
    rng = np.random.default_rng(31 + dim)
    Q = smooth_euler_state(disc, seed=12)
    P = disc.equation.vars_cons2prim(Q)
    P[:, 1] = 2.6 * np.sin(np.pi * disc.coords[:, 0] + 0.4) + 0.1 * P[:, 1]   # |u| up to 2.6 > a ≈ 1.2
    Q = np.asfortranarray(disc.equation.vars_prim2cons(P))
    lam = rng.standard_normal(Q.shape)
    dQ = rng.standard_normal(Q.shape)
    c = np.ones(disc.mesh.nelements)
    Qbar = torch.empty(Q.shape[::-1], dtype=torch.float64, device="cuda")
    disc.ctx.rhs_vjp(Qbar, None, _dev(Q), _dev(lam))
    _, dR = oracle_for(disc).rhs_jvp(Q, dQ, c, 0.0 * c)
    lhs, rhs = np.sum(_host(Qbar) * dQ), np.sum(lam * dR)
    assert abs(lhs - rhs) <= 1e-12 * np.sum(np.abs(lam * dR)), (lhs, rhs)
    with pytest.raises(F.FlouError):   # HLL/HLLC carry no dissipation scale to differentiate
        disc.ctx.set_dissipation(c)


@pytest.mark.parametrize("op", ["split_sd", "strong_sd", "split_md", "strong_md"])
@pytest.mark.parametrize("dim", [1, 2, 3])
def test_dissipation_flux_vjp_with_jumps(dim, op):
    """ScalarDissipation and MatrixDissipation (Euler.jl:228-380) on a state whose traces jump at
    every interface, so the dissipation terms (D and the wave-speed factor; R|Λ|TRᵀ applied to the
    entropy-variable jump) all act, against the oracle's dual numbers."""
    disc = build(dim, 4, (3,) * dim, F.EulerEquation(dim, 1.4), OPERATORS[op]())
    rng = np.random.default_rng(41 + dim)
    eq = disc.equation
    P = eq.vars_cons2prim(smooth_euler_state(disc, seed=dim))
    P += np.repeat(0.05 * rng.standard_normal((disc.mesh.nelements, dim + 2)), disc.std.n ** dim, axis=0)
    Q = np.asfortranarray(eq.vars_prim2cons(P))
    lam = rng.standard_normal(Q.shape)
    dQ = rng.standard_normal(Q.shape)
    c = np.ones(disc.mesh.nelements)
    Qbar = torch.empty(Q.shape[::-1], dtype=torch.float64, device="cuda")
    disc.ctx.rhs_vjp(Qbar, None, _dev(Q), _dev(lam))
    _, dR = oracle_for(disc).rhs_jvp(Q, dQ, c, 0.0 * c)
    lhs, rhs = np.sum(_host(Qbar) * dQ), np.sum(lam * dR)
    assert abs(lhs - rhs) <= 1e-12 * np.sum(np.abs(lam * dR)), (lhs, rhs)


def _functional_inputs(disc, seed):
    rng = np.random.default_rng(seed)
    w = np.tile(disc.std.omega, disc.mesh.nelements) * disc.J
    rho_t = 1.0 + 0.05 * rng.standard_normal(disc.ndofs)
    return rho_t, w


def test_adjoint_solve_against_dual_numbers():
    eq = F.EulerEquation(2, 1.4)
    disc = build(2, 4, (4, 3), eq, _lxf(), box=((-5.0, -5.0), (5.0, 5.0)))
    Q0 = np.asfortranarray(F.initial.vortex_bump(eq, disc.coords, (0.3, -0.4), 4.0, 0.05, period=(10.0, 10.0)))
    rng = np.random.default_rng(3)
    c = 1.0 + 0.2 * rng.random(disc.mesh.nelements)
    disc.ctx.set_dissipation(c)
    rho_t, w = _functional_inputs(disc, 5)
    dt = 0.3 * disc.ctx.max_dt(Q0, 1.0)
    nsteps = 12
    g = torch.empty(Q0.shape[::-1], dtype=torch.float64, device="cuda")
    gc = torch.empty(disc.mesh.nelements, dtype=torch.float64, device="cuda")
    J, nfwd = disc.ctx.adjoint_solve(_dev(Q0), dt, nsteps, 3, _dev(rho_t), _dev(w), g, gc)
    o = oracle_for(disc)
    for k in range(3):
        dQ = rng.standard_normal(Q0.shape)
        dc = rng.standard_normal(c.shape)
        Jo, dJo = o.solve_jvp(Q0, dQ, c, dc, dt, nsteps, rho_t, w)
        assert abs(J - Jo) <= 1e-12 * abs(Jo)
        ours = np.sum(_host(g) * dQ) + np.sum(gc.cpu().numpy() * dc)
        assert abs(ours - dJo) <= 1e-10 * abs(dJo), (ours, dJo)


def test_snapshot_budget_does_not_change_the_gradient():
    eq = F.EulerEquation(2, 1.4)
    disc = build(2, 3, (3, 3), eq, _lxf())
    Q0 = smooth_euler_state(disc, seed=4)
    c = np.ones(disc.mesh.nelements)
    disc.ctx.set_dissipation(c)
    rho_t, w = _functional_inputs(disc, 6)
    dt = 0.3 * disc.ctx.max_dt(Q0, 1.0)
    res = []
    for nsnap in (0, 2, 5, 15):
        g = torch.empty(Q0.shape[::-1], dtype=torch.float64, device="cuda")
        gc = torch.empty(disc.mesh.nelements, dtype=torch.float64, device="cuda")
        J, nfwd = disc.ctx.adjoint_solve(_dev(Q0), dt, 16, nsnap, _dev(rho_t), _dev(w), g, gc)
        res.append((J, g, gc, nfwd))
    for J, g, gc, _ in res[1:]:
        assert J == res[0][0]
        assert torch.equal(g, res[0][1]) and torch.equal(gc, res[0][2])
    nf = [r[3] for r in res]
    assert nf[0] == 16 * 15 // 2 and nf[-1] == 15 and nf[1] > nf[2] > nf[3]


def test_adjoint_against_central_differences():
    eq = F.EulerEquation(2, 1.4)
    disc = build(2, 5, (6, 6), eq, _lxf(), box=((-5.0, -5.0), (5.0, 5.0)))
    Q0 = np.asfortranarray(F.initial.vortex_bump(eq, disc.coords, (0.5, 0.1), 5.0, 0.08, period=(10.0, 10.0)))
    rng = np.random.default_rng(9)
    c = 1.0 + 0.1 * rng.random(disc.mesh.nelements)
    disc.ctx.set_dissipation(c)
    rho_t, w = _functional_inputs(disc, 8)
    dt = 0.4 * disc.ctx.max_dt(Q0, 1.0)
    nsteps = 20
    g = torch.empty(Q0.shape[::-1], dtype=torch.float64, device="cuda")
    gc = torch.empty(disc.mesh.nelements, dtype=torch.float64, device="cuda")
    disc.ctx.adjoint_solve(_dev(Q0), dt, nsteps, 4, _dev(rho_t), _dev(w), g, gc)
    wd, rtd = _dev(w), _dev(rho_t)

    def Jof(Q, cc):
        disc.ctx.set_dissipation(cc)
        q = _dev(Q)
        disc.ctx.step(q, dt, nsteps)
        r = q[0] - rtd
        return float(0.5 * torch.sum(wd * r * r))

    h = 1e-6
    for k in range(3):
        dQ = rng.standard_normal(Q0.shape)
        dc = rng.standard_normal(c.shape) * 0.1
        fd = (Jof(Q0 + h * dQ, c + h * dc) - Jof(Q0 - h * dQ, c - h * dc)) / (2 * h)
        ours = np.sum(_host(g) * dQ) + np.sum(gc.cpu().numpy() * dc)
        assert abs(ours - fd) <= 1e-6 * abs(fd), (ours, fd)


@pytest.mark.parametrize("op", ["split", "split_stdface", "split_hllc", "split_kg", "split_std"])
def test_split_rhs_vjp_columns(op):
    """Every column of the transposed Jacobian at once on a small 3D case: (∂R/∂Q)ᵀ λ against
    the dual-number JVPs of all unit directions of one element's nodes."""
    case = dict(dim=3, n=3, ne=(2, 2, 2), periodic=True, bcs=None)
    disc = _disc(case, op)
    rng = np.random.default_rng(21)
    Q = smooth_euler_state(disc, seed=2, amp=0.3)
    c = _with_c(disc, op, 1.0 + 0.3 * rng.random(disc.mesh.nelements))
    lam = rng.standard_normal(Q.shape)
    Qbar = torch.empty(Q.shape[::-1], dtype=torch.float64, device="cuda")
    cbar = None if op in HLL_FAMILY else torch.empty(disc.mesh.nelements, dtype=torch.float64, device="cuda")
    disc.ctx.rhs_vjp(Qbar, cbar, _dev(Q), _dev(lam))
    Qb = _host(Qbar)
    o = oracle_for(disc)
    npe = disc.std.n ** 3
    for v in range(Q.shape[1]):
        for i in range(npe):
            dQ = np.zeros_like(Q)
            dQ[i, v] = 1.0
            _, dR = o.rhs_jvp(Q, dQ, c, 0.0 * c)
            col = np.sum(lam * dR)
            assert abs(Qb[i, v] - col) <= 1e-12 * max(1.0, np.sum(np.abs(lam * dR))), (v, i, Qb[i, v], col)


def _general(dim, n, op, walls, seed=5):
    """A perturbed box whose elements are randomly rotated (every master2slave orientation occurs
    in 3D) and whose interior nodes are displaced: J, the metric, the face frames and the surface
    Jacobians vary per node.  Walls: slip on the odd boundaries, outflow on the even ones."""
    from test_unstructured import _std
    eq = F.EulerEquation(dim, 1.4)
    mesh = F.perturbed_box(dim, 3, (0.0,) * dim, (1.0,) * dim, amp=0.12, seed=seed)
    bcs = {str(k): (F.EulerSlipBC() if walls and k % 2 else F.EulerOutflowBC()) for k in range(1, 2 * dim + 1)}
    return F.MultielementDisc(mesh, _std(dim, n, dim + 2, "GLL"), eq, OPERATORS[op](), bcs)


GENERAL_OPS = ["strong", "split", "split_stdface", "split_hllc", "strong_hllc", "strong_hll", "split_kg", "split_std",
               "split_sd", "split_md", "strong_md"]


@pytest.mark.parametrize("op", GENERAL_OPS)
@pytest.mark.parametrize("dim,n,walls", [(2, 4, False), (2, 5, True), (3, 3, True), (3, 4, False)])
def test_general_geometry_rhs_vjp_dot_product(dim, n, walls, op):
    """The residual VJP on general geometry (the CURV kernels: contravariant fluxes with the
    per-node metric, pair fluxes along the averaged metric columns, slave traces through the
    orientation, per-node face frames), against the oracle's dual numbers."""
    from test_unstructured import _state
    disc = _general(dim, n, op, walls)
    if dim == 3:
        assert len(set(disc.mesh.orientation.tolist())) == 8
    rng = np.random.default_rng(40 + dim + n)
    Q = _state(disc, seed=dim + n)
    lam = rng.standard_normal(Q.shape)
    dQ = rng.standard_normal(Q.shape)
    c = _with_c(disc, op, 1.0 + 0.3 * rng.random(disc.mesh.nelements))
    hll = op in HLL_FAMILY
    dc = 0.0 * c if hll else rng.standard_normal(c.shape)
    Qbar = torch.empty(Q.shape[::-1], dtype=torch.float64, device="cuda")
    cbar = None if hll else torch.empty(disc.mesh.nelements, dtype=torch.float64, device="cuda")
    disc.ctx.rhs_vjp(Qbar, cbar, _dev(Q), _dev(lam))
    lhs = np.sum(_host(Qbar) * dQ) + (0.0 if hll else np.sum(cbar.cpu().numpy() * dc))
    R, dR = oracle_for(disc).rhs_jvp(Q, dQ, c, dc)
    rhs = np.sum(lam * dR)
    assert abs(lhs - rhs) <= 1e-12 * np.sum(np.abs(lam * dR)), (lhs, rhs)


@pytest.mark.parametrize("op", ["split", "strong", "split_kg", "split_std"])
def test_general_geometry_rhs_vjp_columns(op):
    """Every column of one element's transposed Jacobian on a rotated 3D mesh, against the
    dual-number JVPs of the unit directions (catches a cotangent sent to the wrong slave node)."""
    from test_unstructured import _state
    disc = _general(3, 3, op, walls=True, seed=8)
    rng = np.random.default_rng(23)
    Q = _state(disc, seed=4)
    c = _with_c(disc, op, 1.0 + 0.3 * rng.random(disc.mesh.nelements))
    lam = rng.standard_normal(Q.shape)
    Qbar = torch.empty(Q.shape[::-1], dtype=torch.float64, device="cuda")
    cbar = None if op in HLL_FAMILY else torch.empty(disc.mesh.nelements, dtype=torch.float64, device="cuda")
    disc.ctx.rhs_vjp(Qbar, cbar, _dev(Q), _dev(lam))
    Qb = _host(Qbar)
    o = oracle_for(disc)
    npe = disc.std.n ** 3
    e = 13   # the middle element: all its faces are interior
    for v in range(Q.shape[1]):
        for i in range(e * npe, (e + 1) * npe):
            dQ = np.zeros_like(Q)
            dQ[i, v] = 1.0
            _, dR = o.rhs_jvp(Q, dQ, c, 0.0 * c)
            col = np.sum(lam * dR)
            assert abs(Qb[i, v] - col) <= 1e-12 * max(1.0, np.sum(np.abs(lam * dR))), (v, i, Qb[i, v], col)


@pytest.mark.parametrize("op", ["split_hllc", "strong", "split_kg"])
def test_general_geometry_adjoint_solve_against_dual_numbers(op):
    from test_unstructured import _state
    disc = _general(3, 4, op, walls=True)
    Q0 = _state(disc, seed=9)
    rng = np.random.default_rng(29)
    hll = op in HLL_FAMILY
    c = _with_c(disc, op, 1.0 + 0.2 * rng.random(disc.mesh.nelements))
    rho_t, w = _functional_inputs(disc, 5)
    dt = 0.3 * disc.ctx.max_dt(Q0, 1.0)
    nsteps = 8
    g = torch.empty(Q0.shape[::-1], dtype=torch.float64, device="cuda")
    gc = None if hll else torch.empty(disc.mesh.nelements, dtype=torch.float64, device="cuda")
    J, nfwd = disc.ctx.adjoint_solve(_dev(Q0), dt, nsteps, 3, _dev(rho_t), _dev(w), g, gc)
    o = oracle_for(disc)
    for k in range(2):
        dQ = rng.standard_normal(Q0.shape)
        dc = rng.standard_normal(c.shape) * (0.0 if hll else 1.0)
        Jo, dJo = o.solve_jvp(Q0, dQ, c, dc, dt, nsteps, rho_t, w)
        assert abs(J - Jo) <= 1e-12 * abs(Jo)
        ours = np.sum(_host(g) * dQ) + (0.0 if hll else np.sum(gc.cpu().numpy() * dc))
        assert abs(ours - dJo) <= 1e-10 * abs(dJo), (ours, dJo)


def _fixed_state_bcs(dim, eq, field):
    """Boundary 1: an inflow state; boundary 2: a state that varies along the boundary (a
    boundary-state field, flou_set_bc_field) or an outflow; slip and outflow walls elsewhere."""
    Pin = np.zeros(dim + 2)
    Pin[0], Pin[1], Pin[-1] = 1.05, 0.25, 1.1
    bcs = {"1": F.EulerInflowBC(eq.vars_prim2cons(Pin)), "2": F.EulerOutflowBC()}
    if field:
        def qext(_q, x, _f, _t, _e):
            P = np.zeros(dim + 2)
            P[0], P[1], P[-1] = 1.0 + 0.2 * np.sin(2 * np.pi * x[1]), 0.3, 1.0 + 0.1 * x[1]
            if dim > 1:
                P[2] = 0.1 * np.cos(2 * np.pi * x[1])
            return eq.vars_prim2cons(P)
        bcs["2"] = F.GenericBC(qext)
    for k in range(3, 2 * dim + 1):
        bcs[str(k)] = F.EulerSlipBC() if k % 2 else F.EulerOutflowBC()
    return bcs


@pytest.mark.parametrize("op", ["strong", "split", "split_hllc", "strong_hll", "split_md", "split_kg"])
@pytest.mark.parametrize("dim,general,field", [(2, False, True), (3, False, False), (2, True, True),
                                               (3, True, True)])
def test_rhs_vjp_with_inflow_and_state_field_boundaries(dim, general, field, op):
    """Fixed external states (an inflow boundary, and a boundary-state field that varies along
    the boundary) enter the face flux as constants: only the interior trace's cotangent remains."""
    from test_unstructured import _state, _std
    eq = F.EulerEquation(dim, 1.4)
    bcs = _fixed_state_bcs(dim, eq, field)
    if general:
        mesh = F.perturbed_box(dim, 3, (0.0,) * dim, (1.0,) * dim, amp=0.12, seed=6)
        disc = F.MultielementDisc(mesh, _std(dim, 4, dim + 2, "GLL"), eq, OPERATORS[op](), bcs)
        Q = _state(disc, seed=3)
    else:
        disc = build(dim, 4, (3,) * dim, eq, OPERATORS[op](), periodic=(), bcs=bcs,
                     box=((0.0,) * dim, (1.0,) * dim))
        Q = smooth_euler_state(disc, seed=5)
    if field:
        assert any(isinstance(b, F.equations.StateFieldBC) for b in disc.bcs)
    rng = np.random.default_rng(50 + dim)
    lam = rng.standard_normal(Q.shape)
    dQ = rng.standard_normal(Q.shape)
    c = _with_c(disc, op, 1.0 + 0.3 * rng.random(disc.mesh.nelements))
    hll = op in HLL_FAMILY
    dc = 0.0 * c if hll else rng.standard_normal(c.shape)
    Qbar = torch.empty(Q.shape[::-1], dtype=torch.float64, device="cuda")
    cbar = None if hll else torch.empty(disc.mesh.nelements, dtype=torch.float64, device="cuda")
    disc.ctx.rhs_vjp(Qbar, cbar, _dev(Q), _dev(lam))
    lhs = np.sum(_host(Qbar) * dQ) + (0.0 if hll else np.sum(cbar.cpu().numpy() * dc))
    R, dR = oracle_for(disc).rhs_jvp(Q, dQ, c, dc)
    rhs = np.sum(lam * dR)
    assert abs(lhs - rhs) <= 1e-12 * np.sum(np.abs(lam * dR)), (lhs, rhs)


def test_adjoint_solve_with_inflow_and_state_field_boundaries():
    eq = F.EulerEquation(2, 1.4)
    disc = build(2, 4, (4, 3), eq, OPERATORS["split_hllc"](), periodic=(), bcs=_fixed_state_bcs(2, eq, True),
                 box=((0.0, 0.0), (1.0, 1.0)))
    Q0 = smooth_euler_state(disc, seed=12)
    rng = np.random.default_rng(33)
    rho_t, w = _functional_inputs(disc, 7)
    dt = 0.3 * disc.ctx.max_dt(Q0, 1.0)
    nsteps = 10
    g = torch.empty(Q0.shape[::-1], dtype=torch.float64, device="cuda")
    J, nfwd = disc.ctx.adjoint_solve(_dev(Q0), dt, nsteps, 3, _dev(rho_t), _dev(w), g, None)
    o = oracle_for(disc)
    c1 = np.ones(disc.mesh.nelements)
    for k in range(2):
        dQ = rng.standard_normal(Q0.shape)
        Jo, dJo = o.solve_jvp(Q0, dQ, c1, 0.0 * c1, dt, nsteps, rho_t, w)
        assert abs(J - Jo) <= 1e-12 * abs(Jo)
        ours = np.sum(_host(g) * dQ)
        assert abs(ours - dJo) <= 1e-10 * abs(dJo), (ours, dJo)


GAUSS_OPS = ["strong", "strong_hll", "strong_hllc", "strong_sd", "strong_md"]


@pytest.mark.parametrize("op", GAUSS_OPS)
@pytest.mark.parametrize("dim,n,general,walls", [(1, 5, False, True), (2, 4, False, False), (2, 5, False, True),
                                                 (3, 3, False, True), (2, 4, True, True), (3, 4, True, False)])
def test_gauss_nodes_strong_rhs_vjp_dot_product(dim, n, general, walls, op):
    """The strong form on Gauss nodes: the traces are interpolations Σ l_p U_p and the lift
    reaches every node of a line, so the face VJP gathers the whole line and the element VJP
    scatters the trace cotangents back through l."""
    from test_unstructured import _state, _std
    eq = F.EulerEquation(dim, 1.4)
    if general:
        mesh = F.perturbed_box(dim, 3, (0.0,) * dim, (1.0,) * dim, amp=0.12, seed=7)
        bcs = _fixed_state_bcs(dim, eq, True) if walls else \
            {str(k): F.EulerOutflowBC() for k in range(1, 2 * dim + 1)}
        disc = F.MultielementDisc(mesh, _std(dim, n, dim + 2, "GL"), eq, OPERATORS[op](), bcs)
        Q = _state(disc, seed=dim + n)
    else:
        bcs = None
        if walls:
            bcs = {str(k): (F.EulerSlipBC() if k % 2 else F.EulerOutflowBC()) for k in range(1, 2 * dim + 1)}
        disc = build(dim, n, (3,) * dim, eq, OPERATORS[op](), periodic=() if walls else True, bcs=bcs, basis="GL")
        Q = smooth_euler_state(disc, seed=dim + n)
        if walls:
            P = eq.vars_cons2prim(Q)
            P[:, 1:1 + dim] *= 0.2
            Q = np.asfortranarray(eq.vars_prim2cons(P))
    rng = np.random.default_rng(70 + dim + n)
    lam = rng.standard_normal(Q.shape)
    dQ = rng.standard_normal(Q.shape)
    c = _with_c(disc, op, 1.0 + 0.3 * rng.random(disc.mesh.nelements))
    hll = op in HLL_FAMILY
    dc = 0.0 * c if hll else rng.standard_normal(c.shape)
    Qbar = torch.empty(Q.shape[::-1], dtype=torch.float64, device="cuda")
    cbar = None if hll else torch.empty(disc.mesh.nelements, dtype=torch.float64, device="cuda")
    disc.ctx.rhs_vjp(Qbar, cbar, _dev(Q), _dev(lam))
    lhs = np.sum(_host(Qbar) * dQ) + (0.0 if hll else np.sum(cbar.cpu().numpy() * dc))
    R, dR = oracle_for(disc).rhs_jvp(Q, dQ, c, dc)
    rhs = np.sum(lam * dR)
    assert abs(lhs - rhs) <= 1e-12 * np.sum(np.abs(lam * dR)), (lhs, rhs)


def test_gauss_nodes_strong_rhs_vjp_columns():
    disc = build(2, 4, (3, 3), F.EulerEquation(2, 1.4), _lxf(), basis="GL")
    rng = np.random.default_rng(24)
    Q = smooth_euler_state(disc, seed=5, amp=0.3)
    c = _with_c(disc, "strong", 1.0 + 0.3 * rng.random(disc.mesh.nelements))
    lam = rng.standard_normal(Q.shape)
    Qbar = torch.empty(Q.shape[::-1], dtype=torch.float64, device="cuda")
    disc.ctx.rhs_vjp(Qbar, None, _dev(Q), _dev(lam))
    Qb = _host(Qbar)
    o = oracle_for(disc)
    npe = disc.std.n ** 2
    e = 4
    for v in range(Q.shape[1]):
        for i in range(e * npe, (e + 1) * npe):
            dQ = np.zeros_like(Q)
            dQ[i, v] = 1.0
            _, dR = o.rhs_jvp(Q, dQ, c, 0.0 * c)
            col = np.sum(lam * dR)
            assert abs(Qb[i, v] - col) <= 1e-12 * max(1.0, np.sum(np.abs(lam * dR))), (v, i, Qb[i, v], col)


@pytest.mark.parametrize("op,dim", [("strong", 2), ("strong_hllc", 3)])
def test_gauss_nodes_adjoint_solve_against_dual_numbers(op, dim):
    eq = F.EulerEquation(dim, 1.4)
    if dim == 2:
        disc = build(2, 5, (4, 3), eq, OPERATORS[op](), box=((-5.0, -5.0), (5.0, 5.0)), basis="GL")
        Q0 = np.asfortranarray(F.initial.vortex_bump(eq, disc.coords, (0.3, -0.4), 4.0, 0.05, period=(10.0, 10.0)))
    else:
        disc = build(3, 4, (2, 3, 2), eq, OPERATORS[op](), box=((0.0,) * 3, (2 * np.pi,) * 3), basis="GL")
        Q0 = _tgv_state(disc, 0.3, 4)
    rng = np.random.default_rng(41)
    hll = op in HLL_FAMILY
    c = _with_c(disc, op, 1.0 + 0.2 * rng.random(disc.mesh.nelements))
    rho_t, w = _functional_inputs(disc, 9)
    dt = 0.2 * disc.ctx.max_dt(Q0, 1.0)
    nsteps = 8
    g = torch.empty(Q0.shape[::-1], dtype=torch.float64, device="cuda")
    gc = None if hll else torch.empty(disc.mesh.nelements, dtype=torch.float64, device="cuda")
    J, nfwd = disc.ctx.adjoint_solve(_dev(Q0), dt, nsteps, 3, _dev(rho_t), _dev(w), g, gc)
    o = oracle_for(disc)
    for k in range(2):
        dQ = rng.standard_normal(Q0.shape)
        dc = rng.standard_normal(c.shape) * (0.0 if hll else 1.0)
        Jo, dJo = o.solve_jvp(Q0, dQ, c, dc, dt, nsteps, rho_t, w)
        assert abs(J - Jo) <= 1e-12 * abs(Jo)
        ours = np.sum(_host(g) * dQ) + (0.0 if hll else np.sum(gc.cpu().numpy() * dc))
        assert abs(ours - dJo) <= 1e-10 * abs(dJo), (ours, dJo)


GAUSS_SPLIT_OPS = ["split", "split_stdface", "split_hllc", "split_kg", "split_std", "split_md", "split_sd"]


@pytest.mark.parametrize("op", GAUSS_SPLIT_OPS)
@pytest.mark.parametrize("dim,n,walls", [(1, 4, True), (2, 4, False), (2, 5, True), (3, 3, False), (3, 4, True)])
def test_gauss_nodes_split_rhs_vjp_dot_product(dim, n, walls, op):
    """The split form on Gauss nodes: the entropy-projected coupling (OpDivergence.jl:301-437)
    transposed -- the pair fluxes of every node with its line's two projected states, the
    projections' sums, the state of the projected entropy variables and the entropy variables of
    every node -- against the oracle's dual numbers."""
    eq = F.EulerEquation(dim, 1.4)
    bcs = None
    if walls:
        bcs = {str(k): (F.EulerSlipBC() if k % 2 else F.EulerOutflowBC()) for k in range(1, 2 * dim + 1)}
    disc = build(dim, n, (3,) * dim, eq, OPERATORS[op](), periodic=() if walls else True, bcs=bcs, basis="GL")
    Q = smooth_euler_state(disc, seed=dim + n)
    if walls:
        P = eq.vars_cons2prim(Q)
        P[:, 1:1 + dim] *= 0.2
        Q = np.asfortranarray(eq.vars_prim2cons(P))
    rng = np.random.default_rng(80 + dim + n)
    lam = rng.standard_normal(Q.shape)
    dQ = rng.standard_normal(Q.shape)
    c = _with_c(disc, op, 1.0 + 0.3 * rng.random(disc.mesh.nelements))
    hll = op in HLL_FAMILY
    dc = 0.0 * c if hll else rng.standard_normal(c.shape)
    Qbar = torch.empty(Q.shape[::-1], dtype=torch.float64, device="cuda")
    cbar = None if hll else torch.empty(disc.mesh.nelements, dtype=torch.float64, device="cuda")
    disc.ctx.rhs_vjp(Qbar, cbar, _dev(Q), _dev(lam))
    lhs = np.sum(_host(Qbar) * dQ) + (0.0 if hll else np.sum(cbar.cpu().numpy() * dc))
    R, dR = oracle_for(disc).rhs_jvp(Q, dQ, c, dc)
    rhs = np.sum(lam * dR)
    assert abs(lhs - rhs) <= 1e-12 * np.sum(np.abs(lam * dR)), (lhs, rhs)


@pytest.mark.parametrize("op", ["split", "split_kg", "split_std"])
def test_gauss_nodes_split_rhs_vjp_columns(op):
    disc = build(2, 4, (3, 3), F.EulerEquation(2, 1.4), OPERATORS[op](), basis="GL")
    rng = np.random.default_rng(26)
    Q = smooth_euler_state(disc, seed=6, amp=0.3)
    c = _with_c(disc, op, 1.0 + 0.3 * rng.random(disc.mesh.nelements))
    lam = rng.standard_normal(Q.shape)
    Qbar = torch.empty(Q.shape[::-1], dtype=torch.float64, device="cuda")
    disc.ctx.rhs_vjp(Qbar, None, _dev(Q), _dev(lam))
    Qb = _host(Qbar)
    o = oracle_for(disc)
    npe = disc.std.n ** 2
    e = 4
    for v in range(Q.shape[1]):
        for i in range(e * npe, (e + 1) * npe):
            dQ = np.zeros_like(Q)
            dQ[i, v] = 1.0
            _, dR = o.rhs_jvp(Q, dQ, c, 0.0 * c)
            col = np.sum(lam * dR)
            assert abs(Qb[i, v] - col) <= 1e-12 * max(1.0, np.sum(np.abs(lam * dR))), (v, i, Qb[i, v], col)


@pytest.mark.parametrize("op", ["split_hllc", "split_kg"])
def test_gauss_nodes_split_adjoint_solve_against_dual_numbers(op):
    eq = F.EulerEquation(3, 1.4)
    disc = build(3, 4, (2, 3, 2), eq, OPERATORS[op](), box=((0.0,) * 3, (2 * np.pi,) * 3), basis="GL")
    Q0 = _tgv_state(disc, 0.3, 5)
    rng = np.random.default_rng(43)
    hll = op in HLL_FAMILY
    c = _with_c(disc, op, 1.0 + 0.2 * rng.random(disc.mesh.nelements))
    rho_t, w = _functional_inputs(disc, 10)
    dt = 0.2 * disc.ctx.max_dt(Q0, 1.0)
    nsteps = 6
    g = torch.empty(Q0.shape[::-1], dtype=torch.float64, device="cuda")
    gc = None if hll else torch.empty(disc.mesh.nelements, dtype=torch.float64, device="cuda")
    J, nfwd = disc.ctx.adjoint_solve(_dev(Q0), dt, nsteps, 2, _dev(rho_t), _dev(w), g, gc)
    o = oracle_for(disc)
    for k in range(2):
        dQ = rng.standard_normal(Q0.shape)
        dc = rng.standard_normal(c.shape) * (0.0 if hll else 1.0)
        Jo, dJo = o.solve_jvp(Q0, dQ, c, dc, dt, nsteps, rho_t, w)
        assert abs(J - Jo) <= 1e-12 * abs(Jo)
        ours = np.sum(_host(g) * dQ) + (0.0 if hll else np.sum(gc.cpu().numpy() * dc))
        assert abs(ours - dJo) <= 1e-10 * abs(dJo), (ours, dJo)


def test_gauss_nodes_split_adjoint_3d_p7_kennedy_gruber():
    """The Kennedy-Gruber 3D p=7 tile on Gauss nodes, whose pair cotangents go in two chunks of
    lines (all at once they exceed shared memory), against the oracle's dual numbers."""
    disc = build(3, 8, (2, 2, 1), F.EulerEquation(3, 1.4), OPERATORS["split_kg"](), basis="GL")
    Q = smooth_euler_state(disc, seed=31, amp=0.2)
    rng = np.random.default_rng(131)
    lam = rng.standard_normal(Q.shape)
    dQ = rng.standard_normal(Q.shape)
    c = _with_c(disc, "split_kg", 1.0 + 0.3 * rng.random(disc.mesh.nelements))
    dc = rng.standard_normal(c.shape)
    Qbar = torch.empty(Q.shape[::-1], dtype=torch.float64, device="cuda")
    cbar = torch.empty(disc.mesh.nelements, dtype=torch.float64, device="cuda")
    disc.ctx.rhs_vjp(Qbar, cbar, _dev(Q), _dev(lam))
    lhs = np.sum(_host(Qbar) * dQ) + np.sum(cbar.cpu().numpy() * dc)
    R, dR = oracle_for(disc).rhs_jvp(Q, dQ, c, dc)
    rhs = np.sum(lam * dR)
    assert abs(lhs - rhs) <= 1e-12 * np.sum(np.abs(lam * dR)), (lhs, rhs)


HYBRID_OPS = {
    # blend 0.5 with HLLC: the δ = ½ clip is active at some interfaces and not at others
    "hybrid_hllc": lambda: F.HybridDivOperator(F.ChandrasekharAverage(), F.HLLC(),
                                               F.LxF(F.ChandrasekharAverage(), 1.0), 0.5),
    "hybrid_md": lambda: F.HybridDivOperator(F.MatrixDissipation(F.ChandrasekharAverage(), 1.0), 1.0),
    "hybrid_kg": lambda: F.HybridDivOperator(F.KennedyGruberAverage(), F.LxF(F.StdAverage(), 1.0), 1e-3),
    "hybrid_std_hll": lambda: F.HybridDivOperator(F.StdAverage(), F.HLL(), F.HLL(), 0.1),
}


def _hybrid_disc(dim, n, op, walls, seed, basis="GLL"):
    eq = F.EulerEquation(dim, 1.4)
    bcs = None
    if walls:
        bcs = {str(k): (F.EulerSlipBC() if k % 2 else F.EulerOutflowBC()) for k in range(1, 2 * dim + 1)}
    disc = build(dim, n, (3,) * dim, eq, HYBRID_OPS[op](), periodic=() if walls else True, bcs=bcs, basis=basis)
    Q = smooth_euler_state(disc, seed=seed, amp=0.3)
    if walls:
        P = eq.vars_cons2prim(Q)
        P[:, 1:1 + dim] *= 0.2
        Q = np.asfortranarray(eq.vars_prim2cons(P))
    return disc, Q


def _hybrid_c(disc, op, c):
    """Sets the per-element dissipation scale where the interface flux has one (LxF)."""
    if op in ("hybrid_kg",):
        disc.ctx.set_dissipation(c)
        return c, False
    return np.ones_like(c), True


@pytest.mark.parametrize("op", sorted(HYBRID_OPS))
@pytest.mark.parametrize("dim,n,walls", [(1, 5, True), (2, 4, False), (2, 5, True), (3, 3, True), (3, 4, False)])
def test_hybrid_rhs_vjp_dot_product(dim, n, walls, op):
    """HybridDivOperator on Gauss-Lobatto nodes: the blended subcell fluxes transposed (the FV
    flux VJP, Fisher's indicator through the entropy variables, the ½ clip, the telescoped
    high-order subcell fluxes as weighted split-form pairs), against the oracle's dual numbers."""
    disc, Q = _hybrid_disc(dim, n, op, walls, seed=dim + n)
    rng = np.random.default_rng(90 + dim + n)
    lam = rng.standard_normal(Q.shape)
    dQ = rng.standard_normal(Q.shape)
    c, noc = _hybrid_c(disc, op, 1.0 + 0.3 * rng.random(disc.mesh.nelements))
    dc = 0.0 * c if noc else rng.standard_normal(c.shape)
    Qbar = torch.empty(Q.shape[::-1], dtype=torch.float64, device="cuda")
    cbar = None if noc else torch.empty(disc.mesh.nelements, dtype=torch.float64, device="cuda")
    disc.ctx.rhs_vjp(Qbar, cbar, _dev(Q), _dev(lam))
    lhs = np.sum(_host(Qbar) * dQ) + (0.0 if noc else np.sum(cbar.cpu().numpy() * dc))
    R, dR = oracle_for(disc).rhs_jvp(Q, dQ, c, dc)
    rhs = np.sum(lam * dR)
    assert abs(lhs - rhs) <= 1e-12 * np.sum(np.abs(lam * dR)), (lhs, rhs)


@pytest.mark.parametrize("op", ["hybrid_hllc", "hybrid_md"])
def test_hybrid_rhs_vjp_columns(op):
    disc, Q = _hybrid_disc(2, 4, op, False, seed=7)
    rng = np.random.default_rng(27)
    c, _ = _hybrid_c(disc, op, 1.0 + 0.3 * rng.random(disc.mesh.nelements))
    lam = rng.standard_normal(Q.shape)
    Qbar = torch.empty(Q.shape[::-1], dtype=torch.float64, device="cuda")
    disc.ctx.rhs_vjp(Qbar, None, _dev(Q), _dev(lam))
    Qb = _host(Qbar)
    o = oracle_for(disc)
    npe = disc.std.n ** 2
    e = 4
    for v in range(Q.shape[1]):
        for i in range(e * npe, (e + 1) * npe):
            dQ = np.zeros_like(Q)
            dQ[i, v] = 1.0
            _, dR = o.rhs_jvp(Q, dQ, c, 0.0 * c)
            col = np.sum(lam * dR)
            assert abs(Qb[i, v] - col) <= 1e-12 * max(1.0, np.sum(np.abs(lam * dR))), (v, i, Qb[i, v], col)


@pytest.mark.parametrize("op", ["hybrid_hllc", "hybrid_kg"])
def test_hybrid_adjoint_solve_against_dual_numbers(op):
    eq = F.EulerEquation(3, 1.4)
    disc = build(3, 4, (2, 3, 2), eq, HYBRID_OPS[op](), box=((0.0,) * 3, (2 * np.pi,) * 3))
    Q0 = _tgv_state(disc, 0.3, 6)
    rng = np.random.default_rng(47)
    c, noc = _hybrid_c(disc, op, 1.0 + 0.2 * rng.random(disc.mesh.nelements))
    rho_t, w = _functional_inputs(disc, 11)
    dt = 0.2 * disc.ctx.max_dt(Q0, 1.0)
    nsteps = 6
    g = torch.empty(Q0.shape[::-1], dtype=torch.float64, device="cuda")
    gc = None if noc else torch.empty(disc.mesh.nelements, dtype=torch.float64, device="cuda")
    J, nfwd = disc.ctx.adjoint_solve(_dev(Q0), dt, nsteps, 2, _dev(rho_t), _dev(w), g, gc)
    o = oracle_for(disc)
    for k in range(2):
        dQ = rng.standard_normal(Q0.shape)
        dc = rng.standard_normal(c.shape) * (0.0 if noc else 1.0)
        Jo, dJo = o.solve_jvp(Q0, dQ, c, dc, dt, nsteps, rho_t, w)
        assert abs(J - Jo) <= 1e-12 * abs(Jo)
        ours = np.sum(_host(g) * dQ) + (0.0 if noc else np.sum(gc.cpu().numpy() * dc))
        assert abs(ours - dJo) <= 1e-10 * abs(dJo), (ours, dJo)


@pytest.mark.parametrize("dim,n,walls,op",
                         [(d, n, w, op) for op in sorted(HYBRID_OPS)
                          for d, n, w in [(1, 5, True), (2, 4, False), (2, 5, True), (3, 3, True), (3, 4, False)]] +
                         [(3, 7, False, "hybrid_hllc"), (2, 8, True, "hybrid_kg")])
def test_gauss_nodes_hybrid_rhs_vjp_dot_product(dim, n, walls, op):
    """HybridDivOperator on Gauss nodes: the blended scan that starts from the element's own face
    flux, run backwards (the face-flux cotangents handed to the face VJP), the projected-state
    pairs weighted by l/ω, the FV fluxes and Fisher's indicator, against the oracle's dual
    numbers."""
    disc, Q = _hybrid_disc(dim, n, op, walls, seed=dim + n, basis="GL")
    rng = np.random.default_rng(190 + dim + n)
    lam = rng.standard_normal(Q.shape)
    dQ = rng.standard_normal(Q.shape)
    c, noc = _hybrid_c(disc, op, 1.0 + 0.3 * rng.random(disc.mesh.nelements))
    dc = 0.0 * c if noc else rng.standard_normal(c.shape)
    Qbar = torch.empty(Q.shape[::-1], dtype=torch.float64, device="cuda")
    cbar = None if noc else torch.empty(disc.mesh.nelements, dtype=torch.float64, device="cuda")
    disc.ctx.rhs_vjp(Qbar, cbar, _dev(Q), _dev(lam))
    lhs = np.sum(_host(Qbar) * dQ) + (0.0 if noc else np.sum(cbar.cpu().numpy() * dc))
    R, dR = oracle_for(disc).rhs_jvp(Q, dQ, c, dc)
    rhs = np.sum(lam * dR)
    assert abs(lhs - rhs) <= 1e-12 * np.sum(np.abs(lam * dR)), (lhs, rhs)


@pytest.mark.parametrize("op", ["hybrid_hllc", "hybrid_std_hll"])
def test_gauss_nodes_hybrid_rhs_vjp_columns(op):
    disc, Q = _hybrid_disc(2, 4, op, True, seed=8, basis="GL")
    rng = np.random.default_rng(28)
    c, _ = _hybrid_c(disc, op, 1.0 + 0.3 * rng.random(disc.mesh.nelements))
    lam = rng.standard_normal(Q.shape)
    Qbar = torch.empty(Q.shape[::-1], dtype=torch.float64, device="cuda")
    disc.ctx.rhs_vjp(Qbar, None, _dev(Q), _dev(lam))
    Qb = _host(Qbar)
    o = oracle_for(disc)
    npe = disc.std.n ** 2
    for e in (0, 4):
        for v in range(Q.shape[1]):
            for i in range(e * npe, (e + 1) * npe):
                dQ = np.zeros_like(Q)
                dQ[i, v] = 1.0
                _, dR = o.rhs_jvp(Q, dQ, c, 0.0 * c)
                col = np.sum(lam * dR)
                assert abs(Qb[i, v] - col) <= 1e-12 * max(1.0, np.sum(np.abs(lam * dR))), (v, i, Qb[i, v], col)


@pytest.mark.parametrize("op", ["hybrid_hllc", "hybrid_kg"])
def test_gauss_nodes_hybrid_adjoint_solve_against_dual_numbers(op):
    eq = F.EulerEquation(3, 1.4)
    disc = build(3, 4, (2, 3, 2), eq, HYBRID_OPS[op](), box=((0.0,) * 3, (2 * np.pi,) * 3), basis="GL")
    Q0 = _tgv_state(disc, 0.3, 7)
    rng = np.random.default_rng(48)
    c, noc = _hybrid_c(disc, op, 1.0 + 0.2 * rng.random(disc.mesh.nelements))
    rho_t, w = _functional_inputs(disc, 13)
    dt = 0.2 * disc.ctx.max_dt(Q0, 1.0)
    nsteps = 6
    g = torch.empty(Q0.shape[::-1], dtype=torch.float64, device="cuda")
    gc = None if noc else torch.empty(disc.mesh.nelements, dtype=torch.float64, device="cuda")
    J, nfwd = disc.ctx.adjoint_solve(_dev(Q0), dt, nsteps, 2, _dev(rho_t), _dev(w), g, gc)
    o = oracle_for(disc)
    for k in range(2):
        dQ = rng.standard_normal(Q0.shape)
        dc = rng.standard_normal(c.shape) * (0.0 if noc else 1.0)
        Jo, dJo = o.solve_jvp(Q0, dQ, c, dc, dt, nsteps, rho_t, w)
        assert abs(J - Jo) <= 1e-12 * abs(Jo)
        ours = np.sum(_host(g) * dQ) + (0.0 if noc else np.sum(gc.cpu().numpy() * dc))
        assert abs(ours - dJo) <= 1e-10 * abs(dJo), (ours, dJo)


@pytest.mark.parametrize("integrator,limited", [("SSPRK3", True), ("ORK256", True), ("CarpenterKennedy2N54", False)])
def test_gauss_nodes_hybrid_adjoint_through_limiter_and_2n_storage(integrator, limited):
    """The Gauss-node hybrid operator's two-pass adjoint stage inside the limited SSP-RK3 and
    2N-storage reverse sweeps, against the oracle's dual numbers through the same method."""
    from flou_cuda import _lib as L
    eq = F.EulerEquation(2, 1.4)
    disc = build(2, 4, (4, 3), eq, HYBRID_OPS["hybrid_hllc"](), box=((-5.0, -5.0), (5.0, 5.0)), basis="GL")
    if limited:   # a smooth state (a one-node dip's entropy variables extrapolate to a
        # non-physical line-end state on Gauss nodes), limited where ρ or p is below 0.82
        Q0 = smooth_euler_state(disc, seed=14, amp=0.2)
        disc.ctx.set_limiter(L.LIMITER_ZHANG_SHU, 0.82)
    else:
        Q0 = np.asfortranarray(F.initial.vortex_bump(eq, disc.coords, (0.3, -0.4), 4.0, 0.05, period=(10.0, 10.0)))
    m = None if integrator == "SSPRK3" else getattr(F, integrator)()
    if m is not None:
        disc.ctx.set_integrator(m.A, m.B)
    c = np.ones(disc.mesh.nelements)
    rho_t, w = _functional_inputs(disc, 9)
    dt = 0.2 * disc.ctx.max_dt(Q0, 1.0)
    nsteps = 6
    o = oracle_for(disc)
    args = () if m is None else (m.A, m.B, m.c)
    lim = dict(minval=0.82, omega_tp=disc.std.omega) if limited else {}
    if limited:   # the limiter acts along this trajectory
        J0, _ = o.solve_jvp_lsrk(Q0, 0 * Q0, c, 0 * c, dt, nsteps, rho_t, w, *args)
        J1, _ = o.solve_jvp_lsrk(Q0, 0 * Q0, c, 0 * c, dt, nsteps, rho_t, w, *args, **lim)
        assert abs(J1 - J0) > 1e-6 * abs(J0)
    rng = np.random.default_rng(72)
    for nsnap in (2, nsteps - 1):
        g = torch.empty(Q0.shape[::-1], dtype=torch.float64, device="cuda")
        J, nfwd = disc.ctx.adjoint_solve(_dev(Q0), dt, nsteps, nsnap, _dev(rho_t), _dev(w), g)
        dQ = rng.standard_normal(Q0.shape)
        Jo, dJo = o.solve_jvp_lsrk(Q0, dQ, c, 0 * c, dt, nsteps, rho_t, w, *args, **lim)
        assert abs(J - Jo) <= 1e-12 * abs(Jo)
        ours = np.sum(_host(g) * dQ)
        assert abs(ours - dJo) <= 1e-10 * abs(dJo), (nsnap, ours, dJo)
    disc.ctx.set_limiter(L.LIMITER_NONE)
    if m is not None:
        disc.ctx.set_integrator(None)


@pytest.mark.parametrize("op,basis", [("hybrid_hllc", "GL"), ("hybrid_kg", "GL"), ("hybrid_std_hll", "GL"),
                                      ("hybrid_kg", "GLL"), ("hybrid_md", "GLL")])
def test_hybrid_adjoint_3d_p7(op, basis):
    """The 3D p=7 hybrid tiles: on Gauss nodes (every two-point flux) and with the Kennedy-Gruber
    flux the pair cotangents go in two chunks of lines; the MatrixDissipation tile on Gauss-Lobatto
    nodes keeps the nodes' entropy variables in the last 198 bytes of shared memory.  Against the
    oracle's dual numbers."""
    eq = F.EulerEquation(3, 1.4)
    disc = build(3, 8, (2, 2, 1), eq, HYBRID_OPS[op](), basis=basis)
    Q = smooth_euler_state(disc, seed=32, amp=0.3)
    rng = np.random.default_rng(132)
    lam = rng.standard_normal(Q.shape)
    dQ = rng.standard_normal(Q.shape)
    c, noc = _hybrid_c(disc, op, 1.0 + 0.3 * rng.random(disc.mesh.nelements))
    dc = 0.0 * c if noc else rng.standard_normal(c.shape)
    Qbar = torch.empty(Q.shape[::-1], dtype=torch.float64, device="cuda")
    cbar = None if noc else torch.empty(disc.mesh.nelements, dtype=torch.float64, device="cuda")
    disc.ctx.rhs_vjp(Qbar, cbar, _dev(Q), _dev(lam))
    lhs = np.sum(_host(Qbar) * dQ) + (0.0 if noc else np.sum(cbar.cpu().numpy() * dc))
    R, dR = oracle_for(disc).rhs_jvp(Q, dQ, c, dc)
    rhs = np.sum(lam * dR)
    assert abs(lhs - rhs) <= 1e-12 * np.sum(np.abs(lam * dR)), (lhs, rhs)


def _maybe_c(disc, c):
    """The per-element dissipation scale where the interface flux takes one (LxF): (c, False);
    else (ones, True)."""
    try:
        disc.ctx.set_dissipation(c)
        return c, False
    except F.FlouError:
        return np.ones_like(c), True


@pytest.mark.parametrize("op,basis", [("split_chandra_lxfc", "GL"), ("split_kg_lxf", "GL"), ("split_std_lxf", "GL"),
                                      ("split_chandra_md", "GL"), ("hybrid_hllc", "GLL"), ("hybrid_md", "GLL"),
                                      ("hybrid_kg", "GLL"), ("hybrid_hllc", "GL"), ("hybrid_md", "GL"),
                                      ("hybrid_kg", "GL")])
@pytest.mark.parametrize("dim,n", [(2, 4), (3, 3), (3, 4)])
def test_general_geometry_gauss_split_and_hybrid_rhs_vjp(dim, n, op, basis):
    """General geometry for the split form on Gauss nodes (the projected states' pairs along
    (Ja_j + n Js)/2 with the line end's subcell normal) and for the hybrid operator (the subcell
    FV fluxes in the uploaded subcell frames; on Gauss nodes also the face fluxes' cotangents to
    a slave side through the orientation), against the oracle's dual numbers."""
    from test_gpu_unstructured import _disc as _udisc
    from test_unstructured import _state
    disc = _udisc(dim, n, op, basis=basis)
    if dim == 3:
        assert len(set(disc.mesh.orientation.tolist())) == 8
    rng = np.random.default_rng(100 + dim + n)
    Q = _state(disc, seed=dim * 3 + n)
    lam = rng.standard_normal(Q.shape)
    dQ = rng.standard_normal(Q.shape)
    c, noc = _maybe_c(disc, 1.0 + 0.3 * rng.random(disc.mesh.nelements))
    dc = 0.0 * c if noc else rng.standard_normal(c.shape)
    Qbar = torch.empty(Q.shape[::-1], dtype=torch.float64, device="cuda")
    cbar = None if noc else torch.empty(disc.mesh.nelements, dtype=torch.float64, device="cuda")
    disc.ctx.rhs_vjp(Qbar, cbar, _dev(Q), _dev(lam))
    lhs = np.sum(_host(Qbar) * dQ) + (0.0 if noc else np.sum(cbar.cpu().numpy() * dc))
    R, dR = oracle_for(disc).rhs_jvp(Q, dQ, c, dc)
    rhs = np.sum(lam * dR)
    assert abs(lhs - rhs) <= 1e-12 * np.sum(np.abs(lam * dR)), (lhs, rhs)


@pytest.mark.parametrize("op,basis", [("split_kg_lxf", "GL"), ("hybrid_hllc", "GL"), ("hybrid_kg", "GLL")])
def test_general_geometry_3d_p7_tiles_rhs_vjp(op, basis):
    """The chunked 3D p=7 tiles on rotated general elements (every orientation), against the
    oracle's dual numbers."""
    from test_gpu_unstructured import _disc as _udisc
    from test_unstructured import _state
    disc = _udisc(3, 8, op, basis=basis, nel=2)
    rng = np.random.default_rng(140)
    Q = _state(disc, seed=41)
    lam = rng.standard_normal(Q.shape)
    dQ = rng.standard_normal(Q.shape)
    c, noc = _maybe_c(disc, 1.0 + 0.3 * rng.random(disc.mesh.nelements))
    dc = 0.0 * c if noc else rng.standard_normal(c.shape)
    Qbar = torch.empty(Q.shape[::-1], dtype=torch.float64, device="cuda")
    cbar = None if noc else torch.empty(disc.mesh.nelements, dtype=torch.float64, device="cuda")
    disc.ctx.rhs_vjp(Qbar, cbar, _dev(Q), _dev(lam))
    lhs = np.sum(_host(Qbar) * dQ) + (0.0 if noc else np.sum(cbar.cpu().numpy() * dc))
    R, dR = oracle_for(disc).rhs_jvp(Q, dQ, c, dc)
    rhs = np.sum(lam * dR)
    assert abs(lhs - rhs) <= 1e-12 * np.sum(np.abs(lam * dR)), (lhs, rhs)


@pytest.mark.parametrize("op,basis", [("split_chandra_lxfc", "GL"), ("hybrid_hllc", "GLL"), ("hybrid_hllc", "GL")])
def test_general_geometry_gauss_split_and_hybrid_adjoint_solve(op, basis):
    from test_gpu_unstructured import _disc as _udisc
    from test_unstructured import _state
    disc = _udisc(3, 4, op, basis=basis)
    Q0 = _state(disc, seed=5)
    rng = np.random.default_rng(53)
    c, noc = _maybe_c(disc, 1.0 + 0.2 * rng.random(disc.mesh.nelements))
    rho_t, w = _functional_inputs(disc, 12)
    dt = 0.2 * disc.ctx.max_dt(Q0, 1.0)
    nsteps = 5
    g = torch.empty(Q0.shape[::-1], dtype=torch.float64, device="cuda")
    gc = None if noc else torch.empty(disc.mesh.nelements, dtype=torch.float64, device="cuda")
    J, nfwd = disc.ctx.adjoint_solve(_dev(Q0), dt, nsteps, 2, _dev(rho_t), _dev(w), g, gc)
    o = oracle_for(disc)
    for k in range(2):
        dQ = rng.standard_normal(Q0.shape)
        dc = rng.standard_normal(c.shape) * (0.0 if noc else 1.0)
        Jo, dJo = o.solve_jvp(Q0, dQ, c, dc, dt, nsteps, rho_t, w)
        assert abs(J - Jo) <= 1e-12 * abs(Jo)
        ours = np.sum(_host(g) * dQ) + (0.0 if noc else np.sum(gc.cpu().numpy() * dc))
        assert abs(ours - dJo) <= 1e-10 * abs(dJo), (ours, dJo)


@pytest.mark.parametrize("integrator", ["SSPRK3", "ORK256"])
@pytest.mark.parametrize("op,dim", [("strong", 2), ("split", 2), ("split_hllc", 3), ("strong", 1)])
def test_limited_adjoint_solve_against_dual_numbers(integrator, op, dim):
    """The Zhang-Shu stage limiter (after every stage, as Flou's stage_limiter!) differentiated:
    a state with a density dip and a pressure dip and minval = 0.5 keep two elements limited
    through the solve; against the oracle's dual numbers through the same limited method."""
    from flou_cuda import _lib as L
    from test_oracle_kat import _dipped_state
    eq = F.EulerEquation(dim, 1.4)
    disc = build(dim, 4, (3,) * dim, eq, OPERATORS[op]())
    Q0 = _dipped_state(disc, seed=10 + dim)
    minval = 0.5
    disc.ctx.set_limiter(L.LIMITER_ZHANG_SHU, minval)
    m = None if integrator == "SSPRK3" else F.ORK256()
    if m is not None:
        disc.ctx.set_integrator(m.A, m.B)
    rng = np.random.default_rng(71)
    hll = op in HLL_FAMILY
    c = _with_c(disc, op, 1.0 + 0.2 * rng.random(disc.mesh.nelements))
    rho_t, w = _functional_inputs(disc, 4)
    dt = 0.2 * disc.ctx.max_dt(Q0, 1.0)
    nsteps = 6
    o = oracle_for(disc)
    args = () if m is None else (m.A, m.B, m.c)
    # the limiter acts along this trajectory
    J0, _ = o.solve_jvp_lsrk(Q0, 0 * Q0, c, 0 * c, dt, nsteps, rho_t, w, *args)
    J1, _ = o.solve_jvp_lsrk(Q0, 0 * Q0, c, 0 * c, dt, nsteps, rho_t, w, *args, minval=minval,
                             omega_tp=disc.std.omega)
    assert not np.isfinite(J0) or abs(J1 - J0) > 1e-6 * abs(J0)   # (unlimited, some runs break down)
    for nsnap in (2, nsteps - 1):
        g = torch.empty(Q0.shape[::-1], dtype=torch.float64, device="cuda")
        gc = None if hll else torch.empty(disc.mesh.nelements, dtype=torch.float64, device="cuda")
        J, nfwd = disc.ctx.adjoint_solve(_dev(Q0), dt, nsteps, nsnap, _dev(rho_t), _dev(w), g, gc)
        assert abs(J - J1) <= 1e-12 * abs(J1)
        for k in range(2):
            dQ = rng.standard_normal(Q0.shape)
            dc = rng.standard_normal(c.shape) * (0.0 if hll else 1.0)
            Jo, dJo = o.solve_jvp_lsrk(Q0, dQ, c, dc, dt, nsteps, rho_t, w, *args, minval=minval,
                                       omega_tp=disc.std.omega)
            ours = np.sum(_host(g) * dQ) + (0.0 if hll else np.sum(gc.cpu().numpy() * dc))
            assert abs(ours - dJo) <= 1e-10 * abs(dJo), (nsnap, ours, dJo)
    disc.ctx.set_limiter(L.LIMITER_NONE)
    if m is not None:
        disc.ctx.set_integrator(None)


def test_limited_adjoint_against_central_differences():
    from flou_cuda import _lib as L
    from test_oracle_kat import _dipped_state
    eq = F.EulerEquation(2, 1.4)
    disc = build(2, 5, (4, 4), eq, _lxf())
    Q0 = _dipped_state(disc, seed=21)
    disc.ctx.set_limiter(L.LIMITER_ZHANG_SHU, 0.5)
    rng = np.random.default_rng(81)
    c = 1.0 + 0.1 * rng.random(disc.mesh.nelements)
    disc.ctx.set_dissipation(c)
    rho_t, w = _functional_inputs(disc, 8)
    dt = 0.2 * disc.ctx.max_dt(Q0, 1.0)
    nsteps = 8
    g = torch.empty(Q0.shape[::-1], dtype=torch.float64, device="cuda")
    gc = torch.empty(disc.mesh.nelements, dtype=torch.float64, device="cuda")
    disc.ctx.adjoint_solve(_dev(Q0), dt, nsteps, 3, _dev(rho_t), _dev(w), g, gc)
    wd, rtd = _dev(w), _dev(rho_t)

    def Jof(Q, cc):
        disc.ctx.set_dissipation(cc)
        q = _dev(Q)
        disc.ctx.step(q, dt, nsteps)
        r = q[0] - rtd
        return float(0.5 * torch.sum(wd * r * r))

    h = 1e-6
    for k in range(3):
        dQ = rng.standard_normal(Q0.shape)
        dc = rng.standard_normal(c.shape) * 0.1
        fd = (Jof(Q0 + h * dQ, c + h * dc) - Jof(Q0 - h * dQ, c - h * dc)) / (2 * h)
        ours = np.sum(_host(g) * dQ) + np.sum(gc.cpu().numpy() * dc)
        assert abs(ours - fd) <= 1e-6 * abs(fd), (ours, fd)
    disc.ctx.set_limiter(L.LIMITER_NONE)


@pytest.mark.parametrize("solver", ["ORK256", "CarpenterKennedy2N54"])
@pytest.mark.parametrize("op,dim", [("strong", 2), ("split_hllc", 2), ("split", 3), ("split_kg", 3)])
def test_lowstorage_adjoint_solve_against_dual_numbers(solver, op, dim):
    """The discrete adjoint of the 2N-storage methods (flou_set_integrator): each reverse stage
    Ū_i = Ū_(i+1) + dt (∂L/∂u)(u_i)ᵀ k̄ with k̄ carried as A_i k̄ + B_(i-1) Ū_i, against the oracle's
    dual numbers through the same method, with snapshots and recomputation."""
    eq = F.EulerEquation(dim, 1.4)
    if dim == 2:
        disc = build(2, 4, (4, 3), eq, OPERATORS[op](), box=((-5.0, -5.0), (5.0, 5.0)))
        Q0 = np.asfortranarray(F.initial.vortex_bump(eq, disc.coords, (0.3, -0.4), 4.0, 0.05, period=(10.0, 10.0)))
    else:
        disc = build(3, 4, (2, 3, 2), eq, OPERATORS[op](), box=((0.0,) * 3, (2 * np.pi,) * 3))
        Q0 = _tgv_state(disc, 0.3, 2)
    m = getattr(F, solver)()
    disc.ctx.set_integrator(m.A, m.B)
    rng = np.random.default_rng(61)
    hll = op in HLL_FAMILY
    c = _with_c(disc, op, 1.0 + 0.2 * rng.random(disc.mesh.nelements))
    rho_t, w = _functional_inputs(disc, 3)
    dt = 0.3 * disc.ctx.max_dt(Q0, 1.0)
    nsteps = 9
    o = oracle_for(disc)
    for nsnap in (2, 8):
        g = torch.empty(Q0.shape[::-1], dtype=torch.float64, device="cuda")
        gc = None if hll else torch.empty(disc.mesh.nelements, dtype=torch.float64, device="cuda")
        J, nfwd = disc.ctx.adjoint_solve(_dev(Q0), dt, nsteps, nsnap, _dev(rho_t), _dev(w), g, gc)
        for k in range(2):
            dQ = rng.standard_normal(Q0.shape)
            dc = rng.standard_normal(c.shape) * (0.0 if hll else 1.0)
            Jo, dJo = o.solve_jvp_lsrk(Q0, dQ, c, dc, dt, nsteps, rho_t, w, m.A, m.B, m.c)
            assert abs(J - Jo) <= 1e-12 * abs(Jo)
            ours = np.sum(_host(g) * dQ) + (0.0 if hll else np.sum(gc.cpu().numpy() * dc))
            assert abs(ours - dJo) <= 1e-10 * abs(dJo), (nsnap, ours, dJo)
    disc.ctx.set_integrator(None)


def test_lowstorage_adjoint_against_central_differences():
    eq = F.EulerEquation(2, 1.4)
    disc = build(2, 5, (6, 6), eq, _lxf(), box=((-5.0, -5.0), (5.0, 5.0)))
    Q0 = np.asfortranarray(F.initial.vortex_bump(eq, disc.coords, (0.5, 0.1), 5.0, 0.08, period=(10.0, 10.0)))
    m = F.ORK256()
    disc.ctx.set_integrator(m.A, m.B)
    rng = np.random.default_rng(19)
    c = 1.0 + 0.1 * rng.random(disc.mesh.nelements)
    disc.ctx.set_dissipation(c)
    rho_t, w = _functional_inputs(disc, 8)
    dt = 0.4 * disc.ctx.max_dt(Q0, 1.0)
    nsteps = 12
    g = torch.empty(Q0.shape[::-1], dtype=torch.float64, device="cuda")
    gc = torch.empty(disc.mesh.nelements, dtype=torch.float64, device="cuda")
    disc.ctx.adjoint_solve(_dev(Q0), dt, nsteps, 3, _dev(rho_t), _dev(w), g, gc)
    wd, rtd = _dev(w), _dev(rho_t)

    def Jof(Q, cc):
        disc.ctx.set_dissipation(cc)
        q = _dev(Q)
        disc.ctx.step(q, dt, nsteps)
        r = q[0] - rtd
        return float(0.5 * torch.sum(wd * r * r))

    h = 1e-6
    for k in range(3):
        dQ = rng.standard_normal(Q0.shape)
        dc = rng.standard_normal(c.shape) * 0.1
        fd = (Jof(Q0 + h * dQ, c + h * dc) - Jof(Q0 - h * dQ, c - h * dc)) / (2 * h)
        ours = np.sum(_host(g) * dQ) + np.sum(gc.cpu().numpy() * dc)
        assert abs(ours - fd) <= 1e-6 * abs(fd), (ours, fd)
    disc.ctx.set_integrator(None)


def _tgv_state(disc, mach, seed):
    """Taylor-Green vortex with a small random smooth perturbation of every primitive variable.
    The plain vortex is symmetric: interface wave speeds tie exactly (|u_L| + a_L = |u_R| + a_R)
    on its symmetry planes, where LxF's max is not differentiable and a one-ulp difference in a
    stage state picks the other branch.  The perturbation moves the trajectory off the ties."""
    eq = disc.equation
    P = eq.vars_cons2prim(F.initial.taylor_green(eq, disc.coords, mach))
    rng = np.random.default_rng(seed)
    X = disc.coords
    for v in range(P.shape[1]):
        k = rng.integers(1, 3, size=3)
        ph = rng.uniform(0, 2 * np.pi, size=3)
        wave = np.prod([np.sin(k[i] * X[:, i] + ph[i]) for i in range(3)], axis=0)
        scale = 0.05 * (np.max(np.abs(P[:, v])) if v in (0, 4) else 1.0)
        P[:, v] = P[:, v] + scale * wave
    return np.asfortranarray(eq.vars_prim2cons(P))


@pytest.mark.parametrize("op", ["split", "strong", "split_hllc", "split_kg", "split_sd", "split_md", "split_std"])
def test_3d_adjoint_solve_against_dual_numbers(op):
    eq = F.EulerEquation(3, 1.4)
    L = 2 * np.pi
    disc = build(3, 4, (2, 3, 2), eq, OPERATORS[op](), box=((0.0,) * 3, (L,) * 3))
    Q0 = _tgv_state(disc, 0.3, 0)
    rng = np.random.default_rng(13)
    hll = op in HLL_FAMILY
    c = _with_c(disc, op, 1.0 + 0.2 * rng.random(disc.mesh.nelements))
    rho_t, w = _functional_inputs(disc, 5)
    dt = 0.3 * disc.ctx.max_dt(Q0, 1.0)
    nsteps = 10
    g = torch.empty(Q0.shape[::-1], dtype=torch.float64, device="cuda")
    gc = None if hll else torch.empty(disc.mesh.nelements, dtype=torch.float64, device="cuda")
    J, nfwd = disc.ctx.adjoint_solve(_dev(Q0), dt, nsteps, 3, _dev(rho_t), _dev(w), g, gc)
    o = oracle_for(disc)
    for k in range(3):
        dQ = rng.standard_normal(Q0.shape)
        dc = rng.standard_normal(c.shape) * (0.0 if hll else 1.0)
        Jo, dJo = o.solve_jvp(Q0, dQ, c, dc, dt, nsteps, rho_t, w)
        assert abs(J - Jo) <= 1e-12 * abs(Jo)
        ours = np.sum(_host(g) * dQ) + (0.0 if hll else np.sum(gc.cpu().numpy() * dc))
        assert abs(ours - dJo) <= 1e-10 * abs(dJo), (ours, dJo)


@pytest.mark.parametrize("op", ["split", "split_hllc"])
def test_split_adjoint_against_central_differences(op):
    eq = F.EulerEquation(3, 1.4)
    L = 2 * np.pi
    disc = build(3, 5, (3, 3, 3), eq, OPERATORS[op](), box=((0.0,) * 3, (L,) * 3))
    Q0 = _tgv_state(disc, 0.2, 1)
    rng = np.random.default_rng(17)
    hll = op in HLL_FAMILY
    c = _with_c(disc, op, 1.0 + 0.1 * rng.random(disc.mesh.nelements))
    rho_t, w = _functional_inputs(disc, 8)
    dt = 0.2 * disc.ctx.max_dt(Q0, 1.0)
    nsteps = 12
    g = torch.empty(Q0.shape[::-1], dtype=torch.float64, device="cuda")
    gc = None if hll else torch.empty(disc.mesh.nelements, dtype=torch.float64, device="cuda")
    disc.ctx.adjoint_solve(_dev(Q0), dt, nsteps, 4, _dev(rho_t), _dev(w), g, gc)
    wd, rtd = _dev(w), _dev(rho_t)

    def Jof(Q, cc):
        if not hll:
            disc.ctx.set_dissipation(cc)
        q = _dev(Q)
        disc.ctx.step(q, dt, nsteps)
        r = q[0] - rtd
        return float(0.5 * torch.sum(wd * r * r))

    h = 1e-6
    for k in range(3):
        dQ = rng.standard_normal(Q0.shape)
        dc = rng.standard_normal(c.shape) * (0.0 if hll else 0.1)
        fd = (Jof(Q0 + h * dQ, c + h * dc) - Jof(Q0 - h * dQ, c - h * dc)) / (2 * h)
        ours = np.sum(_host(g) * dQ) + (0.0 if hll else np.sum(gc.cpu().numpy() * dc))
        assert abs(ours - fd) <= 1e-6 * abs(fd), (ours, fd)
