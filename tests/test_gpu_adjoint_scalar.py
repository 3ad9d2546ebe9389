"""Discrete adjoint of the scalar equations (linear advection 1D-3D, Burgers 1D): the residual VJP
and the checkpointed gradient, against the oracle's dual numbers and central differences."""
import numpy as np
import pytest

import flou_cuda as F
from cases import build, oracle_for

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

from test_gpu_adjoint import _dev, _host, _functional_inputs  # noqa: E402

OPS = {
    "strong_lxf": lambda: F.StrongDivOperator(F.LxF(F.StdAverage(), 1.0)),
    "strong_central": lambda: F.StrongDivOperator(F.StdAverage()),
    "split_lxf": lambda: F.SplitDivOperator(F.LxF(F.StdAverage(), 1.0)),
}


def _disc(eq_name, dim, n, op, walls, basis="GLL"):
    if eq_name == "burgers":
        eq = F.BurgersEquation()
    else:
        eq = F.LinearAdvection(*([1.0, -0.6, 0.4][:dim]))
    bcs = None
    if walls:
        bcs = {str(k): (F.DirichletBC([0.5 + 0.1 * k]) if k % 2 else F.OutflowBC()) for k in range(1, 2 * dim + 1)}
    disc = build(dim, n, (4,) + (3,) * (dim - 1), eq, OPS[op](), periodic=() if walls else True, bcs=bcs,
                 basis=basis)
    X = disc.coords
    rng = np.random.default_rng(dim + n)
    ph = rng.uniform(0, 6, size=dim)
    # Burgers: a state that changes sign, so both branches of λ = max(|q_l|, |q_r|) occur
    base = 0.2 if eq_name == "burgers" else 1.0
    Q = base + 0.8 * np.prod([np.sin(2.0 * X[:, d] + ph[d]) for d in range(dim)], axis=0)
    return disc, np.asfortranarray(Q[:, None])


def _with_c(disc, op, c):
    if op.endswith("lxf"):
        disc.ctx.set_dissipation(c)
        return c, False
    return np.ones_like(c), True


CASES = [("advection", 1, 5, True, "GLL"), ("advection", 2, 4, False, "GLL"), ("advection", 2, 5, True, "GLL"),
         ("advection", 3, 3, True, "GLL"), ("advection", 2, 4, True, "GL"), ("advection", 3, 4, False, "GL"),
         ("burgers", 1, 6, False, "GLL"), ("burgers", 1, 5, True, "GLL"), ("burgers", 1, 5, False, "GL")]


# (the split form of the scalar equations needs boundary nodes: no split case on Gauss nodes)
@pytest.mark.parametrize("case,op", [(c, op) for c in CASES for op in sorted(OPS)
                                     if not (op.startswith("split") and c[4] == "GL")],
                         ids=lambda x: x if isinstance(x, str) else "%s_%dd_n%d_%s%s" % (
                             x[0], x[1], x[2], x[4], "_walls" if x[3] else ""))
def test_scalar_rhs_vjp_dot_product(case, op):
    eqn, dim, n, walls, basis = case
    disc, Q = _disc(eqn, dim, n, op, walls, basis)
    rng = np.random.default_rng(5 + dim + n)
    lam = rng.standard_normal(Q.shape)
    dQ = rng.standard_normal(Q.shape)
    c, noc = _with_c(disc, op, 1.0 + 0.3 * rng.random(disc.mesh.nelements))
    dc = 0.0 * c if noc else rng.standard_normal(c.shape)
    Qbar = torch.empty(Q.shape[::-1], dtype=torch.float64, device="cuda")
    cbar = None if noc else torch.empty(disc.mesh.nelements, dtype=torch.float64, device="cuda")
    disc.ctx.rhs_vjp(Qbar, cbar, _dev(Q), _dev(lam))
    lhs = np.sum(_host(Qbar) * dQ) + (0.0 if noc else np.sum(cbar.cpu().numpy() * dc))
    R, dR = oracle_for(disc).rhs_jvp(Q, dQ, c, dc)
    rhs = np.sum(lam * dR)
    assert abs(lhs - rhs) <= 1e-12 * np.sum(np.abs(lam * dR)), (lhs, rhs)


@pytest.mark.parametrize("eqn,dim,op", [("advection", 2, "strong_lxf"), ("advection", 3, "split_lxf"),
                                        ("burgers", 1, "split_lxf"), ("burgers", 1, "strong_lxf")])
def test_scalar_adjoint_solve_against_dual_numbers(eqn, dim, op):
    disc, Q0 = _disc(eqn, dim, 5, op, walls=dim == 2)
    rng = np.random.default_rng(91)
    c, noc = _with_c(disc, op, 1.0 + 0.2 * rng.random(disc.mesh.nelements))
    rho_t, w = _functional_inputs(disc, 3)
    dt = 0.3 * disc.ctx.max_dt(Q0, 1.0)
    nsteps = 12
    o = oracle_for(disc)
    for nsnap in (3, nsteps - 1):
        g = torch.empty(Q0.shape[::-1], dtype=torch.float64, device="cuda")
        gc = None if noc else torch.empty(disc.mesh.nelements, dtype=torch.float64, device="cuda")
        J, nfwd = disc.ctx.adjoint_solve(_dev(Q0), dt, nsteps, nsnap, _dev(rho_t), _dev(w), g, gc)
        for k in range(2):
            dQ = rng.standard_normal(Q0.shape)
            dc = rng.standard_normal(c.shape) * (0.0 if noc else 1.0)
            Jo, dJo = o.solve_jvp(Q0, dQ, c, dc, dt, nsteps, rho_t, w)
            assert abs(J - Jo) <= 1e-12 * abs(Jo)
            ours = np.sum(_host(g) * dQ) + (0.0 if noc else np.sum(gc.cpu().numpy() * dc))
            assert abs(ours - dJo) <= 1e-10 * abs(dJo), (nsnap, ours, dJo)


def test_scalar_adjoint_against_central_differences():
    disc, Q0 = _disc("advection", 2, 5, "strong_lxf", walls=False)
    rng = np.random.default_rng(17)
    c = 1.0 + 0.2 * rng.random(disc.mesh.nelements)
    disc.ctx.set_dissipation(c)
    rho_t, w = _functional_inputs(disc, 6)
    dt = 0.3 * disc.ctx.max_dt(Q0, 1.0)
    nsteps = 15
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


def _general(dim, n, op, basis, walls):
    from test_unstructured import _std
    mesh = F.perturbed_box(dim, 3, (0.0,) * dim, (1.0,) * dim, amp=0.12, seed=4 + dim)
    bcs = {str(k): (F.DirichletBC([0.5 + 0.1 * k]) if walls and k % 2 else F.OutflowBC())
           for k in range(1, 2 * dim + 1)}
    disc = F.MultielementDisc(mesh, _std(dim, n, 1, basis), F.LinearAdvection(*([1.0, -0.6, 0.4][:dim])),
                              OPS[op](), bcs)
    X = disc.coords
    Q = 1.0 + 0.5 * np.prod([np.cos(3.0 * X[:, d] + d) for d in range(dim)], axis=0)
    return disc, np.asfortranarray(Q[:, None])


@pytest.mark.parametrize("op,basis", [("strong_lxf", "GLL"), ("strong_central", "GLL"), ("split_lxf", "GLL"),
                                      ("strong_lxf", "GL")])
@pytest.mark.parametrize("dim,n,walls", [(2, 4, True), (2, 5, False), (3, 3, True), (3, 4, False)])
def test_scalar_general_geometry_rhs_vjp(dim, n, walls, op, basis):
    """Linear advection on perturbed, rotated elements (every orientation in 3D): contravariant
    fluxes with the node's metric, pairs along the averaged columns, the face nodes' normals and
    surface Jacobians, slave traces through the orientation."""
    disc, Q = _general(dim, n, op, basis, walls)
    if dim == 3:
        assert len(set(disc.mesh.orientation.tolist())) == 8
    rng = np.random.default_rng(110 + dim + n)
    lam = rng.standard_normal(Q.shape)
    dQ = rng.standard_normal(Q.shape)
    c, noc = _with_c(disc, op, 1.0 + 0.3 * rng.random(disc.mesh.nelements))
    dc = 0.0 * c if noc else rng.standard_normal(c.shape)
    Qbar = torch.empty(Q.shape[::-1], dtype=torch.float64, device="cuda")
    cbar = None if noc else torch.empty(disc.mesh.nelements, dtype=torch.float64, device="cuda")
    disc.ctx.rhs_vjp(Qbar, cbar, _dev(Q), _dev(lam))
    lhs = np.sum(_host(Qbar) * dQ) + (0.0 if noc else np.sum(cbar.cpu().numpy() * dc))
    R, dR = oracle_for(disc).rhs_jvp(Q, dQ, c, dc)
    rhs = np.sum(lam * dR)
    assert abs(lhs - rhs) <= 1e-12 * np.sum(np.abs(lam * dR)), (lhs, rhs)


def test_scalar_general_geometry_adjoint_solve():
    disc, Q0 = _general(3, 4, "split_lxf", "GLL", True)
    rng = np.random.default_rng(93)
    c, _ = _with_c(disc, "split_lxf", 1.0 + 0.2 * rng.random(disc.mesh.nelements))
    rho_t, w = _functional_inputs(disc, 5)
    dt = 0.3 * disc.ctx.max_dt(Q0, 1.0)
    nsteps = 8
    g = torch.empty(Q0.shape[::-1], dtype=torch.float64, device="cuda")
    gc = torch.empty(disc.mesh.nelements, dtype=torch.float64, device="cuda")
    J, nfwd = disc.ctx.adjoint_solve(_dev(Q0), dt, nsteps, 3, _dev(rho_t), _dev(w), g, gc)
    o = oracle_for(disc)
    for k in range(2):
        dQ = rng.standard_normal(Q0.shape)
        dc = rng.standard_normal(c.shape)
        Jo, dJo = o.solve_jvp(Q0, dQ, c, dc, dt, nsteps, rho_t, w)
        assert abs(J - Jo) <= 1e-12 * abs(Jo)
        ours = np.sum(_host(g) * dQ) + np.sum(gc.cpu().numpy() * dc)
        assert abs(ours - dJo) <= 1e-10 * abs(dJo), (ours, dJo)
