"""General geometry on the GPU: unstructured straight-sided meshes whose elements are randomly
rotated (every master2slave orientation occurs in 3D) and whose interior nodes are displaced,
so J, the metric, the face frames and the surface Jacobians vary per node.  The residual and
SSP-RK3 steps are checked against the oracle (which runs the reference's general loops)."""
import numpy as np
import pytest

import flou_cuda as F
from flou_cuda import _lib as L
from cases import build, oracle_for, rel_linf
from test_unstructured import _state, _std

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _ops():
    return {
        "strong_lxf": lambda: F.StrongDivOperator(F.LxF(F.StdAverage(), 1.0)),
        "strong_hllc": lambda: F.StrongDivOperator(F.HLLC()),
        "split_chandra_lxfc": lambda: F.SplitDivOperator(F.ChandrasekharAverage(), F.LxF(F.ChandrasekharAverage(), 1.0)),
        "split_chandra_md": lambda: F.SplitDivOperator(F.MatrixDissipation(F.ChandrasekharAverage(), 1.0)),
        "split_kg_lxf": lambda: F.SplitDivOperator(F.KennedyGruberAverage(), F.LxF(F.StdAverage(), 1.0)),
        "split_std_lxf": lambda: F.SplitDivOperator(F.LxF(F.StdAverage(), 1.0)),
        # blend 0.5: dδ/db ~ 1/√c, so a small blending constant amplifies round-off in the indicator
        "hybrid_hllc": lambda: F.HybridDivOperator(F.ChandrasekharAverage(), F.HLLC(),
                                                   F.LxF(F.ChandrasekharAverage(), 1.0), 0.5),
        "hybrid_md": lambda: F.HybridDivOperator(F.MatrixDissipation(F.ChandrasekharAverage(), 1.0), 1.0),
        "hybrid_kg": lambda: F.HybridDivOperator(F.KennedyGruberAverage(), F.LxF(F.StdAverage(), 1.0), 1e-3),
    }


def _bcs(dim, eq, walls):
    if not walls:
        return {str(k): F.EulerOutflowBC() for k in range(1, 2 * dim + 1)}
    Pin = np.zeros(dim + 2)
    Pin[0], Pin[1], Pin[-1] = 1.05, 0.2, 1.1
    b = {"1": F.EulerInflowBC(eq.vars_prim2cons(Pin)), "2": F.EulerOutflowBC(), "3": F.EulerSlipBC(),
         "4": F.EulerSlipBC()}
    if dim == 3:
        b.update({"5": F.EulerSlipBC(), "6": F.EulerOutflowBC()})
    return b


def _disc(dim, n, op, walls=False, nel=3, seed=5, amp=0.12, basis="GLL"):
    eq = F.EulerEquation(dim, 1.4)
    mesh = F.perturbed_box(dim, nel, (0.0,) * dim, (1.0,) * dim, amp=amp, seed=seed)
    return F.MultielementDisc(mesh, _std(dim, n, dim + 2, basis), eq, _ops()[op](), _bcs(dim, eq, walls))


def _check(disc, Q, nsteps=4):
    o = oracle_for(disc)
    ref = o.rhs(Q)
    dQ = disc.new_state()
    disc.ctx.rhs(dQ, Q)
    assert rel_linf(dQ, ref) <= 1e-12, rel_linf(dQ, ref)
    dt = 0.2 * disc.ctx.max_dt(Q, 1.0)
    assert abs(dt - 0.2 * o.max_dt(Q, 1.0, disc.std.omega)) <= 1e-14 * dt
    Qg = Q.copy(order="F")
    disc.ctx.step(Qg, dt, nsteps)
    assert rel_linf(Qg, o.ssprk3(Q, dt, nsteps)) <= 1e-10


@pytest.mark.parametrize("dim,n,op", [(2, 4, "strong_lxf"), (2, 5, "split_chandra_lxfc"), (2, 3, "strong_hllc"),
                                      (2, 4, "split_kg_lxf"), (2, 4, "split_std_lxf"), (2, 4, "split_chandra_md"),
                                      (3, 3, "strong_lxf"), (3, 4, "split_chandra_lxfc"), (3, 3, "strong_hllc"),
                                      (3, 3, "split_kg_lxf"), (3, 4, "split_std_lxf"), (3, 3, "split_chandra_md"),
                                      (3, 6, "split_chandra_lxfc"), (2, 8, "strong_lxf")])
def test_unstructured_euler(dim, n, op):
    disc = _disc(dim, n, op)
    if dim == 3:
        assert len(set(disc.mesh.orientation.tolist())) == 8
    assert disc.ctx is not None
    _check(disc, _state(disc, seed=dim + n))


@pytest.mark.parametrize("dim,n,op", [(2, 4, "hybrid_hllc"), (2, 5, "hybrid_md"), (2, 6, "hybrid_kg"),
                                      (3, 3, "hybrid_hllc"), (3, 4, "hybrid_md"), (3, 5, "hybrid_kg"),
                                      (3, 7, "hybrid_hllc")])
def test_unstructured_hybrid(dim, n, op):
    """HybridDivOperator on perturbed, rotated elements: the subcell FV fluxes in the uploaded
    subcell-interface frames (flou_set_subgrid), against the oracle."""
    disc = _disc(dim, n, op, nel=2 if n > 6 else 3)
    _check(disc, _state(disc, seed=dim * 3 + n))


@pytest.mark.parametrize("dim,n,op", [(2, 4, "strong_lxf"), (2, 5, "split_chandra_lxfc"), (2, 4, "split_kg_lxf"),
                                      (2, 4, "hybrid_md"), (3, 3, "strong_hllc"), (3, 4, "split_chandra_lxfc"),
                                      (3, 3, "split_std_lxf"), (3, 4, "hybrid_hllc"), (3, 6, "split_chandra_md")])
def test_unstructured_gauss_nodes(dim, n, op):
    """Gauss nodes on perturbed, rotated elements: interpolated traces through master2slave, the
    general lift, and for the split and hybrid forms the projected states with the subcell normals
    of the line ends (flou_set_subgrid)."""
    disc = _disc(dim, n, op, basis="GL")
    _check(disc, _state(disc, seed=dim * 5 + n))


def test_unstructured_gauss_nodes_walls():
    disc = _disc(2, 4, "split_chandra_lxfc", walls=True, basis="GL")
    _check(disc, _state(disc, seed=12))


def test_unstructured_hybrid_p7_against_the_oracles_conditioning():
    """p = 7 on curved 3D elements: the oracle's own residual moves by ~5e-13 when its input is
    perturbed by one ulp (the split form's too), so the device is held to four times that spread."""
    disc = _disc(3, 8, "hybrid_hllc", nel=2)
    Q = _state(disc, seed=17)
    o = oracle_for(disc)
    ref = o.rhs(Q)
    rng = np.random.default_rng(0)
    spread = rel_linf(o.rhs(Q * (1 + 2.2e-16 * rng.choice([-1.0, 1.0], size=Q.shape))), ref)
    dQ = disc.new_state()
    disc.ctx.rhs(dQ, Q)
    assert rel_linf(dQ, ref) <= max(1e-12, 4 * spread)
    dt = 0.2 * disc.ctx.max_dt(Q, 1.0)
    Qg = Q.copy(order="F")
    disc.ctx.step(Qg, dt, 3)
    assert rel_linf(Qg, o.ssprk3(Q, dt, 3)) <= 1e-10


@pytest.mark.parametrize("dim,op", [(2, "strong_lxf"), (2, "split_chandra_lxfc"), (3, "split_chandra_lxfc"),
                                    (3, "strong_hllc"), (2, "hybrid_md"), (3, "hybrid_hllc")])
def test_unstructured_walls_inflow_outflow(dim, op):
    disc = _disc(dim, 4, op, walls=True)
    _check(disc, _state(disc, seed=11))


@pytest.mark.parametrize("dim,op", [(2, "strong"), (2, "split"), (3, "strong"), (3, "split")])
def test_unstructured_linear_advection(dim, op):
    eq = F.LinearAdvection(*([1.0, -0.5, 0.3][:dim]))
    mesh = F.perturbed_box(dim, 3, (0.0,) * dim, (1.0,) * dim, amp=0.1, seed=2)
    nf = F.LxF(F.StdAverage(), 1.0)
    oper = F.StrongDivOperator(nf) if op == "strong" else F.SplitDivOperator(nf)
    bcs = {str(k): F.DirichletBC([1.0]) for k in range(1, 2 * dim + 1)}
    disc = F.MultielementDisc(mesh, _std(dim, 4, 1), eq, oper, bcs)
    X = disc.coords
    Q = np.asfortranarray((1.0 + 0.3 * np.sin(3 * X[:, 0]) * np.cos(2 * X[:, 1]))[:, None])
    o = oracle_for(disc)
    dQ = disc.new_state()
    disc.ctx.rhs(dQ, Q)
    assert rel_linf(dQ, o.rhs(Q)) <= 1e-12
    dt = 1e-3
    Qg = Q.copy(order="F")
    disc.ctx.step(Qg, dt, 4)
    assert rel_linf(Qg, o.ssprk3(Q, dt, 4)) <= 1e-10


def test_unstructured_freestream_on_gpu():
    disc = _disc(3, 4, "split_chandra_lxfc", amp=0.2)
    P = np.zeros((disc.ndofs, 5))
    P[:, 0], P[:, 1:4], P[:, 4] = 1.2, (0.3, -0.2, 0.1), 1.7
    Q = np.asfortranarray(disc.equation.vars_prim2cons(P))
    dQ = disc.new_state()
    disc.ctx.rhs(dQ, Q)
    assert np.max(np.abs(dQ)) < 1e-11


def test_unstructured_limiter_and_monitors():
    disc = _disc(2, 4, "split_chandra_lxfc")
    Q = _state(disc, seed=3)
    P = disc.equation.vars_cons2prim(Q)
    P[20, 0] = 0.02
    Q = np.asfortranarray(disc.equation.vars_prim2cons(P))
    o = oracle_for(disc)
    disc.ctx.set_limiter(L.LIMITER_ZHANG_SHU, 0.1)
    Qg = Q.copy(order="F")
    disc.ctx.limit(Qg)
    assert rel_linf(Qg, o.limit(Q, 0.1, disc.std.omega)) <= 1e-13
    disc.ctx.set_limiter(L.LIMITER_NONE)
    for which in (L.MONITOR_KINETIC_ENERGY, L.MONITOR_ENTROPY):
        ref = o.monitor(Q, which, disc.std.omega)
        assert abs(disc.ctx.monitor(Q, which) - ref) <= 1e-13 * abs(ref)


def test_general_geometry_is_rejected_where_not_covered():
    # a batch is all Cartesian or all on general geometry
    disc = _disc(2, 4, "strong_lxf")
    Q = torch.from_numpy(np.ascontiguousarray(_state(disc).T)).cuda()
    cart = build(2, 4, (3, 3), F.EulerEquation(2, 1.4), _ops()["strong_lxf"]())
    Qc = torch.from_numpy(np.ascontiguousarray(_state(cart).T)).cuda()
    with pytest.raises(F.FlouError) as ei:
        F.Batch([disc, cart], [Q, Qc], [1e-3, 1e-3])
    assert ei.value.status == L.FLOU_ERR_ARG
    # the split form of a scalar equation has no Gauss-node form (no entropy variables)
    mesh = F.perturbed_box(2, 3, (0.0, 0.0), (1.0, 1.0), amp=0.1, seed=1)
    b = F.LagrangeBasis("GL", 4)
    adv = F.MultielementDisc(mesh, F.StdQuad(b, F.DGSEMrec(b), 1), F.LinearAdvection(1.0, 0.5),
                             F.SplitDivOperator(F.StdAverage(), F.StdAverage()),
                             {str(k): F.DirichletBC([1.0]) for k in range(1, 5)})
    with pytest.raises(F.FlouError) as ei:
        adv.ctx
    assert ei.value.status == L.FLOU_ERR_UNSUPPORTED
