"""GPU parity: libflou_cuda against the CPU oracle on the same inputs, through the C ABI.

Bars: one residual to <= 1e-12 relative L-inf per variable, N SSP-RK3 steps to
<= 1e-10; connectivity/index work is bit-exact (set-up tests).  Relative L-inf is
max_v max_i |a - b| / max_i |b| per variable.
"""
import numpy as np
import pytest

import flou_cuda as F
import oracle_ref
from cases import build, oracle_for, rel_linf, smooth_euler_state

pytestmark = pytest.mark.gpu

RES_TOL = 1e-12
STEP_TOL = 1e-10


def _euler(dim):
    return F.EulerEquation(dim, 1.4)


def _ops():
    return {
        "strong_lxf": lambda: F.StrongDivOperator(F.LxF(F.StdAverage(), 1.0)),
        "strong_lxf_half": lambda: F.StrongDivOperator(F.LxF(F.StdAverage(), 0.5)),
        "strong_hllc": lambda: F.StrongDivOperator(F.HLLC()),
        "strong_hll": lambda: F.StrongDivOperator(F.HLL()),
        "strong_std": lambda: F.StrongDivOperator(F.StdAverage()),
        "split_chandra_hllc": lambda: F.SplitDivOperator(F.ChandrasekharAverage(), F.HLLC()),
        "split_chandra_chandra": lambda: F.SplitDivOperator(F.ChandrasekharAverage(), F.ChandrasekharAverage()),
        "split_chandra_lxfc": lambda: F.SplitDivOperator(F.LxF(F.ChandrasekharAverage(), 1.0)),
        "split_kg_lxf": lambda: F.SplitDivOperator(F.KennedyGruberAverage(), F.LxF(F.StdAverage(), 1.0)),
        "split_std_lxf": lambda: F.SplitDivOperator(F.LxF(F.StdAverage(), 1.0)),
        "split_chandra_md": lambda: F.SplitDivOperator(F.MatrixDissipation(F.ChandrasekharAverage(), 1.0)),
        "split_chandra_sd": lambda: F.SplitDivOperator(F.ScalarDissipation(F.ChandrasekharAverage(), 1.0)),
        "strong_md_std": lambda: F.StrongDivOperator(F.MatrixDissipation(F.StdAverage(), 0.7)),
        "strong_sd_std": lambda: F.StrongDivOperator(F.ScalarDissipation(F.StdAverage(), 1.0)),
        "hybrid_chandra_lxfc": lambda: F.HybridDivOperator(F.ChandrasekharAverage(),
                                                           F.LxF(F.ChandrasekharAverage(), 1.0), 1e-3),
        "hybrid_chandra_hllc_fv": lambda: F.HybridDivOperator(F.ChandrasekharAverage(), F.HLLC(),
                                                              F.LxF(F.ChandrasekharAverage(), 1.0), 0.1),
        "hybrid_kg_lxf": lambda: F.HybridDivOperator(F.KennedyGruberAverage(), F.LxF(F.StdAverage(), 1.0), 1e-2),
        "hybrid_md": lambda: F.HybridDivOperator(F.MatrixDissipation(F.ChandrasekharAverage(), 1.0), 1.0),
        "hybrid_highorder": lambda: F.HybridDivOperator(F.ChandrasekharAverage(),
                                                        F.LxF(F.ChandrasekharAverage(), 1.0), 1e30),
    }


EULER_CASES = [
    (1, 6, (7,), "split_chandra_lxfc"),
    (1, 4, (5,), "strong_lxf"),
    (1, 5, (6,), "strong_hllc"),
    (2, 5, (4, 4), "strong_lxf"),
    (2, 5, (3, 4), "strong_hllc"),
    (2, 4, (3, 3), "strong_hll"),
    (2, 3, (4, 3), "strong_std"),
    (2, 5, (3, 3), "split_chandra_lxfc"),
    (2, 6, (3, 2), "split_chandra_chandra"),
    (2, 4, (3, 3), "split_kg_lxf"),
    (2, 4, (3, 3), "split_std_lxf"),
    (2, 5, (3, 3), "strong_lxf_half"),
    (3, 4, (3, 3, 3), "split_chandra_hllc"),
    (3, 8, (2, 2, 2), "split_chandra_hllc"),
    (3, 3, (3, 2, 3), "strong_lxf"),
    (3, 3, (2, 3, 2), "split_chandra_chandra"),
    (3, 5, (2, 2, 2), "split_kg_lxf"),
    (3, 4, (2, 2, 2), "split_std_lxf"),
]


def _check(disc, Q, nsteps=5, res_tol=RES_TOL, step_tol=STEP_TOL, arrays=None, cfl=0.3):
    o = oracle_for(disc, arrays)
    ref = o.rhs(Q)
    dQ = disc.new_state()
    disc.ctx.rhs(dQ, Q)
    e_res = rel_linf(dQ, ref)
    assert e_res <= res_tol, "residual rel err %.3e" % e_res
    dt = cfl * disc.ctx.max_dt(Q, 1.0)
    Qg = Q.copy(order="F")
    disc.ctx.step(Qg, dt, nsteps)
    e_step = rel_linf(Qg, o.ssprk3(Q, dt, nsteps))
    assert e_step <= step_tol, "%d-step rel err %.3e" % (nsteps, e_step)
    return e_res, e_step


@pytest.mark.parametrize("dim,n,ne,op", EULER_CASES)
def test_euler_periodic(dim, n, ne, op):
    disc = build(dim, n, ne, _euler(dim), _ops()[op]())
    _check(disc, smooth_euler_state(disc, seed=dim * 10 + n))


def _jumpy_state(disc, seed):
    """A smooth state plus a different constant offset of the primitives in every element, so the
    traces jump at every interface (the dissipation terms act)."""
    eq = disc.equation
    d = disc.mesh.dim
    P = eq.vars_cons2prim(smooth_euler_state(disc, seed=seed))
    rng = np.random.default_rng(seed)
    P += np.repeat(0.05 * rng.standard_normal((disc.mesh.nelements, d + 2)), disc.std.n ** d, axis=0)
    return np.asfortranarray(eq.vars_prim2cons(P))


@pytest.mark.parametrize("dim,n,ne,op", [(1, 5, (6,), "split_chandra_md"), (1, 4, (5,), "split_chandra_sd"),
                                         (2, 5, (3, 4), "split_chandra_md"), (2, 4, (3, 3), "split_chandra_sd"),
                                         (2, 4, (3, 3), "strong_md_std"), (2, 3, (4, 3), "strong_sd_std"),
                                         (3, 4, (2, 3, 2), "split_chandra_md"), (3, 3, (3, 2, 2), "split_chandra_sd"),
                                         (3, 5, (2, 2, 2), "strong_md_std")])
def test_euler_dissipation_fluxes(dim, n, ne, op):
    """ScalarDissipation / MatrixDissipation (Euler.jl:228-380) on states whose traces jump."""
    disc = build(dim, n, ne, _euler(dim), _ops()[op]())
    _check(disc, _jumpy_state(disc, seed=dim * 7 + n))


@pytest.mark.parametrize("dim,n,ne,op", [(1, 5, (6,), "hybrid_chandra_lxfc"), (2, 4, (3, 3), "hybrid_chandra_lxfc"),
                                         (2, 5, (3, 2), "hybrid_chandra_hllc_fv"), (2, 4, (3, 3), "hybrid_kg_lxf"),
                                         (2, 4, (3, 3), "hybrid_md"), (3, 3, (2, 3, 2), "hybrid_chandra_lxfc"),
                                         (3, 5, (2, 2, 2), "hybrid_chandra_hllc_fv"), (3, 8, (2, 1, 1), "hybrid_kg_lxf"),
                                         (3, 4, (2, 2, 2), "hybrid_highorder")])
def test_euler_hybrid_operator(dim, n, ne, op):
    """HybridDivOperator (OpDivergence.jl:442-604) on states whose traces jump, against the
    oracle's literal restatement (the reference's O(n³) subcell sums)."""
    disc = build(dim, n, ne, _euler(dim), _ops()[op]())
    # CFL 0.2: with element jumps, p = 7 blows up at 0.3 on the oracle too
    _check(disc, _jumpy_state(disc, seed=dim * 5 + n), cfl=0.2)


GAUSS_CASES = [
    (1, 4, (5,), "split_chandra_lxfc"), (1, 5, (4,), "hybrid_md"), (1, 2, (6,), "split_std_lxf"),
    (2, 4, (3, 3), "split_chandra_chandra"), (2, 5, (3, 2), "split_kg_lxf"), (2, 3, (3, 3), "split_std_lxf"),
    (2, 4, (3, 3), "hybrid_chandra_hllc_fv"), (2, 6, (2, 2), "hybrid_kg_lxf"), (2, 8, (2, 2), "hybrid_highorder"),
    (3, 3, (2, 2, 2), "split_chandra_hllc"), (3, 4, (2, 2, 2), "hybrid_chandra_lxfc"),
    (3, 8, (2, 1, 1), "split_chandra_lxfc"), (3, 8, (1, 1, 2), "hybrid_md"), (3, 5, (2, 2, 1), "split_std_lxf"),
]


@pytest.mark.parametrize("dim,n,ne,op", GAUSS_CASES)
def test_euler_gauss_nodes(dim, n, ne, op):
    """Split and hybrid operators on Gauss nodes: the entropy-projected coupling of
    OpDivergence.jl:301-437 / 614-780, on states whose traces jump."""
    disc = build(dim, n, ne, _euler(dim), _ops()[op](), basis="GL")
    _check(disc, _jumpy_state(disc, seed=dim * 11 + n), cfl=0.2)


def test_euler_gauss_nodes_walls():
    eq = _euler(2)
    Pin = np.array([1.1, 0.0, 0.3, 1.05])
    bcs = {"1": F.EulerSlipBC(), "2": F.EulerSlipBC(), "3": F.EulerInflowBC(eq.vars_prim2cons(Pin)),
           "4": F.EulerOutflowBC()}
    for op in ("split_chandra_md", "hybrid_chandra_lxfc"):
        disc = build(2, 4, (3, 3), eq, _ops()[op](), periodic=(), bcs=bcs, basis="GL")
        _check(disc, _jumpy_state(disc, seed=4), cfl=0.2)


def test_euler_dissipation_fluxes_walls():
    eq = _euler(2)
    Pin = np.array([1.1, 0.0, 0.3, 1.05])
    bcs = {"1": F.EulerSlipBC(), "2": F.EulerSlipBC(), "3": F.EulerInflowBC(eq.vars_prim2cons(Pin)),
           "4": F.EulerOutflowBC()}
    disc = build(2, 4, (3, 3), eq, _ops()["split_chandra_md"](), periodic=(), bcs=bcs)
    _check(disc, _jumpy_state(disc, seed=3))


@pytest.mark.parametrize("n", range(2, 9))
def test_euler2d_strong_all_orders(n):
    disc = build(2, n, (3, 2), _euler(2), _ops()["strong_lxf"]())
    _check(disc, smooth_euler_state(disc, seed=n))


@pytest.mark.parametrize("n", range(2, 9))
def test_euler3d_split_all_orders(n):
    disc = build(3, n, (2, 2, 2), _euler(3), _ops()["split_chandra_hllc"]())
    _check(disc, smooth_euler_state(disc, seed=100 + n), nsteps=3)


@pytest.mark.parametrize("dim,op", [(2, "strong_lxf"), (2, "split_chandra_hllc"), (3, "split_chandra_hllc"),
                                    (1, "strong_hllc")])
def test_euler_walls_inflow_outflow(dim, op):
    eq = _euler(dim)
    # x: slip walls; y: inflow / outflow; z: periodic
    per = (2,) if dim == 3 else ()
    mesh_bcs = {"1": F.EulerSlipBC(), "2": F.EulerSlipBC()}
    if dim >= 2:
        Pin = np.zeros(dim + 2)
        Pin[0], Pin[2], Pin[-1] = 1.1, 0.3, 1.05
        mesh_bcs["3"] = F.EulerInflowBC(eq.vars_prim2cons(Pin))
        mesh_bcs["4"] = F.EulerOutflowBC()
    disc = build(dim, 4, (3,) * dim, eq, _ops()[op](), periodic=per, bcs=mesh_bcs)
    _check(disc, smooth_euler_state(disc, seed=7))


@pytest.mark.parametrize("dim,op", [(2, "split_chandra_lxfc"), (3, "split_chandra_hllc"), (2, "strong_hllc"),
                                    (2, "hybrid_chandra_lxfc")])
def test_euler_generic_bc_varying_state(dim, op):
    """GenericBC(Qext) with a state that varies along the boundary (FlouSpatial.jl:80-91): the
    device reads one state per boundary face node from flou_set_bc_field."""
    eq = _euler(dim)

    def prim(x):
        P = np.zeros(dim + 2)
        P[0] = 1.0 + 0.3 * np.sin(2 * np.pi * x[1]) * (np.cos(2 * np.pi * x[2]) if dim == 3 else 1.0)
        P[1], P[2], P[-1] = 0.4, 0.1 * np.cos(2 * np.pi * x[1]), 1.0 + 0.1 * x[1]
        return eq.vars_prim2cons(P)

    qext = lambda _q, x, _f, _t, _e: prim(x)
    disc = build(dim, 4, (3,) * dim, eq, _ops()[op](), periodic=tuple(range(2, dim)),
                 bcs={"1": F.GenericBC(qext), "2": F.GenericBC(qext), "3": F.EulerSlipBC(),
                      "4": F.EulerSlipBC()}, box=((0.0,) * dim, (1.0,) * dim))
    assert isinstance(disc.bcs[0], F.equations.StateFieldBC)
    _check(disc, smooth_euler_state(disc, seed=13))


def test_oracle_built_operators_general_path():
    """Flou-style fitted operators (tiny non-zero off-end entries) take the general
    interpolation path on the GPU."""
    disc = build(2, 5, (3, 3), _euler(2), _ops()["strong_lxf"]())
    a = disc.abi_arrays()
    o = oracle_ref.operators(5, True)
    for k in ("D", "Ds", "Dsharp", "omega", "l_l", "l_r", "dg_l", "dg_r"):
        a[k] = o[k]
    disc._ctx = F.Context(disc.config, a, disc.mesh.nelements, disc.mesh.nfaces)
    _check(disc, smooth_euler_state(disc, seed=5), arrays=a)


@pytest.mark.parametrize("dim,basis,op", [(1, "GL", "strong"), (2, "GL", "strong"), (3, "GLL", "strong"),
                                          (2, "GLL", "split"), (3, "GLL", "split"), (1, "GLL", "strong")])
def test_linear_advection(dim, basis, op):
    eq = F.LinearAdvection(*[1.0, -0.7, 0.4][:dim])
    o = (F.StrongDivOperator(F.LxF(F.StdAverage(), 1.0)) if op == "strong"
         else F.SplitDivOperator(F.LxF(F.StdAverage(), 1.0)))
    disc = build(dim, 5, (3,) * dim, eq, o, basis=basis)
    Q = np.asfortranarray(1.0 + 0.3 * np.sin(np.pi * disc.coords[:, :1]).prod(axis=1, keepdims=True))
    _check(disc, Q)


def test_linear_advection_dirichlet():
    eq = F.LinearAdvection(1.0, 0.5)
    bcs = {"1": F.DirichletBC([0.5]), "2": F.OutflowBC(), "3": F.DirichletBC([0.25]), "4": F.OutflowBC()}
    disc = build(2, 4, (3, 3), eq, F.StrongDivOperator(F.LxF(F.StdAverage(), 1.0)), periodic=(), bcs=bcs)
    Q = np.asfortranarray(1.0 + 0.2 * np.cos(disc.coords[:, :1]))
    _check(disc, Q)


@pytest.mark.parametrize("op", ["strong", "split"])
def test_burgers(op):
    eq = F.BurgersEquation()
    o = (F.StrongDivOperator(F.LxF(F.StdAverage(), 1.0)) if op == "strong"
         else F.SplitDivOperator(F.LxF(F.StdAverage(), 1.0)))
    disc = build(1, 6, (8,), eq, o)
    Q = np.asfortranarray(1.5 + 0.5 * np.sin(np.pi * disc.coords[:, :1]))
    _check(disc, Q)


def test_max_dt_matches_oracle():
    eq = _euler(2)
    disc = build(2, 5, (8, 8), eq, _ops()["strong_lxf"](), box=((-5.0, -5.0), (5.0, 5.0)))
    Q = np.asfortranarray(F.initial.isentropic_vortex(eq, disc.coords, (1.0, 2.0), period=(10, 10)))
    dt = disc.ctx.max_dt(Q, 0.5)
    ref = oracle_for(disc).max_dt(Q, 0.5, disc.std.omega)
    assert abs(dt - ref) <= 4e-16 * ref


def test_nonphysical_state_raises_domain_error():
    eq = _euler(2)
    disc = build(2, 4, (3, 3), eq, _ops()["strong_lxf"]())
    Q = smooth_euler_state(disc, seed=2)
    Q[17, 0] = -1.0   # negative density, planted on the host
    with pytest.raises(F.DomainError) as ei:
        disc.ctx.rhs(disc.new_state(), Q)
    assert "element 2" in str(ei.value)   # node 17 of 16-node elements
    # the context stays usable
    Q[17, 0] = 1.0
    disc.ctx.rhs(disc.new_state(), Q)


def test_device_pointers_and_determinism():
    torch = pytest.importorskip("torch")
    eq = _euler(3)
    disc = build(3, 4, (3, 3, 3), eq, _ops()["split_chandra_hllc"]())
    Q = smooth_euler_state(disc, seed=9)
    Qd = torch.from_numpy(np.ascontiguousarray(Q.T)).cuda()
    dQd = torch.empty_like(Qd)
    disc.ctx.rhs(dQd, Qd)
    ref = oracle_for(disc).rhs(Q)
    assert rel_linf(dQd.cpu().numpy().T, ref) <= RES_TOL
    again = torch.empty_like(Qd)
    disc.ctx.rhs(again, Qd)
    assert torch.equal(again, dQd)   # bitwise reproducible (no atomics on the data path)
    a, b = Qd.clone(), Qd.clone()
    disc.ctx.step(a, 1e-3, 4)
    disc.ctx.step(b, 1e-3, 2)
    disc.ctx.step(b, 1e-3, 2)
    assert torch.equal(a, b)   # graph replays are deterministic


@pytest.mark.parametrize("basis,eta,op", [("GLL", "SD", "strong_lxf"), ("GLL", "SD", "split_chandra_lxfc"),
                                          ("GLL", 0.3, "hybrid_chandra_lxfc"), ("GL", "SD", "split_kg_lxf"),
                                          ("GL", 0.0, "strong_hllc")])
def test_vcjh_reconstructions(basis, eta, op):
    """VCJHrec lifts (Reconstruction.jl:69-110) reach every node of a line (on Gauss-Lobatto nodes
    Huynh's η is DGSEM again, so SD and η = 0.3 are used there); the split and hybrid kernels keep
    their volume terms and take the general lift, the hybrid's telescoped sums use 2D - B with
    DGSEM's corner B as the reference's 2 ω_l D_lk sums do."""
    eq = _euler(2)
    mesh = F.CartesianMesh((-1.0, -1.0), (1.0, 1.0), (3, 3))
    F.apply_periodicBCs(mesh, ("1", "2"), ("3", "4"))
    b = F.LagrangeBasis(basis, 5)
    std = F.StdQuad(b, F.VCJHrec(5, eta), 4)
    disc = F.MultielementDisc(mesh, std, eq, _ops()[op](), {})
    assert np.abs(disc.std.dg[0][1:]).max() > 1e-3   # the lift is not confined to the end nodes
    _check(disc, smooth_euler_state(disc, seed=13), cfl=0.2)


def test_refined_reciprocal_and_square_root_within_one_ulp():
    """The kernels' reciprocal and square root (the MUFU approximations rcp.approx.ftz.f64 /
    rsqrt.approx.ftz.f64 refined by one third-order step) against CUDA's correctly rounded 1/x
    and sqrt(x) on 2^26 doubles with exponents in [2^-40, 2^40]: within 1 ulp (2 units of 2^-53)."""
    import ctypes
    lib = F.load()
    a, b = ctypes.c_double(), ctypes.c_double()
    assert lib.flou_check_refined_math(1 << 26, ctypes.byref(a), ctypes.byref(b)) == 0
    assert 0.0 < a.value <= 2.0 and 0.0 < b.value <= 2.0, (a.value, b.value)
