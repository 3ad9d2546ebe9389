"""The benchmark configurations at full size.

The 2D vortex (16² elements, p=4, strong form, Rusanov, 100 SSP-RK3 steps) against the
oracle; the 3D Taylor-Green meshes (32³ p=3 and 16³ p=7, split form Chandrashekar + HLLC,
2,097,152 nodes each) through one residual (backward error and relative L-inf against the
oracle's own conditioning floor) and the configuration's 50 SSP-RK3 steps against the oracle,
and size-independent properties: discrete conservation, freestream preservation, bitwise
determinism.
"""
import math

import numpy as np
import pytest

import flou_cuda as F
from cases import oracle_for, rel_linf

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def test_config1_vortex_100_steps():
    eq = F.EulerEquation(2, 1.4)
    mesh = F.CartesianMesh((-5.0, -5.0), (5.0, 5.0), (16, 16))
    F.apply_periodicBCs(mesh, ("1", "2"), ("3", "4"))
    b = F.LagrangeBasis("GLL", 5)
    disc = F.MultielementDisc(mesh, F.StdQuad(b, F.DGSEMrec(b), 4), eq, F.StrongDivOperator(F.LxF(F.StdAverage(), 1.0)))
    rng = np.random.default_rng(1)
    Q0 = np.asfortranarray(F.initial.isentropic_vortex(eq, disc.coords, rng.uniform(-1, 1, 2), beta=5.0,
                                                       period=(10.0, 10.0)))
    dt = F.get_max_dt(Q0, disc, eq, 0.4)   # CFL 0.5 is unstable with SSP-RK3 here (also on the oracle)
    sol, _ = F.timeintegrate(Q0, disc, eq, F.SSPRK33(), 100 * dt, dt=dt)
    ref = oracle_for(disc).ssprk3(Q0, dt, 100)
    assert rel_linf(sol.u[-1], ref) <= 1e-10


@pytest.fixture(scope="module", params=[(32, 4), (16, 8)], ids=["32c_p3", "16c_p7"])
def tgv(request):
    import bench
    nel, n = request.param
    disc, Q0 = bench.make_tgv(nel, n)
    return disc, Q0


def _term_scale(disc, Q):
    """Size of the terms the residual sums, per variable: max |F| x max row sum |D♯| x max Ja/J x d.
    At Mach 0.1 the pressure (p0 = 1/(γM²) ≈ 71) makes these ~1e4 times the residual itself, so two
    evaluations that round differently differ by ε times this, not by ε times the result."""
    eq = disc.equation
    P = eq.vars_cons2prim(Q)
    p = P[:, 4]
    F = np.stack([np.abs(Q[:, 1]), np.abs(Q[:, 1] * P[:, 1]) + np.abs(p), np.abs(Q[:, 2] * P[:, 1]) + np.abs(p),
                  np.abs(Q[:, 3] * P[:, 1]) + np.abs(p), np.abs((Q[:, 4] + p) * P[:, 1])], axis=1)
    D = np.max(np.sum(np.abs(disc.std.Dsharp), axis=1))
    JaJ = np.max(disc.Ja[:, 0]) / np.min(disc.J)
    return np.max(F, axis=0) * D * JaJ * disc.mesh.dim


def test_tgv_residual_against_oracle(tgv):
    disc, Q0 = tgv
    Qd = torch.from_numpy(np.ascontiguousarray(Q0.T)).cuda()
    dQ = torch.empty_like(Qd)
    disc.ctx.rhs(dQ, Qd)
    ref = oracle_for(disc).rhs(Q0)
    err = np.max(np.abs(dQ.cpu().numpy().T - ref), axis=0)
    assert np.all(err <= 1e-14 * _term_scale(disc, Q0)), (err, _term_scale(disc, Q0))


def test_tgv_residual_relative_linf_against_the_oracles_own_spread(tgv):
    """The relative L-inf error per DOF of one residual, against the oracle.  At Mach 0.1 the
    residual is ~1e4 times smaller than the terms it sums, so this is held to the larger of 1e-12
    and four times the oracle's own spread: the change of the oracle's residual when its input
    moves by one ulp (relative perturbations of 1.1e-16 times a standard normal), the
    conditioning floor of the problem itself."""
    disc, Q0 = tgv
    Qd = torch.from_numpy(np.ascontiguousarray(Q0.T)).cuda()
    dQ = torch.empty_like(Qd)
    disc.ctx.rhs(dQ, Qd)
    o = oracle_for(disc)
    ref = o.rhs(Q0)
    err = rel_linf(dQ.cpu().numpy().T, ref)
    rng = np.random.default_rng(0)
    spread = rel_linf(o.rhs(np.asfortranarray(Q0 * (1 + 1.1e-16 * rng.standard_normal(Q0.shape)))), ref)
    print("TGV %s residual: relative L-inf %.3e, oracle spread under 1-ulp input changes %.3e"
          % (disc.mesh.nelements, err, spread))
    assert err <= max(1e-12, 4.0 * spread), (err, spread)


def test_tgv_50_steps_against_oracle(tgv):
    """The configuration's 50 SSP-RK3 steps at the benchmark's fixed dt (CFL 0.15 in get_max_dt's
    definition) on the full mesh, against the oracle's 50 steps: relative L-inf <= 1e-10."""
    import bench
    disc, Q0 = tgv
    Qd = torch.from_numpy(np.ascontiguousarray(Q0.T)).cuda()
    dt = bench.TGV_CFL * disc.ctx.max_dt(Qd, 1.0)
    disc.ctx.step(Qd, dt, 50)
    ref = oracle_for(disc).ssprk3(Q0, dt, 50)
    err = rel_linf(Qd.cpu().numpy().T, ref)
    print("TGV %s after 50 SSP-RK3 steps: relative L-inf %.3e" % (disc.mesh.nelements, err))
    assert err <= 1e-10


def test_tgv_conservation_freestream_determinism(tgv):
    """Discrete conservation: the weighted sum of the residual over the periodic box is round-off.
    Its round-off is set by the summed terms (fluxes of ~p0 = 71 times D♯), not by the residual, so
    the bar is the larger of 1e-12 of Σ w|dQ| and three times the oracle's own sum (the reference's
    evaluation order on the CPU: 6.5e-12 and 9.0e-12 for the momenta at 16³ p=7).  Dropping the
    diagonal D♯_ii F̃_i term breaks it (4e-11 at 16³ p=7)."""
    disc, Q0 = tgv
    eq = disc.equation
    Qd = torch.from_numpy(np.ascontiguousarray(Q0.T)).cuda()
    dQ = torch.empty_like(Qd)
    disc.ctx.rhs(dQ, Qd)
    wn = np.tile(disc.std.omega, disc.mesh.nelements) * disc.J
    w = torch.from_numpy(wn).cuda()
    ref = oracle_for(disc).rhs(Q0)
    scales = [float(torch.sum(w * torch.abs(dQ[v]))) for v in range(5)]
    for v in range(5):
        total = float(torch.sum(w * dQ[v]))
        bar = max(1e-12 * max(scales[v], 1e-3 * max(scales)), 3.0 * abs(float(np.sum(wn * ref[:, v]))))
        assert abs(total) <= bar, (v, total, bar)
    again = torch.empty_like(Qd)
    disc.ctx.rhs(again, Qd)
    assert torch.equal(again, dQ)
    P = np.zeros((disc.ndofs, 5))
    P[:, 0], P[:, 1:4], P[:, 4] = 1.0, (0.3, -0.2, 0.1), 1.0 / (1.4 * 0.01)
    Uf = torch.from_numpy(np.ascontiguousarray(eq.vars_prim2cons(P).T)).cuda()
    disc.ctx.rhs(dQ, Uf)
    assert float(torch.max(torch.abs(dQ))) <= 1e-10   # freestream preserved (fluxes are O(1e2))
    # kinetic energy of the inviscid TGV is nearly conserved over a few steps
    q = Qd.clone()
    dt = 0.3 * disc.ctx.max_dt(q, 1.0)
    ke = lambda u: float(torch.sum(w * (u[1] ** 2 + u[2] ** 2 + u[3] ** 2) / (2 * u[0])))
    k0 = ke(q)
    disc.ctx.step(q, dt, 10)
    assert abs(ke(q) - k0) <= 1e-4 * k0
