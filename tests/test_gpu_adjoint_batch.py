"""Batched discrete adjoint: many independent solves reversed in lockstep under one
device-memory budget (flou_adjoint_solve_batch).  Each instance's gradient must be
bit-identical to its own single-instance checkpointed solve (the checkpoint schedule does not
change the arithmetic) and agree with the dual-number oracle; the budget sets the number of
snapshots."""
import re

import numpy as np
import pytest

import flou_cuda as F
from cases import build, oracle_for, smooth_euler_state

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

from test_gpu_adjoint import _dev, _host, _split, _lxf, _functional_inputs, _tgv_state  # noqa: E402


def _instances():
    L = 2 * np.pi
    out = []
    for k, (dim, n, ne, op) in enumerate([(3, 4, (3, 2, 2), _split), (3, 5, (2, 2, 2), _split),
                                          (3, 3, (3, 3, 3), _split), (2, 4, (4, 3), _lxf)]):
        eq = F.EulerEquation(dim, 1.4)
        if dim == 3:
            disc = build(3, n, ne, eq, op(), box=((0.0,) * 3, (L,) * 3))
            Q0 = _tgv_state(disc, 0.1 + 0.05 * k, k)
        else:
            disc = build(2, n, ne, eq, op(), box=((-5.0, -5.0), (5.0, 5.0)))
            Q0 = np.asfortranarray(F.initial.vortex_bump(eq, disc.coords, (0.3, -0.4), 4.0, 0.05,
                                                         period=(10.0, 10.0)))
        rng = np.random.default_rng(40 + k)
        c = 1.0 + 0.2 * rng.random(disc.mesh.nelements)
        disc.ctx.set_dissipation(c)
        rho_t, w = _functional_inputs(disc, 50 + k)
        dt = 0.2 * disc.ctx.max_dt(Q0, 1.0)   # c up to 1.2 widens LxF's spectrum: 0.3 is unstable at p = 4
        out.append(dict(disc=disc, Q0=Q0, c=c, rho_t=rho_t, w=w, dt=dt))
    return out


def _run_batch(inst, nsteps, budget, nstreams=3):
    g = [torch.empty(x["Q0"].shape[::-1], dtype=torch.float64, device="cuda") for x in inst]
    gc = [torch.empty(x["disc"].mesh.nelements, dtype=torch.float64, device="cuda") for x in inst]
    J, nf, ns = F.adjoint_solve_batch([x["disc"] for x in inst], [_dev(x["Q0"]) for x in inst],
                                      [x["dt"] for x in inst], nsteps, budget,
                                      [_dev(x["rho_t"]) for x in inst], [_dev(x["w"]) for x in inst], g, gc,
                                      nstreams=nstreams)
    return J, g, gc, nf, ns


def _snap_bytes(inst):
    return sum((x["disc"].ndofs * x["disc"].nvariables * 8 + 255) // 256 * 256 for x in inst)


def test_batched_adjoint_matches_single_solves_and_oracle():
    inst = _instances()
    nsteps = 8
    J, g, gc, nf, ns = _run_batch(inst, nsteps, 8 << 30)
    assert ns == nsteps - 1 and nf == nsteps - 1
    for k, x in enumerate(inst):
        d = x["disc"]
        g1 = torch.empty_like(g[k])
        gc1 = torch.empty_like(gc[k])
        J1, _ = d.ctx.adjoint_solve(_dev(x["Q0"]), x["dt"], nsteps, 3, _dev(x["rho_t"]), _dev(x["w"]), g1, gc1)
        assert J[k] == J1
        assert torch.equal(g[k], g1) and torch.equal(gc[k], gc1)
    x = inst[0]
    rng = np.random.default_rng(1)
    dQ = rng.standard_normal(x["Q0"].shape)
    dc = rng.standard_normal(x["c"].shape)
    Jo, dJo = oracle_for(x["disc"]).solve_jvp(x["Q0"], dQ, x["c"], dc, x["dt"], nsteps, x["rho_t"], x["w"])
    ours = np.sum(_host(g[0]) * dQ) + np.sum(gc[0].cpu().numpy() * dc)
    assert abs(J[0] - Jo) <= 1e-12 * abs(Jo)
    assert abs(ours - dJo) <= 1e-10 * abs(dJo), (ours, dJo)


def test_budget_sets_the_snapshots():
    inst = _instances()
    nsteps = 10
    with pytest.raises(F.FlouError) as ei:
        _run_batch(inst, nsteps, 0)
    m = re.search(r"below the (\d+) bytes", str(ei.value))
    assert m, str(ei.value)
    fixed = int(m.group(1))
    J0, g0, gc0, nf0, ns0 = _run_batch(inst, nsteps, fixed + 2 * _snap_bytes(inst))
    assert ns0 == 2 and nf0 > nsteps - 1
    J1, g1, gc1, nf1, ns1 = _run_batch(inst, nsteps, fixed)   # no snapshot: recompute from Q0
    assert ns1 == 0 and nf1 == nsteps * (nsteps - 1) // 2
    J2, g2, gc2, nf2, ns2 = _run_batch(inst, nsteps, 8 << 30, nstreams=1)
    assert ns2 == nsteps - 1
    for k in range(len(inst)):
        assert J0[k] == J1[k] == J2[k]
        assert torch.equal(g0[k], g1[k]) and torch.equal(g0[k], g2[k])
        assert torch.equal(gc0[k], gc1[k]) and torch.equal(gc0[k], gc2[k])


def test_batched_adjoint_with_2n_storage_and_limiter_instances():
    """Instances stepping with ORK256, with the Zhang-Shu limiter, with both, and plain SSP-RK3
    in one lockstep sweep (a stream holding a 2N-storage instance keeps its own register): each
    gradient is bit-identical to its single solve, and the limited 2N-storage one agrees with the
    dual-number oracle through the same limited method."""
    from flou_cuda import _lib as L
    from test_oracle_kat import _dipped_state
    inst = _instances()
    m = F.ORK256()
    eq = F.EulerEquation(2, 1.4)
    extra = []
    for k, (lsrk, lim) in enumerate([(True, False), (False, True), (True, True)]):
        disc = build(2, 4, (3, 3), eq, _lxf())
        Q0 = _dipped_state(disc, seed=30 + k) if lim else smooth_euler_state(disc, seed=30 + k)
        c = 1.0 + 0.1 * np.random.default_rng(60 + k).random(disc.mesh.nelements)
        disc.ctx.set_dissipation(c)
        if lsrk:
            disc.ctx.set_integrator(m.A, m.B)
        if lim:
            disc.ctx.set_limiter(L.LIMITER_ZHANG_SHU, 0.5)
        rho_t, w = _functional_inputs(disc, 70 + k)
        dt = 0.2 * disc.ctx.max_dt(Q0, 1.0)
        extra.append(dict(disc=disc, Q0=Q0, c=c, rho_t=rho_t, w=w, dt=dt, lsrk=lsrk, lim=lim))
    inst = inst[:2] + extra
    nsteps = 6
    for budget in (8 << 30, None):
        if budget is None:   # two snapshots: recomputation through the limited / 2N-storage steps
            with pytest.raises(F.FlouError) as ei:
                _run_batch(inst, nsteps, 0)
            budget = int(re.search(r"below the (\d+) bytes", str(ei.value)).group(1)) + 2 * _snap_bytes(inst)
        J, g, gc, nf, ns = _run_batch(inst, nsteps, budget)
        for k, x in enumerate(inst):
            d = x["disc"]
            g1 = torch.empty_like(g[k])
            gc1 = torch.empty_like(gc[k])
            J1, _ = d.ctx.adjoint_solve(_dev(x["Q0"]), x["dt"], nsteps, 3, _dev(x["rho_t"]), _dev(x["w"]), g1, gc1)
            assert J[k] == J1
            assert torch.equal(g[k], g1) and torch.equal(gc[k], gc1)
    x = inst[-1]
    rng = np.random.default_rng(2)
    dQ = rng.standard_normal(x["Q0"].shape)
    dc = rng.standard_normal(x["c"].shape)
    Jo, dJo = oracle_for(x["disc"]).solve_jvp_lsrk(x["Q0"], dQ, x["c"], dc, x["dt"], nsteps, x["rho_t"], x["w"],
                                                   m.A, m.B, m.c, minval=0.5, omega_tp=x["disc"].std.omega)
    ours = np.sum(_host(g[-1]) * dQ) + np.sum(gc[-1].cpu().numpy() * dc)
    assert abs(J[-1] - Jo) <= 1e-12 * abs(Jo)
    assert abs(ours - dJo) <= 1e-10 * abs(dJo), (ours, dJo)
    for x in extra:
        x["disc"].ctx.set_limiter(L.LIMITER_NONE)
        x["disc"].ctx.set_integrator(None)


def test_batched_adjoint_mixes_operators_and_node_sets():
    """One lockstep reverse sweep over the hybrid operator on Gauss nodes (two element passes a
    stage), the hybrid operator on Gauss-Lobatto nodes and the Gauss-node split form: every
    instance bitwise its own single solve, the Gauss hybrid one also against the dual numbers."""
    from test_gpu_adjoint import HYBRID_OPS, _hybrid_c
    L = 2 * np.pi
    specs = [(4, (2, 2, 2), "GL", HYBRID_OPS["hybrid_md"]), (3, (3, 2, 2), "GL", HYBRID_OPS["hybrid_kg"]),
             (4, (2, 3, 2), "GLL", HYBRID_OPS["hybrid_hllc"]),
             (4, (2, 2, 2), "GL", lambda: F.SplitDivOperator(F.ChandrasekharAverage(), F.HLLC()))]
    inst = []
    for k, (n, ne, basis, op) in enumerate(specs):
        disc = build(3, n, ne, F.EulerEquation(3, 1.4), op(), box=((0.0,) * 3, (L,) * 3), basis=basis)
        Q0 = _tgv_state(disc, 0.2 + 0.05 * k, 60 + k)
        rng = np.random.default_rng(70 + k)
        c, noc = _hybrid_c(disc, "hybrid_kg" if k == 1 else "", 1.0 + 0.2 * rng.random(disc.mesh.nelements))
        rho_t, w = _functional_inputs(disc, 80 + k)
        inst.append(dict(disc=disc, Q0=Q0, c=c, noc=noc, rho_t=rho_t, w=w, dt=0.2 * disc.ctx.max_dt(Q0, 1.0)))
    nsteps = 6
    g = [torch.empty(x["Q0"].shape[::-1], dtype=torch.float64, device="cuda") for x in inst]
    gc = [None if x["noc"] else torch.empty(x["disc"].mesh.nelements, dtype=torch.float64, device="cuda")
          for x in inst]
    J, nf, ns = F.adjoint_solve_batch([x["disc"] for x in inst], [_dev(x["Q0"]) for x in inst],
                                      [x["dt"] for x in inst], nsteps, 8 << 30, [_dev(x["rho_t"]) for x in inst],
                                      [_dev(x["w"]) for x in inst], g, gc, nstreams=2)
    for k, x in enumerate(inst):
        g1 = torch.empty_like(g[k])
        gc1 = None if gc[k] is None else torch.empty_like(gc[k])
        J1, _ = x["disc"].ctx.adjoint_solve(_dev(x["Q0"]), x["dt"], nsteps, 2, _dev(x["rho_t"]), _dev(x["w"]), g1,
                                            gc1)
        assert J[k] == J1
        assert torch.equal(g[k], g1) and (gc1 is None or torch.equal(gc[k], gc1))
    x = inst[0]
    dQ = np.random.default_rng(3).standard_normal(x["Q0"].shape)
    Jo, dJo = oracle_for(x["disc"]).solve_jvp(x["Q0"], dQ, x["c"], 0.0 * x["c"], x["dt"], nsteps, x["rho_t"],
                                              x["w"])
    ours = np.sum(_host(g[0]) * dQ)
    assert abs(J[0] - Jo) <= 1e-12 * abs(Jo)
    assert abs(ours - dJo) <= 1e-10 * abs(dJo), (ours, dJo)
