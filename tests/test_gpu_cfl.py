"""GPU: CFL-limited stepping (get_cfl_callback, FlouTime.jl:92-105) with the step control on the
device, snapshot callbacks (get_save_callback, FlouTime.jl:67-90), and the reference's
convergence study (examples/src/Convergence.jl) run through timeintegrate.

The oracle loop recomputes dt = min(get_max_dt(Q, cfl), dtmax) before every step and cuts the
last step to land on tfinal, as OrdinaryDiffEq does with the reference's callback."""
import math
import os

import numpy as np
import pytest

import flou_cuda as F
from cases import build, oracle_for, rel_linf, smooth_euler_state

pytestmark = pytest.mark.gpu

STEP_TOL = 1e-10


def _oracle_cfl(disc, Q, t0, tf, cfl, dtmax=math.inf, method=None, minval=None):
    o = oracle_for(disc)
    w = disc.std.omega
    t, times = t0, []
    Q = np.array(Q, order="F", copy=True)
    while t < tf:
        dt = min(o.max_dt(Q, cfl, w), dtmax)
        if t + dt >= tf:
            dt, t = tf - t, tf
        else:
            t = t + dt
        if method is None:
            Q = o.ssprk3(Q, dt, 1) if minval is None else o.ssprk3_limited(Q, dt, 1, minval, w)
        else:
            Q = o.lsrk2n(Q, dt, 1, method.A, method.B, method.c, minval=minval,
                         omega_tp=w if minval is not None else None)
        times.append(t)
    return Q, times


def _disc2d(op=None, n=4, ne=(3, 3)):
    op = op or F.SplitDivOperator(F.LxF(F.ChandrasekharAverage(), 1.0))
    return build(2, n, ne, F.EulerEquation(2, 1.4), op)


def test_cfl_stepping_matches_oracle():
    disc = _disc2d()
    Q0 = smooth_euler_state(disc, seed=21)
    tf = 12.5 * disc.ctx.max_dt(Q0, 0.4)   # a fractional number of steps: the last one is cut
    mon, out = F.get_monitor_callback(float, float, disc, disc.equation, "entropy")
    sol, _ = F.timeintegrate(Q0, disc, disc.equation, F.SSPRK33(), tf,
                             callback=F.make_callback_list(F.get_cfl_callback(0.4), mon))
    ref, times = _oracle_cfl(disc, Q0, 0.0, tf, 0.4)
    assert sol.t[-1] == tf
    assert rel_linf(sol.u[-1], ref) <= STEP_TOL
    assert out.iter == list(range(1, len(times) + 1))
    assert np.allclose(out.time, times, rtol=1e-13, atol=0)
    assert out.time[-1] == tf
    o = oracle_for(disc)
    assert abs(out.value[-1] - o.monitor(ref, 2, disc.std.omega)) < 1e-10 * abs(out.value[-1])


def test_cfl_dtmax_lowstorage_limiter_on_device_tensor():
    torch = pytest.importorskip("torch")
    disc = _disc2d()
    Q0 = smooth_euler_state(disc, seed=5, amp=0.6)
    bound = disc.ctx.max_dt(Q0, 0.3)
    dtmax, tf = 0.5 * bound, 7.25 * bound
    lim = F.get_limiter_callback(disc, disc.equation, "zhang_shu", 0.6)
    Qt = torch.tensor(np.ascontiguousarray(Q0.T), device="cuda")
    sol, _ = F.timeintegrate(Qt, disc, disc.equation, F.ORK256(stage_limiter=lim), tf,
                             callback=F.get_cfl_callback(0.3, dtmax))
    ref, times = _oracle_cfl(disc, Q0, 0.0, tf, 0.3, dtmax, method=F.ORK256(), minval=0.6)
    assert len(times) == 15   # 14 steps of dtmax, then the cut one
    assert rel_linf(sol.u[-1].cpu().numpy().T, ref) <= STEP_TOL


def test_cfl_max_steps_resumes():
    """flou_step_cfl stops after max_steps and resumes from the time it reached."""
    disc = _disc2d(F.StrongDivOperator(F.HLLC()))
    Q0 = smooth_euler_state(disc, seed=9)
    tf = 9.3 * disc.ctx.max_dt(Q0, 0.5)
    Qa = Q0.copy(order="F")
    n1, t1 = disc.ctx.step_cfl(Qa, 0.0, tf, 0.5, max_steps=4)
    assert n1 == 4 and 0.0 < t1 < tf
    n2, t2 = disc.ctx.step_cfl(Qa, t1, tf, 0.5)
    assert t2 == tf
    Qb = Q0.copy(order="F")
    n, t = disc.ctx.step_cfl(Qb, 0.0, tf, 0.5)
    assert n == n1 + n2 and t == tf
    assert np.array_equal(Qa, Qb)
    ref, times = _oracle_cfl(disc, Q0, 0.0, tf, 0.5)
    assert len(times) == n and rel_linf(Qb, ref) <= STEP_TOL
    # the fixed-dt graph still works after the CFL one
    Qc = Q0.copy(order="F")
    dt = disc.ctx.max_dt(Q0, 0.5)
    disc.ctx.step(Qc, dt, 2)
    assert rel_linf(Qc, oracle_for(disc).ssprk3(Q0, dt, 2)) <= STEP_TOL


def test_cfl_broken_state_reports_nonphysical():
    disc = _disc2d(F.StrongDivOperator(F.LxF(F.StdAverage(), 1.0)))
    Q = smooth_euler_state(disc, seed=2)
    Q[3, 0] = -1.0   # negative density: no positive time step
    with pytest.raises(F.DomainError):
        disc.ctx.step_cfl(Q, 0.0, 1.0, 0.5)


def test_save_callback_writes_selected_steps(tmp_path):
    disc = _disc2d()
    Q0 = smooth_euler_state(disc, seed=3)
    dt = 0.3 * disc.ctx.max_dt(Q0, 1.0)
    base = os.path.join(tmp_path, "sol")
    cb = F.get_save_callback(base, iter=[2, 5])
    sol, _ = F.timeintegrate(Q0, disc, disc.equation, F.SSPRK33(), 6 * dt, dt=dt, callback=cb)
    assert [os.path.basename(f) for f in cb.files] == ["sol_%010d.hdf" % i for i in (0, 2, 5)]
    d = F.io.read_vtkhdf(cb.files[1])
    assert abs(d["FieldData"]["Time"][0] - 2 * dt) < 1e-15
    ref2 = oracle_for(disc).ssprk3(Q0, dt, 2)
    # the snapshot holds the state resampled to equispaced nodes; the density at the element
    # corners (shared by both node sets on Gauss-Lobatto nodes) equals the state's
    assert abs(d["PointData"]["rho"][0] - ref2[0, 0]) < 1e-12
    assert rel_linf(sol.u[-1], oracle_for(disc).ssprk3(Q0, dt, 6)) <= STEP_TOL
    base2 = os.path.join(tmp_path, "cfl")
    cb2 = F.get_save_callback(base2)
    tf = 3.5 * disc.ctx.max_dt(Q0, 0.4)
    F.timeintegrate(Q0, disc, disc.equation, F.SSPRK33(), tf, callback=[F.get_cfl_callback(0.4), cb2])
    assert len(cb2.files) == 5   # the start and 4 steps
    assert abs(F.io.read_vtkhdf(cb2.files[-1])["FieldData"]["Time"][0] - tf) == 0.0


@pytest.mark.parametrize("basis", ["GLL", "GL"])
def test_reference_convergence_study(basis):
    """examples/src/Convergence.jl on the device: the 1D density wave ρ = 2 + sin(π(x - t)),
    u = p = 1, SplitDivOperator(LxF(ChandrasekharAverage(), 1)), CarpenterKennedy2N54 with a
    CFL callback of 0.125, order 3 (4 nodes) on 8 / 16 / 32 elements: the error falls at the
    design order p + 1 = 4."""
    eq = F.EulerEquation(1, 1.4)
    errs = []
    for ne in (8, 16, 32):
        mesh = F.CartesianMesh((-1.0,), (1.0,), (ne,))
        F.apply_periodicBCs(mesh, ("1", "2"))
        b = F.LagrangeBasis(basis, 4)
        std = F.StdSegment(b, F.DGSEMrec(b), 3)
        disc = F.MultielementDisc(mesh, std, eq, F.SplitDivOperator(F.LxF(F.ChandrasekharAverage(), 1.0)), {})
        x = disc.coords[:, 0]
        exact = lambda t: eq.vars_prim2cons(np.column_stack([2 + np.sin(np.pi * (x - t)), np.ones_like(x),
                                                            np.ones_like(x)]))
        tf = 0.7
        sol, _ = F.timeintegrate(np.asfortranarray(exact(0.0)), disc, eq, F.CarpenterKennedy2N54(), tf,
                                 callback=F.get_cfl_callback(0.125, 1.0), alias_u0=True, dt=1.0)
        assert sol.t[-1] == tf
        errs.append(np.sqrt(np.mean((sol.u[-1] - exact(tf)) ** 2)))
    rates = np.log2(np.array(errs[:-1]) / np.array(errs[1:]))
    assert rates.min() > 3.5, (errs, rates)
