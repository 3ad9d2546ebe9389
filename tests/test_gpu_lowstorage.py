"""GPU: 2N-storage Runge-Kutta stepping (ORK256, CarpenterKennedy2N54) through flou_step against
the oracle, and the reference's own golden problems (Sod tube, 2D normal shock; test/tests.jl:
90-181, test/runtests.jl:34-45) run end to end through timeintegrate on the device.

Bars: N steps to <= 1e-10 relative L-inf against the oracle; the golden minimum / maximum to the
reference's rtol 1e-7."""
import numpy as np
import pytest

import flou_cuda as F
import reference_problems as RP
from cases import build, oracle_for, rel_linf, smooth_euler_state

pytestmark = pytest.mark.gpu

STEP_TOL = 1e-10

CASES = [
    (1, 5, (6,), lambda: F.StrongDivOperator(F.LxF(F.StdAverage(), 1.0))),
    (2, 5, (3, 4), lambda: F.SplitDivOperator(F.LxF(F.ChandrasekharAverage(), 1.0))),
    (2, 4, (3, 3), lambda: F.HybridDivOperator(F.MatrixDissipation(F.ChandrasekharAverage(), 1.0), 0.5)),
    (3, 4, (2, 3, 2), lambda: F.SplitDivOperator(F.ChandrasekharAverage(), F.HLLC())),
    (3, 3, (3, 2, 2), lambda: F.StrongDivOperator(F.HLL())),
]


@pytest.mark.parametrize("solver", ["ORK256", "CarpenterKennedy2N54"])
@pytest.mark.parametrize("case", range(len(CASES)))
def test_lowstorage_steps_match_oracle(case, solver):
    dim, n, ne, op = CASES[case]
    disc = build(dim, n, ne, F.EulerEquation(dim, 1.4), op())
    Q = smooth_euler_state(disc, seed=3 * case + 1)
    m = getattr(F, solver)()
    dt = 0.3 * disc.ctx.max_dt(Q, 1.0)
    Qg = Q.copy(order="F")
    disc.ctx.set_integrator(m.A, m.B)
    try:
        disc.ctx.step(Qg, dt, 6)
    finally:
        disc.ctx.set_integrator(None)
    ref = oracle_for(disc).lsrk2n(Q, dt, 6, m.A, m.B, m.c)
    assert rel_linf(Qg, ref) <= STEP_TOL
    # the default method is back: SSP-RK3
    Qs = Q.copy(order="F")
    disc.ctx.step(Qs, dt, 2)
    assert rel_linf(Qs, oracle_for(disc).ssprk3(Q, dt, 2)) <= STEP_TOL


def test_lowstorage_with_limiter_and_device_state():
    """ORK256 with the Zhang-Shu stage limiter (examples/src/3D_Euler.jl:77-80) on a CUDA tensor."""
    torch = pytest.importorskip("torch")
    disc = build(2, 4, (4, 3), F.EulerEquation(2, 1.4), F.SplitDivOperator(F.LxF(F.ChandrasekharAverage(), 1.0)))
    Q = smooth_euler_state(disc, seed=7, amp=0.6)
    minval = 0.6
    dt = 0.2 * disc.ctx.max_dt(Q, 1.0)
    lim = F.get_limiter_callback(disc, disc.equation, "zhang_shu", minval)
    Qt = torch.tensor(np.ascontiguousarray(Q.T), device="cuda")
    sol, _ = F.timeintegrate(Qt, disc, disc.equation, F.ORK256(stage_limiter=lim), 4 * dt, dt=dt)
    m = F.ORK256()
    ref = oracle_for(disc).lsrk2n(Q, dt, 4, m.A, m.B, m.c, minval=minval, omega_tp=disc.std.omega)
    got = sol.u[-1].cpu().numpy().T
    assert rel_linf(got, ref) <= STEP_TOL
    no_lim = oracle_for(disc).lsrk2n(Q, dt, 4, m.A, m.B, m.c)
    assert rel_linf(no_lim, ref) > 1e-8   # the limiter acted


def test_sod_tube_golden_on_device():
    disc, Q0, dt, tf = RP.sod_tube()
    sol, _ = F.timeintegrate(Q0, disc, disc.equation, F.ORK256(williamson_condition=False), tf, dt=dt)
    Q = sol.u[-1]
    assert RP.isclose(Q.min(), RP.SOD_MIN, 1e-7), Q.min()
    assert RP.isclose(Q.max(), RP.SOD_MAX, 1e-7), Q.max()
    m = F.ORK256()
    ref = oracle_for(disc).lsrk2n(Q0, dt, int(round(tf / dt)), m.A, m.B, m.c)
    assert rel_linf(Q, ref) <= STEP_TOL


def test_shockwave2d_golden_on_device():
    disc, Q0, dt, tf = RP.shockwave_2d()
    sol, _ = F.timeintegrate(Q0, disc, disc.equation, F.ORK256(williamson_condition=False), tf, dt=dt)
    Q = sol.u[-1]
    assert RP.isclose(Q.max(), RP.SHOCK_MAX, 1e-7), Q.max()
    assert RP.isclose(Q.min(), RP.SHOCK_MIN, 1.0), Q.min()
    m = F.ORK256()
    o = oracle_for(disc)
    nsteps = int(round(tf / dt))
    ref = o.lsrk2n(Q0, dt, nsteps, m.A, m.B, m.c)
    # The shock's blending indicator switches on round-off: the oracle itself moves by ~2e-9
    # when its initial state is perturbed by 1e-16 relative.  The device must stay within ten
    # times that spread of the problem's own conditioning.
    rng = np.random.default_rng(0)
    spread = rel_linf(o.lsrk2n(Q0 * (1 + 1e-16 * rng.standard_normal(Q0.shape)), dt, nsteps, m.A, m.B, m.c), ref)
    assert rel_linf(Q, ref) <= max(STEP_TOL, 10 * spread)


def test_integrator_rejects_too_many_stages():
    """(The batched launch and both adjoint solves step with the 2N-storage methods too:
    test_gpu_batch.py, test_gpu_adjoint.py, test_gpu_adjoint_batch.py.)"""
    from flou_cuda import _lib as L
    disc = build(2, 4, (3, 3), F.EulerEquation(2, 1.4), F.StrongDivOperator(F.LxF(F.StdAverage(), 1.0)))
    with pytest.raises(F.FlouError) as ei:
        disc.ctx.set_integrator([0.0] * 17, [0.1] * 17)
    assert ei.value.status == L.FLOU_ERR_ARG
    disc.ctx.set_integrator(None)
