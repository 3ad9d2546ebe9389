"""Zhang-Shu positivity limiter and integral monitors (src/FlouSpatial/Equations/Euler.jl:541-654)
as Flou's stage limiter and monitor callbacks (src/FlouTime/FlouTime.jl:107-148), against the
oracle's restatement."""
import numpy as np
import pytest

import flou_cuda as F
from flou_cuda import _lib as L
from cases import build, oracle_for, rel_linf
from test_oracle_kat import _dipped_state

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _disc(dim, n=4, ne=3, op=None):
    eq = F.EulerEquation(dim, 1.4)
    op = op or F.SplitDivOperator(F.LxF(F.ChandrasekharAverage(), 1.0))
    return build(dim, n, (ne,) * dim, eq, op)


@pytest.mark.parametrize("dim", [1, 2, 3])
def test_limit_matches_oracle(dim):
    disc = _disc(dim)
    Q = _dipped_state(disc, seed=dim)
    minval = 0.1
    disc.ctx.set_limiter(L.LIMITER_ZHANG_SHU, minval)
    Qg = Q.copy(order="F")
    disc.ctx.limit(Qg)
    ref = oracle_for(disc).limit(Q, minval, disc.std.omega)
    npe = disc.std.n ** dim
    touched = [e for e in range(disc.mesh.nelements)
               if not np.array_equal(ref[e * npe:(e + 1) * npe], Q[e * npe:(e + 1) * npe])]
    assert len(touched) == 2
    assert rel_linf(Qg, ref) <= 1e-13
    for e in range(disc.mesh.nelements):   # elements the limiter leaves alone are untouched
        if e not in touched:
            assert np.array_equal(Qg[e * npe:(e + 1) * npe], Q[e * npe:(e + 1) * npe])


@pytest.mark.parametrize("dim", [2, 3])
def test_limited_steps_match_oracle(dim):
    disc = _disc(dim)
    Q = _dipped_state(disc, seed=10 + dim)
    o = oracle_for(disc)
    dt = 0.2 * disc.ctx.max_dt(Q, 1.0)
    minval = 0.5   # the dips fill within a stage; 0.5 keeps the two dipped elements limited
    disc.ctx.set_limiter(L.LIMITER_ZHANG_SHU, minval)
    Qg = Q.copy(order="F")
    disc.ctx.step(Qg, dt, 4)
    ref = o.ssprk3_limited(Q, dt, 4, minval, disc.std.omega)
    assert rel_linf(Qg, ref) <= 1e-10
    assert rel_linf(ref, o.ssprk3(Q, dt, 4)) > 1e-6   # the limiter did act
    disc.ctx.set_limiter(L.LIMITER_NONE)
    Qn = Q.copy(order="F")
    disc.ctx.step(Qn, dt, 4)
    assert rel_linf(Qn, o.ssprk3(Q, dt, 4)) <= 1e-10


@pytest.mark.parametrize("dim", [1, 2, 3])
def test_monitors_match_oracle(dim):
    disc = _disc(dim)
    Q = _dipped_state(disc, seed=20 + dim)
    o = oracle_for(disc)
    for which in (L.MONITOR_KINETIC_ENERGY, L.MONITOR_ENTROPY):
        ref = o.monitor(Q, which, disc.std.omega)
        val = disc.ctx.monitor(Q, which)
        assert abs(val - ref) <= 1e-13 * abs(ref), (which, val, ref)
    Qd = torch.from_numpy(np.ascontiguousarray(Q.T)).cuda()   # device pointers too
    assert abs(disc.ctx.monitor(Qd, L.MONITOR_ENTROPY) - o.monitor(Q, 2, disc.std.omega)) <= 1e-13 * abs(
        o.monitor(Q, 2, disc.std.omega))


def test_monitors_recorded_every_step_inside_the_graph():
    disc = _disc(2)
    Q = _dipped_state(disc, seed=31)
    o = oracle_for(disc)
    dt = 0.2 * disc.ctx.max_dt(Q, 1.0)
    disc.ctx.set_monitors(L.MONITOR_KINETIC_ENERGY | L.MONITOR_ENTROPY, 16)
    Qg = Q.copy(order="F")
    disc.ctx.step(Qg, dt, 3)
    disc.ctx.step(Qg, dt, 2)   # the same graph replayed: the record continues
    vals = disc.ctx.take_monitors()
    assert vals.shape == (5, 2)
    Qo = Q.copy(order="F")
    for k in range(5):
        Qo = o.ssprk3(Qo, dt, 1)
        assert abs(vals[k, 0] - o.monitor(Qo, 1, disc.std.omega)) <= 1e-11 * abs(vals[k, 0])
        assert abs(vals[k, 1] - o.monitor(Qo, 2, disc.std.omega)) <= 1e-11 * abs(vals[k, 1])
    assert disc.ctx.take_monitors().shape == (0, 2)   # taking restarts the record
    disc.ctx.step(Qg, dt, 20)                          # more steps than the capacity
    with pytest.raises(F.FlouError):
        disc.ctx.take_monitors()


def test_flou_style_callbacks():
    """timeintegrate(Q0, disc, eq, SSPRK33(stage_limiter=...), tf; callback=monitor) as Flou's
    examples/src/3D_Euler.jl:72-87 with get_monitor_callback and get_limiter_callback."""
    disc = _disc(2)
    eq = disc.equation
    Q = _dipped_state(disc, seed=41)
    o = oracle_for(disc)
    dt = 0.2 * disc.ctx.max_dt(Q, 1.0)
    mb, mvals = F.get_monitor_callback(float, float, disc, eq, ":entropy")
    zs = F.get_limiter_callback(disc, eq, ":zhang_shu", 0.5)
    sol, _ = F.timeintegrate(Q, disc, eq, F.SSPRK33(stage_limiter=zs), 3 * dt, dt=dt, callback=mb)
    ref = Q.copy(order="F")
    ents = []
    for _ in range(3):
        ref = o.ssprk3_limited(ref, dt, 1, 0.5, disc.std.omega)
        ents.append(o.monitor(ref, 2, disc.std.omega))
    assert rel_linf(sol.u[-1], ref) <= 1e-10
    assert mvals.iter == [1, 2, 3]
    assert np.allclose(mvals.value, ents, rtol=1e-11)


def test_limiter_applies_to_the_euler_equations_only():
    """(The batched launch runs the limiter and the monitors too: test_gpu_batch.py.)"""
    adv = build(1, 4, (3,), F.LinearAdvection(1.0), F.StrongDivOperator(F.LxF(F.StdAverage(), 1.0)))
    with pytest.raises(F.FlouError) as ei:
        adv.ctx.set_limiter(L.LIMITER_ZHANG_SHU, 0.1)
    assert ei.value.status == L.FLOU_ERR_UNSUPPORTED
