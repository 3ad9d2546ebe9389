"""timeintegrate with the Shu-Osher SSP-RK3 integrator, on the GPU.

Reference: src/FlouTime/FlouTime.jl:34-54 (timeintegrate -> ODEProblem(rhs!, ...) + solve).
Flou hands the stepping to OrdinaryDiffEq; here the solver is SSPRK33 (Shu & Osher 1988),
fixed step, run by flou_step with each stage fused into the residual kernel.
"""
import math

from . import _lib as L


class SSPRK33:
    """Three-stage, third-order strong-stability-preserving Runge-Kutta (fixed dt).

    SSPRK33(stage_limiter=get_limiter_callback(disc, eq, "zhang_shu", minval)) applies the limiter
    after every stage, as OrdinaryDiffEq's stage_limiter! does (FlouTime.jl:136-148)."""

    def __init__(self, stage_limiter=None):
        self.stage_limiter = stage_limiter


class LimiterCallback:
    def __init__(self, kind, minval):
        self.kind = kind
        self.minval = minval


def get_limiter_callback(disc, equation, name, p=None):
    """get_limiter_callback(disc, equation, :zhang_shu, minval) (FlouTime.jl:136-148,
    Euler.jl:595-654): the Zhang-Shu positivity limiter with minimum value `p`."""
    if name not in ("zhang_shu", ":zhang_shu"):
        raise ValueError("Unknown limiter '%s'." % name)
    if p is None:
        raise ValueError("The minimum value must be specified when using the limiter of Zhang & Shu.")
    return LimiterCallback(L.LIMITER_ZHANG_SHU, float(p))


class MonitorOutput:
    """MonitorOutput(time, iter, value) (FlouTime.jl:101-105), filled by timeintegrate."""

    def __init__(self):
        self.time, self.iter, self.value = [], [], []


class MonitorCallback:
    def __init__(self, which, out):
        self.which = which
        self.out = out


def get_monitor_callback(timetype, valuetype, disc, equation, name, p=None, iter=True):
    """get_monitor_callback(Float64, Float64, disc, equation, :entropy) -> (callback, monitor)
    (FlouTime.jl:107-134).  `:energy` / `:kinetic_energy` and `:entropy` (Euler.jl:541-590) are
    recorded after every step."""
    key = str(name).lstrip(":")
    which = {"energy": L.MONITOR_KINETIC_ENERGY, "kinetic_energy": L.MONITOR_KINETIC_ENERGY,
             "entropy": L.MONITOR_ENTROPY}.get(key)
    if which is None:
        raise ValueError("Unknown monitor '%s'." % name)
    if iter is not True:
        raise ValueError("only iter=true (every step) is implemented")
    out = MonitorOutput()
    return MonitorCallback(which, out), out


class Solution:
    def __init__(self, t, u):
        self.t = t
        self.u = u


def timeintegrate(Q0, disc, equation, solver, tfinal, dt=None, alias_u0=False, t0=0.0, cfl=None, callback=None):
    """timeintegrate(Q0, disc, equation, solver, tfinal; dt, alias_u0, callback) -> (sol, exetime).

    Q0 is a column-major (ndofs, nvars) numpy matrix or a CUDA tensor (nvars, ndofs).
    With `cfl` set and no `dt`, the step is fixed once from get_max_dt(Q0, cfl).
    `callback`: monitor callbacks (one or a list) from get_monitor_callback.
    """
    import time as _time

    if not isinstance(solver, SSPRK33):
        raise L.FlouError(L.FLOU_ERR_UNSUPPORTED, "only SSPRK33 is implemented")
    ctx = disc.ctx
    if dt is None:
        if cfl is None:
            raise ValueError("give dt or cfl")
        dt = ctx.max_dt(Q0, cfl)
    nsteps = int(math.floor((tfinal - t0) / dt + 0.5))
    if abs(t0 + nsteps * dt - tfinal) > 1e-12 * max(1.0, abs(tfinal)):
        raise ValueError("tfinal - t0 must be a whole number of steps of size dt")
    Q = Q0 if alias_u0 else Q0.copy(order="F") if hasattr(Q0, "flags") else Q0.clone()
    u0 = None if alias_u0 else Q0
    lim = solver.stage_limiter
    ctx.set_limiter(lim.kind, lim.minval) if lim is not None else ctx.set_limiter(L.LIMITER_NONE)
    mons = [] if callback is None else (list(callback) if isinstance(callback, (list, tuple)) else [callback])
    mask = 0
    for m in mons:
        mask |= m.which
    ctx.set_monitors(mask, max(nsteps, 1))
    start = _time.perf_counter()
    try:
        ctx.step(Q, dt, nsteps, t0)
    finally:
        vals = ctx.take_monitors(max(nsteps, 1)) if mask else None
        ctx.set_monitors(0, 1)
        ctx.set_limiter(L.LIMITER_NONE)
    exetime = _time.perf_counter() - start
    for m in mons:
        col = 0 if m.which == L.MONITOR_KINETIC_ENERGY else 1
        for k in range(vals.shape[0]):
            m.out.time.append(t0 + (k + 1) * dt)
            m.out.iter.append(k + 1)
            m.out.value.append(float(vals[k, col]))
    return Solution([t0, tfinal], [u0, Q]), exetime
