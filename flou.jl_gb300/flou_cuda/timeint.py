"""timeintegrate with the Shu-Osher SSP-RK3 integrator, on the GPU.

Reference: src/FlouTime/FlouTime.jl:34-54 (timeintegrate -> ODEProblem(rhs!, ...) + solve).
Flou hands the stepping to OrdinaryDiffEq; here the solver is SSPRK33 (Shu & Osher 1988),
fixed step, run by flou_step with each stage fused into the residual kernel.
"""
import math

from . import _lib as L


class SSPRK33:
    """Three-stage, third-order strong-stability-preserving Runge-Kutta (fixed dt)."""


class Solution:
    def __init__(self, t, u):
        self.t = t
        self.u = u


def timeintegrate(Q0, disc, equation, solver, tfinal, dt=None, alias_u0=False, t0=0.0, cfl=None):
    """timeintegrate(Q0, disc, equation, solver, tfinal; dt, alias_u0) -> (sol, exetime).

    Q0 is a column-major (ndofs, nvars) numpy matrix or a CUDA tensor (nvars, ndofs).
    With `cfl` set and no `dt`, the step is fixed once from get_max_dt(Q0, cfl).
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
    start = _time.perf_counter()
    try:
        ctx.step(Q, dt, nsteps, t0)
    except L.DomainError:
        raise
    exetime = _time.perf_counter() - start
    return Solution([t0, tfinal], [u0, Q]), exetime
