"""timeintegrate on the GPU, with the fixed-step explicit Runge-Kutta methods the reference uses.

Reference: src/FlouTime/FlouTime.jl:34-54 (timeintegrate -> ODEProblem(rhs!, ...) + solve).
Flou hands the stepping to OrdinaryDiffEq (6.49.1); here the solver is SSPRK33 (Shu & Osher
1988) or a 2N-storage method (Williamson 1980: ORK256, CarpenterKennedy2N54, or any
LowStorageRK2N tableau), run by flou_step with each stage fused into the residual kernel.
"""
import math

from . import _lib as L


class SSPRK33:
    """Three-stage, third-order strong-stability-preserving Runge-Kutta (fixed dt).

    SSPRK33(stage_limiter=get_limiter_callback(disc, eq, "zhang_shu", minval)) applies the limiter
    after every stage, as OrdinaryDiffEq's stage_limiter! does (FlouTime.jl:136-148)."""

    def __init__(self, stage_limiter=None):
        self.stage_limiter = stage_limiter


class LowStorageRK2N:
    """A 2N-storage Runge-Kutta method (Williamson 1980) in OrdinaryDiffEq's LowStorageRK2N form
    with williamson_condition = false:
        k = dt L(u); u += B_1 k;   k = A_i k + dt L(u); u += B_i k   (i = 2..s).
    `A[0]` is not used.  The stage limiter, when given, acts after every stage."""

    def __init__(self, A, B, stage_limiter=None, williamson_condition=False):
        if len(A) != len(B) or not 1 <= len(B) <= 16:
            raise ValueError("a 2N-storage method takes 1..16 stages with one A and one B each")
        self.A = [0.0] + [float(a) for a in A[1:]]
        self.B = [float(b) for b in B]
        self.stage_limiter = stage_limiter
        self.williamson_condition = williamson_condition   # an implementation choice; no effect here

    @property
    def c(self):
        """Stage abscissae c_i = Σ_j a_ij of the equivalent Butcher tableau (unused by the
        stepping: no boundary condition on this path depends on time)."""
        s = len(self.B)
        alpha = [[0.0] * s for _ in range(s)]
        beta = [0.0] * s
        out = []
        for i in range(s):
            out.append(sum(beta))
            for j in range(s):
                alpha[i][j] = (self.A[i] * alpha[i - 1][j] if i else 0.0) + (1.0 if i == j else 0.0)
                beta[j] += self.B[i] * alpha[i][j]
        return out


class ORK256(LowStorageRK2N):
    """Five-stage, second-order 2N-storage method of Allampalli, Hixon, Nallasamy and Sawyer
    (J. Comput. Phys. 228, 2009), the solver of the reference's tests (test/tests.jl:19,56,93,139)
    and examples (examples/src/3D_Euler.jl:77)."""

    def __init__(self, stage_limiter=None, williamson_condition=False):
        super().__init__([0.0, -1.0, -1.55798, -1.0, -0.45031], [0.2, 0.83204, 0.6, 0.35394, 0.2],
                         stage_limiter, williamson_condition)


class CarpenterKennedy2N54(LowStorageRK2N):
    """Five-stage, fourth-order 2N-storage method of Carpenter and Kennedy (NASA TM-109112,
    1994), solution 3."""

    def __init__(self, stage_limiter=None, williamson_condition=False):
        super().__init__(
            [0.0, -567301805773 / 1357537059087, -2404267990393 / 2016746695238,
             -3550918686646 / 2091501179385, -1275806237668 / 842570457699],
            [1432997174477 / 9575080441755, 5161836677717 / 13612068292357, 1720146321549 / 2090206949498,
             3134564353537 / 4481467310338, 2277821191437 / 14882151754819],
            stage_limiter, williamson_condition)


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


class CFLCallback:
    def __init__(self, cfl, dtmax):
        self.cfl = cfl
        self.dtmax = dtmax


def get_cfl_callback(cfl, dtmax=math.inf, iter=True):
    """get_cfl_callback(cfl, Δtmax=Inf; iter=true) (FlouTime.jl:92-105): before every step
    dt = min(get_max_dt(Q, cfl), Δtmax), the last step cut to land on tfinal.  The step control
    runs on the device (flou_step_cfl): no host round trip per step."""
    if iter is not True:
        raise ValueError("only iter=true (every step) is implemented")
    if not cfl > 0 or not dtmax > 0:
        raise ValueError("cfl and Δtmax must be positive")
    return CFLCallback(float(cfl), float(dtmax))


class SaveCallback:
    def __init__(self, basename, iter):
        self.basename = basename
        self.iter = iter if iter is True else set(int(i) for i in iter)
        self.files = []

    def selected(self, it):
        return self.iter is True or it in self.iter

    def next_after(self, it):
        if self.iter is True:
            return it + 1
        later = [i for i in self.iter if i > it]
        return min(later) if later else math.inf

    def save(self, disc, Q, it, t):
        from .io import write_vtkhdf
        path = "%s_%010d.hdf" % (self.basename, it)
        write_vtkhdf(path, disc, Q, time=t)
        self.files.append(path)


def get_save_callback(basename, iter=True):
    """get_save_callback(basename; iter=true) (FlouTime.jl:67-90): the solution at the start and
    after every selected step, with its time, as the VTKHDF file `basename_%010d.hdf` that
    FlouTime.jl:70-75 writes (Lagrange cells on equispaced nodes, FieldData/Time)."""
    return SaveCallback(basename, iter)


class CallbackList(list):
    pass


def make_callback_list(*callbacks):
    """make_callback_list(callbacks...) (FlouTime.jl:150-156): None when empty."""
    return CallbackList(callbacks) if callbacks else None


def _flatten(callback):
    if callback is None:
        return []
    if isinstance(callback, (list, tuple)):
        out = []
        for c in callback:
            out += _flatten(c)
        return out
    return [callback]


class Solution:
    def __init__(self, t, u):
        self.t = t
        self.u = u


def timeintegrate(Q0, disc, equation, solver, tfinal, dt=None, alias_u0=False, t0=0.0, cfl=None, callback=None,
                  maxiters=10 ** 6, **_ignored):
    """timeintegrate(Q0, disc, equation, solver, tfinal; dt, alias_u0, callback) -> (sol, exetime).

    Q0 is a column-major (ndofs, nvars) numpy matrix or a CUDA tensor (nvars, ndofs).
    With `cfl` set and no `dt`, the step is fixed once from get_max_dt(Q0, cfl).
    `callback`: one callback, a list or make_callback_list(...) of get_monitor_callback,
    get_cfl_callback (then dt is ignored: the step follows the CFL bound on the device) and
    get_save_callback callbacks.  Other keyword arguments of the reference's call (saveat,
    adaptive=false, save_everystep, ...) do not change the result and are accepted.
    """
    import time as _time

    if not isinstance(solver, (SSPRK33, LowStorageRK2N)):
        raise L.FlouError(L.FLOU_ERR_UNSUPPORTED, "the solvers are SSPRK33 and the 2N-storage methods "
                                                  "(ORK256, CarpenterKennedy2N54, LowStorageRK2N)")
    cbs = _flatten(callback)
    for c in cbs:
        if not isinstance(c, (MonitorCallback, CFLCallback, SaveCallback)):
            raise TypeError("unknown callback %r" % (c,))
    cflcb = [c for c in cbs if isinstance(c, CFLCallback)]
    mons = [c for c in cbs if isinstance(c, MonitorCallback)]
    saves = [c for c in cbs if isinstance(c, SaveCallback)]
    if len(cflcb) > 1:
        raise ValueError("one CFL callback at most")
    ctx = disc.ctx
    if cflcb:
        nsteps, capacity = None, int(min(maxiters, 10 ** 6))
    else:
        if dt is None:
            if cfl is None:
                raise ValueError("give dt or cfl")
            dt = ctx.max_dt(Q0, cfl)
        nsteps = int(math.floor((tfinal - t0) / dt + 0.5))
        if abs(t0 + nsteps * dt - tfinal) > 1e-12 * max(1.0, abs(tfinal)):
            raise ValueError("tfinal - t0 must be a whole number of steps of size dt")
        capacity = max(nsteps, 1)
    Q = Q0 if alias_u0 else Q0.copy(order="F") if hasattr(Q0, "flags") else Q0.clone()
    u0 = None if alias_u0 else Q0
    lim = solver.stage_limiter
    ctx.set_limiter(lim.kind, lim.minval) if lim is not None else ctx.set_limiter(L.LIMITER_NONE)
    mask = 0
    for m in mons:
        mask |= m.which
    ctx.set_monitors(mask, capacity)
    lowstorage = isinstance(solver, LowStorageRK2N)
    if lowstorage:
        ctx.set_integrator(solver.A, solver.B)

    def next_stop(it):
        return min([s.next_after(it) for s in saves] + [math.inf])

    start = _time.perf_counter()
    it, t = 0, t0
    try:
        for s in saves:
            s.save(disc, Q, it, t)
        if cflcb:
            c = cflcb[0]
            while t < tfinal and it < maxiters:
                k = min(next_stop(it), maxiters) - it
                n, t = ctx.step_cfl(Q, t, tfinal, c.cfl, c.dtmax, max_steps=int(min(k, 2 ** 62)))
                it += n
                if n == 0:
                    break
                for s in saves:
                    if s.selected(it):
                        s.save(disc, Q, it, t)
            if t < tfinal:
                raise L.FlouError(L.FLOU_ERR_STATE, "maxiters = %d steps reached at t = %.17g" % (maxiters, t))
        else:
            while it < nsteps:
                k = int(min(next_stop(it), nsteps)) - it
                ctx.step(Q, dt, k, t0 + it * dt)
                it += k
                t = t0 + it * dt
                for s in saves:
                    if s.selected(it):
                        s.save(disc, Q, it, t)
    finally:
        vals, times = ctx.take_monitors(capacity, with_times=True) if mask else (None, None)
        ctx.set_monitors(0, 1)
        ctx.set_limiter(L.LIMITER_NONE)
        if lowstorage:
            ctx.set_integrator(None)
    exetime = _time.perf_counter() - start
    for m in mons:
        col = 0 if m.which == L.MONITOR_KINETIC_ENERGY else 1
        for k in range(vals.shape[0]):
            m.out.time.append(float(times[k]) if cflcb else t0 + (k + 1) * dt)
            m.out.iter.append(k + 1)
            m.out.value.append(float(vals[k, col]))
    return Solution([t0, t], [u0, Q]), exetime
