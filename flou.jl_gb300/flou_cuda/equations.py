"""Equations, boundary conditions and numerical-flux / operator descriptors, mirroring Flou.

Reference: src/FlouCommon/Euler.jl:16-24 (EulerEquation), :142-155 (pressure), :237-271
(primitive <-> conservative); src/FlouCommon/LinearAdvection.jl:16-26;
src/FlouCommon/Burgers.jl:16; src/FlouSpatial/Equations/Euler.jl:69-94 (BCs);
src/FlouSpatial/Interfaces.jl:16-23 (StdAverage, LxF); Euler.jl:167,228,303 (flux types);
src/FlouSpatial/Equations/OpDivergence.jl:105-107,184-194 (operators).
These objects only describe the configuration; all arithmetic runs in libflou_cuda.
"""
import numpy as np

from . import _lib as L


class LinearAdvection:
    """LinearAdvection(a1[, a2[, a3]])."""

    def __init__(self, *velocity):
        if not 1 <= len(velocity) <= 3:
            raise ValueError("Linear advection is implemented in 1D, 2D and 3D.")
        self.a = np.asarray(velocity, dtype=np.float64)
        self.dim = len(velocity)
        self.nvariables = 1
        self.kind = L.EQ_LINEAR_ADVECTION


class BurgersEquation:
    """BurgersEquation() (1D)."""

    def __init__(self):
        self.dim = 1
        self.nvariables = 1
        self.kind = L.EQ_BURGERS


class EulerEquation:
    """EulerEquation{ND}(γ) -> EulerEquation(ND, gamma)."""

    def __init__(self, nd, gamma=1.4):
        if not 1 <= nd <= 3:
            raise ValueError("The Euler equations are only implemented in 1D, 2D and 3D.")
        self.dim = nd
        self.gamma = float(gamma)
        self.nvariables = nd + 2
        self.kind = L.EQ_EULER

    # host-side conversions (set-up and diagnostics only)
    def pressure(self, Q):
        Q = np.asarray(Q)
        rho = Q[..., 0]
        m2 = np.sum(Q[..., 1:1 + self.dim] ** 2, axis=-1)
        return (self.gamma - 1) * (Q[..., self.dim + 1] - m2 / (2 * rho))

    def vars_prim2cons(self, P):
        P = np.asarray(P, dtype=np.float64)
        rho = P[..., 0]
        v = P[..., 1:1 + self.dim]
        p = P[..., self.dim + 1]
        out = np.empty_like(P)
        out[..., 0] = rho
        out[..., 1:1 + self.dim] = rho[..., None] * v
        out[..., self.dim + 1] = p / (self.gamma - 1) + rho * np.sum(v * v, axis=-1) / 2
        return out

    def vars_cons2prim(self, Q):
        Q = np.asarray(Q, dtype=np.float64)
        out = np.empty_like(Q)
        out[..., 0] = Q[..., 0]
        out[..., 1:1 + self.dim] = Q[..., 1:1 + self.dim] / Q[..., :1]
        out[..., self.dim + 1] = self.pressure(Q)
        return out


# ---- boundary conditions -------------------------------------------------------------
class EulerInflowBC:
    def __init__(self, Qext):
        self.kind = L.BC_INFLOW
        self.state = np.asarray(Qext, dtype=np.float64)


class EulerOutflowBC:
    def __init__(self):
        self.kind = L.BC_OUTFLOW
        self.state = None


class EulerSlipBC:
    def __init__(self):
        self.kind = L.BC_SLIP
        self.state = None


class GenericBC:
    """GenericBC(Qext) with Qext(Qin, x, frame, time, equation) (FlouSpatial.jl:80-91).
    MultielementDisc evaluates Qext at every face node of the boundary (Qin = frame = None,
    time = 0): one state everywhere acts as EulerInflowBC(state); a state varying along the
    boundary is uploaded per face node (FLOU_BC_STATE_FIELD).  A Qext that reads the interior
    state or the frame is rejected; one that depends on time is evaluated at t = 0."""

    def __init__(self, Qext):
        self.Qext = Qext
        self.kind = L.BC_INFLOW
        self.state = None


class StateFieldBC:
    """A GenericBC resolved per face node: `states` maps each of the boundary's face nodes
    (face index, face dof) to its external state."""

    def __init__(self, states):
        self.kind = L.BC_STATE_FIELD
        self.state = None
        self.states = states


DirichletBC = EulerInflowBC   # constant state for the scalar equations
OutflowBC = EulerOutflowBC


# ---- numerical fluxes ----------------------------------------------------------------
class StdAverage:
    code = L.NF_STD_AVERAGE
    tpcode = L.TP_STD_AVERAGE


class ChandrasekharAverage:
    code = L.NF_CHANDRASHEKAR
    tpcode = L.TP_CHANDRASHEKAR


class KennedyGruberAverage:
    """Kennedy & Gruber (2008) split flux; a two-point volume flux only (no Flou counterpart)."""
    code = None
    tpcode = L.TP_KENNEDY_GRUBER


class LxF:
    """LxF(avg, intensity): Rusanov / local Lax-Friedrichs."""
    code = L.NF_LXF

    def __init__(self, avg, intensity=1.0):
        self.avg = avg
        self.intensity = float(intensity)


class ScalarDissipation:
    """ScalarDissipation(avg, intensity): central flux `avg` minus λ/2 times the entropy-stable
    scalar dissipation (Euler only; Euler.jl:228-301)."""
    code = L.NF_SCALAR_DISSIPATION

    def __init__(self, avg, intensity=1.0):
        self.avg = avg
        self.intensity = float(intensity)


class MatrixDissipation:
    """MatrixDissipation(avg, intensity): central flux `avg` plus R|Λ|TRᵀ(W_l - W_r)/2, the
    entropy-stable matrix dissipation (Euler only; Euler.jl:303-380)."""
    code = L.NF_MATRIX_DISSIPATION

    def __init__(self, avg, intensity=1.0):
        self.avg = avg
        self.intensity = float(intensity)


class HLL:
    code = L.NF_HLL
    avg = StdAverage()


class HLLC:
    code = L.NF_HLLC
    avg = StdAverage()


# ---- divergence operators ------------------------------------------------------------
class StrongDivOperator:
    def __init__(self, numflux):
        self.numflux = numflux
        self.code = L.OP_STRONG
        self.tpflux = StdAverage()


class HybridDivOperator:
    """HybridDivOperator([tpflux=numflux.avg, [fvflux=numflux]], numflux, blend)
    (OpDivergence.jl:439-472): the split form in telescopic (subcell) form, blended with the
    subcell finite-volume flux `fvflux` by the entropy indicator with constant `blend`."""

    def __init__(self, *args):
        if len(args) == 2:
            self.numflux, self.blend = args
            self.tpflux, self.fvflux = self.numflux.avg, self.numflux
        elif len(args) == 3:
            self.tpflux, self.numflux, self.blend = args
            self.fvflux = self.numflux
        elif len(args) == 4:
            self.tpflux, self.fvflux, self.numflux, self.blend = args
        else:
            raise ValueError("HybridDivOperator([tpflux, [fvflux]], numflux, blend)")
        self.blend = float(self.blend)
        self.code = L.OP_HYBRID


class SplitDivOperator:
    """SplitDivOperator([tpflux=numflux.avg], numflux)."""

    def __init__(self, *args):
        if len(args) == 1:
            self.numflux = args[0]
            self.tpflux = args[0].avg
        elif len(args) == 2:
            self.tpflux, self.numflux = args
        else:
            raise ValueError("SplitDivOperator([tpflux], numflux)")
        self.code = L.OP_SPLIT
