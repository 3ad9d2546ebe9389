"""ctypes front-end of the CPU oracle (oracle/liboracle.so) for the tests.

Test infrastructure: the oracle the CUDA library is compared against.
"""
import ctypes
import os

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
_lib = None

D = ctypes.POINTER(ctypes.c_double)
I32 = ctypes.POINTER(ctypes.c_int32)
U8 = ctypes.POINTER(ctypes.c_uint8)


def lib():
    global _lib
    if _lib is None:
        path = os.path.join(ROOT, "oracle", "liboracle.so")
        _lib = ctypes.CDLL(path)
        _lib.oracle_mesh_new.restype = ctypes.c_void_p
        _lib.oracle_mesh_new.argtypes = [ctypes.c_int, D, D, I32, ctypes.c_int, I32]
        _lib.oracle_mesh_free.argtypes = [ctypes.c_void_p]
        _lib.oracle_mesh_sizes.argtypes = [ctypes.c_void_p] + [ctypes.POINTER(ctypes.c_int)] * 4
        _lib.oracle_mesh_get.argtypes = [ctypes.c_void_p, I32, I32, I32, I32, U8, I32, I32, I32]
        _lib.oracle_geometry.argtypes = [ctypes.c_void_p, ctypes.c_int, D, D, D, D, D, D]
        _lib.oracle_std_operators.argtypes = [ctypes.c_int, ctypes.c_int] + [D] * 9
        _lib.oracle_disc_new.restype = ctypes.c_void_p
        _lib.oracle_disc_new.argtypes = ([ctypes.c_int, ctypes.c_int, ctypes.c_double, D, ctypes.c_int, ctypes.c_int,
                                          ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_int] + [D] * 6 +
                                         [ctypes.c_int, ctypes.c_int, I32, I32, I32, I32, U8, I32, ctypes.c_int,
                                          I32, D, D, D, D, D])
        _lib.oracle_disc_free.argtypes = [ctypes.c_void_p]
        _lib.oracle_rhs.argtypes = [ctypes.c_void_p, D, D, ctypes.c_double]
        _lib.oracle_ssprk3.argtypes = [ctypes.c_void_p, D, ctypes.c_double, ctypes.c_int, ctypes.c_double]
        _lib.oracle_max_dt.restype = ctypes.c_double
        _lib.oracle_max_dt.argtypes = [ctypes.c_void_p, D, ctypes.c_double, D]
        _lib.oracle_limit.argtypes = [ctypes.c_void_p, D, ctypes.c_double, D]
        _lib.oracle_set_hybrid.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                           ctypes.c_double, D, D]
        _lib.oracle_monitor.restype = ctypes.c_double
        _lib.oracle_monitor.argtypes = [ctypes.c_void_p, D, ctypes.c_int, D]
        _lib.oracle_ssprk3_limited.argtypes = [ctypes.c_void_p, D, ctypes.c_double, ctypes.c_int, ctypes.c_double,
                                               ctypes.c_double, D]
        _lib.oracle_set_subgrid.argtypes = [ctypes.c_void_p, D, D]
        _lib.oracle_set_bc_field.argtypes = [ctypes.c_void_p, D]
        _lib.oracle_lsrk2n.argtypes = [ctypes.c_void_p, D, ctypes.c_double, ctypes.c_int, ctypes.c_double,
                                       ctypes.c_int, D, D, D, ctypes.c_double, D]
        _lib.oracle_count_rhs.argtypes = [ctypes.c_void_p, D, ctypes.c_double, ctypes.POINTER(ctypes.c_longlong)]
        _lib.oracle_set_threads.argtypes = [ctypes.c_int]
        _lib.oracle_rhs_jvp.argtypes = [ctypes.c_void_p, D, D, D, D, D, D]
        _lib.oracle_solve_jvp.argtypes = [ctypes.c_void_p, D, D, D, D, ctypes.c_double, ctypes.c_int, D, D, D, D]
        _lib.oracle_solve_jvp_lsrk.argtypes = [ctypes.c_void_p, D, D, D, D, ctypes.c_double, ctypes.c_int, D, D,
                                               ctypes.c_int, D, D, D, D, D, ctypes.c_double, D]
    return _lib


def _d(a):
    return a.ctypes.data_as(D)


def _i(a):
    return a.ctypes.data_as(I32)


def mesh(dim, start, finish, n, periodic=()):
    """Cartesian mesh by the reference's own procedure; returns a dict of 1-based arrays."""
    L = lib()
    st = np.asarray(start, dtype=np.float64).reshape(-1)
    fi = np.asarray(finish, dtype=np.float64).reshape(-1)
    nn = np.asarray(n, dtype=np.int32).reshape(-1)
    pp = np.asarray(periodic, dtype=np.int32).reshape(-1)
    h = L.oracle_mesh_new(dim, _d(st), _d(fi), _i(nn), len(periodic), _i(pp) if len(pp) else None)
    if not h:
        raise ValueError("oracle rejected the mesh")
    ne, nf, ni, nb = (ctypes.c_int() for _ in range(4))
    L.oracle_mesh_sizes(h, ctypes.byref(ne), ctypes.byref(nf), ctypes.byref(ni), ctypes.byref(nb))
    ne, nf, ni = ne.value, nf.value, ni.value
    out = dict(
        faceinds=np.zeros((ne, 2 * dim), np.int32), facepos=np.zeros((ne, 2 * dim), np.int32),
        eleminds=np.zeros((nf, 2), np.int32), elempos=np.zeros((nf, 2), np.int32),
        orientation=np.zeros(nf, np.uint8), bdface_index=np.zeros(nf, np.int32),
        intfaces=np.zeros(max(ni, 1), np.int32), bdindex_of_id=np.zeros(2 * dim, np.int32))
    L.oracle_mesh_get(h, _i(out["faceinds"]), _i(out["facepos"]), _i(out["eleminds"]), _i(out["elempos"]),
                      out["orientation"].ctypes.data_as(U8), _i(out["bdface_index"]), _i(out["intfaces"]),
                      _i(out["bdindex_of_id"]))
    out["intfaces"] = out["intfaces"][:ni]
    out["nelem"], out["nfaces"], out["dim"] = ne, nf, dim
    out["_handle"] = h
    return out


def geometry(m, n, xi):
    L = lib()
    dim = m["dim"]
    nd = m["nelem"] * n ** dim
    nfd = m["nfaces"] * n ** (dim - 1)
    J, Ja, X = np.zeros(nd), np.zeros((nd, dim * dim)), np.zeros((nd, 3))
    fr, fJ = np.zeros((nfd, 9)), np.zeros(nfd)
    L.oracle_geometry(m["_handle"], n, _d(np.ascontiguousarray(xi, dtype=np.float64)), _d(J), _d(Ja), _d(X),
                      _d(fr), _d(fJ))
    return dict(J=J, Ja=Ja, coords=X, frames=fr, faceJ=fJ)


def operators(n, lobatto=True):
    L = lib()
    out = {k: np.zeros(n) for k in ("xi", "omega", "l_l", "l_r", "dg_l", "dg_r")}
    for k in ("D", "Ds", "Dsharp"):
        out[k] = np.zeros((n, n), order="F")
    L.oracle_std_operators(n, int(lobatto), _d(out["xi"]), _d(out["omega"]), _d(out["D"]), _d(out["Ds"]),
                           _d(out["Dsharp"]), _d(out["l_l"]), _d(out["l_r"]), _d(out["dg_l"]), _d(out["dg_r"]))
    return out


class Disc:
    """Oracle discretization fed with the same set-up arrays as the C ABI."""

    def __init__(self, cfg, a, nelem, nfaces):
        L = lib()
        self.L = L
        adv = np.array([cfg.advection[k] for k in range(3)], dtype=np.float64)
        self._keep = (adv, a)
        self.dim = cfg.dim
        self.nv = cfg.dim + 2 if cfg.equation == 2 else 1
        self.n = cfg.nnodes
        self.ndofs = nelem * self.n ** self.dim
        self.h = L.oracle_disc_new(
            cfg.dim, cfg.equation, cfg.gamma, _d(adv), cfg.volume_op, cfg.twopoint_flux, cfg.numflux,
            cfg.numflux_avg, cfg.numflux_intensity, cfg.nnodes, _d(a["Ds"]), _d(a["Dsharp"]), _d(a["l_l"]),
            _d(a["l_r"]), _d(a["dg_l"]), _d(a["dg_r"]), nelem, nfaces, _i(a["faceinds"]), _i(a["facepos"]),
            _i(a["eleminds"]), _i(a["elempos"]), a["orientation"].ctypes.data_as(U8), _i(a["bdface_index"]),
            len(a["bc_kinds"]), _i(a["bc_kinds"]), _d(a["bc_states"]), _d(a["J"]), _d(a["Ja"]), _d(a["frames"]),
            _d(a["faceJ"]))
        if a.get("hybrid") is not None:
            fv, fvavg, fvint, blend = a["hybrid"]
            om = np.ascontiguousarray(a["omega"], dtype=np.float64)
            Dm = np.asfortranarray(a["D"], dtype=np.float64)
            self._keep = (adv, a, om, Dm)
            L.oracle_set_hybrid(self.h, int(fv), int(fvavg), float(fvint), float(blend), _d(om), _d(Dm))
        if a.get("subgrid") is not None:
            fr, jac = a["subgrid"]
            L.oracle_set_subgrid(self.h, _d(np.ascontiguousarray(fr)), _d(np.ascontiguousarray(jac)))
        if a.get("bc_field") is not None:
            L.oracle_set_bc_field(self.h, _d(np.ascontiguousarray(a["bc_field"])))

    def __del__(self):
        if getattr(self, "h", None):
            self.L.oracle_disc_free(self.h)
            self.h = None

    def rhs(self, Q, t=0.0):
        Q = np.asfortranarray(Q, dtype=np.float64)
        dQ = np.zeros_like(Q, order="F")
        if self.L.oracle_rhs(self.h, _d(dQ), _d(Q), t) != 0:
            raise RuntimeError("oracle rhs failed")
        return dQ

    def ssprk3(self, Q, dt, nsteps, t0=0.0):
        Q = np.array(Q, dtype=np.float64, order="F", copy=True)
        if self.L.oracle_ssprk3(self.h, _d(Q), dt, nsteps, t0) != 0:
            raise RuntimeError("oracle ssprk3 failed")
        return Q

    def limit(self, Q, minval, omega_tp):
        """Zhang–Shu limiter (Euler.jl:611-654) applied once; returns the limited copy."""
        Q = np.array(Q, dtype=np.float64, order="F", copy=True)
        self.L.oracle_limit(self.h, _d(Q), minval, _d(np.ascontiguousarray(omega_tp)))
        return Q

    def monitor(self, Q, which, omega_tp):
        """1: kinetic energy, 2: mathematical entropy (Euler.jl:560-590)."""
        Q = np.asfortranarray(Q, dtype=np.float64)
        return self.L.oracle_monitor(self.h, _d(Q), int(which), _d(np.ascontiguousarray(omega_tp)))

    def ssprk3_limited(self, Q, dt, nsteps, minval, omega_tp, t0=0.0):
        Q = np.array(Q, dtype=np.float64, order="F", copy=True)
        if self.L.oracle_ssprk3_limited(self.h, _d(Q), dt, nsteps, t0, minval,
                                        _d(np.ascontiguousarray(omega_tp))) != 0:
            raise RuntimeError("oracle ssprk3 failed")
        return Q

    def lsrk2n(self, Q, dt, nsteps, A, B, c, t0=0.0, minval=None, omega_tp=None):
        """`nsteps` steps of the 2N-storage method (A, B, c); the limiter after every stage when
        `minval` is given."""
        Q = np.array(Q, dtype=np.float64, order="F", copy=True)
        A, B, c = (np.ascontiguousarray(x, dtype=np.float64) for x in (A, B, c))
        w = None if minval is None else np.ascontiguousarray(omega_tp, dtype=np.float64)
        if self.L.oracle_lsrk2n(self.h, _d(Q), dt, nsteps, t0, len(B), _d(A), _d(B), _d(c),
                                0.0 if minval is None else float(minval), _d(w) if w is not None else None) != 0:
            raise RuntimeError("oracle lsrk2n failed")
        return Q

    def max_dt(self, Q, cfl, omega_tp):
        Q = np.asfortranarray(Q, dtype=np.float64)
        return self.L.oracle_max_dt(self.h, _d(Q), cfl, _d(np.ascontiguousarray(omega_tp)))

    def rhs_jvp(self, Q, dQ, c=None, dc=None):
        """(rhs, directional derivative) at (Q, c) along (dQ, dc) -- forward-mode duals."""
        Q = np.asfortranarray(Q, dtype=np.float64)
        dQ = np.asfortranarray(dQ, dtype=np.float64)
        R, dR = np.zeros_like(Q, order="F"), np.zeros_like(Q, order="F")
        cc = None if c is None else np.ascontiguousarray(c, dtype=np.float64)
        dcc = None if dc is None else np.ascontiguousarray(dc, dtype=np.float64)
        self.L.oracle_rhs_jvp(self.h, _d(Q), _d(dQ), _d(cc) if cc is not None else None,
                              _d(dcc) if dcc is not None else None, _d(R), _d(dR))
        return R, dR

    def solve_jvp(self, Q0, dQ0, c, dc, dt, nsteps, rho_t, w):
        """(J, dJ): J = 1/2 Σ w (ρ(T) - ρt)² after nsteps SSP-RK3 steps, and its derivative."""
        Q0 = np.asfortranarray(Q0, dtype=np.float64)
        dQ0 = np.asfortranarray(dQ0, dtype=np.float64)
        J, dJ = ctypes.c_double(), ctypes.c_double()
        args = [np.ascontiguousarray(x, dtype=np.float64) if x is not None else None for x in (c, dc, rho_t, w)]
        p = lambda a: _d(a) if a is not None else None
        self.L.oracle_solve_jvp(self.h, _d(Q0), _d(dQ0), p(args[0]), p(args[1]), dt, nsteps, p(args[2]),
                                p(args[3]), ctypes.byref(J), ctypes.byref(dJ))
        return J.value, dJ.value

    def solve_jvp_lsrk(self, Q0, dQ0, c, dc, dt, nsteps, rho_t, w, A=None, B=None, cst=None, minval=None,
                       omega_tp=None):
        """solve_jvp for nsteps steps of the 2N-storage method (A, B, c), or of SSP-RK3 when A is
        None; with the Zhang-Shu stage limiter when minval is given."""
        Q0 = np.asfortranarray(Q0, dtype=np.float64)
        dQ0 = np.asfortranarray(dQ0, dtype=np.float64)
        J, dJ = ctypes.c_double(), ctypes.c_double()
        args = [np.ascontiguousarray(x, dtype=np.float64) if x is not None else None
                for x in (c, dc, rho_t, w, A, B, cst, omega_tp if minval is not None else None)]
        p = lambda a: _d(a) if a is not None else None
        self.L.oracle_solve_jvp_lsrk(self.h, _d(Q0), _d(dQ0), p(args[0]), p(args[1]), dt, nsteps, p(args[2]),
                                     p(args[3]), 0 if A is None else len(args[5]), p(args[4]), p(args[5]),
                                     p(args[6]), ctypes.byref(J), ctypes.byref(dJ),
                                     0.0 if minval is None else float(minval), p(args[7]))
        return J.value, dJ.value

    def count(self, Q, t=0.0):
        out = (ctypes.c_longlong * 6)()
        Q = np.asfortranarray(Q, dtype=np.float64)
        self.L.oracle_count_rhs(self.h, _d(Q), t, out)
        return dict(zip(("add", "mul", "div", "sqrt", "log", "cmp"), list(out)))
