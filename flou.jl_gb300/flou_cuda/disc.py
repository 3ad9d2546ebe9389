"""MultielementDisc / EquationConfig / rhs! / get_max_dt on top of libflou_cuda.

Reference: src/FlouSpatial/MultielementDiscontinuous.jl:29-92 (MultielementDisc),
src/FlouCommon/FlouCommon.jl:92-102 (EquationConfig, rhs!),
src/FlouSpatial/Equations/Hyperbolic.jl:31-69 (the residual), MultielementDiscontinuous.jl:162-178
(get_max_dt), src/FlouSpatial/PhysicalRegions.jl:370-408,541-696 (Cartesian geometry).

States are Flou's (ndofs, nvars) column-major matrices: a numpy array in Fortran order
(host memory) or a CUDA tensor laid out as (nvars, ndofs) row-major, which is the same
memory.  Every residual runs on the GPU; there is no CPU path.
"""
import ctypes

import numpy as np

from . import _lib as L
from .unstructured import UnstructuredMesh, unstructured_geometry, unstructured_subgrid
from .equations import (BurgersEquation, ChandrasekharAverage, EulerEquation, EulerInflowBC, GenericBC, HLL, HLLC,
                        LinearAdvection, LxF, SplitDivOperator, StateFieldBC, StdAverage, StrongDivOperator)


class DofHandler:
    def __init__(self, nelem, nfaces, npe, nfd):
        self.nelements = nelem
        self.nfaces = nfaces
        self.elem_dofs = npe
        self.face_dofs = nfd

    @property
    def ndofs(self):
        return self.nelements * self.elem_dofs


def cartesian_geometry(mesh, std):
    """Per-node J and metric, per-face-node frame and surface Jacobian of a CartesianMesh
    (PhysicalRegions.jl:370-408 and :541-696), plus node coordinates."""
    d, n = mesh.dim, std.n
    dx = mesh.dx
    npe, nfd = n ** d, n ** (d - 1)
    nd = mesh.nelements * npe
    nfd_tot = mesh.nfaces * nfd
    if d == 1:
        jac, M = dx[0] / 2, np.array([[1.0]])
    elif d == 2:
        jac = (dx[0] * dx[1]) / 4
        M = np.array([[dx[1] / 2, 0.0], [0.0, dx[0] / 2]])
    else:
        jac = (dx[0] * dx[1] * dx[2]) / 8
        M = np.diag([dx[1] * dx[2] / 4, dx[0] * dx[2] / 4, dx[0] * dx[1] / 4])
    J = np.full(nd, jac)
    Ja = np.broadcast_to(M.ravel(order="F"), (nd, d * d)).copy()
    # frames and surface Jacobians from the master side's local face position
    tab = {
        1: {1: ((-1, 0, 0), (0, 0, 0), (0, 0, 0)), 2: ((1, 0, 0), (0, 0, 0), (0, 0, 0))},
        2: {1: ((-1, 0, 0), (0, -1, 0), (0, 0, 0)), 2: ((1, 0, 0), (0, 1, 0), (0, 0, 0)),
            3: ((0, -1, 0), (1, 0, 0), (0, 0, 0)), 4: ((0, 1, 0), (-1, 0, 0), (0, 0, 0))},
        3: {1: ((-1, 0, 0), (0, -1, 0), (0, 0, 1)), 2: ((1, 0, 0), (0, 1, 0), (0, 0, 1)),
            3: ((0, -1, 0), (0, 0, -1), (1, 0, 0)), 4: ((0, 1, 0), (0, 0, 1), (1, 0, 0)),
            5: ((0, 0, -1), (-1, 0, 0), (0, 1, 0)), 6: ((0, 0, 1), (1, 0, 0), (0, 1, 0))},
    }[d]
    if d == 1:
        fj = {1: 1.0, 2: 1.0}
    elif d == 2:
        fj = {1: dx[1] / 2, 2: dx[1] / 2, 3: dx[0] / 2, 4: dx[0] / 2}
    else:
        fj = {1: dx[1] * dx[2] / 4, 2: dx[1] * dx[2] / 4, 3: dx[0] * dx[2] / 4, 4: dx[0] * dx[2] / 4,
              5: dx[0] * dx[1] / 4, 6: dx[0] * dx[1] / 4}
    pos = mesh.elempos[:, 0]
    frames_f = np.array([np.array(tab[p], dtype=np.float64).ravel() for p in range(1, 2 * d + 1)])[pos - 1]
    frames = np.repeat(frames_f, nfd, axis=0)
    faceJ = np.repeat(np.array([fj[p] for p in range(1, 2 * d + 1)])[pos - 1], nfd)
    # node coordinates (x fastest within an element)
    org = mesh.element_origin()
    r = (std.xi1d + 1.0) / 2.0
    idx = np.array(np.unravel_index(np.arange(npe), (n,) * d, order="F"))   # (d, npe)
    coords = np.zeros((nd, 3))
    for k in range(d):
        local = r[idx[k]] * dx[k]
        coords[:, k] = (org[:, k][:, None] + local[None, :]).ravel()
    return J, Ja, frames, faceJ, coords


class MultielementDisc:
    """MultielementDisc(mesh, std, equation, operator, bcs) on the GPU.

    `bcs` maps boundary names ("1".."2d") to EulerInflowBC / EulerOutflowBC / EulerSlipBC / GenericBC.
    """

    def __init__(self, mesh, std, equation, operator, bcs=None):
        bcs = dict(bcs or {})
        if mesh.dim != std.dim or mesh.dim != equation.dim:
            raise ValueError("mesh, standard region and equation dimensions differ")
        if len(bcs) != mesh.nboundaries:
            raise ValueError("The number of BCs does not match the number of boundaries.")
        self.mesh, self.std, self.equation, self.operator = mesh, std, equation, operator
        self.bcs = [None] * mesh.nboundaries
        for key, value in bcs.items():
            b = mesh.boundary_index(key) if hasattr(mesh, "boundary_index") else mesh.bdmap[int(key)]
            self.bcs[b - 1] = value
        n, d = std.n, mesh.dim
        self.dofhandler = DofHandler(mesh.nelements, mesh.nfaces, n ** d, n ** (d - 1))
        if isinstance(mesh, UnstructuredMesh):
            self.J, self.Ja, self.frames, self.faceJ, self.coords = unstructured_geometry(mesh, std)
        else:
            self.J, self.Ja, self.frames, self.faceJ, self.coords = cartesian_geometry(mesh, std)
        self._resolve_generic_bcs()
        self.config = self._config()
        self._ctx = None

    def _boundary_face_coords(self, ib):
        """(faces, coordinates) of the face nodes of boundary `ib` (1-based): the boundary's face
        indices (0-based) and, per face in face-dof order, the trace Σ_i l_i x_i of the master
        element's node coordinates across the face (Interfaces.jl:51-109; exact for the linear
        element mappings)."""
        m, s = self.mesh, self.std
        n, d = s.n, m.dim
        faces = np.nonzero(np.asarray(m.bdface_index) == ib)[0]
        out = []
        for f in faces:
            e, pos = int(m.eleminds[f, 0]) - 1, int(m.elempos[f, 0]) - 1
            X = self.coords[e * n ** d:(e + 1) * n ** d, :d].reshape((n,) * d + (d,), order="F")
            lv = s.l[pos % 2]
            # the remaining axes in order, the first fastest: the face-dof (line) order
            out.append(np.tensordot(X, lv, axes=([pos // 2], [0])).reshape(-1, d, order="F"))
        return faces, (np.stack(out) if out else np.zeros((0, n ** (d - 1), d)))

    def _resolve_generic_bcs(self):
        for ib, bc in enumerate(self.bcs):
            if not isinstance(bc, GenericBC):
                continue
            faces, X = self._boundary_face_coords(ib + 1)
            try:
                vals = np.array([[np.asarray(bc.Qext(None, x, None, 0.0, self.equation), dtype=np.float64)
                                  for x in Xf] for Xf in X])
            except Exception as exc:   # Qext reads the interior state or the frame
                raise L.FlouError(L.FLOU_ERR_UNSUPPORTED, "GenericBC on boundary %d: Qext must give the external "
                                  "state from the position alone (%s)" % (ib + 1, exc)) from exc
            flat = vals.reshape(-1, vals.shape[-1]) if vals.size else vals
            if vals.size and np.all(flat == flat[0]):
                self.bcs[ib] = EulerInflowBC(flat[0])
            else:
                self.bcs[ib] = StateFieldBC({int(f): v for f, v in zip(faces, vals)})

    def _bc_field(self):
        """flou_set_bc_field's array (nfaces·n^(d-1) x 5) when a boundary holds a varying state."""
        fields = [b for b in self.bcs if isinstance(b, StateFieldBC)]
        if not fields:
            return None
        nfd = self.std.n ** (self.mesh.dim - 1)
        out = np.zeros((self.mesh.nfaces * nfd, 5))
        for b in fields:
            for f, v in b.states.items():
                out[f * nfd:(f + 1) * nfd, :v.shape[1]] = v
        return out

    # -- C ABI configuration ------------------------------------------------------------
    def _config(self):
        eq, op = self.equation, self.operator
        cfg = L.FlouConfig()
        cfg.dim = self.mesh.dim
        cfg.equation = eq.kind
        cfg.gamma = getattr(eq, "gamma", 1.4)
        adv = getattr(eq, "a", np.zeros(0))
        for k in range(3):
            cfg.advection[k] = float(adv[k]) if k < len(adv) else 0.0
        cfg.volume_op = op.code
        cfg.twopoint_flux = op.tpflux.tpcode if op.code in (L.OP_SPLIT, L.OP_HYBRID) else L.TP_STD_AVERAGE
        nf = op.numflux
        if nf.code is None:
            raise ValueError("%s is not a numerical flux" % type(nf).__name__)
        cfg.numflux = nf.code
        avg = getattr(nf, "avg", StdAverage())
        cfg.numflux_avg = L.NF_CHANDRASHEKAR if isinstance(avg, ChandrasekharAverage) else L.NF_STD_AVERAGE
        cfg.numflux_intensity = getattr(nf, "intensity", 1.0)
        cfg.nnodes = self.std.n
        return cfg

    def abi_arrays(self):
        """The set-up arrays exactly as the C ABI receives them."""
        m, s = self.mesh, self.std
        kinds = np.array([b.kind for b in self.bcs], dtype=np.int32)
        states = np.zeros((max(len(self.bcs), 1), 5))
        for i, b in enumerate(self.bcs):
            if b.state is not None:
                states[i, :len(b.state)] = b.state
        return dict(
            D=np.asfortranarray(s.D), Ds=np.asfortranarray(s.Ds), Dsharp=np.asfortranarray(s.Dsharp),
            omega=s.omega1d.copy(), l_l=s.l[0].copy(), l_r=s.l[1].copy(), dg_l=s.dg[0].copy(), dg_r=s.dg[1].copy(),
            faceinds=np.ascontiguousarray(m.faceinds, dtype=np.int32),
            facepos=np.ascontiguousarray(m.facepos, dtype=np.int32),
            eleminds=np.ascontiguousarray(m.eleminds, dtype=np.int32),
            elempos=np.ascontiguousarray(m.elempos, dtype=np.int32),
            orientation=np.ascontiguousarray(m.orientation, dtype=np.uint8),
            bdface_index=np.ascontiguousarray(m.bdface_index, dtype=np.int32),
            bc_kinds=kinds, bc_states=np.ascontiguousarray(states),
            J=self.J, Ja=np.ascontiguousarray(self.Ja), frames=np.ascontiguousarray(self.frames), faceJ=self.faceJ,
            hybrid=self._hybrid_params(),
            subgrid=self._subgrid(),
            bc_field=self._bc_field(),
        )

    def _subgrid(self):
        """Subcell-interface frames and Jacobians (flou_set_subgrid layout) on an UnstructuredMesh for
        the hybrid operator, and for the split form on a basis without boundary nodes (its projected
        states' normals); else None (Cartesian elements use the axes)."""
        code = getattr(self.operator, "code", None)
        gauss_split = code == L.OP_SPLIT and not self.std.basis.hasboundaries
        if not isinstance(self.mesh, UnstructuredMesh) or not (code == L.OP_HYBRID or gauss_split):
            return None
        if getattr(self, "_subgrid_cache", None) is None:
            fr, jac = unstructured_subgrid(self.mesh, self.std)
            self._subgrid_cache = (np.ascontiguousarray(fr.reshape(-1, 9)), np.ascontiguousarray(jac.ravel()))
        return self._subgrid_cache

    def _hybrid_params(self):
        """(fvflux, its central flux, intensity, blend) of a HybridDivOperator, else None."""
        op = self.operator
        if getattr(op, "code", None) != L.OP_HYBRID:
            return None
        fv = op.fvflux
        avg = getattr(fv, "avg", StdAverage())
        return (fv.code, L.NF_CHANDRASHEKAR if isinstance(avg, ChandrasekharAverage) else L.NF_STD_AVERAGE,
                float(getattr(fv, "intensity", 1.0)), op.blend)

    @property
    def ctx(self):
        if self._ctx is None:
            self._ctx = Context(self.config, self.abi_arrays(), self.mesh.nelements, self.mesh.nfaces)
        return self._ctx

    @property
    def ndofs(self):
        return self.dofhandler.ndofs

    @property
    def nvariables(self):
        return self.equation.nvariables

    def new_state(self):
        return np.zeros((self.ndofs, self.nvariables), order="F")


def _torch_stream_sync(t):
    """Inputs written by torch on its current stream are complete before a call on the context's
    own stream reads them (the context's stream does not order itself after torch's)."""
    if getattr(t, "is_cuda", False):
        import torch
        torch.cuda.current_stream(t.device).synchronize()


class Context:
    """Owns one flou_ctx (create + uploads); destroyed with the object."""

    def __init__(self, cfg, a, nelem, nfaces):
        lib = L.load()
        self._lib = lib
        h = ctypes.c_void_p()
        st = lib.flou_create(ctypes.byref(cfg), ctypes.byref(h))
        if st != L.FLOU_OK:
            raise L.FlouError(st, "flou_create rejected the configuration")
        self.h = h
        self.cfg = cfg
        d = L.dptr
        i32 = lambda x: x.ctypes.data_as(L._I32)
        L.check(lib.flou_set_operators(h, d(a["D"]), d(a["Ds"]), d(a["Dsharp"]), d(a["omega"]), d(a["l_l"]),
                                       d(a["l_r"]), d(a["dg_l"]), d(a["dg_r"])), h)
        L.check(lib.flou_set_mesh(h, nelem, nfaces, i32(a["faceinds"]), i32(a["facepos"]), i32(a["eleminds"]),
                                  i32(a["elempos"]), a["orientation"].ctypes.data_as(L._U8),
                                  i32(a["bdface_index"])), h)
        L.check(lib.flou_set_bcs(h, len(a["bc_kinds"]), i32(a["bc_kinds"]), d(a["bc_states"])), h)
        L.check(lib.flou_set_geometry(h, d(a["J"]), d(a["Ja"]), d(a["frames"]), d(a["faceJ"])), h)
        if a.get("hybrid") is not None:
            fv, fvavg, fvint, blend = a["hybrid"]
            L.check(lib.flou_set_hybrid(h, int(fv), int(fvavg), float(fvint), float(blend)), h)
        if a.get("subgrid") is not None:
            fr, jac = a["subgrid"]
            L.check(lib.flou_set_subgrid(h, d(fr), d(jac)), h)
        if a.get("bc_field") is not None:
            L.check(lib.flou_set_bc_field(h, d(np.ascontiguousarray(a["bc_field"]))), h)
        nd = ctypes.c_int64()
        nv = ctypes.c_int32()
        L.check(lib.flou_sizes(h, ctypes.byref(nd), ctypes.byref(nv), None, None), h)
        self.ndofs, self.nvars = nd.value, nv.value

    def __del__(self):
        h = getattr(self, "h", None)
        if h is not None and h.value:
            self._lib.flou_destroy(h)
            self.h = None

    def _ptr(self, a, writable=False):
        """(pointer, kind) of a state array: numpy (host) or CUDA tensor (device)."""
        if isinstance(a, np.ndarray):
            if a.dtype != np.float64 or a.size != self.ndofs * self.nvars:
                raise ValueError("state must be float64 with %d x %d entries" % (self.ndofs, self.nvars))
            if a.ndim == 2 and a.shape == (self.ndofs, self.nvars):
                if not a.flags.f_contiguous:
                    raise ValueError("host state must be a column-major (ndofs, nvars) matrix")
            elif not a.flags.c_contiguous:
                raise ValueError("host state must be contiguous")
            if writable and not a.flags.writeable:
                raise ValueError("state is read-only")
            return ctypes.c_void_p(a.ctypes.data), L.PTR_HOST
        # torch tensor: CUDA (device pointer) or CPU, e.g. pinned (host pointer)
        if not hasattr(a, "data_ptr"):
            raise TypeError("state must be a numpy array or a torch tensor")
        if a.numel() != self.ndofs * self.nvars or not a.is_contiguous() or str(a.dtype) != "torch.float64":
            raise ValueError("state tensor must be a contiguous float64 tensor (nvars, ndofs)")
        if a.is_cuda:   # torch's pending writes to `a` complete first, unless both share a stream
            import torch
            if torch.cuda.current_stream(a.device).cuda_stream != getattr(self, "_stream", 0):
                _torch_stream_sync(a)
        return ctypes.c_void_p(a.data_ptr()), (L.PTR_DEVICE if a.is_cuda else L.PTR_HOST)

    def set_stream(self, stream_ptr):
        L.check(self._lib.flou_set_stream(self.h, ctypes.c_void_p(stream_ptr)), self.h)
        self._stream = int(stream_ptr or 0)

    def rhs(self, dQ, Q, t=0.0):
        pd, kd = self._ptr(dQ, True)
        pq, kq = self._ptr(Q)
        if kd != kq:
            raise ValueError("dQ and Q must both live on the host or both on the device")
        L.check(self._lib.flou_rhs(self.h, pd, pq, float(t), kd), self.h)

    def step(self, Q, dt, nsteps, t0=0.0):
        pq, kq = self._ptr(Q, True)
        L.check(self._lib.flou_step(self.h, pq, float(dt), float(t0), int(nsteps), kq), self.h)

    def step_cfl(self, Q, t0, tfinal, cfl, dtmax=float("inf"), max_steps=100000):
        """CFL-limited steps from t0 towards tfinal (at most max_steps); returns (steps, t reached)."""
        pq, kq = self._ptr(Q, True)
        n, t = ctypes.c_int64(), ctypes.c_double()
        L.check(self._lib.flou_step_cfl(self.h, pq, float(t0), float(tfinal), float(cfl), float(dtmax),
                                        int(max_steps), kq, ctypes.byref(n), ctypes.byref(t)), self.h)
        return n.value, t.value

    def step_async(self, Q, dt, nsteps, t0=0.0):
        """Queue `nsteps` steps (and, for host memory, the copies) without waiting; see wait()."""
        pq, kq = self._ptr(Q, True)
        L.check(self._lib.flou_step_async(self.h, pq, float(dt), float(t0), int(nsteps), kq), self.h)

    def wait(self):
        L.check(self._lib.flou_wait(self.h), self.h)

    def set_integrator(self, A=None, B=None):
        """The step method of step(): a 2N-storage method (A[0] unused), or SSP-RK3 when None."""
        if B is None:
            L.check(self._lib.flou_set_integrator(self.h, 0, None, None), self.h)
            return
        A = np.ascontiguousarray(A, dtype=np.float64)
        B = np.ascontiguousarray(B, dtype=np.float64)
        if A.shape != B.shape:
            raise ValueError("A and B must have one coefficient per stage")
        dp = ctypes.POINTER(ctypes.c_double)
        L.check(self._lib.flou_set_integrator(self.h, len(B), A.ctypes.data_as(dp), B.ctypes.data_as(dp)), self.h)

    def set_limiter(self, kind, minval=0.0):
        """FLOU_LIMITER_ZHANG_SHU with its minimum value, or FLOU_LIMITER_NONE."""
        L.check(self._lib.flou_set_limiter(self.h, int(kind), float(minval)), self.h)

    def limit(self, Q):
        """The set limiter applied once to Q in place."""
        pq, kq = self._ptr(Q, True)
        L.check(self._lib.flou_limit(self.h, pq, kq), self.h)

    def monitor(self, Q, which):
        pq, kq = self._ptr(Q)
        v = ctypes.c_double()
        L.check(self._lib.flou_monitor(self.h, pq, int(which), ctypes.byref(v), kq), self.h)
        return v.value

    def set_monitors(self, mask, capacity=1024):
        L.check(self._lib.flou_set_monitors(self.h, int(mask), int(capacity)), self.h)

    def take_monitors(self, max_steps=1 << 20, with_times=False):
        """(nsteps, 2) array of (kinetic energy, entropy) recorded after each step since the last take;
        with_times: also the time after each step (CFL stepping; NaN after fixed steps)."""
        out = np.zeros((max_steps, 2))
        times = np.zeros(max_steps)
        n = ctypes.c_int32()
        L.check(self._lib.flou_take_monitors_timed(self.h, out.ctypes.data_as(L._D),
                                                   times.ctypes.data_as(L._D) if with_times else None,
                                                   int(max_steps), ctypes.byref(n)), self.h)
        vals = out[:n.value].copy()
        return (vals, times[:n.value].copy()) if with_times else vals

    def max_dt(self, Q, cfl):
        pq, kq = self._ptr(Q)
        out = ctypes.c_double()
        L.check(self._lib.flou_max_dt(self.h, pq, float(cfl), ctypes.byref(out), kq), self.h)
        return out.value

    def set_dissipation(self, c):
        """Per-element LxF dissipation scale (numpy or CUDA tensor, nelem entries); None removes it."""
        if c is None:
            L.check(self._lib.flou_set_dissipation(self.h, None, L.PTR_HOST), self.h)
            return
        if isinstance(c, np.ndarray):
            c = np.ascontiguousarray(c, dtype=np.float64)
            self._c_keep = c
            L.check(self._lib.flou_set_dissipation(self.h, ctypes.c_void_p(c.ctypes.data), L.PTR_HOST), self.h)
        else:
            L.check(self._lib.flou_set_dissipation(self.h, ctypes.c_void_p(c.data_ptr()),
                                                   L.PTR_DEVICE if c.is_cuda else L.PTR_HOST), self.h)

    def rhs_vjp(self, Qbar, cbar, Q, lam):
        """Qbar = (∂rhs/∂Q)ᵀ lam, cbar = (∂rhs/∂c)ᵀ lam (CUDA tensors; cbar may be None)."""
        p = lambda t: ctypes.c_void_p(t.data_ptr()) if t is not None else None
        _torch_stream_sync(Q)
        L.check(self._lib.flou_rhs_vjp(self.h, p(Qbar), p(cbar), p(Q), p(lam)), self.h)

    def adjoint_solve(self, Q0, dt, nsteps, nsnap, rho_target, weights, dJdQ0, dJdc=None):
        """Returns (J, recomputed forward steps); fills dJdQ0 (and dJdc) -- CUDA tensors."""
        p = lambda t: ctypes.c_void_p(t.data_ptr()) if t is not None else None
        J = ctypes.c_double()
        nf = ctypes.c_int64()
        _torch_stream_sync(Q0)
        L.check(self._lib.flou_adjoint_solve(self.h, p(Q0), float(dt), int(nsteps), int(nsnap), p(rho_target),
                                             p(weights), ctypes.byref(J), p(dJdQ0), p(dJdc), ctypes.byref(nf)),
                self.h)
        return J.value, nf.value

    def time_kernels(self, Q, nrep=3):
        """Mean launch durations (ms) of the face kernel and the element kernel (CUDA events)."""
        pq, kq = self._ptr(Q)
        if kq != L.PTR_DEVICE:
            raise ValueError("time_kernels needs a device state")
        f, e = ctypes.c_double(), ctypes.c_double()
        L.check(self._lib.flou_time_kernels(self.h, pq, int(nrep), ctypes.byref(f), ctypes.byref(e)), self.h)
        return f.value, e.value

    def take_status(self):
        f, e = ctypes.c_int32(), ctypes.c_int32()
        L.check(self._lib.flou_take_status(self.h, ctypes.byref(f), ctypes.byref(e)), self.h)
        return f.value, e.value


class EquationConfig:
    """EquationConfig(disc, equation)."""

    def __init__(self, disc, equation):
        self.disc = disc
        self.equation = equation


def rhs_(dQ, Q, p, time=0.0):
    """rhs!(dQ, Q, p::EquationConfig, t): overwrites dQ with the semidiscrete residual."""
    p.disc.ctx.rhs(dQ, Q, time)
    return None


def get_max_dt(q, disc, equation, cfl):
    """get_max_dt(q, disc, eq, cfl) (MultielementDiscontinuous.jl:162-178)."""
    return disc.ctx.max_dt(q, cfl)
