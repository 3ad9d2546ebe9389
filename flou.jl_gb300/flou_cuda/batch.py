"""Batched mode: many independent discretizations advanced by one persistent launch per
SSP-RK3 stage (flou_batch_* in include/flou_cuda.h).  No counterpart in Flou, which solves one
problem at a time; each instance is an ordinary MultielementDisc."""
import ctypes

import numpy as np

from . import _lib as L


class Batch:
    """Batch(discs, states, dts): `states` are CUDA tensors (nvars, ndofs), advanced in place."""

    def __init__(self, discs, states, dts):
        lib = L.load()
        self._lib = lib
        self.discs = list(discs)
        self.states = list(states)
        n = len(self.discs)
        ctxs = (ctypes.c_void_p * n)(*[d.ctx.h.value for d in self.discs])
        h = ctypes.c_void_p()
        st = lib.flou_batch_create(n, ctxs, ctypes.byref(h))
        self.h = h
        self._check(st)
        for d, q in zip(self.discs, self.states):
            if not getattr(q, "is_cuda", False) or q.numel() != d.ndofs * d.nvariables:
                raise ValueError("batch states must be CUDA tensors of each instance's size")
        self.set_states(self.states, dts)

    def _check(self, st):
        if st == L.FLOU_OK:
            return
        msg = ""
        if self.h is not None and self.h.value:
            raw = self._lib.flou_batch_last_error(self.h)
            msg = raw.decode() if raw else ""
        cls = L.DomainError if st == L.FLOU_ERR_NONPHYSICAL else L.FlouError
        raise cls(st, msg)

    def set_states(self, states, dts):
        self.states = list(states)
        n = len(self.states)
        ptrs = (ctypes.c_void_p * n)(*[q.data_ptr() for q in self.states])
        self._dts = np.ascontiguousarray(dts, dtype=np.float64)
        self._check(self._lib.flou_batch_set_states(self.h, ptrs, L.dptr(self._dts)))

    def set_stream(self, stream_ptr):
        self._check(self._lib.flou_batch_set_stream(self.h, ctypes.c_void_p(stream_ptr)))

    def step(self, nsteps=1):
        self._check(self._lib.flou_batch_step(self.h, int(nsteps)))

    def autotune(self):
        """Times the candidate launch shapes and keeps the fastest: threads per block (which sets
        the elements per tile of every order), resident blocks per SM, the element-item order, and
        per order the number of element tiles one work item holds."""
        out = (ctypes.c_int32 * 3)()
        self._check(self._lib.flou_batch_autotune(self.h, out))
        return {"threads_per_block": out[0], "blocks_per_sm": out[1], "order": "by_order_desc" if out[2] else "by_instance",
                "tiles_per_item": self.tiles_per_item()}

    def set_tiles_per_item(self, tiles):
        """Fixes the element tiles per work item: an int for every order or {p: tiles}."""
        t = (ctypes.c_int32 * 7)(*[int(tiles.get(p, 1) if isinstance(tiles, dict) else tiles) for p in range(1, 8)])
        self._check(self._lib.flou_batch_set_tiles(self.h, t))

    def tiles_per_item(self):
        """{p: element tiles per work item} for the orders p = 1..7."""
        t = (ctypes.c_int32 * 7)()
        self._check(self._lib.flou_batch_tiles(self.h, t))
        return {n + 1: t[n] for n in range(7)}

    def test_skip_faces(self, inst):
        self._check(self._lib.flou_batch_test_skip_faces(self.h, int(inst)))

    def __del__(self):
        h = getattr(self, "h", None)
        if h is not None and h.value:
            self._lib.flou_batch_destroy(h)
            self.h = None


def adjoint_solve_batch(discs, Q0s, dts, nsteps, budget_bytes, rho_targets, weights, dJdQ0s, dJdcs=None,
                        nstreams=8):
    """Gradients of J_k = 1/2 Σ w (ρ(T) - ρt)² for every instance k in one lockstep reverse sweep
    under one device-memory budget (flou_adjoint_solve_batch).  All arrays are CUDA tensors;
    dJdQ0s (and dJdcs) are filled.  Returns (J list, recomputed forward steps per instance,
    snapshots used)."""
    import torch

    lib = L.load()
    n = len(discs)
    vp = lambda ts: (ctypes.c_void_p * n)(*[t.data_ptr() if t is not None else None for t in ts])
    ctxs = (ctypes.c_void_p * n)(*[d.ctx.h.value for d in discs])
    dt = np.ascontiguousarray(dts, dtype=np.float64)
    J = np.zeros(n)
    nf = ctypes.c_int64()
    ns = ctypes.c_int32()
    torch.cuda.synchronize()   # inputs written on torch's stream are complete
    st = lib.flou_adjoint_solve_batch(n, ctxs, vp(Q0s), L.dptr(dt), int(nsteps), int(budget_bytes), int(nstreams),
                                      vp(rho_targets), vp(weights), L.dptr(J), vp(dJdQ0s),
                                      vp(dJdcs) if dJdcs is not None else None, ctypes.byref(nf),
                                      ctypes.byref(ns))
    L.check(st, discs[0].ctx.h)
    return list(J), nf.value, ns.value
