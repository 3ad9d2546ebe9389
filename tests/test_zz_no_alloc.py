"""flou_rhs_noalloc: the residual without any device allocation, against flou_rhs.

flou_rhs allocates its face-flux buffer with cudaMalloc the first time it runs.  A caller
whose device memory is owned by another allocator (CUDA.jl's memory pool in a Julia
session, PyTorch's caching allocator here) may have no free memory left for that, or may
not allow allocations outside its pool once the solve has started.  flou_rhs_noalloc keeps
the face fluxes in a fixed array inside the library instead.  These tests call it through
the C ABI and compare it with flou_rhs, twice in a row, across contexts, and check that an
oversized mesh is rejected.  This file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

import flou_cuda as F
from flou_cuda import _lib
from cases import build, rel_linf, smooth_euler_state

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _noalloc(disc, out, Q):
    lib = F.load()
    return lib.flou_rhs_noalloc(disc.ctx.h, ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(Q.data_ptr()), 0.0)


def _case(dim, n, ne, op, seed, periodic=True, bcs=None):
    torch = pytest.importorskip("torch")
    disc = build(dim, n, ne, F.EulerEquation(dim, 1.4), op, periodic=periodic, bcs=bcs)
    Q = smooth_euler_state(disc, seed=seed)
    Qd = torch.from_numpy(np.ascontiguousarray(Q.T)).cuda()
    ref = torch.empty_like(Qd)
    disc.ctx.rhs(ref, Qd)
    return disc, Qd, ref.cpu().numpy().T


def test_noalloc_matches_rhs_two_calls_in_a_row():
    torch = pytest.importorskip("torch")
    disc, Qd, ref = _case(3, 4, (3, 3, 3), F.SplitDivOperator(F.ChandrasekharAverage(), F.HLLC()), seed=1)
    for _ in range(2):
        out = torch.full_like(Qd, float("nan"))
        assert _noalloc(disc, out, Qd) == _lib.FLOU_OK, F.load().flou_last_error(disc.ctx.h)
        assert rel_linf(out.cpu().numpy().T, ref) <= TOL


def test_noalloc_shared_scratch_across_contexts():
    torch = pytest.importorskip("torch")
    walls = {"1": F.EulerSlipBC(), "2": F.EulerSlipBC(), "3": F.EulerOutflowBC(), "4": F.EulerOutflowBC()}
    a = _case(2, 5, (4, 3), F.StrongDivOperator(F.LxF(F.StdAverage(), 1.0)), seed=2, periodic=(), bcs=walls)
    b = _case(3, 8, (2, 2, 2), F.SplitDivOperator(F.ChandrasekharAverage(), F.HLLC()), seed=3)
    for disc, Qd, ref in (a, b, a, b):
        out = torch.full_like(Qd, float("nan"))
        assert _noalloc(disc, out, Qd) == _lib.FLOU_OK
        assert rel_linf(out.cpu().numpy().T, ref) <= TOL


def test_noalloc_rejects_meshes_beyond_the_fixed_scratch():
    torch = pytest.importorskip("torch")
    disc = build(2, 8, (130, 130), F.EulerEquation(2, 1.4), F.StrongDivOperator(F.LxF(F.StdAverage(), 1.0)))
    Qd = torch.ones((4, disc.ndofs), dtype=torch.float64, device="cuda")
    out = torch.empty_like(Qd)
    assert _noalloc(disc, out, Qd) == _lib.FLOU_ERR_ARG
    assert b"fixed scratch holds at most 1048576" in F.load().flou_last_error(disc.ctx.h)
