"""flou_rhs_noalloc: the residual without any device allocation, against flou_rhs.

flou_rhs allocates its face-flux buffer with cudaMalloc the first time it runs.  A caller
whose device memory is owned by another allocator (CUDA.jl's memory pool in a Julia
session, PyTorch's caching allocator here) may have no free memory left for that, or may
not allow allocations outside its pool once the solve has started.  flou_rhs_noalloc keeps
the face fluxes in a fixed array inside the library instead.  These tests call it through
the C ABI and compare it with flou_rhs, twice in a row, across contexts and over every
kind of context the residual serves (strong, split and hybrid operators; Cartesian and
general geometry; Gauss-Lobatto and Gauss nodes; a boundary state that varies along the
boundary).  They also check that it turns away, on the host and before any launch, the
contexts flou_rhs turns away, and that an oversized mesh is rejected.  This file is
collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

import flou_cuda as F
from flou_cuda import _lib
from cases import build, rel_linf, smooth_euler_state

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _noalloc(disc_or_ctx, out, Q):
    h = getattr(disc_or_ctx, "ctx", disc_or_ctx).h
    return F.load().flou_rhs_noalloc(h, ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(Q.data_ptr()), 0.0)


def _rhs(ctx, out, Q):
    return F.load().flou_rhs(ctx.h, ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(Q.data_ptr()), 0.0,
                             _lib.PTR_DEVICE)


def _device(Q):
    torch = pytest.importorskip("torch")
    return torch.from_numpy(np.ascontiguousarray(Q.T)).cuda()


def _reference(disc, Q):
    """(device state, flou_rhs residual as an (ndofs, nvars) array)."""
    torch = pytest.importorskip("torch")
    Qd = _device(Q)
    ref = torch.empty_like(Qd)
    disc.ctx.rhs(ref, Qd)
    return Qd, ref.cpu().numpy().T


def _case(dim, n, ne, op, seed, periodic=True, bcs=None):
    disc = build(dim, n, ne, F.EulerEquation(dim, 1.4), op, periodic=periodic, bcs=bcs)
    Q = smooth_euler_state(disc, seed=seed)
    return (disc,) + _reference(disc, Q)


def _general(dim, n, op, basis="GLL"):
    """A perturbed box whose elements are randomly rotated (general geometry)."""
    from test_gpu_unstructured import _disc
    from test_unstructured import _state
    disc = _disc(dim, n, op, basis=basis)
    return (disc,) + _reference(disc, _state(disc, seed=dim + n))


def _state_field_case():
    eq = F.EulerEquation(2, 1.4)

    def qext(_q, x, _f, _t, _e):
        return eq.vars_prim2cons(np.array([1.0 + 0.3 * np.sin(2 * np.pi * x[1]), 0.4,
                                           0.1 * np.cos(2 * np.pi * x[1]), 1.0 + 0.1 * x[1]]))

    disc = build(2, 4, (3, 3), eq, F.SplitDivOperator(F.ChandrasekharAverage(), F.HLLC()), periodic=(),
                 bcs={"1": F.GenericBC(qext), "2": F.GenericBC(qext), "3": F.EulerSlipBC(), "4": F.EulerSlipBC()},
                 box=((0.0, 0.0), (1.0, 1.0)))
    assert isinstance(disc.bcs[0], F.equations.StateFieldBC)
    return (disc,) + _reference(disc, smooth_euler_state(disc, seed=13))


def _hybrid_hllc():
    return F.HybridDivOperator(F.ChandrasekharAverage(), F.HLLC(), F.LxF(F.ChandrasekharAverage(), 1.0), 0.5)


CASES = {
    "hybrid_2d": lambda: _case(2, 5, (3, 3), _hybrid_hllc(), seed=4),
    "hybrid_md_3d": lambda: _case(3, 4, (2, 2, 2),
                                  F.HybridDivOperator(F.MatrixDissipation(F.ChandrasekharAverage(), 1.0), 1.0), seed=5),
    "gauss_split_2d": lambda: (lambda d: (d,) + _reference(d, smooth_euler_state(d, seed=6)))(
        build(2, 4, (3, 3), F.EulerEquation(2, 1.4), F.SplitDivOperator(F.ChandrasekharAverage(), F.HLLC()),
              basis="GL")),
    "general_split_3d": lambda: _general(3, 4, "split_chandra_lxfc"),
    "general_hybrid_2d": lambda: _general(2, 4, "hybrid_hllc"),
    "general_gauss_split_2d": lambda: _general(2, 4, "split_chandra_lxfc", basis="GL"),
    "state_field_bc_2d": _state_field_case,
}


def test_noalloc_matches_rhs_two_calls_in_a_row():
    torch = pytest.importorskip("torch")
    disc, Qd, ref = _case(3, 4, (3, 3, 3), F.SplitDivOperator(F.ChandrasekharAverage(), F.HLLC()), seed=1)
    for _ in range(2):
        out = torch.full_like(Qd, float("nan"))
        assert _noalloc(disc, out, Qd) == _lib.FLOU_OK, F.load().flou_last_error(disc.ctx.h)
        assert rel_linf(out.cpu().numpy().T, ref) <= TOL


@pytest.mark.parametrize("name", sorted(CASES))
def test_noalloc_matches_rhs_on_every_context_kind(name):
    torch = pytest.importorskip("torch")
    disc, Qd, ref = CASES[name]()
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


def _incomplete_context(disc, drop):
    """A context of disc's set-up with one set-up call left out."""
    a = dict(disc.abi_arrays())
    assert a[drop] is not None
    a[drop] = None
    return F.Context(disc.config, a, disc.mesh.nelements, disc.mesh.nfaces)


@pytest.mark.parametrize("which", ["hybrid", "subgrid"])
def test_noalloc_rejects_the_contexts_rhs_rejects(which):
    """A hybrid context without flou_set_hybrid, or a general-geometry hybrid context without
    flou_set_subgrid, is turned away by both entry points with FLOU_ERR_STATE before anything
    is launched (the output keeps its NaN fill)."""
    torch = pytest.importorskip("torch")
    if which == "hybrid":
        disc = build(2, 4, (3, 3), F.EulerEquation(2, 1.4), _hybrid_hllc())
        Q = smooth_euler_state(disc, seed=7)
    else:
        from test_gpu_unstructured import _disc
        from test_unstructured import _state
        disc = _disc(2, 4, "hybrid_hllc")
        Q = _state(disc, seed=7)
    ctx = _incomplete_context(disc, which)
    Qd = _device(Q)
    for call in (_noalloc, _rhs):
        out = torch.full_like(Qd, float("nan"))
        assert call(ctx, out, Qd) == _lib.FLOU_ERR_STATE
        assert ("flou_set_" + which).encode() in F.load().flou_last_error(ctx.h)
        torch.cuda.synchronize()
        assert torch.isnan(out).all()


def test_noalloc_rejects_meshes_beyond_the_fixed_scratch():
    torch = pytest.importorskip("torch")
    disc = build(2, 8, (130, 130), F.EulerEquation(2, 1.4), F.StrongDivOperator(F.LxF(F.StdAverage(), 1.0)))
    Qd = torch.ones((4, disc.ndofs), dtype=torch.float64, device="cuda")
    out = torch.empty_like(Qd)
    assert _noalloc(disc, out, Qd) == _lib.FLOU_ERR_ARG
    assert b"fixed scratch holds at most 1048576" in F.load().flou_last_error(disc.ctx.h)
