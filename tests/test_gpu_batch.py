"""Batched mode: one persistent launch per SSP-RK3 stage over many uneven instances.

The batched result must equal, bit for bit, each instance stepped on its own with the plain
kernels (the same tile code runs in both), agree with the oracle, survive the autotuner's
re-tiling, and report a bounded-wait timeout as FLOU_ERR_TIMEOUT without hanging.
"""
import numpy as np
import pytest

import flou_cuda as F
from flou_cuda import _lib
from cases import build, oracle_for, rel_linf, smooth_euler_state

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _instances_2d(seed=0, count=8):
    """Small instances of the batched configuration: periodic or slip-walled [-5,5]² boxes,
    orders p = 2..7, isentropic vortex + Gaussian density bump."""
    rng = np.random.default_rng(seed)
    eq = F.EulerEquation(2, 1.4)
    box = ((-5.0, -5.0), (5.0, 5.0))
    op = lambda: F.StrongDivOperator(F.LxF(F.StdAverage(), 1.0))
    out = []
    for k in range(count):
        n = int(rng.integers(3, 9))          # p = 2..7
        ne = tuple(int(x) for x in rng.integers(2, 6, size=2))
        walls = bool(k % 2)
        if walls:
            bcs = {str(b): F.EulerSlipBC() for b in range(1, 5)}
            disc = build(2, n, ne, eq, op(), periodic=(), bcs=bcs, box=box)
        else:
            disc = build(2, n, ne, eq, op(), box=box)
        Q = np.asfortranarray(F.initial.vortex_bump(
            eq, disc.coords, rng.uniform(-1, 1, 2), rng.uniform(1, 6), rng.uniform(0, 0.1),
            uinf=(0.0, 0.0) if walls else (1.0, 1.0), period=None if walls else (10.0, 10.0)))
        dt = 0.3 * disc.ctx.max_dt(Q, 1.0)
        out.append((disc, Q, dt))
    return out


def _device(Q):
    return torch.from_numpy(np.ascontiguousarray(Q.T)).cuda()


def _serial(insts, nsteps):
    res = []
    for disc, Q, dt in insts:
        q = _device(Q)
        disc.ctx.step(q, dt, nsteps)
        res.append(q)
    return res


def test_batch_2d_matches_serial_bitwise():
    insts = _instances_2d(seed=1)
    ref = _serial(insts, 3)
    states = [_device(Q) for _, Q, _ in insts]
    b = F.Batch([d for d, _, _ in insts], states, [dt for _, _, dt in insts])
    b.step(3)
    for q, r in zip(states, ref):
        assert torch.equal(q, r)


def test_batch_autotune_keeps_results():
    insts = _instances_2d(seed=2, count=6)
    ref = _serial(insts, 2)
    states = [_device(Q) for _, Q, _ in insts]
    b = F.Batch([d for d, _, _ in insts], states, [dt for _, _, dt in insts])
    choice = b.autotune()
    assert choice["threads_per_block"] in (128, 256) and choice["blocks_per_sm"] >= 1
    assert set(choice["tiles_per_item"].values()) <= {1, 2, 4}
    b.step(2)
    for q, r in zip(states, ref):
        assert torch.equal(q, r)


@pytest.mark.parametrize("tiles", [3, 8, {1: 2, 2: 4, 3: 1, 4: 5, 5: 2, 6: 3, 7: 8}])
def test_batch_tiles_per_item_keep_results(tiles):
    """Work items of several element tiles (the last tile of an instance may run past its
    elements) give the serial results bit for bit."""
    insts = _instances_2d(seed=4, count=6)
    ref = _serial(insts, 2)
    states = [_device(Q) for _, Q, _ in insts]
    b = F.Batch([d for d, _, _ in insts], states, [dt for _, _, dt in insts])
    b.set_tiles_per_item(tiles)
    assert b.tiles_per_item() == ({p: tiles for p in range(1, 8)} if isinstance(tiles, int) else tiles)
    b.step(2)
    for q, r in zip(states, ref):
        assert torch.equal(q, r)
    with pytest.raises(F.FlouError):
        b.set_tiles_per_item(9)


def test_batch_instance_against_oracle():
    insts = _instances_2d(seed=3, count=4)
    states = [_device(Q) for _, Q, _ in insts]
    b = F.Batch([d for d, _, _ in insts], states, [dt for _, _, dt in insts])
    b.step(4)
    for (disc, Q, dt), q in zip(insts, states):
        ref = oracle_for(disc).ssprk3(Q, dt, 4)
        assert rel_linf(q.cpu().numpy().T, ref) <= 1e-10


def test_batch_3d_split_matches_serial():
    eq = F.EulerEquation(3, 1.4)
    insts = []
    for k, (n, ne) in enumerate(((4, (2, 3, 2)), (5, (2, 2, 2)), (6, (1, 2, 2)), (4, (3, 3, 3)))):
        disc = build(3, n, ne, eq, F.SplitDivOperator(F.ChandrasekharAverage(), F.HLLC()))
        Q = smooth_euler_state(disc, seed=40 + k)
        insts.append((disc, Q, 0.3 * disc.ctx.max_dt(Q, 1.0)))
    ref = _serial(insts, 2)
    states = [_device(Q) for _, Q, _ in insts]
    b = F.Batch([d for d, _, _ in insts], states, [dt for _, _, dt in insts])
    b.step(2)
    for q, r in zip(states, ref):
        assert torch.equal(q, r)


def test_batch_wait_timeout_is_reported_and_recoverable():
    insts = _instances_2d(seed=4, count=3)
    states = [_device(Q) for _, Q, _ in insts]
    b = F.Batch([d for d, _, _ in insts], states, [dt for _, _, dt in insts])
    b.test_skip_faces(1)   # instance 1's face items never report: its tiles' waits run out
    with pytest.raises(F.FlouError) as ei:
        b.step(1)
    assert ei.value.status == _lib.FLOU_ERR_TIMEOUT
    b.test_skip_faces(-1)
    fresh = [_device(Q) for _, Q, _ in insts]
    b.set_states(fresh, [dt for _, _, dt in insts])
    b.step(1)
    ref = _serial(insts, 1)
    for q, r in zip(fresh, ref):
        assert torch.equal(q, r)


def test_batch_rejects_mixed_operators():
    eq = F.EulerEquation(2, 1.4)
    a = build(2, 4, (2, 2), eq, F.StrongDivOperator(F.LxF(F.StdAverage(), 1.0)))
    c = build(2, 4, (2, 2), eq, F.SplitDivOperator(F.ChandrasekharAverage(), F.HLLC()))
    qa, qc = _device(smooth_euler_state(a)), _device(smooth_euler_state(c))
    with pytest.raises(F.FlouError):
        F.Batch([a, c], [qa, qc], [1e-3, 1e-3])


@pytest.mark.parametrize("method", ["ORK256", "CarpenterKennedy2N54"])
def test_batch_2n_storage_matches_serial_bitwise(method):
    """Instances stepping with a 2N-storage method: one persistent launch per stage, every stage
    in place with the register in the stage buffer, bit for bit the serial steps; the autotuner
    times its own set (the first SSP-RK3 stage) and leaves the states alone."""
    insts = _instances_2d(seed=5, count=6)
    m = getattr(F, method)()
    for d, _, _ in insts:
        d.ctx.set_integrator(m.A, m.B)
    try:
        ref = _serial(insts, 3)
        states = [_device(Q) for _, Q, _ in insts]
        b = F.Batch([d for d, _, _ in insts], states, [dt for _, _, dt in insts])
        b.autotune()
        for q, (_, Q, _) in zip(states, insts):
            assert torch.equal(q, _device(Q))
        b.step(3)
        for q, r in zip(states, ref):
            assert torch.equal(q, r)
    finally:
        for d, _, _ in insts:
            d.ctx.set_integrator(None)


def test_batch_limiter_matches_serial_bitwise():
    """Instances with the Zhang-Shu stage limiter (some with it, some without), with SSP-RK3 and
    with ORK256: the limiter runs after every stage of the limited instances, bit for bit the
    serial steps, and it acts."""
    from test_oracle_kat import _dipped_state
    eq = F.EulerEquation(2, 1.4)
    op = lambda: F.StrongDivOperator(F.LxF(F.StdAverage(), 1.0))
    for method in (None, F.ORK256()):
        insts = []
        for k in range(4):
            disc = build(2, 4 + k % 2, (3, 3), eq, op())
            Q = _dipped_state(disc, seed=40 + k)
            if k % 2 == 0:
                disc.ctx.set_limiter(_lib.LIMITER_ZHANG_SHU, 0.5)
            if method is not None:
                disc.ctx.set_integrator(method.A, method.B)
            insts.append((disc, Q, 0.2 * disc.ctx.max_dt(Q, 1.0)))
        ref = _serial(insts[::2], 3)
        states = [_device(Q) for _, Q, _ in insts[::2]]
        b = F.Batch([d for d, _, _ in insts[::2]], states, [dt for _, _, dt in insts[::2]])
        b.step(3)
        for q, r in zip(states, ref):
            assert torch.equal(q, r)
        d0, Q0, dt0 = insts[0]
        o = oracle_for(d0)
        lim = (o.ssprk3_limited(Q0, dt0, 3, 0.5, d0.std.omega) if method is None else
               o.lsrk2n(Q0, dt0, 3, method.A, method.B, method.c, minval=0.5, omega_tp=d0.std.omega))
        assert rel_linf(states[0].cpu().numpy().T, lim) <= 1e-10
        for d, _, _ in insts:
            d.ctx.set_limiter(_lib.LIMITER_NONE)
            d.ctx.set_integrator(None)


def test_batch_rejects_mixed_integrators():
    eq = F.EulerEquation(2, 1.4)
    a = build(2, 4, (2, 2), eq, F.StrongDivOperator(F.LxF(F.StdAverage(), 1.0)))
    c = build(2, 4, (2, 2), eq, F.StrongDivOperator(F.LxF(F.StdAverage(), 1.0)))
    m = F.ORK256()
    c.ctx.set_integrator(m.A, m.B)
    qa, qc = _device(smooth_euler_state(a)), _device(smooth_euler_state(c))
    with pytest.raises(F.FlouError):
        F.Batch([a, c], [qa, qc], [1e-3, 1e-3])
    c.ctx.set_integrator(None)


def test_batch_general_geometry_matches_serial_bitwise():
    """Instances on perturbed, rotated meshes (the general-geometry tiles and face nodes of the
    persistent kernel): 2D strong form of uneven orders, and 3D split form."""
    from test_gpu_unstructured import _disc as _udisc
    from test_unstructured import _state
    for dim, cases in ((2, [(3, "strong_lxf"), (5, "strong_lxf"), (4, "strong_lxf"), (7, "strong_lxf")]),
                       (3, [(3, "split_chandra_lxfc"), (4, "split_chandra_lxfc"), (5, "split_chandra_lxfc")])):
        insts = []
        for k, (n, op) in enumerate(cases):
            disc = _udisc(dim, n, op, nel=2 + k % 2, seed=3 + k)
            Q = _state(disc, seed=k)
            insts.append((disc, Q, 0.2 * disc.ctx.max_dt(Q, 1.0)))
        ref = _serial(insts, 3)
        states = [_device(Q) for _, Q, _ in insts]
        b = F.Batch([d for d, _, _ in insts], states, [dt for _, _, dt in insts])
        b.step(3)
        for q, r in zip(states, ref):
            assert torch.equal(q, r)


def test_batch_records_monitors_like_serial():
    insts = _instances_2d(seed=7, count=4)
    for d, _, _ in insts[::2]:
        d.ctx.set_monitors(_lib.MONITOR_KINETIC_ENERGY | _lib.MONITOR_ENTROPY)
    ref_states = _serial(insts, 3)
    ref = [d.ctx.take_monitors() for d, _, _ in insts[::2]]
    states = [_device(Q) for _, Q, _ in insts]
    b = F.Batch([d for d, _, _ in insts], states, [dt for _, _, dt in insts])
    b.step(3)
    for q, r in zip(states, ref_states):
        assert torch.equal(q, r)
    for (d, _, _), r in zip(insts[::2], ref):
        got = d.ctx.take_monitors()
        assert got.shape == (3, 2) and np.array_equal(got, r)
        d.ctx.set_monitors(0)
