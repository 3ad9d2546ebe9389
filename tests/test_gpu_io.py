"""Snapshots and restarts from device buffers: the equispaced resampling runs on the GPU and
gives the host path's values; a restart of a device state reproduces it bit for bit."""
import numpy as np
import pytest

import flou_cuda as F
from flou_cuda import io as fio
from cases import build, smooth_euler_state

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def test_device_snapshot_and_restart(tmp_path):
    eq = F.EulerEquation(3, 1.4)
    disc = build(3, 5, (2, 2, 2), eq, F.SplitDivOperator(F.LxF(F.ChandrasekharAverage(), 1.0)))
    Q = smooth_euler_state(disc, seed=2)
    Qd = torch.from_numpy(np.ascontiguousarray(Q.T)).cuda()
    disc.ctx.step(Qd, 1e-3, 3)
    Qh = np.asfortranarray(Qd.cpu().numpy().T)
    fio.write_vtu(str(tmp_path / "d.vtu"), disc, Qd, time=3e-3)
    fio.write_vtu(str(tmp_path / "h.vtu"), disc, Qh, time=3e-3)
    vd, vh = fio.read_vtu(str(tmp_path / "d.vtu")), fio.read_vtu(str(tmp_path / "h.vtu"))
    for name in fio.variablenames(eq):
        assert np.allclose(vd[name], vh[name], rtol=1e-13, atol=1e-14)
    fio.write_vtkhdf(str(tmp_path / "d.hdf"), disc, Qd, time=3e-3)
    hd = fio.read_vtkhdf(str(tmp_path / "d.hdf"))
    for name in fio.variablenames(eq):
        assert np.allclose(hd["PointData"][name], vh[name], rtol=1e-13, atol=1e-14)
    fio.save_restart(str(tmp_path / "r.bin"), disc, Qd, time=3e-3, iteration=3)
    R, t, it = fio.load_restart(str(tmp_path / "r.bin"), disc)
    assert np.array_equal(R, Qh) and it == 3
