"""The index-checked build: libflou_cuda_checked.so, compiled with -DFLOU_CUDA_CHECKED.

Every kernel of that build checks the indices it computes (elements and local faces decoded
from the connectivity, trace nodes, face-flux offsets, orientation-mapped lines, batched
instance numbers, adjoint trace cotangents) against the sizes of the arrays they address.  An
index out of range sets bit 2 of the status word, the access is skipped, and the call returns
FLOU_ERR_INDEX; nothing traps.  This stands in for a memory checker on the device.

test_checked_build_runs_the_device_suites runs the device parity suites and an all-orders
sweep on tiny meshes in a child process with FLOU_CUDA_CHECKED=1, which makes flou_cuda load
the checked library; every call must come back with a clean status word.  The sweep itself only
runs in that child process.
"""
import os
import subprocess
import sys

import numpy as np
import pytest

import flou_cuda as F
from flou_cuda import _lib
from cases import build, smooth_euler_state

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SUITES = ["tests/test_gpu_parity.py", "tests/test_gpu_unstructured.py", "tests/test_gpu_batch.py",
          "tests/test_gpu_adjoint.py", "tests/test_gpu_adjoint_scalar.py", "tests/test_gpu_adjoint_batch.py", "tests/test_gpu_limiter.py",
          "tests/test_gpu_cfl.py", "tests/test_gpu_lowstorage.py", "tests/test_zz_no_alloc.py"]


def test_checked_build_runs_the_device_suites():
    lib = os.path.join(ROOT, "flou.jl_gb300", "lib", "libflou_cuda_checked.so")
    assert os.path.exists(lib), "build() builds the checked library beside the default one"
    env = dict(os.environ, FLOU_CUDA_CHECKED="1")
    cmd = [sys.executable, "-m", "pytest", "-q", "-x", "-m", "gpu", "-p", "no:cacheprovider"] + SUITES + \
          ["tests/test_gpu_checked.py::test_all_orders_sweep_under_checks"]
    p = subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=1500)
    tail = "\n".join((p.stdout + p.stderr).splitlines()[-25:])
    assert p.returncode == 0, tail
    assert " passed" in tail and "skipped" not in tail.split("\n")[-1], tail


def _ops(dim):
    hyb = F.HybridDivOperator(F.ChandrasekharAverage(), F.HLLC(), F.LxF(F.ChandrasekharAverage(), 1.0), 0.5)
    return {"strong_lxf": F.StrongDivOperator(F.LxF(F.StdAverage(), 1.0)),
            "split_hllc": F.SplitDivOperator(F.ChandrasekharAverage(), F.HLLC()),
            "split_md": F.SplitDivOperator(F.MatrixDissipation(F.ChandrasekharAverage(), 1.0)),
            "hybrid": hyb}


@pytest.mark.skipif(not _lib.CHECKED, reason="runs in the child process that loads the checked build")
@pytest.mark.parametrize("dim", [1, 2, 3])
def test_all_orders_sweep_under_checks(dim):
    """p = 1..7 on one- and two-element meshes (walls, and periodic), every volume operator, both
    node sets: a residual, two SSP-RK3 steps and a time-step estimate, each status-checked."""
    torch = pytest.importorskip("torch")
    assert _lib.LIB_PATH.endswith("libflou_cuda_checked.so")
    eq = F.EulerEquation(dim, 1.4)
    walls = {str(k): (F.EulerSlipBC() if k % 2 else F.EulerOutflowBC()) for k in range(1, 2 * dim + 1)}
    for n in range(2, 9):
        for basis in ("GLL", "GL"):
            for name, op in _ops(dim).items():
                for ne, periodic, bcs in (((1,) * dim, (), walls), ((2,) + (1,) * (dim - 1), (0,), walls)):
                    disc = build(dim, n, ne, eq, op, periodic=periodic,
                                 bcs={k: v for k, v in bcs.items() if periodic == () or k not in ("1", "2")},
                                 basis=basis)
                    Q = smooth_euler_state(disc, seed=n)
                    Qd = torch.from_numpy(np.ascontiguousarray(Q.T)).cuda()
                    dQ = torch.empty_like(Qd)
                    disc.ctx.rhs(dQ, Qd)
                    dt = 0.1 * disc.ctx.max_dt(Qd, 1.0)
                    disc.ctx.step(Qd, dt, 2)
                    assert bool(torch.isfinite(Qd).all())
