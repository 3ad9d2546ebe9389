"""GPU: the reference's own examples (examples/src/1D_Burgers.jl, 2D_LinearAdvection.jl) set up
through the flou_cuda host side exactly as the scripts do, run with ORK256 through timeintegrate
(a shorter final time), against the oracle stepping the same method."""
import os

import numpy as np
import pytest

import flou_cuda as F
from cases import oracle_for, rel_linf

pytestmark = pytest.mark.gpu


def test_example_1d_burgers():
    """1D_Burgers.jl: GLL 4 nodes, 20 periodic elements on [0, 1], StrongDivOperator(LxF(StdAverage,
    1)), a Gaussian bump (x0 0.4, s 0.1, h 1), ORK256 with dt 1e-4 (tf 0.15 there; 0.02 here)."""
    eq = F.BurgersEquation()
    basis = F.LagrangeBasis("GLL", 4)
    std = F.StdSegment(basis, F.DGSEMrec(basis), eq.nvariables)
    mesh = F.CartesianMesh((0.0,), (1.0,), (20,))
    F.apply_periodicBCs(mesh, ("1", "2"))
    dg = F.MultielementDisc(mesh, std, eq, F.StrongDivOperator(F.LxF(F.StdAverage(), 1.0)), {})
    Q = np.asfortranarray(F.initial.gaussian_bump(dg.coords[:, :1], (0.4,), (0.1,), 1.0)[:, None])
    dt, tf = 1e-4, 0.02
    sol, _ = F.timeintegrate(Q.copy(order="F"), dg, eq, F.ORK256(williamson_condition=False), tf, dt=dt,
                             alias_u0=True)
    m = F.ORK256()
    ref = oracle_for(dg).lsrk2n(Q, dt, int(round(tf / dt)), m.A, m.B, m.c)
    assert rel_linf(sol.u[-1], ref) <= 1e-10
    assert sol.u[-1].max() < 1.0 and sol.u[-1].max() > 0.9   # the bump steepens and moves


def test_example_2d_linear_advection(tmp_path):
    """2D_LinearAdvection.jl: a = (2, -1), GL 4 nodes, 10 x 10 periodic elements on [0, 1]²,
    StrongDivOperator(LxF(StdAverage, 1)), ORK256 with dt 1e-3 and a save callback every 50 steps
    (range(0, 1000, 21) there; tf 1 there, 0.1 here)."""
    eq = F.LinearAdvection(2.0, -1.0)
    basis = F.LagrangeBasis("GL", 4)
    std = F.StdQuad(basis, F.DGSEMrec(basis), eq.nvariables)
    mesh = F.CartesianMesh((0.0, 0.0), (1.0, 1.0), (10, 10))
    F.apply_periodicBCs(mesh, ("1", "2"), ("3", "4"))
    dg = F.MultielementDisc(mesh, std, eq, F.StrongDivOperator(F.LxF(F.StdAverage(), 1.0)), {})
    Q = np.asfortranarray(F.initial.gaussian_bump(dg.coords[:, :2], (0.5, 0.5), (0.1, 0.1), 1.0)[:, None])
    dt, tf = 1e-3, 0.1
    sb = F.get_save_callback(os.path.join(tmp_path, "solution"), iter=range(0, 1000, 50))
    sol, _ = F.timeintegrate(Q.copy(order="F"), dg, eq, F.ORK256(williamson_condition=False), tf, dt=dt,
                             alias_u0=True, save_everystep=False, adaptive=False, callback=sb)
    m = F.ORK256()
    ref = oracle_for(dg).lsrk2n(Q, dt, int(round(tf / dt)), m.A, m.B, m.c)
    assert rel_linf(sol.u[-1], ref) <= 1e-10
    assert [os.path.basename(f) for f in sb.files] == ["solution_%010d.hdf" % i for i in (0, 50, 100)]
    assert abs(F.io.read_vtkhdf(sb.files[-1])["FieldData"]["Time"][0] - tf) < 1e-15
