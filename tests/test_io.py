"""Snapshots (VTK Lagrange cells on equispaced nodes, the content of Flou's VTKHDF writer,
src/FlouSpatial/IO.jl:16-126) and restart files."""
import os

import numpy as np
import pytest

import flou_cuda as F
from flou_cuda import io as fio
from cases import build, smooth_euler_state


def _disc(dim, n=4, unstructured=False):
    eq = F.EulerEquation(dim, 1.4)
    op = F.StrongDivOperator(F.LxF(F.StdAverage(), 1.0))
    if unstructured:
        mesh = F.perturbed_box(dim, 2, (0.0,) * dim, (1.0,) * dim, amp=0.1, seed=3)
        b = F.LagrangeBasis("GLL", n)
        std = {2: F.StdQuad, 3: F.StdHex}[dim](b, F.DGSEMrec(b), dim + 2)
        return F.MultielementDisc(mesh, std, eq, op, {k: F.EulerOutflowBC() for k in mesh.bdnames})
    return build(dim, n, (2,) * dim, eq, op)


def test_restart_round_trip(tmp_path):
    disc = _disc(2)
    Q = smooth_euler_state(disc, seed=1)
    p = str(tmp_path / "r.bin")
    fio.save_restart(p, disc, Q, time=0.25, iteration=17)
    R, t, it = fio.load_restart(p, disc)
    assert np.array_equal(R, Q) and t == 0.25 and it == 17
    raw = bytearray(open(p, "rb").read())
    raw[100] ^= 1                                      # flip one bit of the state
    open(p, "wb").write(bytes(raw))
    with pytest.raises(ValueError):
        fio.load_restart(p, disc)
    with pytest.raises(ValueError):
        fio.save_restart(p, disc, Q)
        fio.load_restart(p, _disc(2, n=5))


@pytest.mark.parametrize("dim,unstructured", [(1, False), (2, False), (3, False), (2, True), (3, True)])
def test_vtu_snapshot(tmp_path, dim, unstructured):
    disc = _disc(dim, unstructured=unstructured)
    n, npe, ne = disc.std.n, disc.std.n ** dim, disc.mesh.nelements
    # a state linear in the coordinates is reproduced exactly at the equispaced nodes
    X = disc.coords
    P = np.zeros((disc.ndofs, dim + 2))
    P[:, 0] = 1.0 + 0.1 * X[:, 0]
    P[:, -1] = 2.0
    Q = np.asfortranarray(disc.equation.vars_prim2cons(P))
    p = str(tmp_path / "s.vtu")
    fio.write_vtu(p, disc, Q, time=0.5)
    v = fio.read_vtu(p)
    assert v["npoints"] == ne * npe and v["ncells"] == ne
    assert set(fio.variablenames(disc.equation)) <= set(v)
    assert np.all(v["types"] == fio.VTK_TYPE[dim]) and v["Time"][0] == 0.5
    conn = v["connectivity"]
    assert len(conn) == ne * npe and conn.min() == 0 and conn.max() == ne * npe - 1
    assert np.array_equal(np.sort(conn), np.arange(ne * npe))
    assert np.array_equal(v["offsets"], np.arange(1, ne + 1) * npe)
    pts = v["Points"]
    assert np.allclose(v["rho"], 1.0 + 0.1 * pts[:, 0], atol=1e-13)
    # the first point of each cell is the element's first corner (an LGL node: unchanged)
    first = conn[::npe]
    assert np.allclose(pts[first, :dim], X[np.arange(ne) * npe, :dim], atol=1e-13)
    # equispaced: the second corner along x is n-1 spacings away
    if dim == 2 and not unstructured:
        c = conn[:npe]
        assert np.allclose(pts[c[1], 0] - pts[c[0], 0], disc.mesh.dx[0], atol=1e-13)


def test_vtk_point_order_lagrange_hexahedron():
    """VTK's Lagrange hexahedron: 8 corners, 12 edges, 6 faces (x-, x+, y-, y+, z-, z+), interior."""
    n = 4
    order = fio.vtk_connectivity(3, n)
    assert sorted(order) == list(range(n ** 3))
    coords = [np.unravel_index(i, (n,) * 3, order="F") for i in order]
    corners = {(0, 0, 0), (3, 0, 0), (3, 3, 0), (0, 3, 0), (0, 0, 3), (3, 0, 3), (3, 3, 3), (0, 3, 3)}
    assert {tuple(int(v) for v in c) for c in coords[:8]} == corners
    assert tuple(int(v) for v in coords[8]) == (1, 0, 0) and tuple(int(v) for v in coords[8 + 12 * 2]) == (0, 1, 1)
