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


def test_lookup3_published_vectors():
    """The checksum HDF5 uses (Bob Jenkins' lookup3 hashlittle), against the test vectors printed
    by lookup3.c's own driver."""
    from flou_cuda.hdf5 import lookup3
    assert lookup3(b"") == 0xDEADBEEF
    assert lookup3(b"Four score and seven years ago") == 0x17770551
    assert lookup3(b"Four score and seven years ago", 1) == 0xCD628161


@pytest.mark.parametrize("dim,unstructured", [(1, False), (2, False), (3, False), (3, True)])
def test_vtkhdf_snapshot_has_flous_layout(tmp_path, dim, unstructured):
    """write_vtkhdf writes the groups, datasets and attributes of Flou's VTKHDF writer
    (IO.jl:16-126, FlouBiz.jl:38-113, FlouTime.jl:70-75), read back with the same encoder."""
    disc = _disc(dim, unstructured=unstructured)
    npe, ne = disc.std.n ** dim, disc.mesh.nelements
    X = disc.coords
    P = np.zeros((disc.ndofs, dim + 2))
    P[:, 0] = 1.0 + 0.1 * X[:, 0]
    P[:, -1] = 2.0
    Q = np.asfortranarray(disc.equation.vars_prim2cons(P))
    p = str(tmp_path / "s.hdf")
    fio.write_vtkhdf(p, disc, Q, time=0.5)
    v = fio.read_vtkhdf(p)
    assert set(v) == {"@attrs", "NumberOfPoints", "Points", "NumberOfConnectivityIds", "Connectivity",
                      "NumberOfCells", "Types", "Offsets", "CellData", "FieldData", "PointData"}
    assert list(v["@attrs"]["Version"]) == [1, 0] and v["@attrs"]["Type"] == b"UnstructuredGrid"
    assert v["NumberOfPoints"].tolist() == [ne * npe] and v["NumberOfCells"].tolist() == [ne]
    assert v["Points"].shape == (ne * npe, 3) and v["Points"].dtype == np.float64
    assert np.all(v["Points"][:, dim:] == 0.0)
    assert v["NumberOfConnectivityIds"].tolist() == [ne * npe]
    assert np.array_equal(v["Connectivity"], fio.cell_connectivity(dim, disc.std.n, ne))
    assert np.array_equal(v["Offsets"], np.arange(ne + 1) * npe)
    assert v["Types"].dtype == np.uint8 and np.all(v["Types"] == fio.VTK_TYPE[dim])
    assert v["CellData"]["Region"].tolist() == [1] * ne
    assert v["FieldData"]["Time"].tolist() == [0.5]
    assert tuple(v["PointData"]) == fio.variablenames(disc.equation)
    assert np.allclose(v["PointData"]["rho"], 1.0 + 0.1 * v["Points"][:, 0], atol=1e-13)
    # the same values as the .vtu writer
    q = str(tmp_path / "s.vtu")
    fio.write_vtu(q, disc, Q, time=0.5)
    u = fio.read_vtu(q)
    for name in fio.variablenames(disc.equation):
        assert np.array_equal(u[name], v["PointData"][name])
    assert np.array_equal(u["Points"], v["Points"])


def test_hdf5_encoder_structure_and_checksums(tmp_path):
    """Superblock version 2 and version-2 object headers: the signature, the end-of-file address,
    and every checksum are checked on reading; one flipped byte anywhere in a header is caught."""
    from flou_cuda import hdf5
    p = str(tmp_path / "t.h5")
    tree = {"@attrs": {"a": np.array([3], dtype=np.int64)},
            "g": {"x": np.arange(5, dtype=np.float64), "s": {"y": np.array([7, 8], dtype=np.uint8)}},
            "m": np.arange(6, dtype=np.int64).reshape(2, 3)}
    hdf5.write(p, tree)
    raw = open(p, "rb").read()
    assert raw[:8] == b"\x89HDF\r\n\x1a\n" and raw[8] == 2
    import struct
    assert struct.unpack_from("<Q", raw, 28)[0] == len(raw)          # end-of-file address
    back = hdf5.read(p)
    assert back["@attrs"]["a"].tolist() == [3]
    assert back["g"]["x"].tolist() == list(range(5)) and back["g"]["s"]["y"].tolist() == [7, 8]
    assert back["m"].shape == (2, 3) and back["m"].tolist() == [[0, 1, 2], [3, 4, 5]]
    for at in (20, raw.index(b"OHDR") + 10, raw.rindex(b"OHDR") + 12):
        bad = bytearray(raw)
        bad[at] ^= 0x40
        open(p, "wb").write(bytes(bad))
        with pytest.raises(ValueError):
            hdf5.read(p)
