"""Fault injection on the host: corrupted connectivity or non-Cartesian geometry is rejected by
the same validator flou_set_mesh / flou_set_geometry run, before anything reaches a GPU."""
import ctypes

import numpy as np
import pytest

import flou_cuda as F
from flou_cuda import _lib as L


def _mesh_args(disc):
    return {k: v for k, v in disc.abi_arrays().items() if v is not None}


def _check_mesh(dim, a):
    lib = F.load()
    buf = ctypes.create_string_buffer(256)
    i32 = lambda x: np.ascontiguousarray(x, dtype=np.int32).ctypes.data_as(L._I32)
    keep = [np.ascontiguousarray(a[k], dtype=np.int32) for k in ("faceinds", "facepos", "eleminds", "elempos",
                                                                  "bdface_index")]
    orient = np.ascontiguousarray(a["orientation"], dtype=np.uint8)
    st = lib.flou_check_mesh(dim, a["faceinds"].shape[0], a["eleminds"].shape[0],
                             *[k.ctypes.data_as(L._I32) for k in keep[:4]], orient.ctypes.data_as(L._U8),
                             keep[4].ctypes.data_as(L._I32), buf, 256)
    return st, buf.value.decode()


def _check_geom(dim, n, a, J=None, Ja=None, frames=None, faceJ=None):
    lib = F.load()
    buf = ctypes.create_string_buffer(256)
    ep = np.ascontiguousarray(a["elempos"], dtype=np.int32)
    arrs = [np.ascontiguousarray(x, dtype=np.float64) for x in
            (a["omega"], a["J"] if J is None else J, a["Ja"] if Ja is None else Ja,
             a["frames"] if frames is None else frames, a["faceJ"] if faceJ is None else faceJ)]
    st = lib.flou_check_geometry(dim, n, a["faceinds"].shape[0], a["eleminds"].shape[0], ep.ctypes.data_as(L._I32),
                                 *[x.ctypes.data_as(L._D) for x in arrs], buf, 256)
    return st, buf.value.decode()


def _disc(dim, periodic=True):
    eq = F.EulerEquation(dim, 1.4)
    mesh = F.CartesianMesh((0.0,) * dim, (1.0,) * dim, (3,) * dim)
    if periodic:
        for d in range(dim):
            F.apply_periodicBCs(mesh, (str(2 * d + 1), str(2 * d + 2)))
    b = F.LagrangeBasis("GLL", 4)
    std = {1: F.StdSegment, 2: F.StdQuad, 3: F.StdHex}[dim](b, F.DGSEMrec(b))
    bcs = {str(k): F.EulerSlipBC() for k in mesh.bdmap}
    return F.MultielementDisc(mesh, std, eq, F.StrongDivOperator(F.LxF(F.StdAverage(), 1.0)), bcs)


@pytest.mark.parametrize("dim", [1, 2, 3])
@pytest.mark.parametrize("periodic", [True, False])
def test_valid_setup_passes(dim, periodic):
    d = _disc(dim, periodic)
    a = _mesh_args(d)
    assert _check_mesh(dim, a) == (L.FLOU_OK, "")
    assert _check_geom(dim, 4, a) == (L.FLOU_OK, "")


def test_corrupted_connectivity_is_rejected():
    d = _disc(2, periodic=False)
    a = _mesh_args(d)
    b = {k: v.copy() for k, v in a.items()}
    b["faceinds"][4, 1] = b["faceinds"][4, 0]          # element 5 points at the wrong face
    st, msg = _check_mesh(2, b)
    assert st == L.FLOU_ERR_ARG and "face" in msg
    b = {k: v.copy() for k, v in a.items()}
    b["eleminds"][3, 0] = 999                             # element out of range
    st, msg = _check_mesh(2, b)
    assert st == L.FLOU_ERR_ARG and "out of range" in msg
    b = {k: v.copy() for k, v in a.items()}
    b["orientation"][2] = 4                               # a 2D face takes orientation 0 or 1
    st, msg = _check_mesh(2, b)
    assert st == L.FLOU_ERR_ARG and "orientation" in msg
    b = {k: v.copy() for k, v in a.items()}
    b["orientation"][2] = 1                               # reversed face: valid (general geometry)
    assert _check_mesh(2, b)[0] == L.FLOU_OK
    b = {k: v.copy() for k, v in a.items()}
    f = int(np.nonzero(b["eleminds"][:, 1] == 0)[0][0])
    b["bdface_index"][f] = 0                              # boundary face without a boundary
    st, msg = _check_mesh(2, b)
    assert st == L.FLOU_ERR_ARG and "boundary face" in msg
    b = {k: v.copy() for k, v in a.items()}
    f = int(np.nonzero(b["eleminds"][:, 1] != 0)[0][0])
    b["bdface_index"][f] = 1                              # interior face marked as boundary
    st, msg = _check_mesh(2, b)
    assert st == L.FLOU_ERR_ARG and "interior face" in msg


def test_geometry_validation():
    """General (curvilinear / unstructured) geometry is accepted; malformed geometry is not."""
    d = _disc(2)
    a = _mesh_args(d)
    Ja = a["Ja"].copy()
    Ja[5, 1] = 1e-3                                       # off-diagonal metric term
    assert _check_geom(2, 4, a, Ja=Ja)[0] == L.FLOU_OK
    J = a["J"].copy()
    J[17] *= 1.01                                         # Jacobian varies inside element 2
    assert _check_geom(2, 4, a, J=J)[0] == L.FLOU_OK
    fr = a["frames"].copy()
    fr[9, 0] = -fr[9, 0]                                  # another (unit) normal
    assert _check_geom(2, 4, a, frames=fr)[0] == L.FLOU_OK
    fr = a["frames"].copy()
    fr[9, 0] = 2.0 * fr[9, 0]                             # not a unit normal
    st, msg = _check_geom(2, 4, a, frames=fr)
    assert st == L.FLOU_ERR_ARG and "unit" in msg
    J = -a["J"]
    st, msg = _check_geom(2, 4, a, J=J)
    assert st == L.FLOU_ERR_ARG and "J <= 0" in msg
    fj = a["faceJ"].copy()
    fj[3] = 0.0
    st, msg = _check_geom(2, 4, a, faceJ=fj)
    assert st == L.FLOU_ERR_ARG and "surface Jacobian" in msg
