"""Solution snapshots and restarts.

Reference: src/FlouSpatial/IO.jl:16-126 and src/FlouBiz/FlouBiz.jl:30-113 write VTKHDF files
(HDF5) with Lagrange cells on equispaced nodes (StdSegment.jl:56-58, vtk_connectivities of
StdQuad.jl:185-195 / StdHex.jl:174-196, vtk_type 68 / 70 / 72), the solution variables under
`variablenames`, the cell region and the time as field data.  `write_vtkhdf` writes the same
file: the /VTKHDF group with its Version and Type attributes, NumberOfPoints, Points,
NumberOfConnectivityIds, Connectivity, NumberOfCells, Types, Offsets, CellData/Region,
FieldData/Time and one PointData dataset per variable, through the HDF5 encoder of
`flou_cuda.hdf5` (no HDF5 library is needed).  `write_vtu` writes the same content as a VTK XML
UnstructuredGrid (.vtu).  A state on the device is resampled to the equispaced nodes on the
device before it is copied out.

Restart files hold the state bit for bit: a 64-byte header (magic, version, dim, nodes per
direction, elements, variables, DOFs, time, iteration, CRC-32 of the data) and the column-major
(ndofs, nvars) float64 state.
"""
import struct
import zlib

import numpy as np

from .std import interp_matrix


def variablenames(equation):
    """variablenames(eq) of src/FlouCommon/Euler.jl:33-54, LinearAdvection.jl:34-40, Burgers.jl:23-29."""
    if hasattr(equation, "gamma"):
        return {1: ("rho", "rhou", "rhoe"), 2: ("rho", "rhou", "rhov", "rhoe"),
                3: ("rho", "rhou", "rhov", "rhow", "rhoe")}[equation.dim]
    return ("u",)


# ---------------------------------------------------------------------------------------
# restart files
# ---------------------------------------------------------------------------------------
_MAGIC = b"FLOURST1"
_HEADER = struct.Struct("<8sIiiqiqdqI")   # 60 bytes, padded to 64


def _host_state(Q, disc):
    if hasattr(Q, "is_cuda"):
        x = Q.detach().cpu().numpy()
        if x.shape == (disc.nvariables, disc.ndofs):
            x = x.T
        return np.asfortranarray(x, dtype=np.float64)
    return np.asfortranarray(Q, dtype=np.float64)


def save_restart(path, disc, Q, time=0.0, iteration=0):
    """Writes Q (numpy (ndofs, nvars) or CUDA tensor (nvars, ndofs)) with its time and step."""
    q = _host_state(Q, disc)
    data = q.tobytes(order="F")
    hdr = _HEADER.pack(_MAGIC, 1, disc.mesh.dim, disc.std.n, disc.mesh.nelements, disc.nvariables, disc.ndofs,
                       float(time), int(iteration), zlib.crc32(data) & 0xFFFFFFFF)
    with open(path, "wb") as f:
        f.write(hdr.ljust(64, b"\0"))
        f.write(data)


def load_restart(path, disc=None):
    """(Q (ndofs, nvars) column-major, time, iteration); checks the sizes against `disc`."""
    with open(path, "rb") as f:
        hdr = f.read(64)
        data = f.read()
    magic, ver, dim, n, nelem, nvars, ndofs, t, it, crc = _HEADER.unpack(hdr[:_HEADER.size])
    if magic != _MAGIC or ver != 1:
        raise ValueError("%s is not a restart file of this format" % path)
    if len(data) != ndofs * nvars * 8 or (zlib.crc32(data) & 0xFFFFFFFF) != crc:
        raise ValueError("%s: the state is truncated or corrupted (CRC mismatch)" % path)
    if disc is not None and (dim, n, nelem, nvars, ndofs) != (disc.mesh.dim, disc.std.n, disc.mesh.nelements,
                                                              disc.nvariables, disc.ndofs):
        raise ValueError("%s was written for another discretization" % path)
    Q = np.frombuffer(data, dtype=np.float64).reshape((ndofs, nvars), order="F").copy(order="F")
    return Q, t, it


# ---------------------------------------------------------------------------------------
# VTK output
# ---------------------------------------------------------------------------------------
VTK_TYPE = {1: 68, 2: 70, 3: 72}   # Lagrange curve / quadrilateral / hexahedron


def vtk_connectivity(dim, n):
    """Local point order of a VTK Lagrange cell over an n^dim equispaced grid (x fastest):
    corners, then edge points, then face points, then interior points."""
    li = lambda *c: int(np.ravel_multi_index(c, (n,) * dim, order="F"))
    r = range(1, n - 1)
    if dim == 1:
        return [li(0), li(n - 1)] + [li(i) for i in r]
    if dim == 2:
        corners = [li(0, 0), li(n - 1, 0), li(n - 1, n - 1), li(0, n - 1)]
        edges = ([li(i, 0) for i in r] + [li(n - 1, j) for j in r] + [li(i, n - 1) for i in r] +
                 [li(0, j) for j in r])
        interior = [li(i, j) for j in r for i in r]
        return corners + edges + interior
    m = n - 1
    corners = [li(0, 0, 0), li(m, 0, 0), li(m, m, 0), li(0, m, 0), li(0, 0, m), li(m, 0, m), li(m, m, m), li(0, m, m)]
    edges = ([li(i, 0, 0) for i in r] + [li(m, j, 0) for j in r] + [li(i, m, 0) for i in r] + [li(0, j, 0) for j in r] +
             [li(i, 0, m) for i in r] + [li(m, j, m) for j in r] + [li(i, m, m) for i in r] + [li(0, j, m) for j in r] +
             [li(0, 0, k) for k in r] + [li(m, 0, k) for k in r] + [li(m, m, k) for k in r] + [li(0, m, k) for k in r])
    faces = ([li(0, j, k) for k in r for j in r] + [li(m, j, k) for k in r for j in r] +
             [li(i, 0, k) for k in r for i in r] + [li(i, m, k) for k in r for i in r] +
             [li(i, j, 0) for j in r for i in r] + [li(i, j, m) for j in r for i in r])
    interior = [li(i, j, k) for k in r for j in r for i in r]
    return corners + edges + faces + interior


def cell_connectivity(dim, n, ne):
    """The connectivity both writers store: element e's local points in VTK order, offset by
    e n^dim (IO.jl:45-46)."""
    local = np.array(vtk_connectivity(dim, n), dtype=np.int64)
    return (np.arange(ne, dtype=np.int64)[:, None] * n ** dim + local[None, :]).ravel()


def _equispaced_operator(disc):
    """Tensor-product interpolation from the solution nodes to n equispaced nodes per
    direction (StdSegment.jl:56-58: range(-1, 1, n))."""
    n, d = disc.std.n, disc.mesh.dim
    I1 = interp_matrix(np.linspace(-1.0, 1.0, n), disc.std.xi1d)   # (n, n)
    I = np.ones((1, 1))
    for _ in range(d):
        I = np.kron(I1, I)   # x fastest
    return I


def _project(disc, A, I):
    """A: (ndofs, k) host array or CUDA tensor (k, ndofs) -> (ndofs, k) host array at the
    equispaced nodes (element by element)."""
    npe, ne = disc.std.n ** disc.mesh.dim, disc.mesh.nelements
    if hasattr(A, "is_cuda"):
        import torch
        At = A.reshape(A.shape[0], ne, npe)
        It = torch.as_tensor(I, dtype=A.dtype, device=A.device)
        out = torch.einsum("ij,kej->kei", It, At).reshape(A.shape[0], ne * npe)
        return out.cpu().numpy().T
    A = np.asarray(A)
    return np.einsum("ij,ejk->eik", I, A.reshape(ne, npe, -1)).reshape(ne * npe, -1)


def write_vtu(path, disc, Q, time=None, names=None):
    """A snapshot of Q (numpy (ndofs, nvars) or a CUDA tensor (nvars, ndofs)) as a VTK XML
    UnstructuredGrid of Lagrange cells on equispaced nodes."""
    d, n = disc.mesh.dim, disc.std.n
    ne, npe = disc.mesh.nelements, n ** d
    I = _equispaced_operator(disc)
    pts = _project(disc, disc.coords, I)                # (ndofs, 3)
    vals = _project(disc, Q, I)                          # (ndofs, nvars)
    names = names or variablenames(disc.equation)
    conn = cell_connectivity(d, n, ne)
    offsets = np.arange(1, ne + 1, dtype=np.int64) * npe
    types = np.full(ne, VTK_TYPE[d], dtype=np.uint8)
    regions = np.ones(ne, dtype=np.int64)
    blocks = []

    def add(arr):
        off = sum(8 + len(b) for b in blocks)
        blocks.append(np.ascontiguousarray(arr).tobytes())
        return off

    fd = ""
    if time is not None:
        fd = ('<FieldData><DataArray type="Float64" Name="Time" NumberOfTuples="1" format="appended" '
              'offset="%d"/></FieldData>' % add(np.array([float(time)])))
    pd = "".join('<DataArray type="Float64" Name="%s" format="appended" offset="%d"/>' % (nm, add(vals[:, k]))
                 for k, nm in enumerate(names))
    xml = ('<?xml version="1.0"?>\n<VTKFile type="UnstructuredGrid" version="1.0" byte_order="LittleEndian" '
           'header_type="UInt64">\n<UnstructuredGrid>%s\n<Piece NumberOfPoints="%d" NumberOfCells="%d">\n'
           '<PointData>%s</PointData>\n<CellData><DataArray type="Int64" Name="Region" format="appended" '
           'offset="%d"/></CellData>\n<Points><DataArray type="Float64" NumberOfComponents="3" format="appended" '
           'offset="%d"/></Points>\n<Cells><DataArray type="Int64" Name="connectivity" format="appended" offset="%d"/>'
           '<DataArray type="Int64" Name="offsets" format="appended" offset="%d"/>'
           '<DataArray type="UInt8" Name="types" format="appended" offset="%d"/></Cells>\n</Piece>\n'
           '</UnstructuredGrid>\n<AppendedData encoding="raw">\n_' %
           (fd, ne * npe, ne, pd, add(regions), add(pts.astype(np.float64)), add(conn), add(offsets), add(types)))
    with open(path, "wb") as f:
        f.write(xml.encode())
        for b in blocks:
            f.write(struct.pack("<Q", len(b)))
            f.write(b)
        f.write(b"\n</AppendedData>\n</VTKFile>\n")


def read_vtu(path):
    """The arrays of a .vtu file written by write_vtu: {name: array} plus 'Points',
    'connectivity', 'offsets', 'types', and the piece sizes."""
    import re
    raw = open(path, "rb").read()
    head, _, rest = raw.partition(b'<AppendedData encoding="raw">\n_')
    text = head.decode()
    out = {}
    m = re.search(r'NumberOfPoints="(\d+)" NumberOfCells="(\d+)"', text)
    out["npoints"], out["ncells"] = int(m.group(1)), int(m.group(2))
    dt = {"Float64": np.float64, "Int64": np.int64, "UInt8": np.uint8}
    for tag in re.finditer(r'<DataArray type="(\w+)"(?: Name="(\w+)")?(?: NumberOfComponents="(\d+)")?'
                           r'(?: NumberOfTuples="\d+")? format="appended" offset="(\d+)"/>', text):
        typ, name, ncomp, off = tag.group(1), tag.group(2) or "Points", tag.group(3), int(tag.group(4))
        nb = struct.unpack("<Q", rest[off:off + 8])[0]
        arr = np.frombuffer(rest[off + 8:off + 8 + nb], dtype=dt[typ])
        out[name] = arr.reshape(-1, int(ncomp)) if ncomp else arr
    return out


def _snapshot_arrays(disc, Q):
    """Points (npoints, 3), values (npoints, nvars), connectivity, offsets (ncells + 1), types,
    regions of a snapshot, element by element as IO.jl:33-66 builds them."""
    d, n = disc.mesh.dim, disc.std.n
    ne, npe = disc.mesh.nelements, n ** d
    I = _equispaced_operator(disc)
    pts = _project(disc, disc.coords, I)
    if pts.shape[1] < 3:   # IO.jl pads the coordinates with zeros to three components
        pts = np.hstack([pts, np.zeros((pts.shape[0], 3 - pts.shape[1]))])
    vals = _project(disc, Q, I)
    conn = cell_connectivity(d, n, ne)
    offsets = np.arange(0, ne + 1, dtype=np.int64) * npe
    types = np.full(ne, VTK_TYPE[d], dtype=np.uint8)
    regions = np.asarray(getattr(disc.mesh, "regions", np.ones(ne)), dtype=np.int64)
    return np.ascontiguousarray(pts, dtype=np.float64), vals, conn, offsets, types, regions


def write_vtkhdf(path, disc, Q, time=None, names=None):
    """A snapshot of Q (numpy (ndofs, nvars) or a CUDA tensor (nvars, ndofs)) as the VTKHDF file
    Flou writes (open_for_write + add_fielddata!(file, [t], "Time") + add_solution!, IO.jl:16-126,
    FlouBiz.jl:38-113, FlouTime.jl:67-80)."""
    from . import hdf5
    pts, vals, conn, offsets, types, regions = _snapshot_arrays(disc, Q)
    names = names or variablenames(disc.equation)
    root = {
        "@attrs": {"Version": np.array([1, 0], dtype=np.int64), "Type": b"UnstructuredGrid"},
        "NumberOfPoints": np.array([pts.shape[0]], dtype=np.int64),
        "Points": pts,
        "NumberOfConnectivityIds": np.array([conn.size], dtype=np.int64),
        "Connectivity": conn,
        "NumberOfCells": np.array([types.size], dtype=np.int64),
        "Types": types,
        "Offsets": offsets,
        "CellData": {"Region": regions},
    }
    if time is not None:
        root["FieldData"] = {"Time": np.array([float(time)])}
    root["PointData"] = {nm: np.ascontiguousarray(vals[:, k]) for k, nm in enumerate(names)}
    hdf5.write(path, {"VTKHDF": root})


def read_vtkhdf(path):
    """The /VTKHDF group of a file written by write_vtkhdf, as a dict of numpy arrays."""
    from . import hdf5
    return hdf5.read(path)["VTKHDF"]
