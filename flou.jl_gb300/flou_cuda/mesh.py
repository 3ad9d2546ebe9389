"""Structured Cartesian meshes, mirroring Flou's CartesianMesh and apply_periodicBCs!.

Reference: src/FlouCommon/CartesianMesh.jl (constructor :38-97, connectivities :152-500) and
src/FlouCommon/Mesh.jl:236-322 (periodic stitching).  The reference builds the faces of the
box, stitches each periodic pair, deletes the duplicate faces and renumbers everything.  Here
the final numbering is computed directly: the faces of one direction form a column-major
grid with one extra layer along that direction, the faces on the `bd2` side of a periodic
pair are dropped, and the kept faces keep their relative order.  The result is the same
1-based connectivity (checked bit-for-bit against the reference's procedure in the tests).
"""
import numpy as np


class CartesianMesh:
    """CartesianMesh{ND,Float64}(start, finish, nxyz)."""

    def __init__(self, start, finish, nxyz):
        start = np.atleast_1d(np.asarray(start, dtype=np.float64))
        finish = np.atleast_1d(np.asarray(finish, dtype=np.float64))
        nxyz = tuple(int(v) for v in np.atleast_1d(nxyz))
        nd = len(nxyz)
        if not 1 <= nd <= 3:
            raise ValueError("The mesh can only have 1, 2 or 3 dimensions.")
        if len(start) != nd or len(finish) != nd:
            raise ValueError("`start` and `finish` must have %d coordinates." % nd)
        if not np.all(start < finish):
            raise ValueError("All components of `start` must be lower than those of `finish`.")
        if any(v < 1 for v in nxyz):
            raise ValueError("At least one element per direction.")
        self.dim = nd
        self.nelements_dir = nxyz
        self.start = start
        self.finish = finish
        self.dx = (finish - start) / np.asarray(nxyz, dtype=np.float64)
        self.periodic = {}
        self._build()

    # -- connectivity -------------------------------------------------------------------
    def _face_shape(self, d):
        s = list(self.nelements_dir)
        s[d] += 1
        return tuple(s)

    def _build(self):
        nd, nx = self.dim, self.nelements_dir
        nelem = int(np.prod(nx))
        counts = [int(np.prod(self._face_shape(d))) for d in range(nd)]
        offs = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
        nfaces0 = int(offs[-1])
        per = [(2 * d + 1) in self.periodic for d in range(nd)]

        ec = np.array(np.unravel_index(np.arange(nelem), nx, order="F"))   # (nd, nelem)
        faceinds = np.zeros((nelem, 2 * nd), dtype=np.int64)
        facepos = np.zeros((nelem, 2 * nd), dtype=np.int64)
        eleminds = np.zeros((nfaces0, 2), dtype=np.int64)
        elempos = np.zeros((nfaces0, 2), dtype=np.int64)
        keep = np.ones(nfaces0, dtype=bool)
        bd_of = np.zeros(nfaces0, dtype=np.int64)   # boundary id (1..2nd) of boundary faces

        elem_id = lambda c: np.ravel_multi_index(tuple(c), nx, order="F") + 1
        for d in range(nd):
            shp = self._face_shape(d)
            fid = lambda c: offs[d] + np.ravel_multi_index(tuple(c), shp, order="F")
            # element faces
            left = fid(ec)
            cr = ec.copy()
            cr[d] += 1
            if per[d]:
                cr[d] = np.where(cr[d] == nx[d], 0, cr[d])
            right = fid(cr)
            faceinds[:, 2 * d] = left
            faceinds[:, 2 * d + 1] = right
            facepos[:, 2 * d] = np.where(ec[d] == 0, 1, 2)
            facepos[:, 2 * d + 1] = np.where(per[d] & (ec[d] == nx[d] - 1), 2, 1)
            # faces of direction d
            fc = np.array(np.unravel_index(np.arange(counts[d]), shp, order="F"))
            f = offs[d] + np.arange(counts[d])
            cd = fc[d]
            interior = (cd > 0) & (cd < nx[d])
            lo = cd == 0
            hi = cd == nx[d]
            cm = fc.copy()
            cm[d] = np.clip(cd - 1, 0, nx[d] - 1)
            cp = fc.copy()
            cp[d] = np.clip(cd, 0, nx[d] - 1)
            e_minus = elem_id(cm)
            e_plus = elem_id(cp)
            # interior: [elem(c - e_d) at position 2d+2, elem(c) at 2d+1]
            eleminds[f[interior], 0] = e_minus[interior]
            elempos[f[interior], 0] = 2 * d + 2
            eleminds[f[interior], 1] = e_plus[interior]
            elempos[f[interior], 1] = 2 * d + 1
            # low boundary: master = elem(c) at 2d+1; periodic slave = elem(c_d = n-1) at 2d+2
            eleminds[f[lo], 0] = e_plus[lo]
            elempos[f[lo], 0] = 2 * d + 1
            if per[d]:
                cw = fc.copy()
                cw[d] = nx[d] - 1
                e_wrap = elem_id(cw)
                eleminds[f[lo], 1] = e_wrap[lo]
                elempos[f[lo], 1] = 2 * d + 2
                keep[f[hi]] = False
            else:
                bd_of[f[lo]] = 2 * d + 1
                eleminds[f[hi], 0] = e_minus[hi]
                elempos[f[hi], 0] = 2 * d + 2
                bd_of[f[hi]] = 2 * d + 2

        newid = np.cumsum(keep).astype(np.int64)   # 1-based id of kept faces
        self.faceinds = newid[faceinds]
        self.facepos = facepos
        self.eleminds = eleminds[keep]
        self.elempos = elempos[keep]
        self.orientation = np.zeros(int(keep.sum()), dtype=np.uint8)
        bd = bd_of[keep]
        # remaining boundaries keep their original order; bdmap: id -> index
        remaining = [b for b in range(1, 2 * nd + 1) if not per[(b - 1) // 2]]
        self.bdmap = {b: i + 1 for i, b in enumerate(remaining)}
        self.bdnames = [str(b) for b in range(1, 2 * nd + 1)]
        self.bdfaces = [np.nonzero(bd == b)[0] + 1 for b in remaining]
        self.bdface_index = np.zeros(len(bd), dtype=np.int64)
        for b, i in self.bdmap.items():
            self.bdface_index[bd == b] = i
        self.intfaces = np.nonzero(self.eleminds[:, 1] != 0)[0] + 1

    # -- sizes --------------------------------------------------------------------------
    @property
    def nelements(self):
        return int(np.prod(self.nelements_dir))

    @property
    def nfaces(self):
        return len(self.orientation)

    @property
    def nboundaries(self):
        return len(self.bdfaces)

    def element_origin(self):
        """Lower corner of every element, (nelem, dim)."""
        ec = np.array(np.unravel_index(np.arange(self.nelements), self.nelements_dir, order="F")).T
        return self.start[None, :] + ec * self.dx[None, :]


def apply_periodicBCs(mesh, *pairs):
    """apply_periodicBCs!(mesh, "1" => "2", ...) (CartesianMesh.jl:127-150).

    Each pair is given as a tuple of boundary names, e.g. ("1", "2").
    """
    for p in pairs:
        a, b = p
        try:
            bd1, bd2 = int(a), int(b)
        except ValueError:
            raise ValueError("Boundary IDs must be integers.")
        nb = 2 * mesh.dim
        if not (1 <= bd1 <= nb and 1 <= bd2 <= nb):
            raise ValueError("Boundary IDs must be between 1 and %d." % nb)
        if not (bd2 % 2 == 0 and bd1 + 1 == bd2):
            raise ValueError("Boundaries %s and %s cannot be made periodic." % (a, b))
        if bd1 in mesh.periodic:
            raise ValueError("Boundaries %s and %s cannot be periodic." % (a, b))
        mesh.periodic[bd1] = bd2
    mesh._build()
    return None
