"""Unstructured straight-sided meshes (lines, quadrilaterals, hexahedra) and their geometry.

Reference: src/FlouCommon/GmshMesh.jl:16-394 (UnstructuredMesh, face maps and orientations),
src/FlouCommon/Mesh.jl:331-487 (linear element mappings, their main and dual bases and
Jacobians) and src/FlouSpatial/PhysicalRegions.jl:438-472 and :756-971 (per-node Jacobian and
metric, per-face-node frame and surface Jacobian).

The reference reads meshes through the Gmsh SDK and numbers the faces with Gmsh's internal
edge/face tags.  Here a mesh comes from node coordinates and element node lists (or a Gmsh .msh
ASCII file, formats 2.2 and 4.1); faces are numbered in order of first appearance while visiting
each element's faces in Gmsh's order, which gives the same master/slave sides as the reference
(the first element that visits a face is its master) with another face numbering.
"""
import itertools

import numpy as np

# Local nodes of each element face (Flou's face positions 1..2d), in the order of the face's
# parametric coordinates on that element: the face-dof order of the face's master.
FACE_NODES = {
    1: ((0,), (1,)),
    2: ((0, 3), (1, 2), (0, 1), (3, 2)),
    3: ((0, 3, 7, 4), (1, 2, 6, 5), (0, 1, 5, 4), (3, 2, 6, 7), (0, 1, 2, 3), (4, 5, 6, 7)),
}
# Order in which an element's faces are visited (Gmsh's edge / face order, GmshMesh.jl:286-295
# and :342-351 map them to Flou's positions).
VISIT = {1: (1, 2), 2: (3, 2, 4, 1), 3: (5, 3, 1, 2, 4, 6)}
# Reference-element corners of the local nodes (Gmsh numbering).
CORNERS = {
    1: ((-1,), (1,)),
    2: ((-1, -1), (1, -1), (1, 1), (-1, 1)),
    3: ((-1, -1, -1), (1, -1, -1), (1, 1, -1), (-1, 1, -1), (-1, -1, 1), (1, -1, 1), (1, 1, 1), (-1, 1, 1)),
}


def master2slave_quad(i, orientation, n):
    """master2slave of a quadrilateral face (StdQuad.jl:161-181), 0-based face dofs, x fastest."""
    m1, m2 = i % n, i // n
    li = lambda a, b: a + n * b
    return {0: i, 1: li(m2, n - 1 - m1), 2: li(n - 1 - m1, n - 1 - m2), 3: li(n - 1 - m2, m1),
            4: li(m2, m1), 5: li(n - 1 - m1, m2), 6: li(n - 1 - m2, n - 1 - m1), 7: li(m1, n - 1 - m2)}[orientation]


_CORNER_DOF = (0, 1, 3, 2)   # face corners (-,-), (+,-), (+,+), (-,+) as dofs of a 2x2 face


def _orientation_3d(master, slave):
    """The orientation code whose master2slave (StdQuad.jl:161-181) sends every corner of the
    master's face-node list onto the same mesh node in the slave's list.  GmshMesh.jl:362-389
    derives the code from the positions of the master's first two nodes in the slave's list; for
    the two quarter turns its table gives code 1 where master2slave's code-1 mapping describes the
    other quarter turn (and 3 for 1), so the code is taken from master2slave itself here."""
    for o in range(8):
        if all(slave[_CORNER_DOF.index(master2slave_quad(_CORNER_DOF[k], o, 2))] == master[k] for k in range(4)):
            return o
    raise ValueError("faces %s and %s do not match" % (master, slave))


class UnstructuredMesh:
    """UnstructuredMesh{ND,Float64}(nodes, elements, boundaries).

    nodes: (npoints, dim) coordinates; elements: (nelem, 2^dim) 0-based node indices in Gmsh's
    local order; boundaries: {name: iterable of boundary faces, each given by its node indices}.
    Every face with a single element must belong to exactly one named boundary.
    """

    def __init__(self, nodes, elements, boundaries):
        nodes = np.asarray(nodes, dtype=np.float64)
        if nodes.ndim == 1:
            nodes = nodes[:, None]
        elements = np.asarray(elements, dtype=np.int64)
        dim = nodes.shape[1]
        if dim not in (1, 2, 3) or elements.shape[1] != 2 ** dim:
            raise ValueError("elements must be lines (1D), quadrilaterals (2D) or hexahedra (3D) with 2^dim nodes")
        self.dim = dim
        self.nodes = nodes
        self.elements = elements
        nelem = elements.shape[0]
        key2face = {}
        face_nodes, eleminds, elempos, orient = [], [], [], []
        faceinds = np.zeros((nelem, 2 * dim), dtype=np.int64)
        facepos = np.zeros((nelem, 2 * dim), dtype=np.int64)
        for e in range(nelem):
            for pos in VISIT[dim]:
                fn = tuple(int(elements[e, k]) for k in FACE_NODES[dim][pos - 1])
                key = tuple(sorted(fn))
                f = key2face.get(key)
                if f is None:
                    f = len(face_nodes)
                    key2face[key] = f
                    face_nodes.append(fn)
                    eleminds.append([e + 1, 0])
                    elempos.append([pos, 0])
                    orient.append(0)
                    side = 1
                else:
                    if eleminds[f][1] != 0:
                        raise ValueError("face %s is shared by more than two elements" % (key,))
                    eleminds[f][1] = e + 1
                    elempos[f][1] = pos
                    master = face_nodes[f]
                    if dim == 2:
                        orient[f] = 0 if fn[0] == master[0] else 1
                    elif dim == 3:
                        orient[f] = _orientation_3d(master, fn)
                    side = 2
                faceinds[e, pos - 1] = f + 1
                facepos[e, pos - 1] = side
        self.faceinds = faceinds
        self.facepos = facepos
        self.eleminds = np.array(eleminds, dtype=np.int64)
        self.elempos = np.array(elempos, dtype=np.int64)
        self.orientation = np.array(orient, dtype=np.uint8)
        self.face_nodes = face_nodes
        self.intfaces = np.nonzero(self.eleminds[:, 1] != 0)[0] + 1
        # boundaries
        self.bdnames = [str(k) for k in boundaries]
        self.bdface_index = np.zeros(len(face_nodes), dtype=np.int64)
        self.bdfaces = []
        for b, name in enumerate(self.bdnames):
            fl = []
            for fn in boundaries[name if name in boundaries else int(name)]:
                key = tuple(sorted(int(v) for v in fn))
                f = key2face.get(key)
                if f is None or self.eleminds[f, 1] != 0:
                    raise ValueError("boundary '%s': %s is not a boundary face of the mesh" % (name, key))
                if self.bdface_index[f]:
                    raise ValueError("face %d belongs to two boundaries" % (f + 1))
                self.bdface_index[f] = b + 1
                fl.append(f + 1)
            self.bdfaces.append(np.array(sorted(fl), dtype=np.int64))
        orphan = np.nonzero((self.eleminds[:, 1] == 0) & (self.bdface_index == 0))[0]
        if len(orphan):
            raise ValueError("%d boundary faces belong to no named boundary (first: face %d)" %
                             (len(orphan), orphan[0] + 1))
        self.bdmap = {i + 1: i + 1 for i in range(len(self.bdnames))}
        self.periodic = {}

    @property
    def nelements(self):
        return self.elements.shape[0]

    @property
    def nfaces(self):
        return len(self.face_nodes)

    @property
    def nboundaries(self):
        return len(self.bdnames)

    def boundary_index(self, key):
        """1-based index of the boundary called `key`."""
        return self.bdnames.index(str(key)) + 1

    @property
    def start(self):
        return self.nodes.min(axis=0)

    @property
    def finish(self):
        return self.nodes.max(axis=0)

    # -- Gmsh files ----------------------------------------------------------------------
    @classmethod
    def from_gmsh(cls, filename, dim):
        """Linear quadrilaterals (2D) / hexahedra (3D) / lines (1D) and the physical groups of
        dimension dim-1 as named boundaries, from a Gmsh .msh ASCII file (format 2.2 or 4.1)."""
        return cls(*read_gmsh(filename, dim))


# ---------------------------------------------------------------------------------------
# Gmsh .msh ASCII (2.2 and 4.1)
# ---------------------------------------------------------------------------------------
_GMSH_TYPE = {1: (1, 2), 3: (2, 4), 5: (3, 8), 15: (0, 1)}   # type -> (dimension, nodes)


def _sections(text):
    out = {}
    lines = text.splitlines()
    i = 0
    while i < len(lines):
        s = lines[i].strip()
        if s.startswith("$") and not s.startswith("$End"):
            name = s[1:]
            j = i + 1
            while not lines[j].strip().startswith("$End" + name):
                j += 1
            out[name] = lines[i + 1:j]
            i = j
        i += 1
    return out


def read_gmsh(filename, dim):
    sec = _sections(open(filename).read())
    version = float(sec["MeshFormat"][0].split()[0])
    phys_names = {}
    for ln in sec.get("PhysicalNames", [])[1:]:
        parts = ln.split(maxsplit=2)
        phys_names[(int(parts[0]), int(parts[1]))] = parts[2].strip().strip('"')
    node_id = {}
    coords = []
    elems = []          # (gmsh type, physical tag, node tags)
    if version < 3:
        nl = sec["Nodes"]
        for ln in nl[1:1 + int(nl[0])]:
            p = ln.split()
            node_id[int(p[0])] = len(coords)
            coords.append([float(v) for v in p[1:4]])
        el = sec["Elements"]
        for ln in el[1:1 + int(el[0])]:
            p = [int(v) for v in ln.split()]
            etype, ntags = p[1], p[2]
            tags = p[3:3 + ntags]
            elems.append((etype, tags[0] if tags else 0, p[3 + ntags:]))
    else:
        ent_phys = {}
        if "Entities" in sec:
            en = sec["Entities"]
            counts = [int(v) for v in en[0].split()]
            row = 1
            for d, cnt in enumerate(counts):
                for _ in range(cnt):
                    p = en[row].split()
                    row += 1
                    tag = int(p[0])
                    if d == 0:
                        nphys = int(p[4])
                        phys = [int(v) for v in p[5:5 + nphys]]
                    else:
                        nphys = int(p[7])
                        phys = [int(v) for v in p[8:8 + nphys]]
                    ent_phys[(d, tag)] = phys[0] if phys else 0
        nl = sec["Nodes"]
        nblocks = int(nl[0].split()[0])
        row = 1
        for _ in range(nblocks):
            p = nl[row].split()
            row += 1
            nn = int(p[3])
            tags = [int(nl[row + k]) for k in range(nn)]
            row += nn
            for k in range(nn):
                node_id[tags[k]] = len(coords)
                coords.append([float(v) for v in nl[row + k].split()[:3]])
            row += nn
        el = sec["Elements"]
        nblocks = int(el[0].split()[0])
        row = 1
        for _ in range(nblocks):
            p = [int(v) for v in el[row].split()]
            row += 1
            edim, etag, etype, ne = p
            phys = ent_phys.get((edim, etag), 0)
            for k in range(ne):
                q = [int(v) for v in el[row + k].split()]
                elems.append((etype, phys, q[1:]))
            row += ne
    coords = np.array(coords)[:, :dim]
    cells = [e for e in elems if e[0] in _GMSH_TYPE and _GMSH_TYPE[e[0]][0] == dim]
    types = {e[0] for e in cells}
    if len(types) != 1:
        raise ValueError("Hybrid meshes are not supported." if types else "no %dD elements" % dim)
    used = sorted({node_id[t] for e in cells for t in e[2]})
    remap = {old: new for new, old in enumerate(used)}
    elements = np.array([[remap[node_id[t]] for t in e[2]] for e in cells], dtype=np.int64)
    # boundaries in the order of their physical tags, as gmsh.model.get_physical_groups lists
    # them to the reference's reader (GmshMesh.jl:112-126)
    groups = {}
    for etype, phys, tags in elems:
        if etype in _GMSH_TYPE and _GMSH_TYPE[etype][0] == dim - 1 and phys:
            groups.setdefault(phys, []).append(tuple(remap[node_id[t]] for t in tags))
    boundaries = {phys_names.get((dim - 1, tag), str(tag)): groups[tag] for tag in sorted(groups)}
    return coords[used], elements, boundaries


def write_gmsh22(filename, mesh):
    """Writes a mesh (nodes, elements, named boundaries) as a Gmsh 2.2 ASCII file."""
    dim = mesh.dim
    etype = {1: 1, 2: 3, 3: 5}[dim]
    btype = {1: 15, 2: 1, 3: 3}[dim]
    with open(filename, "w") as f:
        f.write("$MeshFormat\n2.2 0 8\n$EndMeshFormat\n$PhysicalNames\n%d\n" % (mesh.nboundaries + 1))
        for b, name in enumerate(mesh.bdnames):
            f.write('%d %d "%s"\n' % (dim - 1, b + 1, name))
        f.write('%d %d "domain"\n$EndPhysicalNames\n' % (dim, mesh.nboundaries + 1))
        f.write("$Nodes\n%d\n" % len(mesh.nodes))
        for i, x in enumerate(mesh.nodes):
            xyz = list(x) + [0.0] * (3 - dim)
            f.write("%d %.17g %.17g %.17g\n" % (i + 1, xyz[0], xyz[1], xyz[2]))
        f.write("$EndNodes\n$Elements\n")
        rows = []
        for b in range(mesh.nboundaries):
            for fidx in mesh.bdfaces[b]:
                rows.append((btype, b + 1, [v + 1 for v in mesh.face_nodes[fidx - 1]]))
        for e in mesh.elements:
            rows.append((etype, mesh.nboundaries + 1, [v + 1 for v in e]))
        f.write("%d\n" % len(rows))
        for k, (t, ph, nd) in enumerate(rows):
            f.write("%d %d 2 %d %d %s\n" % (k + 1, t, ph, ph, " ".join(str(v) for v in nd)))
        f.write("$EndElements\n")


# ---------------------------------------------------------------------------------------
# Test meshes: a box with smoothly displaced interior nodes and randomly rotated elements
# ---------------------------------------------------------------------------------------
def _cube_rotations(dim):
    """Permutations of the local nodes that rotate the reference element (orientation kept)."""
    corners = [np.array(c) for c in CORNERS[dim]]
    index = {tuple(c): k for k, c in enumerate(corners)}
    if dim == 1:
        return [tuple(range(2))]
    if dim == 2:
        gens = [np.array([[0, -1], [1, 0]])]
    else:
        gens = [np.array([[1, 0, 0], [0, 0, -1], [0, 1, 0]]), np.array([[0, -1, 0], [1, 0, 0], [0, 0, 1]])]
    group = {tuple(np.eye(dim, dtype=int).ravel())}
    frontier = [np.eye(dim, dtype=int)]
    while frontier:
        R = frontier.pop()
        for G in gens:
            M = G @ R
            k = tuple(M.ravel())
            if k not in group:
                group.add(k)
                frontier.append(M)
    perms = []
    for k in sorted(group):
        R = np.array(k).reshape(dim, dim)
        perms.append(tuple(index[tuple(R @ c)] for c in corners))
    return perms


def perturbed_box(dim, nel, start, finish, amp=0.1, seed=0, rotate=True):
    """A box of nel^dim straight-sided elements whose interior nodes are displaced by a smooth
    field of relative amplitude `amp`, each element's local numbering rotated at random.
    Boundaries "1".."2d" are the x-, x+, y-, y+, z-, z+ sides (CartesianMesh's names)."""
    rng = np.random.default_rng(seed)
    nel = tuple(int(v) for v in (nel if np.ndim(nel) else (nel,) * dim))
    start = np.asarray(start, dtype=np.float64)
    finish = np.asarray(finish, dtype=np.float64)
    npts = tuple(v + 1 for v in nel)
    idx = np.array(np.unravel_index(np.arange(int(np.prod(npts))), npts, order="F")).T   # (npts, dim)
    h = (finish - start) / np.array(nel)
    X = start + idx * h
    interior = np.all((idx > 0) & (idx < np.array(nel)), axis=1)
    L = finish - start
    disp = np.zeros_like(X)
    ph = rng.uniform(0, 2 * np.pi, size=(dim, dim))
    for k in range(dim):
        w = np.ones(len(X))
        for q in range(dim):
            w = w * np.sin(2 * np.pi * (X[:, q] - start[q]) / L[q] + ph[k, q])
        disp[:, k] = amp * h[k] * w
    X = X + np.where(interior[:, None], disp, 0.0)
    node = lambda c: int(np.ravel_multi_index(tuple(c), npts, order="F"))
    eidx = np.array(np.unravel_index(np.arange(int(np.prod(nel))), nel, order="F")).T
    corners = [(np.array(c) + 1) // 2 for c in CORNERS[dim]]
    elements = np.array([[node(ec + c) for c in corners] for ec in eidx], dtype=np.int64)
    if rotate:
        perms = _cube_rotations(dim)
        for e in range(len(elements)):
            p = perms[rng.integers(len(perms))]
            elements[e] = elements[e][list(p)]
    boundaries = {}
    for d in range(dim):
        for side, val in ((0, 0), (1, nel[d])):
            faces = []
            others = [q for q in range(dim) if q != d]
            for c in itertools.product(*[range(nel[q]) for q in others]):
                base = np.zeros(dim, dtype=int)
                base[d] = val
                for q, v in zip(others, c):
                    base[q] = v
                fn = []
                for off in itertools.product((0, 1), repeat=dim - 1):
                    p = base.copy()
                    for q, o in zip(others, off):
                        p[q] += o
                    fn.append(node(p))
                faces.append(tuple(fn))
            boundaries[str(2 * d + side + 1)] = faces
    return UnstructuredMesh(X, elements, boundaries)


# ---------------------------------------------------------------------------------------
# Geometry of the linear mappings (Mesh.jl:380-487, PhysicalRegions.jl:438-472, 756-971)
# ---------------------------------------------------------------------------------------
def _main_basis(dim, P, r):
    """d x / d ξ_k of the linear map at relative coordinates r = (ξ+1)/2 (Mesh.jl:386-475).
    P: corner coordinates, P[k] of shape (..., dim) (vectorised over elements)."""
    if dim == 1:
        return [(P[1] - P[0]) / 2]
    if dim == 2:
        x, y = r
        return [(P[1] - P[0]) / 2 * (1 - y) + (P[2] - P[3]) / 2 * y,
                (P[3] - P[0]) / 2 * (1 - x) + (P[2] - P[1]) / 2 * x]
    x, y, z = r
    a = (1 - z) * ((P[1] - P[0]) / 2 * (1 - y) + (P[2] - P[3]) / 2 * y) + \
        z * ((P[5] - P[4]) / 2 * (1 - y) + (P[6] - P[7]) / 2 * y)
    b = (1 - x) * ((P[3] - P[0]) / 2 * (1 - z) + (P[7] - P[4]) / 2 * z) + \
        x * ((P[2] - P[1]) / 2 * (1 - z) + (P[6] - P[5]) / 2 * z)
    c = (1 - y) * ((P[4] - P[0]) / 2 * (1 - x) + (P[5] - P[1]) / 2 * x) + \
        y * ((P[7] - P[3]) / 2 * (1 - x) + (P[6] - P[2]) / 2 * x)
    return [a, b, c]


def _dual_basis(dim, main):
    """Mesh.jl:391-394, 423-428, 477-483: J ∇ξ_k of the linear map."""
    if dim == 1:
        return [np.ones_like(main[0])]
    if dim == 2:
        return [np.stack([main[1][..., 1], -main[1][..., 0]], -1), np.stack([-main[0][..., 1], main[0][..., 0]], -1)]
    return [np.cross(main[1], main[2]), np.cross(main[2], main[0]), np.cross(main[0], main[1])]


def _jacobian(dim, main):
    """Mesh.jl:396-398, 430-432, 485-487."""
    if dim == 1:
        return main[0][..., 0]
    if dim == 2:
        return main[0][..., 0] * main[1][..., 1] - main[0][..., 1] * main[1][..., 0]
    return np.einsum("...k,...k->...", main[0], np.cross(main[1], main[2]))


def _phys(dim, P, r):
    out = 0.0
    for c, Pk in zip(CORNERS[dim], P):
        v = 1.0
        for q in range(dim):
            v = v * (r[q] if c[q] > 0 else (1 - r[q]))
        out = out + v * Pk
    return out


def unstructured_geometry(mesh, std):
    """Per-node J and metric (columns = dual basis), per-face-node frame (n, t, b) and surface
    Jacobian (master side), and node coordinates of an UnstructuredMesh
    (PhysicalRegions.jl:438-472, 756-971); vectorised over elements and faces."""
    d, n = mesh.dim, std.n
    xi = std.xi1d
    npe, nfd = n ** d, n ** (d - 1)
    ne, nf = mesh.nelements, mesh.nfaces
    P = [mesh.nodes[mesh.elements[:, k]] for k in range(2 ** d)]   # each (ne, d)
    J = np.zeros((ne, npe))
    Ja = np.zeros((ne, npe, d * d))
    coords = np.zeros((ne, npe, 3))
    loc = np.array(np.unravel_index(np.arange(npe), (n,) * d, order="F")).T   # x fastest
    for i in range(npe):
        r = [(xi[loc[i, q]] + 1) / 2 for q in range(d)]
        main = _main_basis(d, P, r)
        dual = _dual_basis(d, main)
        jac = _jacobian(d, main)
        if d < 3:
            jac = np.abs(jac)
        elif not np.all(jac > 0):
            raise ValueError("Found a negative Jacobian in element %d." % (int(np.argmin(jac > 0)) + 1))
        J[:, i] = jac
        Ja[:, i, :] = np.concatenate(dual, axis=-1)    # column-major: column k = dual[k]
        coords[:, i, :d] = _phys(d, P, r)
    frames = np.zeros((nf, nfd, 9))
    faceJ = np.zeros((nf, nfd))
    floc = np.array(np.unravel_index(np.arange(nfd), (n,) * (d - 1), order="F")).T if d > 1 else np.zeros((1, 0), int)
    me = mesh.eleminds[:, 0] - 1
    mpos = mesh.elempos[:, 0]
    tsign2 = {1: -1.0, 2: 1.0, 3: 1.0, 4: -1.0}
    tax3 = {1: 1, 2: 1, 3: 2, 4: 2, 5: 0, 6: 0}
    for pos in range(1, 2 * d + 1):
        fs = np.nonzero(mpos == pos)[0]
        if len(fs) == 0:
            continue
        Pf = [Pk[me[fs]] for Pk in P]
        ax = (pos - 1) // 2
        sgn = -1.0 if pos % 2 == 1 else 1.0
        tang = [q for q in range(d) if q != ax]
        for m in range(nfd):
            xi_e = [0.0] * d
            xi_e[ax] = sgn
            for k, q in enumerate(tang):
                xi_e[q] = xi[floc[m, k]]
            r = [(v + 1) / 2 for v in xi_e]
            main = _main_basis(d, Pf, r)
            dual = _dual_basis(d, main)
            out = np.zeros((len(fs), 9))
            if d == 1:
                s = np.sign(_jacobian(d, main))[:, None]
                nv = sgn * dual[0] * s
            elif d == 2:
                # PhysicalRegions.jl:797-871: n = ±dual[ax] s, t = ±normalize(main[other]) s
                s = np.sign(_jacobian(d, main))[:, None]
                nv = sgn * dual[ax] * s
                mo = main[1 - ax]
                out[:, 3:5] = tsign2[pos] * mo / np.linalg.norm(mo, axis=1)[:, None] * s
            else:
                # PhysicalRegions.jl:873-971: n = ±dual[ax], t = ±normalize(main[next]), b = n × t
                nv = sgn * dual[ax]
                mt = main[tax3[pos]]
                tv = sgn * mt / np.linalg.norm(mt, axis=1)[:, None]
                bv = np.cross(nv, tv)
                out[:, 3:6] = tv
                out[:, 6:9] = bv / np.linalg.norm(bv, axis=1)[:, None]
            jac = np.linalg.norm(nv, axis=1)
            out[:, :d] = nv / jac[:, None]
            frames[fs, m] = out
            faceJ[fs, m] = jac
    return (J.ravel(), Ja.reshape(ne * npe, d * d), frames.reshape(nf * nfd, 9), faceJ.ravel(),
            coords.reshape(ne * npe, 3))


def subgrid_points(omega):
    """The n + 1 subcell interfaces of one direction (StdSegment.jl:60-73): the running sums of the
    weights from both ends, averaged, with the ends at exactly -1 and 1."""
    n = len(omega)
    a = np.empty(n + 1)
    b = np.empty(n + 1)
    a[0], b[n] = -1.0, 1.0
    for i in range(n):
        a[i + 1] = a[i] + omega[i]
    for i in range(n - 1, -1, -1):
        b[i] = b[i + 1] - omega[i]
    c = (a + b) / 2
    c[0], c[n] = -1.0, 1.0
    return c


def unstructured_subgrid(mesh, std):
    """Frames (n, t, b) and surface Jacobians of the subcell interfaces of every element of an
    UnstructuredMesh (PhysicalRegions.jl:180-300), the geometry the hybrid operator's subcell
    finite-volume fluxes use: for direction d, line m (the face-dof order of a face normal to d)
    and interface s = 0..n, the point with ξ_d = ξc[s] and the line's node coordinates on the other
    axes.  Returns frames (nelem, d, n^(d-1), n + 1, 9) and jac (nelem, d, n^(d-1), n + 1)."""
    d, n = mesh.dim, std.n
    xi, xc = std.xi1d, subgrid_points(std.omega1d)
    ne, nfd = mesh.nelements, n ** (d - 1)
    P = [mesh.nodes[mesh.elements[:, k]] for k in range(2 ** d)]
    frames = np.zeros((ne, d, nfd, n + 1, 9))
    jac = np.zeros((ne, d, nfd, n + 1))
    for ax in range(d):
        others = [q for q in range(d) if q != ax]
        for m in range(nfd):
            rest = np.unravel_index(m, (n,) * (d - 1), order="F") if d > 1 else ()
            for s in range(n + 1):
                pt = [0.0] * d
                pt[ax] = xc[s]
                for k, q in enumerate(others):
                    pt[q] = xi[rest[k]]
                main = _main_basis(d, P, [(v + 1) / 2 for v in pt])
                dual = _dual_basis(d, main)
                out = np.zeros((ne, 9))
                if d == 1:
                    sg = np.sign(_jacobian(d, main))[:, None]
                    nv = sg * dual[0][:, None] if dual[0].ndim == 1 else sg * dual[0]
                    jv = np.ones(ne)
                    out[:, :1] = nv
                elif d == 2:
                    sg = np.sign(_jacobian(d, main))[:, None]
                    nv = sg * dual[ax]
                    mo = main[1 - ax]
                    out[:, 3:5] = (1.0 if ax == 0 else -1.0) * sg * mo / np.linalg.norm(mo, axis=1)[:, None]
                    jv = np.linalg.norm(nv, axis=1)
                    out[:, :2] = nv / jv[:, None]
                else:
                    nv = dual[ax]
                    mt = main[(ax + 1) % 3]
                    tv = mt / np.linalg.norm(mt, axis=1)[:, None]
                    bv = np.cross(nv, tv)
                    jv = np.linalg.norm(nv, axis=1)
                    out[:, :3] = nv / jv[:, None]
                    out[:, 3:6] = tv
                    out[:, 6:9] = bv / np.linalg.norm(bv, axis=1)[:, None]
                frames[:, ax, m, s] = out
                jac[:, ax, m, s] = jv
    return frames, jac
