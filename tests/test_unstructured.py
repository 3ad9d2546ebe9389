"""Unstructured straight-sided meshes (GmshMesh.jl:16-394, Mesh.jl:380-487) and their geometry
(PhysicalRegions.jl:438-472, 756-971), checked on the oracle: residuals are invariant under any
rotation of the elements' local numbering (face orientations, master2slave, frames), freestream is
preserved, and an unperturbed unrotated box reproduces CartesianMesh's geometry."""
import os

import numpy as np
import pytest

import flou_cuda as F
from cases import oracle_for, smooth_euler_state

HERE = os.path.dirname(os.path.abspath(__file__))


def _std(d, n, nv, basis="GLL"):
    b = F.LagrangeBasis(basis, n)
    return {1: F.StdSegment, 2: F.StdQuad, 3: F.StdHex}[d](b, F.DGSEMrec(b), nv)


def _disc(mesh, n, op, eq=None, basis="GLL"):
    d = mesh.dim
    eq = eq or F.EulerEquation(d, 1.4)
    bcs = {name: F.EulerOutflowBC() for name in mesh.bdnames}
    return F.MultielementDisc(mesh, _std(d, n, eq.nvariables, basis), eq, op, bcs)


def _state(disc, seed=0):
    """A smooth state defined on physical coordinates (the same at the same point of any mesh)."""
    d = disc.mesh.dim
    X = disc.coords
    rng = np.random.default_rng(seed)
    ph = rng.uniform(0, 6, size=(d + 2, 3))
    P = np.zeros((disc.ndofs, d + 2))
    for v in range(d + 2):
        w = np.ones(disc.ndofs)
        for q in range(d):
            w = w * np.cos(2.0 * X[:, q] + ph[v, q])
        P[:, v] = (1.0 if v in (0, d + 1) else 0.0) + (0.1 if v in (0, d + 1) else 0.3) * w
    return np.asfortranarray(disc.equation.vars_prim2cons(P))


@pytest.mark.parametrize("dim", [1, 2, 3])
def test_mesh_topology(dim):
    nel = 3
    m = F.perturbed_box(dim, nel, (0.0,) * dim, (1.0,) * dim, amp=0.1, seed=2)
    assert m.nfaces == dim * nel ** (dim - 1) * (nel + 1)
    assert len(m.intfaces) == dim * nel ** (dim - 1) * (nel - 1)
    assert sorted(m.bdnames) == [str(k) for k in range(1, 2 * dim + 1)]
    for b in m.bdfaces:
        assert len(b) == nel ** (dim - 1)
    # every element face points back to its element
    for e in range(m.nelements):
        for p in range(2 * dim):
            f, s = m.faceinds[e, p] - 1, m.facepos[e, p] - 1
            assert m.eleminds[f, s] == e + 1 and m.elempos[f, s] == p + 1
    assert int(m.orientation.max()) <= (1 if dim == 2 else 7 if dim == 3 else 0)
    plain = F.perturbed_box(dim, nel, (0.0,) * dim, (1.0,) * dim, amp=0.1, seed=2, rotate=False)
    assert not plain.orientation.any()


@pytest.mark.parametrize("dim", [1, 2, 3])
def test_unperturbed_box_reproduces_cartesian_geometry(dim):
    n, nel = 4, 3
    um = F.perturbed_box(dim, nel, (0.0,) * dim, (2.0,) * dim, amp=0.0, rotate=False)
    cm = F.CartesianMesh((0.0,) * dim, (2.0,) * dim, (nel,) * dim)
    op = F.StrongDivOperator(F.LxF(F.StdAverage(), 1.0))
    du, dc = _disc(um, n, op), _disc(cm, n, op)
    npe = n ** dim
    # same elements in the same order (x fastest) with the same local numbering
    assert np.allclose(du.coords, dc.coords, atol=1e-14)
    assert np.allclose(du.J, dc.J, rtol=1e-14)
    assert np.allclose(du.Ja, dc.Ja, rtol=1e-14, atol=1e-15)
    # faces: compare per (element, position)
    for e in range(um.nelements):
        for p in range(2 * dim):
            fu, fc = um.faceinds[e, p] - 1, cm.faceinds[e, p] - 1
            if um.facepos[e, p] == 1 and cm.facepos[e, p] == 1:
                nfd = n ** (dim - 1)
                assert np.allclose(du.frames[fu * nfd:(fu + 1) * nfd], dc.frames[fc * nfd:(fc + 1) * nfd], atol=1e-14)
                assert np.allclose(du.faceJ[fu * nfd:(fu + 1) * nfd], dc.faceJ[fc * nfd:(fc + 1) * nfd], rtol=1e-14)


def _match(coords_a, coords_b, npe):
    """Index map b -> a of equal points within the same element (elements matched by centroid;
    LGL nodes on element boundaries are shared by several elements)."""
    ne = len(coords_a) // npe
    ca = coords_a.reshape(ne, npe, 3)
    cb = coords_b.reshape(ne, npe, 3)
    ka = {tuple(np.round(c.mean(axis=0), 10)): e for e, c in enumerate(ca)}
    out = np.zeros(len(coords_b), dtype=np.int64)
    for eb in range(ne):
        ea = ka[tuple(np.round(cb[eb].mean(axis=0), 10))]
        kn = {tuple(np.round(c, 10)): i for i, c in enumerate(ca[ea])}
        for i, c in enumerate(cb[eb]):
            out[eb * npe + i] = ea * npe + kn[tuple(np.round(c, 10))]
    return out


OPS = {"strong": lambda: F.StrongDivOperator(F.LxF(F.StdAverage(), 1.0)),
       "split": lambda: F.SplitDivOperator(F.ChandrasekharAverage(), F.LxF(F.ChandrasekharAverage(), 1.0)),
       "split_md": lambda: F.SplitDivOperator(F.MatrixDissipation(F.ChandrasekharAverage(), 1.0)),
       "hybrid": lambda: F.HybridDivOperator(F.ChandrasekharAverage(), F.HLLC(),
                                             F.LxF(F.ChandrasekharAverage(), 1.0), 1e-2),
       "hybrid_md": lambda: F.HybridDivOperator(F.MatrixDissipation(F.ChandrasekharAverage(), 1.0), 1.0),
       # δ -> 1: no blending (OpDivergence.jl:781-801 with a huge constant)
       "hybrid_unblended": lambda: F.HybridDivOperator(F.ChandrasekharAverage(), F.HLLC(),
                                                       F.LxF(F.ChandrasekharAverage(), 1.0), 1e30),
       # HLLC interfaces: rotation-invariant in 3D also when the traces jump (Gauss nodes)
       "split_hllc": lambda: F.SplitDivOperator(F.ChandrasekharAverage(), F.HLLC()),
       "hybrid_unblended_hllc": lambda: F.HybridDivOperator(F.ChandrasekharAverage(), F.HLLC(), F.HLLC(), 1e30)}


@pytest.mark.parametrize("dim,op,basis", [(2, "strong", "GLL"), (2, "split", "GLL"), (3, "strong", "GLL"),
                                          (3, "split", "GLL"), (3, "split_md", "GLL"), (2, "hybrid", "GLL"),
                                          (2, "hybrid_md", "GLL"), (3, "hybrid", "GLL"), (2, "strong", "GL"),
                                          (2, "split", "GL"), (2, "hybrid_unblended", "GL"), (3, "strong", "GL"),
                                          (3, "split_hllc", "GL"), (3, "hybrid_unblended_hllc", "GL")])
def test_residual_is_invariant_under_element_rotations(dim, op, basis):
    """Rotating each element's local numbering permutes the nodes and re-orients the faces
    (all orientation codes occur in 3D); the residual at each physical node must not change.
    For the hybrid operator this also turns the subcell lines (and their subgrid frames).  Not
    for the 3D hybrid with MatrixDissipation(ChandrasekharAverage): the reference's 3D Chandrashekar
    interface flux counts wl² twice (Euler.jl:216), so it changes when the subcell frames' two
    tangents trade places and the states jump between nodes (1.5e-7 here).  Nor for the blended
    hybrid on Gauss nodes: the reference sweeps each line from its first node, every subcell flux
    starting from the blended one before it (OpDivergence.jl:741-769), so reversing a line's
    direction changes the result (1e-3 here); unblended (δ = 1) it is invariant.  On Gauss nodes the
    traces jump, so the 3D cases take HLLC interfaces (the Chandrashekar interface flux's wl² term
    would show, as above)."""
    ops = OPS
    n = 4
    plain = F.perturbed_box(dim, 3, (0.0,) * dim, (1.0,) * dim, amp=0.12, seed=5, rotate=False)
    rot = F.perturbed_box(dim, 3, (0.0,) * dim, (1.0,) * dim, amp=0.12, seed=5, rotate=True)
    if dim == 3:
        assert len(set(rot.orientation.tolist())) == 8
    d0, d1 = _disc(plain, n, ops[op](), basis=basis), _disc(rot, n, ops[op](), basis=basis)
    Q0, Q1 = _state(d0, 3), _state(d1, 3)
    R0 = oracle_for(d0).rhs(Q0)
    R1 = oracle_for(d1).rhs(Q1)
    perm = _match(d0.coords, d1.coords, n ** dim)
    err = np.max(np.abs(R1 - R0[perm])) / np.max(np.abs(R0))
    assert err < 1e-12, err


@pytest.mark.parametrize("dim,n", [(2, 3), (2, 5), (3, 3), (3, 4)])
def test_freestream_on_perturbed_meshes(dim, n):
    m = F.perturbed_box(dim, 3, (0.0,) * dim, (1.0,) * dim, amp=0.15, seed=7)
    for op in (F.StrongDivOperator(F.LxF(F.StdAverage(), 1.0)),
               F.SplitDivOperator(F.ChandrasekharAverage(), F.LxF(F.ChandrasekharAverage(), 1.0))):
        disc = _disc(m, n, op)
        P = np.zeros((disc.ndofs, dim + 2))
        P[:, 0], P[:, 1:1 + dim], P[:, -1] = 1.2, 0.3, 1.7
        Q = np.asfortranarray(disc.equation.vars_prim2cons(P))
        R = oracle_for(disc).rhs(Q)
        assert np.max(np.abs(R)) < 1e-11, np.max(np.abs(R))


def test_gmsh_round_trip(tmp_path):
    m = F.perturbed_box(3, 2, (0.0,) * 3, (1.0,) * 3, amp=0.1, seed=3)
    p = tmp_path / "box.msh"
    F.write_gmsh22(str(p), m)
    r = F.UnstructuredMesh.from_gmsh(str(p), 3)
    assert np.array_equal(r.elements, m.elements) and np.allclose(r.nodes, m.nodes)
    assert r.bdnames == m.bdnames
    assert np.array_equal(r.faceinds, m.faceinds) and np.array_equal(r.orientation, m.orientation)


def test_gmsh41_file():
    """A two-quadrilateral mesh in format 4.1 (entities, node and element blocks, named groups)."""
    m = F.UnstructuredMesh.from_gmsh(os.path.join(HERE, "golden", "two_quads_v41.msh"), 2)
    assert m.nelements == 2 and m.nfaces == 7
    assert sorted(m.bdnames) == ["outlet", "wall"]
    assert len(m.bdfaces[m.boundary_index("wall") - 1]) == 5
    assert len(m.bdfaces[m.boundary_index("outlet") - 1]) == 1
    assert np.allclose(m.nodes[m.elements[1]], [[1, 0], [2, 0], [2, 1], [1, 1]])


# The reference's test/meshes folder, named by FLOU_REFERENCE_MESHES (the test is skipped
# when it is unset or absent).
REF_MESHES = os.environ.get("FLOU_REFERENCE_MESHES", "")


@pytest.mark.skipif(not REF_MESHES or not os.path.isdir(REF_MESHES),
                    reason="FLOU_REFERENCE_MESHES does not name the reference's test/meshes folder")
@pytest.mark.parametrize("name,dim,nelem,names", [
    ("2D_cylinder", 2, 73, ["Bottom", "Right", "Top", "Left", "Hole"]),
    ("3D_bullet", 3, 295, ["Body", "Interior", "Inlet", "Wall", "Outlet", "Left", "Right"]),
])
def test_reference_meshes(name, dim, nelem, names):
    """The reference's own Gmsh 4.1 meshes (test/meshes/*.msh; 3D_bullet is the coarse version of
    the mesh of examples/src/3D_Euler.jl): read in the order of their physical groups, the
    connectivity is consistent, the geometry is valid (positive Jacobians, unit normals) and the
    split form with MatrixDissipation, as the 3D example runs it, preserves a uniform flow."""
    m = F.UnstructuredMesh.from_gmsh(os.path.join(REF_MESHES, name + ".msh"), dim)
    assert m.nelements == nelem and m.bdnames == names
    for f in range(m.nfaces):   # every face is held by the element positions that name it
        for side in range(2):
            e, pos = int(m.eleminds[f, side]), int(m.elempos[f, side])
            if e:
                assert m.faceinds[e - 1, pos - 1] == f + 1
    assert sum(len(b) for b in m.bdfaces) == int(np.sum(m.eleminds[:, 1] == 0))
    op = F.SplitDivOperator(F.MatrixDissipation(F.ChandrasekharAverage(), 1.0))
    disc = _disc(m, 3, op)
    assert np.all(disc.J > 0) and np.all(disc.faceJ > 0)
    fr = np.asarray(disc.frames).reshape(-1, 9)
    assert np.allclose(np.linalg.norm(fr[:, 0:3], axis=1), 1.0)
    P = np.zeros((disc.ndofs, dim + 2))
    P[:, 0], P[:, 1], P[:, -1] = 1.0, 2.0, 1.0   # the example's inflow state (1, 2, 0, 0, 1)
    Q = np.asfortranarray(disc.equation.vars_prim2cons(P))
    R = oracle_for(disc).rhs(Q)
    assert np.max(np.abs(R)) < 1e-10, np.max(np.abs(R))


@pytest.mark.parametrize("dim", [2, 3])
def test_hybrid_subgrid_geometry(dim):
    """The subcell-interface geometry (PhysicalRegions.jl:180-300) of an unperturbed, unrotated box
    is the Cartesian one (axes, Ja_dd), so the hybrid residual equals the Cartesian hybrid's; on
    perturbed elements a uniform flow stays uniform (the subcell metrics are consistent with the
    telescoped volume metrics)."""
    n, nel = 4, 3
    um = F.perturbed_box(dim, nel, (0.0,) * dim, (2.0,) * dim, amp=0.0, rotate=False)
    cm = F.CartesianMesh((0.0,) * dim, (2.0,) * dim, (nel,) * dim)
    du, dc = _disc(um, n, OPS["hybrid"]()), _disc(cm, n, OPS["hybrid"]())
    Qu, Qc = _state(du, 4), _state(dc, 4)
    Ru, Rc = oracle_for(du).rhs(Qu), oracle_for(dc).rhs(Qc)
    assert np.max(np.abs(Ru - Rc)) < 1e-12 * np.max(np.abs(Rc))
    fr, jac = du.abi_arrays()["subgrid"]
    assert np.all(jac > 0) and np.allclose(np.linalg.norm(fr[:, :3], axis=1), 1.0)
    pm = F.perturbed_box(dim, nel, (0.0,) * dim, (1.0,) * dim, amp=0.15, seed=7)
    dp = _disc(pm, n, OPS["hybrid_md"]())
    P = np.zeros((dp.ndofs, dim + 2))
    P[:, 0], P[:, 1:1 + dim], P[:, -1] = 1.2, 0.3, 1.7
    R = oracle_for(dp).rhs(np.asfortranarray(dp.equation.vars_prim2cons(P)))
    assert np.max(np.abs(R)) < 1e-11, np.max(np.abs(R))


@pytest.mark.parametrize("dim", [2, 3])
def test_gauss_nodes_on_general_elements(dim):
    """Gauss nodes on unstructured elements: an unperturbed box reproduces the Cartesian strong,
    split and hybrid residuals (interpolated traces, subcell normals at the line ends), and a
    uniform flow stays uniform on perturbed elements."""
    n, nel = 4, 3
    um = F.perturbed_box(dim, nel, (0.0,) * dim, (2.0,) * dim, amp=0.0, rotate=False)
    cm = F.CartesianMesh((0.0,) * dim, (2.0,) * dim, (nel,) * dim)
    for op in ("strong", "split", "hybrid"):
        du, dc = _disc(um, n, OPS[op](), basis="GL"), _disc(cm, n, OPS[op](), basis="GL")
        Qu, Qc = _state(du, 4), _state(dc, 4)
        Ru, Rc = oracle_for(du).rhs(Qu), oracle_for(dc).rhs(Qc)
        assert np.max(np.abs(Ru - Rc)) < 1e-12 * np.max(np.abs(Rc)), op
    pm = F.perturbed_box(dim, nel, (0.0,) * dim, (1.0,) * dim, amp=0.15, seed=7)
    for op in ("strong", "split", "hybrid_md"):
        dp = _disc(pm, n, OPS[op](), basis="GL")
        P = np.zeros((dp.ndofs, dim + 2))
        P[:, 0], P[:, 1:1 + dim], P[:, -1] = 1.2, 0.3, 1.7
        R = oracle_for(dp).rhs(np.asfortranarray(dp.equation.vars_prim2cons(P)))
        assert np.max(np.abs(R)) < 1e-11, (op, np.max(np.abs(R)))
