"""Host set-up parity: connectivity (bit-exact), operators, geometry against the oracle's
restatement of the reference's procedures (CartesianMesh.jl, Mesh.jl:236-322,
ApproximationBases.jl, StdSegment.jl, PhysicalRegions.jl)."""
import itertools

import numpy as np
import pytest

import flou_cuda as F
import oracle_ref

MESHES = [
    (1, (0.0,), (1.0,), (20,)),
    (1, (0.0,), (1.0,), (1,)),
    (2, (-5.0, -5.0), (5.0, 5.0), (16, 16)),
    (2, (0.0, 0.0), (1.5, 2.0), (20, 10)),
    (2, (0.0, 0.0), (1.0, 1.0), (1, 3)),
    (3, (0.0, 0.0, 0.0), (2 * np.pi,) * 3, (4, 3, 5)),
    (3, (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), (1, 1, 2)),
]


def _periodic_sets(dim):
    dirs = range(dim)
    for r in range(dim + 1):
        for c in itertools.combinations(dirs, r):
            yield c


@pytest.mark.parametrize("dim,start,finish,n", MESHES)
def test_connectivity_bit_exact(dim, start, finish, n):
    for per in _periodic_sets(dim):
        m = F.CartesianMesh(start, finish, n)
        for d in per:
            F.apply_periodicBCs(m, (str(2 * d + 1), str(2 * d + 2)))
        pairs = [(2 * d + 1, 2 * d + 2) for d in per]
        o = oracle_ref.mesh(dim, start, finish, n, pairs)
        assert m.nfaces == o["nfaces"], per
        np.testing.assert_array_equal(m.faceinds, o["faceinds"])
        np.testing.assert_array_equal(m.facepos, o["facepos"])
        np.testing.assert_array_equal(m.eleminds, o["eleminds"])
        np.testing.assert_array_equal(m.elempos, o["elempos"])
        np.testing.assert_array_equal(m.orientation, o["orientation"])
        np.testing.assert_array_equal(m.bdface_index, o["bdface_index"])
        np.testing.assert_array_equal(m.intfaces, o["intfaces"])
        for bid in range(1, 2 * dim + 1):
            assert m.bdmap.get(bid, 0) == o["bdindex_of_id"][bid - 1]


def test_face_counts_of_the_vortex_and_tgv_meshes():
    m = F.CartesianMesh((-5, -5), (5, 5), (16, 16))
    assert m.nfaces == 17 * 16 * 2 == 544
    F.apply_periodicBCs(m, ("1", "2"), ("3", "4"))
    assert m.nfaces == 512
    m3 = F.CartesianMesh((0, 0, 0), (1, 1, 1), (32, 32, 32))
    F.apply_periodicBCs(m3, ("1", "2"), ("3", "4"), ("5", "6"))
    assert m3.nfaces == 3 * 32 ** 3


def test_periodic_argument_errors():
    m = F.CartesianMesh((0, 0), (1, 1), (2, 2))
    with pytest.raises(ValueError):
        F.apply_periodicBCs(m, ("2", "3"))
    with pytest.raises(ValueError):
        F.apply_periodicBCs(m, ("1", "5"))
    with pytest.raises(ValueError):
        F.apply_periodicBCs(m, ("a", "2"))


@pytest.mark.parametrize("n", range(2, 9))
@pytest.mark.parametrize("lobatto", [True, False])
def test_operators_match_reference_construction(n, lobatto):
    b = F.LagrangeBasis("GLL" if lobatto else "GL", n)
    s = F.StdSegment(b, F.DGSEMrec(b))
    o = oracle_ref.operators(n, lobatto)
    tol = 5e-14 * n * n
    np.testing.assert_allclose(b.xi, o["xi"], atol=1e-15)
    np.testing.assert_allclose(b.omega, o["omega"], atol=1e-15)
    for k, v in (("D", s.D), ("Ds", s.Ds), ("Dsharp", s.Dsharp)):
        np.testing.assert_allclose(v, o[k], atol=tol, err_msg=k)
    np.testing.assert_allclose(s.l[0], o["l_l"], atol=1e-14)
    np.testing.assert_allclose(s.l[1], o["l_r"], atol=1e-14)
    np.testing.assert_allclose(s.dg[0], o["dg_l"], atol=1e-12)
    np.testing.assert_allclose(s.dg[1], o["dg_r"], atol=1e-12)


@pytest.mark.parametrize("n", range(2, 9))
def test_operator_exactness(n):
    """D differentiates polynomials of degree < n exactly; LGL weights integrate degree 2n-3,
    GL weights degree 2n-1; SBP property Q + Qᵀ = B for LGL."""
    for nodes, deg in (("GLL", 2 * n - 3), ("GL", 2 * n - 1)):
        b = F.LagrangeBasis(nodes, n)
        s = F.StdSegment(b, F.DGSEMrec(b))
        x = b.xi
        for k in range(n):
            np.testing.assert_allclose(s.D @ x ** k, k * x ** (k - 1) if k else 0 * x, atol=1e-12)
        for k in range(deg + 1):
            exact = (1 - (-1) ** (k + 1)) / (k + 1)
            assert abs(b.omega @ x ** k - exact) < 1e-13
    b = F.LagrangeBasis("GLL", n)
    s = F.StdSegment(b, F.DGSEMrec(b))
    Q = np.diag(b.omega) @ s.D
    B = np.zeros((n, n))
    B[0, 0], B[-1, -1] = -1, 1
    np.testing.assert_allclose(Q + Q.T, B, atol=1e-13)


@pytest.mark.parametrize("dim,start,finish,n", [m for m in MESHES if m[3][0] > 1])
def test_geometry_matches_reference(dim, start, finish, n):
    m = F.CartesianMesh(start, finish, n)
    F.apply_periodicBCs(m, ("1", "2"))
    b = F.LagrangeBasis("GLL", 4)
    std = {1: F.StdSegment, 2: F.StdQuad, 3: F.StdHex}[dim](b, F.DGSEMrec(b))
    eq = F.LinearAdvection(*([1.0] * dim))
    bcs = {str(k): F.OutflowBC() for k in m.bdmap}
    disc = F.MultielementDisc(m, std, eq, F.StrongDivOperator(F.LxF(F.StdAverage(), 1.0)), bcs)
    o = oracle_ref.mesh(dim, start, finish, n, [(1, 2)])
    g = oracle_ref.geometry(o, 4, b.xi)
    np.testing.assert_array_equal(disc.J, g["J"])
    np.testing.assert_array_equal(disc.Ja, g["Ja"])
    np.testing.assert_array_equal(disc.frames, g["frames"])
    np.testing.assert_array_equal(disc.faceJ, g["faceJ"])
    np.testing.assert_allclose(disc.coords, g["coords"], atol=1e-13)
