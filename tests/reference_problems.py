"""The reference's own Euler test problems with golden values (test/tests.jl:90-181,
test/runtests.jl:34-45), set up through the flou_cuda host side: the Sod tube and the 2D
normal shock, both stepped with ORK256 at a fixed dt.  The golden values are the reference's
`minimum(sol.u[end])` / `maximum(sol.u[end])` over the final conservative state."""
import numpy as np

import flou_cuda as F

# test/runtests.jl:36-43
SOD_MIN, SOD_MAX = -0.1662939230897596, 254.90504152149907
SHOCK_MIN, SHOCK_MAX = -4.680030848090326e-13, 12.977466260673845


def sod_tube():
    """SodTube1D (test/tests.jl:90-134): 20 elements on [0, 1], 4 Gauss-Lobatto nodes, split form
    with MatrixDissipation(ChandrasekharAverage(), 1.0), GenericBC with the initial states on both
    ends, dt = 1e-4, tf = 0.018.  Returns (disc, Q0, dt, tf)."""
    eq = F.EulerEquation(1, 1.4)
    left = eq.vars_prim2cons(np.array([1.0, 0.0, 100.0]))
    right = eq.vars_prim2cons(np.array([0.125, 0.0, 10.0]))

    def qext(_q, x, _frame, _t, _eq):
        return left if x[0] < 0.5 else right

    mesh = F.CartesianMesh((0.0,), (1.0,), (20,))
    basis = F.LagrangeBasis("GLL", 4)
    std = F.StdSegment(basis, F.DGSEMrec(basis), eq.nvariables)
    op = F.SplitDivOperator(F.MatrixDissipation(F.ChandrasekharAverage(), 1.0))
    disc = F.MultielementDisc(mesh, std, eq, op, {"1": F.GenericBC(qext), "2": F.GenericBC(qext)})
    # node coordinates as the reference maps them, x = x1 (1 - r) + x2 r with r = (ξ + 1)/2 and the
    # vertices of range(0, 1, 21) (Mesh.jl:380-384): the nodes on x = 0.5 take the right state
    n, ne = std.n, 20
    Q = np.zeros((disc.ndofs, 3), order="F")
    for e in range(ne):
        x1, x2 = e / ne, (e + 1) / ne
        for i in range(n):
            r = (std.xi1d[i] + 1) / 2
            Q[e * n + i] = qext(None, (x1 * (1 - r) + x2 * r,), None, 0.0, eq)
    return disc, Q, 1e-4, 0.018


def normal_shockwave(rho0, u0, p0, gamma):
    """Rankine-Hugoniot state behind a normal shock (src/FlouCommon/Euler.jl:346-359)."""
    a = np.sqrt(gamma * p0 / rho0)
    m0 = u0 / a
    rho1 = rho0 * m0 ** 2 * (gamma + 1) / ((gamma - 1) * m0 ** 2 + 2)
    p1 = p0 * (2 * gamma * m0 ** 2 - (gamma - 1)) / (gamma + 1)
    m1 = np.sqrt(((gamma - 1) * m0 ** 2 + 2) / (2 * gamma * m0 ** 2 - (gamma - 1)))
    return rho1, m1 * np.sqrt(gamma * p1 / rho1), p1


def shockwave_2d():
    """Shockwave2D (test/tests.jl:136-181): 11 x 3 elements on [-1, 1] x [0, 1], periodic in y,
    6 Gauss-Lobatto nodes, HybridDivOperator(MatrixDissipation(ChandrasekharAverage(), 1.0), 1.0),
    a Mach 2 normal shock at x = 0 held by GenericBC states, dt = 1e-2, tf = 1.  Returns
    (disc, Q0, dt, tf)."""
    gamma = 1.4
    eq = F.EulerEquation(2, gamma)
    rho0, p0 = 1.0, 1.0
    u0 = 2.0 * np.sqrt(gamma * p0 / rho0)
    rho1, u1, p1 = normal_shockwave(rho0, u0, p0, gamma)
    q0 = eq.vars_prim2cons(np.array([rho0, u0, 0.0, p0]))
    q1 = eq.vars_prim2cons(np.array([rho1, u1, 0.0, p1]))

    def qext(_q, xy, _frame, _t, _eq):
        return q0 if xy[0] < 0 else q1

    mesh = F.CartesianMesh((-1.0, 0.0), (1.0, 1.0), (11, 3))
    F.apply_periodicBCs(mesh, ("3", "4"))
    basis = F.LagrangeBasis("GLL", 6)
    std = F.StdQuad(basis, F.DGSEMrec(basis), eq.nvariables)
    op = F.HybridDivOperator(F.MatrixDissipation(F.ChandrasekharAverage(), 1.0), 1.0)
    disc = F.MultielementDisc(mesh, std, eq, op, {"1": F.GenericBC(qext), "2": F.GenericBC(qext)})
    # no node lies on x = 0 (11 elements, 6 nodes), so the coordinates' last bits do not matter
    Q = np.asfortranarray(np.array([qext(None, x, None, 0.0, eq) for x in disc.coords[:, :2]]))
    return disc, Q, 1e-2, 1.0


def isclose(a, b, rtol):
    """Julia's isapprox(a, b; rtol) for scalars: |a - b| <= rtol * max(|a|, |b|)."""
    return abs(a - b) <= rtol * max(abs(a), abs(b))
