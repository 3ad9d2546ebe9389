"""Nodal bases and standard regions, mirroring Flou's LagrangeBasis / DGSEMrec / StdSegment /
StdQuad / StdHex.

Reference: src/FlouSpatial/StdRegions/ApproximationBases.jl:68-91,135-186 (nodes, weights,
derivative matrix), Reconstruction.jl:121-134 (DGSEM lifting), StdSegment.jl:35-121 (D, l,
∂g, B, Ds = D - B, D♯ = 2D - B), StdQuad.jl:35-93 and StdHex.jl:36-112 (tensor products
reuse the segment's 1D matrices).

The reference fits monomial Lagrange polynomials (Polynomials.fit) and differentiates and
integrates them; this host code uses the barycentric form (Berrut & Trefethen 2004), which
gives the same matrices to about 1e-15.  The C ABI takes the matrices as inputs, so a Julia
caller passes Flou's own.
"""
import numpy as np


def _legendre(n, x):
    """P_n(x) and P_n'(x) by the three-term recurrence."""
    x = np.asarray(x, dtype=np.float64)
    p0, p1 = np.ones_like(x), x.copy()
    if n == 0:
        return p0, np.zeros_like(x)
    for k in range(2, n + 1):
        p0, p1 = p1, ((2 * k - 1) * x * p1 - (k - 1) * p0) / k
    dp = n * (x * p1 - p0) / np.where(np.abs(x) < 1, x * x - 1, 1.0)
    return p1, dp


def gausslobatto(n):
    """Gauss-Lobatto-Legendre nodes and weights on [-1, 1], ascending."""
    if n < 2:
        raise ValueError("Gauss-Lobatto needs at least 2 nodes")
    m = n - 1
    x = -np.cos(np.pi * np.arange(n) / m)
    for _ in range(100):   # Newton on P'_m, P''_m = (2x P'_m - m(m+1) P_m) / (1 - x²)
        p, dp = _legendre(m, x)
        inner = slice(1, n - 1)
        xi = x[inner]
        d2p = (2 * xi * dp[inner] - m * (m + 1) * p[inner]) / (1 - xi * xi)
        dx = dp[inner] / d2p
        x[inner] = xi - dx
        if len(dx) == 0 or np.max(np.abs(dx)) < 1e-15:
            break
    x[0], x[-1] = -1.0, 1.0
    x = 0.5 * (x - x[::-1])   # exact antisymmetry
    p, _ = _legendre(m, x)
    w = 2.0 / (m * (m + 1) * p * p)
    w = 0.5 * (w + w[::-1])
    return x, w


def gausslegendre(n):
    """Gauss-Legendre nodes and weights on [-1, 1], ascending."""
    x = -np.cos(np.pi * (np.arange(n) + 0.75) / (n + 0.5))
    for _ in range(100):
        p, dp = _legendre(n, x)
        dx = p / dp
        x = x - dx
        if np.max(np.abs(dx)) < 1e-16:
            break
    x = 0.5 * (x - x[::-1])
    _, dp = _legendre(n, x)
    w = 2.0 / ((1 - x * x) * dp * dp)
    w = 0.5 * (w + w[::-1])
    return x, w


def _bary_weights(x):
    n = len(x)
    w = np.ones(n)
    for j in range(n):
        for k in range(n):
            if k != j:
                w[j] /= (x[j] - x[k])
    return w


def interp_matrix(xe, x):
    """Lagrange basis of nodes x evaluated at points xe: P[i, j] = l_j(xe_i)."""
    xe = np.atleast_1d(np.asarray(xe, dtype=np.float64))
    w = _bary_weights(x)
    P = np.zeros((len(xe), len(x)))
    for i, xi in enumerate(xe):
        hit = np.nonzero(xi == x)[0]
        if len(hit):
            P[i, hit[0]] = 1.0
            continue
        t = w / (xi - x)
        P[i] = t / t.sum()
    return P


def derivative_matrix(x):
    """D[i, j] = l_j'(x_i) (ApproximationBases.jl:89-91), barycentric form, negative-sum diagonal."""
    n = len(x)
    w = _bary_weights(x)
    D = np.zeros((n, n))
    for i in range(n):
        for j in range(n):
            if i != j:
                D[i, j] = (w[j] / w[i]) / (x[i] - x[j])
        D[i, i] = -np.sum(D[i, np.arange(n) != i])
    return D


class LagrangeBasis:
    """LagrangeBasis(nodetype, nnodes): nodetype "GLL"/"GaussLobatto" or "GL"/"Gauss"."""

    def __init__(self, nodetype, nnodes):
        name = str(nodetype).lstrip(":")
        if name in ("GLL", "GaussLobatto"):
            self.xi, self.omega = gausslobatto(nnodes)
            self.hasboundaries = True
            self.nname = "Gauss-Lobatto"
        elif name in ("GL", "Gauss"):
            self.xi, self.omega = gausslegendre(nnodes)
            self.hasboundaries = False
            self.nname = "Gauss"
        else:
            raise ValueError("Nodes of type %s cannot be used in Lagrange bases." % nodetype)
        self.bname = "Lagrange"

    @property
    def nnodes(self):
        return len(self.xi)


class DGSEMrec:
    """DGSEMrec(basis): DGSEM lifting (Reconstruction.jl:121-134)."""

    def __init__(self, basis):
        self.basis = basis


class VCJHrec:
    """VCJHrec(p, η) (Reconstruction.jl:69-110): the energy-stable flux-reconstruction correction
    functions of Vincent, Castonguay and Jameson, g_l = (-1)^(p-1) (L_{p-1} - (η L_{p-2} + L_p)/(1+η))/2
    and g_r = (L_{p-1} + (η L_{p-2} + L_p)/(1+η))/2 with Legendre polynomials L_k; η = 0 (:DGSEM_GL)
    is DGSEM on Gauss nodes, η = (p-1)/p (:SD), η = p/(p-1) (:Huynh)."""

    def __init__(self, p, eta):
        self.p = int(p)
        if isinstance(eta, str):
            key = eta.lstrip(":")
            eta = {"DGSEM_GL": 0.0, "SD": (self.p - 1) / self.p, "Huynh": self.p / (self.p - 1)}[key]
        self.eta = float(eta)

    def derivatives(self, x):
        from numpy.polynomial import legendre as Lg
        p, eta = self.p, self.eta
        unit = lambda k: np.eye(k + 1)[k] if k >= 0 else np.zeros(1)
        Lkm, Lk, Lkp = unit(p - 2), unit(p - 1), unit(p)
        mix = Lg.legadd(Lg.legmul(eta, Lkm), Lkp) / (1.0 + eta)
        gl = (-1.0) ** (p - 1) * Lg.legsub(Lk, mix) / 2.0
        gr = Lg.legadd(Lk, mix) / 2.0
        return Lg.legval(x, Lg.legder(gl)), Lg.legval(x, Lg.legder(gr))


class _StdRegion:
    dim = 0

    def __init__(self, basis, rec, nvars=1):
        if not isinstance(rec, (DGSEMrec, VCJHrec)):
            raise ValueError("the reconstructions are DGSEMrec and VCJHrec")
        self.basis = basis
        self.reconstruction = rec
        x, w = basis.xi, basis.omega
        n = len(x)
        self.n = n
        self.xi1d = x
        self.omega1d = w
        ll = interp_matrix([-1.0], x)[0]
        lr = interp_matrix([1.0], x)[0]
        D = derivative_matrix(x)
        if isinstance(rec, VCJHrec):   # StdSegment.jl:82-83: ∂g = (-g_l', g_r')
            gl, gr = rec.derivatives(np.asarray(x))
            dgl, dgr = -gl, gr
        else:
            dgl, dgr = ll / w, lr / w   # StdSegment.jl:84-85: ∂g = (l_l/ω, l_r/ω)
        B = np.outer(dgr, lr) - np.outer(dgl, ll)
        self.D = D
        self.Ds = D - B
        self.Dsharp = 2.0 * D - B
        self.l = (ll, lr)
        self.dg = (dgl, dgr)
        # tensor-product quadrature weights, x fastest (StdQuad.jl:49, StdHex.jl:54)
        W = np.ones(1)
        for _ in range(self.dim):
            W = np.kron(w, W)
        self.omega = W

    @property
    def ndofs(self):
        return self.n ** self.dim

    def dofsize(self):
        return (self.n,) * self.dim


class StdSegment(_StdRegion):
    dim = 1


class StdQuad(_StdRegion):
    dim = 2


class StdHex(_StdRegion):
    dim = 3
