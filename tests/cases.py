"""Shared builders for the parity tests: a product discretization (flou_cuda host side) and
the identical set-up arrays for the oracle."""
import numpy as np

import flou_cuda as F
import oracle_ref


def build(dim, n, nelem, equation, operator, periodic=True, bcs=None, basis="GLL", box=None):
    if box is None:
        box = ((-1.0,) * dim, (1.0,) * dim)
    mesh = F.CartesianMesh(box[0], box[1], nelem)
    if periodic is True:
        periodic = tuple(range(dim))
    for d in periodic or ():
        F.apply_periodicBCs(mesh, (str(2 * d + 1), str(2 * d + 2)))
    b = LagrangeBasis = F.LagrangeBasis(basis, n)
    std = {1: F.StdSegment, 2: F.StdQuad, 3: F.StdHex}[dim](b, F.DGSEMrec(b), equation.nvariables)
    if bcs is None:
        bcs = {}
        for bid in mesh.bdmap:
            bcs[str(bid)] = F.EulerOutflowBC()
    disc = F.MultielementDisc(mesh, std, equation, operator, bcs)
    return disc


def oracle_for(disc, arrays=None):
    a = arrays if arrays is not None else disc.abi_arrays()
    return oracle_ref.Disc(disc.config, a, disc.mesh.nelements, disc.mesh.nfaces)


def smooth_euler_state(disc, seed=0, amp=0.1):
    """A smooth, strictly physical state with random Fourier content."""
    rng = np.random.default_rng(seed)
    X = disc.coords
    d = disc.mesh.dim
    L = disc.mesh.finish - disc.mesh.start
    def wave():
        k = rng.integers(1, 3, size=d)
        ph = rng.uniform(0, 2 * np.pi, size=d)
        return np.prod([np.sin(2 * np.pi * k[i] * (X[:, i] - disc.mesh.start[i]) / L[i] + ph[i]) for i in range(d)],
                       axis=0)
    rho = 1.0 + amp * wave()
    P = np.zeros((disc.ndofs, d + 2))
    P[:, 0] = rho
    for i in range(d):
        P[:, 1 + i] = 0.3 * (i + 1) + amp * wave()
    P[:, d + 1] = 1.0 + amp * wave()
    return np.asfortranarray(disc.equation.vars_prim2cons(P))


def rel_linf(a, b):
    """Relative L-inf error per variable: max_v max_i |a - b| / s_v with s_v = max_i |b_v|, floored
    at 1e-3 of the largest |b| over all variables.  The floor only matters for a component whose
    reference is round-off (e.g. the density residual of a divergence-free field at constant
    density), where a relative error of round-off against round-off carries no information."""
    a = np.asarray(a).reshape(b.shape, order="F") if np.asarray(a).shape != b.shape else np.asarray(a)
    smax = np.max(np.abs(b)) if b.size else 0.0
    out = 0.0
    for v in range(b.shape[1]):
        s = max(np.max(np.abs(b[:, v])), 1e-3 * smax)
        out = max(out, np.max(np.abs(a[:, v] - b[:, v])) / (s if s > 0 else 1.0))
    return out
