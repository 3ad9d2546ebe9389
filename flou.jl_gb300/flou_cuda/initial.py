"""Synthetic initial states of the benchmark configurations (no counterpart in Flou except
gaussian_bump, src/FlouCommon/Utilities.jl:16-32).

  isentropic_vortex: Shu's isentropic vortex (Shu 1998): on a uniform flow (ρ∞, u∞, p∞ = 1),
      δ(u, v) = β/(2π) exp((1 - r²)/2) (-y', x'), T = 1 - (γ-1) β²/(8γπ²) exp(1 - r²),
      ρ = T^(1/(γ-1)), p = ρ^γ.
  taylor_green: the 3D Taylor-Green vortex with ρ0 = 1, p0 = 1/(γ M²), u = sin x cos y cos z,
      v = -cos x sin y cos z, w = 0, p = p0 + (cos 2x + cos 2y)(cos 2z + 2)/16.
"""
import numpy as np


def gaussian_bump(x, x0, s, h):
    """h exp(-Σ (x_k - x0_k)² / (2 s_k²)) (Utilities.jl:16-32)."""
    x = np.atleast_2d(x)
    e = np.zeros(x.shape[0])
    for k in range(len(x0)):
        e -= (x[:, k] - x0[k]) ** 2 / (2 * s[k] ** 2)
    return h * np.exp(e)


def isentropic_vortex(eq, coords, center, beta=5.0, uinf=(1.0, 1.0), rhoinf=1.0, pinf=1.0, period=None):
    """Conservative state (ndofs, 4) of Shu's vortex; `period` (Lx, Ly) wraps the distance."""
    g = eq.gamma
    dx = coords[:, 0] - center[0]
    dy = coords[:, 1] - center[1]
    if period is not None:
        dx = dx - period[0] * np.round(dx / period[0])
        dy = dy - period[1] * np.round(dy / period[1])
    r2 = dx * dx + dy * dy
    f = np.exp(0.5 * (1.0 - r2))
    du = -beta / (2 * np.pi) * f * dy
    dv = beta / (2 * np.pi) * f * dx
    T = (pinf / rhoinf) - (g - 1) * beta ** 2 / (8 * g * np.pi ** 2) * np.exp(1.0 - r2)
    rho = rhoinf * (T / (pinf / rhoinf)) ** (1.0 / (g - 1))
    p = rho * T
    P = np.stack([rho, uinf[0] + du, uinf[1] + dv, p], axis=1)
    return eq.vars_prim2cons(P)


def taylor_green(eq, coords, mach=0.1, rho0=1.0):
    g = eq.gamma
    x, y, z = coords[:, 0], coords[:, 1], coords[:, 2]
    p0 = 1.0 / (g * mach ** 2)
    u = np.sin(x) * np.cos(y) * np.cos(z)
    v = -np.cos(x) * np.sin(y) * np.cos(z)
    w = np.zeros_like(x)
    p = p0 + (np.cos(2 * x) + np.cos(2 * y)) * (np.cos(2 * z) + 2.0) / 16.0
    rho = np.full_like(x, rho0)
    return eq.vars_prim2cons(np.stack([rho, u, v, w, p], axis=1))


def vortex_bump(eq, coords, center, beta, amp, uinf=(1.0, 1.0), period=None, bump_center=(0.0, 0.0), sigma=1.0):
    """Isentropic vortex of strength `beta` plus a Gaussian density perturbation of amplitude
    `amp` (pressure unchanged), the initial state of the batched configuration.  Walled boxes
    use uinf = (0, 0)."""
    Q = isentropic_vortex(eq, coords, center, beta=beta, uinf=uinf, period=period)
    P = eq.vars_cons2prim(Q)
    dx = coords[:, 0] - bump_center[0]
    dy = coords[:, 1] - bump_center[1]
    if period is not None:
        dx = dx - period[0] * np.round(dx / period[0])
        dy = dy - period[1] * np.round(dy / period[1])
    P[:, 0] = P[:, 0] + amp * np.exp(-(dx * dx + dy * dy) / (2 * sigma * sigma))
    return eq.vars_prim2cons(P)
