"""Host-side construction of the benchmark inputs (numpy, float64).

Arrays follow the ns_set_state layout: u faces (n, n+1), v faces (n+1, n),
cell fields (n, n), x fastest; the domain is [0, L]^2 with the MAC faces of
the reference's hybrid_grid_init (fn_init.cpp:61-229, kn_init.H:8-37).
"""
import math

import numpy as np


def tgv_fields(n, length=2.0 * math.pi):
    """Taylor-Green vortex u = sin x cos y, v = -cos x sin y on the faces and
    p = (cos 2x + cos 2y) / 4 at the cell centres."""
    h = length / n
    xf = np.arange(n + 1) * h
    xc = (np.arange(n) + 0.5) * h
    u = np.sin(xf)[None, :] * np.cos(xc)[:, None]
    v = -np.cos(xc)[None, :] * np.sin(xf)[:, None]
    p = 0.25 * (np.cos(2 * xc)[None, :] + np.cos(2 * xc)[:, None])
    return u, v, p


def divfree_perturbation(n, amp=1e-3, seed=0, length=2.0 * math.pi):
    """Periodic, discretely divergence-free perturbation: a streamfunction psi
    on the n x n nodes drawn from the standard normal distribution (numpy
    PCG64 generator, the given seed), du = d psi / dy and dv = -d psi / dx by
    MAC differences, scaled so that max(|du|, |dv|) = amp."""
    h = length / n
    psi = np.random.default_rng(seed).standard_normal((n, n))  # psi[j, i] at node (x_i, y_j)
    psi_n = np.roll(psi, -1, axis=0)  # node (i, j+1)
    psi_e = np.roll(psi, -1, axis=1)  # node (i+1, j)
    du = (psi_n - psi) / h           # u face (i, j), i < n
    dv = -(psi_e - psi) / h          # v face (i, j), j < n
    s = amp / max(np.abs(du).max(), np.abs(dv).max())
    u = np.empty((n, n + 1))
    v = np.empty((n + 1, n))
    u[:, :n] = s * du
    u[:, n] = u[:, 0]  # periodic image of the first face
    v[:n, :] = s * dv
    v[n, :] = v[0, :]
    return u, v


def tgv_perturbed_state(n, amp=1e-3, seed=0, length=2.0 * math.pi):
    """(u, u_prev, p) of the perturbed Taylor-Green run: u^{-1} = u^0."""
    u, v, p = tgv_fields(n, length)
    du, dv = divfree_perturbation(n, amp, seed, length)
    u0 = [u + du, v + dv]
    return u0, [u0[0].copy(), u0[1].copy()], p


def mac_divergence(u, v, length=2.0 * math.pi):
    n = u.shape[0]
    h = length / n
    return (u[:, 1:] - u[:, :-1]) / h + (v[1:, :] - v[:-1, :]) / h


def tgv_amplitude(u, v, length=2.0 * math.pi):
    """Projection of (u, v) on the initial Taylor-Green field (1 at t = 0)."""
    n = u.shape[0]
    ut, vt, _ = tgv_fields(n, length)
    a = u[:, :n] * ut[:, :n]
    b = v[:n, :] * vt[:n, :]
    return float((a.sum() + b.sum()) / ((ut[:, :n] ** 2).sum() + (vt[:n, :] ** 2).sum()))


def lid_controls(nseg=256, sigma=0.05, seed=0):
    """Lid velocities 1 + N(0, sigma^2) (numpy PCG64, the given seed)."""
    return 1.0 + sigma * np.random.default_rng(seed).standard_normal(nseg)


# ---- 3D (arrays indexed [k, j, i]) -------------------------------------------------

def tgv3d_fields(n, length=2.0 * math.pi):
    """u = sin x cos y cos z, v = -cos x sin y cos z, w = 0 on the faces; p =
    (cos 2x + cos 2y)(cos 2z + 2) / 16 at the cell centres."""
    h = length / n
    xf = np.arange(n + 1) * h
    xc = (np.arange(n) + 0.5) * h
    u = np.sin(xf)[None, None, :] * np.cos(xc)[None, :, None] * np.cos(xc)[:, None, None]
    v = -np.cos(xc)[None, None, :] * np.sin(xf)[None, :, None] * np.cos(xc)[:, None, None]
    w = np.zeros((n + 1, n, n))
    p = (np.cos(2 * xc)[None, None, :] + np.cos(2 * xc)[None, :, None]) * (np.cos(2 * xc)[:, None, None] + 2.0) / 16.0
    return [u, v, w], p


def divfree_perturbation3d(n, amp=1e-3, seed=0, length=2.0 * math.pi):
    """Periodic, discretely divergence-free 3D perturbation: the MAC curl of a
    vector potential on the cell edges drawn from the standard normal
    distribution (numpy PCG64, the given seed), scaled to max |du| = amp."""
    h = length / n
    r = np.random.default_rng(seed)
    ax, ay, az = (r.standard_normal((n, n, n)) for _ in range(3))  # [k, j, i]

    def d(a, axis):  # forward difference a(index + 1) - a(index), periodic
        return (np.roll(a, -1, axis=axis) - a) / h

    du = d(az, 1) - d(ay, 0)  # x face (i, j+1/2, k+1/2)
    dv = d(ax, 0) - d(az, 2)  # y face
    dw = d(ay, 2) - d(ax, 1)  # z face
    s = amp / max(np.abs(du).max(), np.abs(dv).max(), np.abs(dw).max())
    u = np.empty((n, n, n + 1)); u[:, :, :n] = s * du; u[:, :, n] = u[:, :, 0]
    v = np.empty((n, n + 1, n)); v[:, :n, :] = s * dv; v[:, n, :] = v[:, 0, :]
    w = np.empty((n + 1, n, n)); w[:n, :, :] = s * dw; w[n, :, :] = w[0, :, :]
    return [u, v, w]


def tgv3d_perturbed_state(n, amp=1e-3, seed=0, length=2.0 * math.pi):
    """(u, u_prev, p) of the perturbed 3D Taylor-Green run: u^{-1} = u^0."""
    u, p = tgv3d_fields(n, length)
    du = divfree_perturbation3d(n, amp, seed, length)
    u0 = [u[m] + du[m] for m in range(3)]
    return u0, [a.copy() for a in u0], p


def mac_divergence3d(u, length=2.0 * math.pi):
    n = u[0].shape[0]
    h = length / n
    return ((u[0][:, :, 1:] - u[0][:, :, :-1]) + (u[1][:, 1:, :] - u[1][:, :-1, :]) + (u[2][1:, :, :] - u[2][:-1, :, :])) / h
