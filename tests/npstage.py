"""Second, independent restatement (vectorised numpy) of one RK pseudo-stage.

Used only to cross-check the C++ oracle: it is written from the reference
formulas (fn_flux_calc.cpp:62-200, 716-764, main.cpp:939-1014,
fn_rhs.cpp:43-61, momentum.cpp:68-79, utilities.cpp:47-261) with ghost-padded
arrays instead of index loops, keeping each expression's operation order.
2D only. Arrays are indexed [j, i].
"""
import numpy as np


def cart_ghost_rule(code, d, side, m, inflow):
    """(kind, add) of the velCart ghost on one side for comp m."""
    if code == 135:
        return "neg", 0.0
    slip = code == -135 or (d == 0 and side == 1 and code == 1)
    if slip:
        return ("neg", 0.0) if m == d else ("pos", 0.0)
    if code == 165 or (code == -165 and d == 0 and side == 0):
        if d == 1 and side == 1:
            return "inlet", 2 * inflow[m]
        return "inlet", 2.0
    raise ValueError(code)


def cont2cart(u, v, n, bc_lo, bc_hi, inflow, periodic):
    g = 2
    c = [np.zeros((n + 2 * g, n + 2 * g)) for _ in range(2)]
    c[0][g:-g, g:-g] = 0.5 * (u[:, :-1] + u[:, 1:])
    c[1][g:-g, g:-g] = 0.5 * (v[:-1, :] + v[1:, :])
    for m in range(2):
        a = c[m]
        if periodic[0]:
            a[g:-g, :g] = a[g:-g, n:n + g]
            a[g:-g, n + g:] = a[g:-g, g:2 * g]
        if periodic[1]:
            a[:g, :] = a[n:n + g, :]
            a[n + g:, :] = a[g:2 * g, :]
    for d in range(2):
        if periodic[d]:
            continue
        for side in range(2):
            code = bc_lo[d] if side == 0 else bc_hi[d]
            for m in range(2):
                kind, add = cart_ghost_rule(code, d, side, m, inflow)
                a = c[m]
                for k in range(g):  # ghost layer index: -1-k or n+k
                    gi = g - 1 - k if side == 0 else n + g + k
                    mi = g + k if side == 0 else n + g - 1 - k
                    if d == 0:
                        q = a[:, mi].copy()
                        a[:, gi] = (add - q) if kind == "inlet" else (-q if kind == "neg" else q)
                    else:
                        q = a[mi, :].copy()
                        a[gi, :] = (add - q) if kind == "inlet" else (-q if kind == "neg" else q)
    return c


def quick(ucf, A, B, C, E):
    ucon = 0.5 * ucf
    ud = ucon + np.abs(ucon)
    up = ucon - np.abs(ucon)
    return up * (0.125 * (-A - 2 * B + 3 * C) + B) + ud * (0.125 * (-E - 2 * C + 3 * B) + C)


def conv_quick_int(u, v, c, n, dx, dy):
    """Convective term of convective_flux_calc_quick (fn_flux_calc.cpp:204-393)
    on one box: first-order upwind face values plus 0.0 times the QUICK
    correction (its weight Real(1/8) is an integer division), face n a copy of
    face 0, and the y differences taken at i+1 through the flat y-face fab,
    whose element (i+1, j) is (0, j+1) at the last column."""
    g = 2
    I = np.arange(n)
    X, Y = [], []
    for m in range(2):
        q = c[m]
        r = q[g:-g]
        vp = r[:, g - 1 + I] + 0.0 * (-r[:, g - 2 + I] - 2 * r[:, g - 1 + I] + 3 * r[:, g + I])
        vm = r[:, g + I] + 0.0 * (3 * r[:, g - 1 + I] - 2 * r[:, g + I] - r[:, g + 1 + I])
        x = np.where(u[:, :n] > 0, vp, vm)
        X.append(np.hstack([x, x[:, :1]]))
        col = q[:, g:-g]
        vp = col[g - 1 + I, :] + 0.0 * (-col[g - 2 + I, :] - 2 * col[g - 1 + I, :] + 3 * col[g + I, :])
        vm = col[g + I, :] + 0.0 * (3 * col[g - 1 + I, :] - 2 * col[g + I, :] - col[g + 1 + I, :])
        y = np.where(v[:n, :] > 0, vp, vm)
        Y.append(np.vstack([y, y[:1, :]]))
    flat = I[:, None] * n + I[None, :] + 1  # element (i+1, j) of an (n+1) x n y-face fab

    def nxt(a):
        return a.ravel()[flat]

    conv0 = (u[:, 1:] * X[0][:, 1:] - u[:, :-1] * X[0][:, :-1]) / dx + (nxt(v) * nxt(Y[0]) - v[:n] * Y[0][:n]) / dy
    conv1 = (c[0][g:-g, g:-g] * (X[1][:, 1:] - X[1][:, :-1])) / dx + (c[1][g:-g, g:-g] * (nxt(Y[1]) - Y[1][:n])) / dy
    return conv0, conv1


def stage(us, ub, un, du, p, n, dx, dy, dt, ren, rk, bc_lo, bc_hi, inflow, periodic, cart=None, conv_scheme=0,
          explicit=False):
    """One RK pseudo-stage; returns (new u*, momentum rhs). conv_scheme: the
    convective routine (0 convective_flux_calc_new_quick, 1
    convective_flux_calc_quick, 2 convective_flux_calc, which leaves the
    total flux without a convective term). explicit=True: the explicit
    predictor instead (PSEUDO_TIMESTEPPING = 0, main.cpp:902-925,
    momentum.cpp:96-192): no reflection of the normal flux (quirk Q3),
    R += du / (2 dt), u* += (dt / 1.5) R."""
    g = 2
    u, v = us
    c = cart if cart is not None else cont2cart(u, v, n, bc_lo, bc_hi, inflow, periodic)
    alt = conv_quick_int(u, v, c, n, dx, dy) if conv_scheme == 1 else None
    total = []
    for m in range(2):
        q = c[m]
        # x-face fluxes at faces i = 0..n of rows j = 0..n-1
        I = np.arange(n + 1) + g
        Bx = q[g:-g][:, I]
        Ax = q[g:-g][:, I + 1]
        Cx = q[g:-g][:, I - 1]
        Ex = q[g:-g][:, I - 2]
        Fx = quick(u, Ax, Bx, Cx, Ex)
        J = np.arange(n + 1) + g
        By = q[J, g:-g]
        Ay = q[J + 1, g:-g]
        Cy = q[J - 1, g:-g]
        Ey = q[J - 2, g:-g]
        Fy = quick(v, Ay, By, Cy, Ey)
        conv = (Fx[:, 1:] - Fx[:, :-1]) / dx + (Fy[1:, :] - Fy[:-1, :]) / dy
        if conv_scheme == 1:
            conv = alt[m]
        elif conv_scheme == 2:
            conv = np.zeros((n, n))
        ce = q[g:-g, g:-g]
        visc = ((q[g:-g, g + 1:n + g + 1] - 2 * ce + q[g:-g, g - 1:n + g - 1]) / (dx * dx)
                + (q[g + 1:n + g + 1, g:-g] - 2 * ce + q[g - 1:n + g - 1, g:-g]) / (dy * dy)) / ren
        t = np.zeros((n + 2, n + 2))
        t[1:-1, 1:-1] = (0.0 - conv) + visc
        total.append(t)
    # flux ghosts: periodic fill then odd reflection of the normal component
    for m in range(2):
        t = total[m]
        if periodic[0]:
            t[1:-1, 0] = t[1:-1, n]
            t[1:-1, n + 1] = t[1:-1, 1]
        if periodic[1]:
            t[0, :] = t[n, :]
            t[n + 1, :] = t[1, :]
    if not explicit:
        total[0][:, 0] = -total[0][:, 1]
        total[0][:, n + 1] = -total[0][:, n]
        total[1][0, :] = -total[1][1, :]
        total[1][n + 1, :] = -total[1][n, :]
    # pressure with mirrored ghosts
    pp = np.zeros((n + 2, n + 2))
    pp[1:-1, 1:-1] = p
    pp[1:-1, 0] = p[:, 0]
    pp[1:-1, -1] = p[:, -1]
    pp[0, :] = pp[1, :]
    pp[-1, :] = pp[-2, :]
    gpx = (pp[1:-1, 1:] - pp[1:-1, :-1]) / dx
    gpy = (pp[1:, 1:-1] - pp[:-1, 1:-1]) / dy
    rx = -gpx + 0.5 * (total[0][1:-1, :-1] + total[0][1:-1, 1:])
    ry = -gpy + 0.5 * (total[1][:-1, 1:-1] + total[1][1:, 1:-1])
    out = []
    rhs = []
    for r, s, b, pn, d in ((rx, u, ub[0], un[0], du[0]), (ry, v, ub[1], un[1], du[1])):
        if explicit:
            r = r + (1.0 / (2.0 * dt)) * d
            rhs.append(r)
            out.append(s + ((dt / 1.5) * r))
            continue
        r = r - (1.5 / dt) * (s - pn) + (0.5 / dt) * d
        rhs.append(r)
        out.append(b + (rk * r))
    return out, rhs
