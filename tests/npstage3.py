"""Independent restatement (vectorised numpy) of one 3D RK pseudo-stage.

Used only to cross-check the C++ oracle's 3D branch: it is written from the
reference formulas with AMREX_SPACEDIM = 3 (fn_flux_calc.cpp:62-200, 716-736,
main.cpp:939-1014, fn_rhs.cpp:43-61, momentum.cpp:68-88, utilities.cpp:47-350)
with ghost-padded arrays instead of index loops, keeping each expression's
operation order. Arrays are indexed [k, j, i] (x fastest), so direction d
(x, y, z) is array axis 2 - d. Only the ghost cells that a stencil reads (one
coordinate outside the box) are filled.
"""
import numpy as np

from tests.npstage import cart_ghost_rule, quick

G = 2  # ghost layers of velCart


def _axis(d):
    return 2 - d


def _box(sl_axis, a, inner):
    """an index tuple: sl_axis along array axis a, inner along the other two"""
    return tuple(sl_axis if e == a else inner for e in range(3))


def cont2cart3(u, n, bc_lo, bc_hi, inflow, periodic):
    """velCart of the face arrays u[0..2] with two ghost layers."""
    inner = slice(G, G + n)
    c = []
    for m in range(3):
        a = _axis(m)
        q = np.zeros((n + 2 * G,) * 3)
        q[(inner,) * 3] = 0.5 * (u[m][_box(slice(0, n), a, slice(None))] + u[m][_box(slice(1, n + 1), a, slice(None))])
        c.append(q)
    for d in range(3):
        a = _axis(d)
        for m in range(3):
            q = c[m]
            for k in range(G):  # ghost layers -1-k and n+k
                lo_g, hi_g = G - 1 - k, n + G + k
                if periodic[d]:
                    q[_box(lo_g, a, inner)] = q[_box(n + G - 1 - k, a, inner)]
                    q[_box(hi_g, a, inner)] = q[_box(G + k, a, inner)]
                    continue
                for side, gi, mi in ((0, lo_g, G + k), (1, hi_g, n + G - 1 - k)):
                    code = bc_lo[d] if side == 0 else bc_hi[d]
                    kind, add = cart_ghost_rule(code, d, side, m, inflow)
                    v = q[_box(mi, a, inner)].copy()
                    q[_box(gi, a, inner)] = (add - v) if kind == "inlet" else (-v if kind == "neg" else v)
    return c


def stage3(us, ub, un, du, p, n, h, dt, ren, rk, bc_lo, bc_hi, inflow, periodic, reflect_periodic=True,
           explicit=False):
    """One 3D RK pseudo-stage; returns (new u*, momentum rhs). h = (dx, dy, dz).
    reflect_periodic=False skips the normal-flux reflection and keeps the
    pressure ghosts' periodic wrap in periodic directions (fix_quirks = 1).
    explicit=True: the explicit predictor (momentum.cpp:96-192) with no
    normal-flux reflection at all (quirk Q3)."""
    c = cont2cart3(us, n, bc_lo, bc_hi, inflow, periodic)
    inner = slice(G, G + n)
    total = []
    for m in range(3):
        q = c[m]

        def cells(a, off, count):  # cells off .. off+count-1 along axis a, the box along the others
            return q[_box(slice(G + off, G + off + count), a, inner)]

        conv = None
        for d in range(3):  # QUICK half-node fluxes at the faces along d, then their difference
            a = _axis(d)
            F = quick(us[d], cells(a, 1, n + 1), cells(a, 0, n + 1), cells(a, -1, n + 1), cells(a, -2, n + 1))
            diff = (F[_box(slice(1, n + 1), a, slice(None))] - F[_box(slice(0, n), a, slice(None))]) / h[d]
            conv = diff if conv is None else conv + diff
        ce = q[(inner,) * 3]
        x, y, z = _axis(0), _axis(1), _axis(2)
        visc = ((cells(x, 1, n) - 2 * ce + cells(x, -1, n)) / (h[0] * h[0])
                + (cells(y, 1, n) - 2 * ce + cells(y, -1, n)) / (h[1] * h[1])) / ren
        visc = visc + ((cells(z, 1, n) - 2 * ce + cells(z, -1, n)) / (h[2] * h[2])) / ren
        t = np.zeros((n + 2,) * 3)
        t[(slice(1, n + 1),) * 3] = (0.0 - conv) + visc
        total.append(t)
    # flux ghosts: periodic fill, then the odd reflection of the normal component at the edges
    box1 = slice(1, n + 1)
    for m in range(3):
        for d in range(3):
            if periodic[d]:
                a = _axis(d)
                total[m][_box(0, a, box1)] = total[m][_box(n, a, box1)]
                total[m][_box(n + 1, a, box1)] = total[m][_box(1, a, box1)]
    for d in range(3):
        if explicit or (periodic[d] and not reflect_periodic):
            continue
        a = _axis(d)
        total[d][_box(0, a, box1)] = -total[d][_box(1, a, box1)]
        total[d][_box(n + 1, a, box1)] = -total[d][_box(n, a, box1)]
    # pressure ghosts: mirrored on every side (the reference mirrors even periodic
    # directions), or wrapped in periodic directions with reflect_periodic=False
    pp = p
    for d in range(3):
        wrap = periodic[d] and not reflect_periodic
        pp = np.pad(pp, [(1, 1) if e == _axis(d) else (0, 0) for e in range(3)], mode="wrap" if wrap else "edge")
    out, rhs = [], []
    for d in range(3):
        a = _axis(d)
        gp = (pp[_box(slice(1, n + 2), a, box1)] - pp[_box(slice(0, n + 1), a, box1)]) / h[d]
        t = total[d]
        r = -gp + 0.5 * (t[_box(slice(0, n + 1), a, box1)] + t[_box(slice(1, n + 2), a, box1)])
        if explicit:
            r = r + (1.0 / (2.0 * dt)) * du[d]
            rhs.append(r)
            out.append(us[d] + ((dt / 1.5) * r))
            continue
        r = r - (1.5 / dt) * (us[d] - un[d]) + (0.5 / dt) * du[d]
        rhs.append(r)
        out.append(ub[d] + (rk * r))
    return out, rhs
