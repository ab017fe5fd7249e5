"""Discrete adjoint of the time advance: dot-product (tangent-linear vs
adjoint) tests of the predictor Jacobian and of one whole step, central
finite differences of the objective through the ns_step_adjoint_fwd /
ns_step_adjoint_bwd pair, and agreement of the checkpoint schedules.

Tolerances: the linearised predictor is solved to ||r|| <= 1e-13 ||b|| and
the Poisson solves to 1e-13, so dot products agree to 1e-10 relative; the
forward runs use momentum_tolerance 1e-13 so that the finite differences
(eps = 1e-6, central) see the converged map, and the gradient must match
them to 1e-6 relative (the accuracy asked of the adjoint).
"""
import numpy as np
import pytest

import amressif_gb300 as ns

pytestmark = pytest.mark.gpu

LIN_TOL = 1e-13


def cavity(n=32, ren=400.0, precision=ns.PREC_FP64, **kw):
    p = ns.default_params(n_cell=n, ren=ren, fixed_dt=0.5 / n, iter_num=400, momentum_tolerance=1e-13,
                          poisson_tol_rel=1e-13, precision=precision, **kw)
    s = ns.Solver(p)
    s.init(ns.INIT_CAVITY)
    return s


def interior(s, rng):
    """random face fields, zero on the boundary faces"""
    n = s.n
    u = rng.standard_normal((n, n + 1))
    v = rng.standard_normal((n + 1, n))
    u[:, 0] = u[:, n] = 0.0
    v[0, :] = v[n, :] = 0.0
    return [u, v]


def dot(a, b):
    return sum(float(np.vdot(x, y)) for x, y in zip(a, b))


def controls(nseg, seed=0):
    rng = np.random.default_rng(seed)
    return 1.0 + 0.05 * rng.standard_normal(nseg)


def advance(s, k):
    for _ in range(k):
        s.step()


def test_operator_dot_product():
    s = cavity(32)
    s.set_controls(controls(8))
    advance(s, 5)
    rng = np.random.default_rng(1)
    x, w = interior(s, rng), interior(s, rng)
    dc = rng.standard_normal(8)
    jx = s.adjoint_op(x, dc=dc)
    jtw, cb = s.adjoint_op(w, transpose=True)
    lhs = dot(jx, w)
    rhs = dot(x, jtw) + float(np.dot(dc, cb))
    assert abs(lhs - rhs) <= 1e-12 * max(abs(lhs), abs(rhs))
    # boundary faces carry nothing
    assert np.all(jx[0][:, 0] == 0) and np.all(jx[0][:, -1] == 0)
    assert np.all(jtw[1][0, :] == 0) and np.all(jtw[1][-1, :] == 0)


def test_operator_matches_finite_difference_of_the_lid_term():
    """J x is linear in x and the lid term enters only the north ghost row:
    the jvp along (0, dc) equals the difference quotient of the predictor
    residual seen through two lid profiles (G is affine in the lid)."""
    s = cavity(32)
    c0 = controls(8)
    s.set_controls(c0)
    advance(s, 3)
    rng = np.random.default_rng(2)
    zero = [np.zeros(s.face_shape(0)), np.zeros(s.face_shape(1))]
    dc = rng.standard_normal(8)
    y1 = s.adjoint_op(zero, dc=dc)
    y2 = s.adjoint_op(zero, dc=2 * dc)
    for a, b in zip(y1, y2):
        np.testing.assert_allclose(2 * a, b, rtol=1e-13, atol=1e-13 * np.abs(b).max())
    # only the faces within reach of the north ghosts (two rows of cells) move
    assert np.abs(y1[0][: s.n - 3, :]).max() == 0.0


def test_step_dot_product():
    s = cavity(32)
    s.set_controls(controls(8))
    advance(s, 4)
    rng = np.random.default_rng(3)
    du, dup = interior(s, rng), interior(s, rng)
    dp = rng.standard_normal((s.n, s.n))
    dc = rng.standard_normal(8)
    ub, upb = interior(s, rng), interior(s, rng)
    pb = rng.standard_normal((s.n, s.n))
    pb -= pb.mean()  # the step leaves the additive constant of p undetermined
    u0, _, p0, _ = s.get_state()
    t0 = s.time
    o, op, odp = s.step_jvp(du, dup, dp, dc)
    a_u, a_up, a_p, a_c = s.step_vjp(ub, upb, pb)
    lhs = dot(o, ub) + dot(op, upb) + float(np.vdot(odp, pb))
    rhs = dot(du, a_u) + dot(dup, a_up) + float(np.vdot(dp, a_p)) + float(np.dot(dc, a_c))
    assert abs(lhs - rhs) <= 1e-10 * max(abs(lhs), abs(rhs))
    # du_prev' = du, and the state is not advanced by the linearised steps
    np.testing.assert_array_equal(op[0], du[0])
    u1, _, p1, _ = s.get_state()
    np.testing.assert_array_equal(u0[0], u1[0])
    np.testing.assert_array_equal(p0, p1)
    assert s.time == t0


def run_J(n, c, nsteps, nsnap=2):
    s = cavity(n)
    J, _ = s.adjoint_fwd(c, nsteps=nsteps, nsnap=nsnap, lin_tol=LIN_TOL)
    s.close()
    return J


@pytest.mark.parametrize("nsnap", [3])
def test_gradient_matches_central_differences(nsnap):
    n, nseg, L = 32, 8, 12
    c = controls(nseg, seed=4)
    s = cavity(n)
    J, fst = s.adjoint_fwd(c, nsteps=L, nsnap=nsnap, lin_tol=LIN_TOL)
    g, bst = s.adjoint_bwd()
    assert J > 0 and np.all(np.isfinite(g))
    assert bst["adjoint_steps"] == L
    assert bst["lin_max_res"] <= 1e-12
    rng = np.random.default_rng(5)
    eps = 1e-6
    for _ in range(3):
        d = rng.standard_normal(nseg)
        d /= np.linalg.norm(d)
        fd = (run_J(n, c + eps * d, L) - run_J(n, c - eps * d, L)) / (2 * eps)
        ad = float(np.dot(g, d))
        assert abs(fd - ad) <= 1e-6 * abs(ad), (fd, ad)


def smooth_direction(n):
    """discretely divergence-free face field from psi = sin^2(pi x) sin^2(pi y)
    on the nodes (zero normal velocity on the walls)"""
    x = np.arange(n + 1) / n
    psi = np.outer(np.sin(np.pi * x) ** 2, np.sin(np.pi * x) ** 2)  # psi[j, i] at node (x_i, y_j)
    u = (psi[1:, :] - psi[:-1, :]) * n   # u at face (i, j): (psi(i, j+1) - psi(i, j)) / dy
    v = -(psi[:, 1:] - psi[:, :-1]) * n  # v at face (i, j): -(psi(i+1, j) - psi(i, j)) / dx
    return [u, v]


def test_gradient_of_the_state():
    """dJ/du^n (ns_adjoint_get_state_grad) against central differences, from
    a developed flow (so that J depends smoothly on the perturbed state)"""
    n, L = 32, 6
    c = controls(4, seed=6)
    s = cavity(n, ren=100.0)
    s.set_controls(c)
    advance(s, 30)
    u, up, p, _ = s.get_state()
    s.set_state(u, up, p)
    s.adjoint_fwd(c, nsteps=L, nsnap=L, lin_tol=LIN_TOL)
    s.adjoint_bwd()
    ub, _, _ = s.adjoint_state_grad()
    d = smooth_direction(n)
    eps = 1e-6

    def J_of(sign):
        t = cavity(n, ren=100.0)
        t.set_state([u[m] + sign * eps * d[m] for m in range(2)], up, p)
        J, _ = t.adjoint_fwd(c, nsteps=L, nsnap=L, lin_tol=LIN_TOL)
        t.close()
        return J

    fd = (J_of(1.0) - J_of(-1.0)) / (2 * eps)
    ad = dot(ub, d)
    assert abs(fd - ad) <= 1e-6 * abs(ad), (fd, ad)


def test_schedules_give_identical_gradients():
    n, nseg, L = 32, 8, 10
    c = controls(nseg, seed=8)
    out = {}
    for nsnap in (1, 3, L):
        s = cavity(n)
        J, _ = s.adjoint_fwd(c, nsteps=L, nsnap=nsnap, lin_tol=LIN_TOL)
        g, st = s.adjoint_bwd()
        out[nsnap] = (J, g, st)
        s.close()
    assert out[L][2]["steps_advanced"] == L  # store-all: no recomputation
    assert out[1][2]["steps_advanced"] > out[3][2]["steps_advanced"] > L
    for k in (1, 3):
        assert out[k][0] == out[L][0]
        np.testing.assert_array_equal(out[k][1], out[L][1])


def test_objective_value_and_final_state():
    n, L = 32, 5
    c = controls(4, seed=9)
    s = cavity(n)
    J, _ = s.adjoint_fwd(c, nsteps=L, nsnap=2, lin_tol=LIN_TOL)
    u, _, _, _ = s.get_state()
    h = n // 2
    dx = 1.0 / n
    cu = 0.5 * (u[0][:h, :h] + u[0][:h, 1:h + 1])
    cv = 0.5 * (u[1][:h, :h] + u[1][1:h + 1, :h])
    ref = 0.5 * float(np.sum(cu * cu + cv * cv)) * dx * dx
    assert abs(J - ref) <= 1e-13 * ref
    # the backward sweep leaves the context at the final state
    s.adjoint_bwd()
    u2, _, _, _ = s.get_state()
    np.testing.assert_array_equal(u[0], u2[0])
    np.testing.assert_array_equal(u[1], u2[1])
