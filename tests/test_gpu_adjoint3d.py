"""3D discrete adjoint (periodic Taylor-Green boxes, physical mode): dot
products of the predictor Jacobian and of one whole step, central
differences of the final-enstrophy gradient with respect to the initial
velocity (u^{-1} tied to u^0, as the perturbed Taylor-Green run starts), and
identical gradients from different checkpoint schedules.

The dot-product and central-difference tests run in FP64 and in the
mixed-precision mode (FP64 residuals of the Jacobian solves refined by FP32
BiCGStab solves). Tolerances as in the 2D adjoint tests: dot products to 1e-12 (operator) and
1e-10 (step), central differences (eps = 1e-6, converged forward runs) to
1e-6. The QUICK flux u_d Q(phi) has a kink where the advecting velocity u_d
changes sign (the upwind switch flips), so the objective is differentiable
only where no face velocity lies within eps of zero; the Taylor-Green box has
such faces (w = 0 plus 1e-3 noise), and the central-difference check runs on
the scaled Taylor-Green field plus a uniform mean flow, where every face
velocity stays above 0.16."""
import math

import numpy as np
import pytest

import amressif_gb300 as ns
from amressif_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

N = 16
LIN_TOL = 1e-13


def shifted_state(n=N):
    """0.3 x (perturbed Taylor-Green) + (0.5, 0.45, 0.4): no face velocity
    near zero, so no upwind switch flips under a small perturbation"""
    u, up, p = wl.tgv3d_perturbed_state(n, amp=1e-3, seed=0)
    u = [0.3 * u[m] + off for m, off in enumerate((0.5, 0.45, 0.4))]
    return u, [a.copy() for a in u], 0.09 * p


def solver(n=N, ren=400.0, state=None, precision=ns.PREC_FP64):
    h = 2 * math.pi / n
    p = ns.default_params(dim=3, n_cell=n, ren=ren, fixed_dt=0.4 * h, iter_num=400, momentum_tolerance=1e-13,
                          precision=precision, prob_hi=(2 * math.pi,) * 3, bc_lo=(111,) * 3, bc_hi=(111,) * 3,
                          fix_quirks=1, poisson_tol_rel=1e-13, max_grid_size=(n, n, n))
    s = ns.Solver(p)
    s.set_state(*(state if state is not None else wl.tgv3d_perturbed_state(n, amp=1e-3, seed=0)))
    return s


def dofs(rng, n=N):
    """random face fields of the periodic degrees of freedom (face n = face 0)"""
    out = []
    for d in range(3):
        shp = [n, n, n]
        shp[2 - d] += 1
        a = rng.standard_normal(shp)
        sl_hi = [slice(None)] * 3
        sl_lo = [slice(None)] * 3
        sl_hi[2 - d] = n
        sl_lo[2 - d] = 0
        a[tuple(sl_hi)] = a[tuple(sl_lo)]
        out.append(a)
    return out


def inner(a, b):
    """sum over the degrees of freedom (the face-n images excluded)"""
    t = 0.0
    for d in range(3):
        sl = [slice(None)] * 3
        sl[2 - d] = slice(0, N)
        t += float(np.vdot(a[d][tuple(sl)], b[d][tuple(sl)]))
    return t


def test_3d_operator_dot_product(gpu_lib):
    s = solver()
    s.step()
    rng = np.random.default_rng(1)
    x, w = dofs(rng), dofs(rng)
    jx = s.adjoint_op(x)
    jtw, _ = s.adjoint_op(w, transpose=True)
    lhs, rhs = inner(jx, w), inner(x, jtw)
    assert abs(lhs - rhs) <= 1e-12 * max(abs(lhs), abs(rhs))


@pytest.mark.parametrize("precision", [ns.PREC_FP64, ns.PREC_MIXED])
def test_3d_step_dot_product(gpu_lib, precision):
    s = solver(precision=precision)
    s.step()
    rng = np.random.default_rng(2)
    du, dup = dofs(rng), dofs(rng)
    dp = rng.standard_normal((N, N, N))
    ub, upb = dofs(rng), dofs(rng)
    pb = rng.standard_normal((N, N, N))
    pb -= pb.mean()
    o, op, odp = s.step_jvp(du, dup, dp)
    a_u, a_up, a_p, _ = s.step_vjp(ub, upb, pb)
    lhs = inner(o, ub) + inner(op, upb) + float(np.vdot(odp, pb))
    rhs = inner(du, a_u) + inner(dup, a_up) + float(np.vdot(dp, a_p))
    assert abs(lhs - rhs) <= 1e-10 * max(abs(lhs), abs(rhs))


def enstrophy_grad(nsnap, L, state=None, precision=ns.PREC_FP64):
    s = solver(state=state, precision=precision)
    J, _ = s.adjoint_fwd(np.zeros(0), nsteps=L, nsnap=nsnap, lin_tol=LIN_TOL)
    _, st = s.adjoint_bwd()
    ub, upb, _ = s.adjoint_state_grad()
    s.close()
    return J, [a + b for a, b in zip(ub, upb)], st


@pytest.mark.parametrize("precision", [ns.PREC_FP64, ns.PREC_MIXED])
def test_3d_enstrophy_gradient_matches_central_differences(gpu_lib, precision):
    L = 4
    J, g, st = enstrophy_grad(2, L, shifted_state(), precision)
    assert J > 0 and st["adjoint_steps"] == L and st["status"] == 0
    d = wl.divfree_perturbation3d(N, amp=1.0, seed=3)  # direction with face n = face 0
    ad = inner(g, d)
    eps = 1e-6

    def J_at(sign):
        u, _, p = shifted_state()
        u = [u[m] + sign * eps * d[m] for m in range(3)]
        t = solver(state=(u, [a.copy() for a in u], p), precision=precision)  # u^{-1} = u^0
        Jx, stx = t.adjoint_fwd(np.zeros(0), nsteps=L, nsnap=L, lin_tol=LIN_TOL)
        assert stx["status"] == 0
        t.close()
        return Jx

    fd = (J_at(1.0) - J_at(-1.0)) / (2 * eps)
    assert abs(fd - ad) <= 1e-6 * abs(ad), (fd, ad)


def test_3d_schedules_give_identical_gradients(gpu_lib):
    L = 5
    res = {k: enstrophy_grad(k, L) for k in (1, 2, L)}
    assert res[L][2]["steps_advanced"] == L
    for k in (1, 2):
        assert res[k][0] == res[L][0]
        for a, b in zip(res[k][1], res[L][1]):
            np.testing.assert_array_equal(a, b)


def test_3d_mixed_gradient_matches_fp64(gpu_lib):
    """Mixed precision (float-float / FP32 predictor, FP32 inner solves of the
    refined Jacobian solves) against FP64 on the perturbed Taylor-Green box:
    the same gradient to 1e-9 (relative L2)."""
    L = 5
    J64, g64, _ = enstrophy_grad(2, L)
    J32, g32, st = enstrophy_grad(2, L, precision=ns.PREC_MIXED)
    assert st["status"] == 0 and st["lin_max_res"] <= LIN_TOL
    assert abs(J32 - J64) <= 1e-12 * abs(J64)
    num = sum(float(np.sum((a - b) ** 2)) for a, b in zip(g32, g64))
    den = sum(float(np.sum(b ** 2)) for b in g64)
    assert math.sqrt(num / den) <= 1e-9, math.sqrt(num / den)
