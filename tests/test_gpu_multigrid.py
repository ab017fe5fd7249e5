"""The fine-level multigrid smoother (the warp-marching kernel used for FP32
levels of 4096^2 and above) on a walled cavity and on a periodic
Taylor-Green box: one 4096^2 step of the mixed-precision solver (FP32
V-cycles inside float-float defect correction) against the plain FP64
solver (FP64 V-cycles with the tiled smoother) from the same state. The two
solve the same discrete Poisson problem to the same tolerance, so pressure
(modulo its constant) and velocity agree to 1e-10 (relative L2) and the
mixed step leaves max|div u| <= 1e-10. The smoothers read one buffer and
write another (no block reads a halo that another block has already
updated), so two runs of the same step are bitwise identical."""
import math

import numpy as np
import pytest

import amressif_gb300 as ns
from amressif_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

N = 4096


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def one_step(precision, case, dc_residual=0):
    if case == "cavity":
        p = ns.default_params(n_cell=N, ren=1000.0, fixed_dt=0.5 / N, iter_num=100, momentum_tolerance=1e-10,
                              max_grid_size=(N, N, N), precision=precision, poisson_tol_rel=1e-11,
                              poisson_tol_div=1e-10, poisson_max_cycles=200, dtau_clip=1, dc_residual=dc_residual)
        s = ns.Solver(p)
        s.init(ns.INIT_CAVITY)
        s.step()  # a developed right-hand side
    else:
        h = 2 * math.pi / N
        p = ns.default_params(n_cell=N, ren=1000.0, fixed_dt=0.5 * h, iter_num=100, momentum_tolerance=1e-10,
                              prob_hi=(2 * math.pi,) * 3, bc_lo=(111,) * 3, bc_hi=(111,) * 3, fix_quirks=1,
                              max_grid_size=(N, N, N), precision=precision, poisson_tol_rel=1e-11,
                              poisson_tol_div=1e-10, poisson_max_cycles=200, dc_residual=dc_residual)
        s = ns.Solver(p)
        s.set_state(*wl.tgv_perturbed_state(N, amp=1e-3, seed=0))
    st = s.step()
    u, _, pp, _ = s.get_state()
    s.close()
    return st, u, pp


@pytest.mark.parametrize("dc_residual", [0, 1])
@pytest.mark.parametrize("case", ["cavity", "tgv"])
def test_fine_level_smoother_mixed_matches_fp64(gpu_lib, case, dc_residual):
    """dc_residual 0: float-float residual and phi; 1: FP64 from the first sweep"""
    sm, um, pm = one_step(ns.PREC_MIXED, case, dc_residual)
    sd, ud, pd = one_step(ns.PREC_FP64, case)
    assert sm["div_after"] <= 1e-10, sm["div_after"]
    assert rel(pm - pm.mean(), pd - pd.mean()) <= 1e-10
    for a, b in zip(um, ud):
        assert rel(a, b) <= 1e-10


def test_mixed_step_is_deterministic(gpu_lib):
    s1, u1, p1 = one_step(ns.PREC_MIXED, "tgv")
    s2, u2, p2 = one_step(ns.PREC_MIXED, "tgv")
    assert s1["poisson_cycles"] == s2["poisson_cycles"] and s1["pseudo_iters"] == s2["pseudo_iters"]
    assert np.array_equal(p1, p2)
    for a, b in zip(u1, u2):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("n", [256, N])
def test_warm_started_mixed_poisson_matches_fp64(gpu_lib, n):
    """poisson_warm_start = 1: the defect correction starts from the previous
    step's phi, with the tolerance still relative to max|f - mean f|. Over
    several steps of the cavity it keeps the pseudo-iteration counts of the
    FP64 solver, u and p within 1e-10 of it and max|div u| <= 1e-10. (The
    V-cycles it saves depend on how much phi changes between steps: about one
    a step on the 4096^2 cavity, none at 256^2.)"""
    steps = 6 if n < N else 3
    out = {}
    for name, prec, warm in (("fp64", ns.PREC_FP64, 0), ("cold", ns.PREC_MIXED, 0), ("warm", ns.PREC_MIXED, 1)):
        p = ns.default_params(n_cell=n, ren=1000.0, fixed_dt=0.5 / n, iter_num=100, momentum_tolerance=1e-10,
                              max_grid_size=(n, n, n), precision=prec, poisson_tol_rel=1e-10, poisson_tol_div=1e-10,
                              poisson_max_cycles=200, dtau_clip=1, poisson_warm_start=warm)
        s = ns.Solver(p)
        s.init(ns.INIT_CAVITY)
        st = [s.step() for _ in range(steps)]
        u, _, pp, _ = s.get_state()
        out[name] = (st, u, pp)
        s.close()
    for name in ("cold", "warm"):
        st, u, pp = out[name]
        assert [x["pseudo_iters"] for x in st] == [x["pseudo_iters"] for x in out["fp64"][0]]
        assert all(x["div_after"] <= 1e-10 for x in st)
        for a, b in zip(u, out["fp64"][1]):
            assert rel(a, b) <= 1e-10, (name, rel(a, b))
        assert rel(pp - pp.mean(), out["fp64"][2] - out["fp64"][2].mean()) <= 1e-10
    cold = [x["poisson_cycles"] for x in out["cold"][0]]
    warm = [x["poisson_cycles"] for x in out["warm"][0]]
    assert warm[0] == cold[0]  # the first step has no previous phi
