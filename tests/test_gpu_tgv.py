"""Doubly periodic Taylor-Green vortex on [0, 2 pi]^2 at 1024^2, Re = 1000,
dt = 0.5 dx, with the seeded divergence-free perturbation of amplitude 1e-3
(amressif_gb300.workloads): per-step parity with the oracle in the
reference's parity mode (quirks Q1/Q2), and the analytic decay exp(-2 nu t)
of the Taylor-Green amplitude over 500 steps in the physical (fixed) mode.

Tolerances: per-step relative L2 <= 1e-10 in u, v and p (p modulo its
constant) with identical pseudo-iteration counts; the amplitude follows
exp(-2 nu t) to 1e-5 relative (the discretisation error of the decay over
t = 1.53 is O(1e-7), the perturbation's projection on the mode O(1e-6)).
"""
import math

import numpy as np
import pytest

import amressif_gb300 as ns
from amressif_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

N = 1024
DT = 0.5 * 2 * math.pi / N
PER = dict(prob_hi=(2 * math.pi,) * 3, bc_lo=(111,) * 3, bc_hi=(111,) * 3)


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def relp(a, b):
    return rel(a - a.mean(), b - b.mean())


def test_tgv1024_perturbed_parity(gpu_lib, oracle_lib):
    from oracle.orc import Oracle

    u, up, p = wl.tgv_perturbed_state(N, amp=1e-3, seed=0)
    o = Oracle(N, ren=1000.0, dt=DT, iter_num=100, poisson_tol=1e-13, max_grid_size=(N, N, N), **PER)
    o.set_state(u, up, p)
    prm = ns.default_params(n_cell=N, ren=1000.0, fixed_dt=DT, iter_num=100, precision=ns.PREC_FP64_EXACT,
                            poisson_tol_rel=1e-12, max_grid_size=(N, N, N), **PER)
    s = ns.Solver(prm)
    s.set_state(u, up, p)
    for step in range(2):
        so = o.step()
        sg = s.step()
        assert sg["pseudo_iters"] == so["pseudo_iters"], (step, sg, so)
        ug, _, pg, _ = s.get_state()
        uo, _, po, _ = o.get_state()
        for d in range(2):
            assert rel(ug[d], uo[d]) <= 1e-10, (step, d, rel(ug[d], uo[d]))
        assert relp(pg, po) <= 1e-10
        # parity mode mirrors phi at the periodic edges (quirk Q2): the
        # projection leaves a divergence at the edge cells, the same on both sides
        assert abs(sg["div_after"] - so["div_after"]) <= 1e-8 * so["div_after"] + 1e-12
    o.close()


@pytest.mark.parametrize("precision", [ns.PREC_FP64, ns.PREC_MIXED])
def test_tgv1024_analytic_decay(gpu_lib, precision):
    nu = 1e-3
    u, up, p = wl.tgv_perturbed_state(N, amp=1e-3, seed=0)
    prm = ns.default_params(n_cell=N, ren=1.0 / nu, fixed_dt=DT, iter_num=100, precision=precision, fix_quirks=1,
                            poisson_tol_rel=1e-10, poisson_tol_div=1e-10, max_grid_size=(N, N, N), **PER)
    s = ns.Solver(prm)
    s.set_state(u, up, p)
    a0 = wl.tgv_amplitude(u[0], u[1])
    worst = 0.0
    for step in range(1, 501):
        st = s.step()
        assert st["div_after"] <= 1e-10
        if step % 100 == 0:
            ug, _, _, _ = s.get_state()
            a = wl.tgv_amplitude(ug[0], ug[1]) / a0
            worst = max(worst, abs(a / math.exp(-2 * nu * s.time) - 1.0))
    assert worst <= 1e-5, worst
