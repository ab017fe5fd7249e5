"""The benchmark workloads over their stated lengths (main.cpp:875-1202).

The 128^2 cavity in four 64^2 boxes (Re 100, dt = 0.5 dx, 200 steps):
the plain FP64 path runs all 200 steps free-running beside the oracle, with
identical pseudo-iteration counts K and a relative L2 <= 1e-10 in u, v and p
(p modulo its constant) after every step.

The perturbed Taylor-Green vortex at 1024^2 (Re 1000, dt = 0.5 dx, parity mode):
20 steps resynced to the oracle (same K, <= 1e-10 per step), and all 500
steps free-running against the oracle's committed per-step history
(tests/golden/tgv1024_parity_history.json, made by make_tgv1024_history.py):
the same K at every step and the kinetic energy, Taylor-Green amplitude and
field norms within 1e-9 relative.

The 512^2 lid-control cavity (Re 400, 400 steps, 256 lid controls, 20 snapshots):
the adjoint gradient against central differences (eps = 1e-6) along the 8
seeded unit directions, to 1e-6 relative, and against the tangent-linear
model (ns_step_jvp chained over the 400 steps) along one seeded direction,
to 1e-9 relative.
"""
import json
import math
import os

import numpy as np
import pytest

import amressif_gb300 as ns
from amressif_gb300 import workloads as wl
from oracle.orc import Oracle

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


def relp(a, b):
    return rel(a - a.mean(), b - b.mean())


def compare(s, o, what, tol=1e-10):
    ug, _, pg, _ = s.get_state()
    uo, _, po, _ = o.get_state()
    errs = [rel(ug[0], uo[0]), rel(ug[1], uo[1]), relp(pg, po)]
    assert max(errs) <= tol, (what, errs)
    return errs


def test_cavity128_4boxes_200_steps(gpu_lib, oracle_lib):
    n, dt = 128, 0.5 / 128
    o = Oracle(n, ren=100.0, dt=dt, iter_num=100, poisson_tol=1e-13, max_grid_size=(64, 64, 64))
    o.init(0)
    p = ns.default_params(n_cell=n, ren=100.0, fixed_dt=dt, iter_num=100, precision=ns.PREC_FP64_EXACT,
                          poisson_tol_rel=1e-13, max_grid_size=(64, 64, 64))
    s = ns.Solver(p)
    s.init(ns.INIT_CAVITY)
    worst = 0.0
    for step in range(1, 201):
        so, sg = o.step(), s.step()
        assert sg["pseudo_iters"] == so["pseudo_iters"], (step, sg["pseudo_iters"], so["pseudo_iters"])
        assert sg["div_after"] <= 1e-10
        worst = max(worst, max(compare(s, o, "step %d" % step)))
    assert s.step_count == 200 and worst <= 1e-10
    o.close()
    s.close()


N2 = 1024
DT2 = 0.5 * 2 * math.pi / N2
PER = dict(prob_hi=(2 * math.pi,) * 3, bc_lo=(111,) * 3, bc_hi=(111,) * 3)


def tgv_solver():
    prm = ns.default_params(n_cell=N2, ren=1000.0, fixed_dt=DT2, iter_num=100, precision=ns.PREC_FP64_EXACT,
                            poisson_tol_rel=1e-13, max_grid_size=(N2, N2, N2), **PER)
    return ns.Solver(prm)


def test_tgv1024_20_resynced_steps(gpu_lib, oracle_lib):
    u, up, p = wl.tgv_perturbed_state(N2, amp=1e-3, seed=0)
    o = Oracle(N2, ren=1000.0, dt=DT2, iter_num=100, poisson_tol=1e-13, max_grid_size=(N2, N2, N2), **PER)
    o.set_state(u, up, p)
    s = tgv_solver()
    for step in range(1, 21):
        uo, upo, po, _ = o.get_state()
        s.set_state(uo, upo, po, time=o_time(step - 1))
        so, sg = o.step(), s.step()
        assert sg["pseudo_iters"] == so["pseudo_iters"], (step, sg, so)
        compare(s, o, "step %d" % step)
        assert abs(sg["div_after"] - so["div_after"]) <= 1e-8 * so["div_after"] + 1e-12
    o.close()
    s.close()


def o_time(k):
    return k * DT2


def history_scalars(u, v, p, h):
    n = u.shape[0]
    return {"ke": 0.5 * h * h * float((u[:, :n] ** 2).sum() + (v[:n, :] ** 2).sum()),
            "amp": wl.tgv_amplitude(u, v), "norm_u": float(np.linalg.norm(u)), "norm_v": float(np.linalg.norm(v)),
            "norm_p": float(np.linalg.norm(p - p.mean()))}


def test_tgv1024_500_steps_against_oracle_history(gpu_lib):
    path = os.path.join(HERE, "golden", "tgv1024_parity_history.json")
    with open(path) as f:
        ref = json.load(f)
    hist = ref["history"]
    assert ref["nsteps"] == 500 and len(hist) == 500
    u, up, p = wl.tgv_perturbed_state(N2, amp=1e-3, seed=0)
    s = tgv_solver()
    s.set_state(u, up, p)
    h = 2 * math.pi / N2
    worst = {}
    for rec in hist:
        st = s.step()
        assert st["pseudo_iters"] == rec["K"], (rec["step"], st["pseudo_iters"], rec["K"])
        ug, _, pg, _ = s.get_state()
        got = history_scalars(ug[0], ug[1], pg, h)
        for k, v in got.items():
            e = abs(v - rec[k]) / abs(rec[k])
            worst[k] = max(worst.get(k, 0.0), e)
        assert abs(st["div_after"] - rec["div_after"]) <= 1e-8 * rec["div_after"] + 1e-12, rec["step"]
    assert max(worst.values()) <= 1e-9, worst
    s.close()


# ---- the 512^2 lid-control cavity ----------------------------------------------

N4, L4, NSEG, SNAP = 512, 400, 256, 20


def cavity4(tol=1e-13):
    p = ns.default_params(n_cell=N4, ren=400.0, fixed_dt=0.5 / N4, iter_num=400, momentum_tolerance=tol,
                          poisson_tol_rel=1e-13, precision=ns.PREC_FP64, max_grid_size=(N4, N4, N4))
    s = ns.Solver(p)
    s.init(ns.INIT_CAVITY)
    return s


def quarter_ke_tangent(u, du, n):
    """dJ = sum over the cells of [0, 1/2]^2 of (phi . dphi) dx dy, phi the
    cell average of the faces (the linearisation of the lid-control cavity's objective)"""
    hh = n // 2
    dx = 1.0 / n
    cu = 0.5 * (u[0][:hh, :hh] + u[0][:hh, 1:hh + 1])
    cv = 0.5 * (u[1][:hh, :hh] + u[1][1:hh + 1, :hh])
    dcu = 0.5 * (du[0][:hh, :hh] + du[0][:hh, 1:hh + 1])
    dcv = 0.5 * (du[1][:hh, :hh] + du[1][1:hh + 1, :hh])
    return float(np.sum(cu * dcu + cv * dcv)) * dx * dx


def test_lid_control_adjoint_full_size(gpu_lib):
    rng = np.random.default_rng(0)
    c = 1.0 + 0.05 * rng.standard_normal(NSEG)
    s = cavity4()
    J, _ = s.adjoint_fwd(c, nsteps=L4, nsnap=SNAP, lin_tol=1e-13)
    g, bst = s.adjoint_bwd()
    s.close()
    assert bst["adjoint_steps"] == L4 and np.all(np.isfinite(g)) and J > 0
    # 8 seeded unit directions (the directions of bench.py's check: the same
    # generator, drawn after the controls)
    errs = []
    for _ in range(8):
        d = rng.standard_normal(NSEG)
        d /= np.linalg.norm(d)
        Js = []
        for sg in (1.0, -1.0):
            t = cavity4()
            Jx, _ = t.adjoint_fwd(c + sg * 1e-6 * d, nsteps=L4, nsnap=2, lin_tol=1e-13)
            t.close()
            Js.append(Jx)
        fd = (Js[0] - Js[1]) / 2e-6
        ad = float(g @ d)
        errs.append(abs(fd - ad) / abs(ad))
    assert max(errs) <= 1e-6, errs
    # tangent-linear model along one more seeded direction: the state tangent
    # starts at zero and is carried step by step by ns_step_jvp at the
    # trajectory's own states
    d = rng.standard_normal(NSEG)
    d /= np.linalg.norm(d)
    t = cavity4()
    t.set_controls(c)
    zf = [np.zeros(t.face_shape(0)), np.zeros(t.face_shape(1))]
    du, dup, dp = [a.copy() for a in zf], [a.copy() for a in zf], np.zeros((N4, N4))
    for _ in range(L4):
        du, dup, dp = t.step_jvp(du, dup, dp, d)
        t.step()
    uf, _, _, _ = t.get_state()
    t.close()
    dj_tlm = quarter_ke_tangent(uf, du, N4)
    ad = float(g @ d)
    assert abs(dj_tlm - ad) <= 1e-9 * abs(ad), (dj_tlm, ad)
