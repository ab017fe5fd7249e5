"""Parity of the CUDA path (through the C ABI) with the CPU oracle.

Tolerances: the FP64 exact mode reproduces the oracle's pseudo-stages bit for
bit (same operation order, no FMA); whole steps differ only through the
Poisson solve (different solver, both converged to <= 1e-12 relative), so u, v
and p (modulo its additive constant) must agree to a relative L2 of 1e-10 per
step, with identical pseudo-iteration counts K.
"""
import math

import numpy as np
import pytest

import amressif_gb300 as ns
from oracle.orc import FIELD_MRHS, FIELD_STAR, Oracle

pytestmark = pytest.mark.gpu

TOL_STEP = 1e-10


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


def relp(a, b):
    return rel(a - a.mean(), b - b.mean())


CASES = {
    # name: (n, oracle kwargs, gpu kwargs, init case)
    "cavity32": (32, dict(ren=100.0, dt=1e-3, max_grid_size=(32, 16, 16)), dict(ren=100.0, fixed_dt=1e-3), 0),
    "cavity40_partial_tiles": (40, dict(ren=100.0, dt=2e-3, max_grid_size=(40, 40, 40)), dict(ren=100.0, fixed_dt=2e-3), 0),
    "cavity128_4boxes": (128, dict(ren=100.0, dt=0.5 / 128, max_grid_size=(64, 64, 64)),
                       dict(ren=100.0, fixed_dt=0.5 / 128, max_grid_size=(64, 64, 64)), 0),
    "tgv64_parity": (64, dict(ren=1000.0, dt=0.5 * 2 * math.pi / 64, prob_hi=(2 * math.pi,) * 3,
                              bc_lo=(111,) * 3, bc_hi=(111,) * 3),
                     dict(ren=1000.0, fixed_dt=0.5 * 2 * math.pi / 64, prob_hi=(2 * math.pi,) * 3,
                          bc_lo=(111,) * 3, bc_hi=(111,) * 3), 1),
    "tgv64_fixed": (64, dict(ren=1000.0, dt=0.5 * 2 * math.pi / 64, prob_hi=(2 * math.pi,) * 3,
                             bc_lo=(111,) * 3, bc_hi=(111,) * 3, fix_quirks=1),
                    dict(ren=1000.0, fixed_dt=0.5 * 2 * math.pi / 64, prob_hi=(2 * math.pi,) * 3,
                         bc_lo=(111,) * 3, bc_hi=(111,) * 3, fix_quirks=1), 1),
    # periodic with partial strips and tiles: 40 is not a multiple of the 32-, 58- or 64-column
    # strips, so the wrap is taken inside a strip and by a lane other than the last
    "tgv40_partial_tiles": (40, dict(ren=1000.0, dt=0.5 * 2 * math.pi / 40, prob_hi=(2 * math.pi,) * 3,
                                     bc_lo=(111,) * 3, bc_hi=(111,) * 3, fix_quirks=1),
                            dict(ren=1000.0, fixed_dt=0.5 * 2 * math.pi / 40, prob_hi=(2 * math.pi,) * 3,
                                 bc_lo=(111,) * 3, bc_hi=(111,) * 3, fix_quirks=1), 1),
}


def make_pair(name, precision=ns.PREC_FP64_EXACT, tol=1e-12, **extra):
    n, okw, gkw, case = CASES[name]
    o = Oracle(n, iter_num=100, poisson_tol=min(tol, 1e-13), **okw)
    o.init(case)
    p = ns.default_params(n_cell=n, iter_num=100, precision=precision, poisson_tol_rel=tol, **gkw, **extra)
    s = ns.Solver(p)
    s.init(case)
    return o, s


def sync_state(o, s):
    u, up, p, _ = o.get_state()
    s.set_state(u, up, p)
    o.set_state(u, up, p)


@pytest.mark.parametrize("name", ["cavity32", "cavity40_partial_tiles", "cavity128_4boxes", "tgv64_parity", "tgv64_fixed",
                                  "tgv40_partial_tiles"])
def test_rk_stages_bit_exact(gpu_lib, oracle_lib, name):
    o, s = make_pair(name)
    for _ in range(3):
        o.step()
    sync_state(o, s)
    o.step_begin()
    s.step_begin()
    for it in range(2):
        for sub in range(4):
            o.rk_stage(sub)
            s.rk_stage(sub)
            for d in range(2):
                np.testing.assert_array_equal(s.get_field(ns.FIELD_VEL_STAR, d), o.field(FIELD_STAR, d),
                                              err_msg="stage %d comp %d" % (sub, d))
        eo = o.pseudo_norm()
        eg = s.pseudo_norm()
        assert abs(eg - eo) <= 1e-13 * abs(eo), (eg, eo)


def test_first_stage_uses_analytic_cell_velocity(gpu_lib, oracle_lib):
    """hybrid_grid_init sets velCart analytically; the first stage must use it."""
    o, s = make_pair("tgv64_parity")
    o.step_begin()
    s.step_begin()
    o.rk_stage(0)
    s.rk_stage(0)
    for d in range(2):
        np.testing.assert_array_equal(s.get_field(ns.FIELD_VEL_STAR, d), o.field(FIELD_STAR, d))


def test_explicit_predictor_bit_exact(gpu_lib, oracle_lib):
    n, okw, gkw, case = CASES["cavity32"]
    o = Oracle(n, iter_num=100, pseudo_timestepping=0, **okw)
    o.init(case)
    for _ in range(2):
        o.step()
    p = ns.default_params(n_cell=n, pseudo_timestepping=0, precision=ns.PREC_FP64_EXACT, **gkw)
    s = ns.Solver(p)
    s.init(case)
    sync_state(o, s)
    o.step_begin()
    s.step_begin()
    eo = o.explicit_predictor()
    eg = s.explicit_predictor()
    for d in range(2):
        np.testing.assert_array_equal(s.get_field(ns.FIELD_VEL_STAR, d), o.field(FIELD_STAR, d))
    assert abs(eg - eo) <= 1e-13 * abs(eo)


@pytest.mark.parametrize("precision", [ns.PREC_FP64, ns.PREC_MIXED])
@pytest.mark.parametrize("name", ["cavity128_4boxes", "tgv64_fixed"])
def test_poisson_and_projection(gpu_lib, oracle_lib, name, precision):
    o, s = make_pair(name, precision=ns.PREC_FP64_EXACT, tol=1e-12)
    for _ in range(2):
        o.step()
    sync_state(o, s)
    o.step_begin()
    s.step_begin()
    for _ in range(200):
        for sub in range(4):
            o.rk_stage(sub)
            s.rk_stage(sub)
        eo, eg = o.pseudo_norm(), s.pseudo_norm()
        if eo <= 1e-10:
            break
    assert eg <= 1e-10
    do, so_ = o.poisson_rhs()
    dg, sg = s.poisson_rhs()
    assert abs(dg - do) <= 1e-14 * abs(do)
    np.testing.assert_array_equal(s.get_field(ns.FIELD_POISSON_RHS), o.field(12))
    o.poisson_solve()
    cyc, res = s.poisson_solve(precision)
    assert res <= 1e-12 and cyc >= 1
    dao = o.project()
    dag = s.project()
    phig, phio = s.get_field(ns.FIELD_PHI), o.field(11)  # userCtx comp 1 after the copy
    assert relp(phig, phio) <= 1e-10
    assert dag <= 1e-10 * max(1.0, 1.5 / o.params.dt) and dag <= 1e-9
    u, _, p, _ = s.get_state()
    uo, _, po, _ = o.get_state()
    for d in range(2):
        assert rel(u[d], uo[d]) <= TOL_STEP
    assert relp(p, po) <= TOL_STEP


@pytest.mark.parametrize("name,nsteps", [("cavity32", 11), ("cavity128_4boxes", 6), ("tgv64_parity", 6), ("tgv64_fixed", 6)])
def test_steps_resynced(gpu_lib, oracle_lib, name, nsteps):
    """Per-step parity: both sides start every step from the oracle's state."""
    o, s = make_pair(name)
    for step in range(nsteps):
        sync_state(o, s)
        so = o.step()
        sg = s.step()
        assert sg["pseudo_iters"] == so["pseudo_iters"], (step, sg, so)
        u, _, p, _ = s.get_state()
        uo, _, po, _ = o.get_state()
        for d in range(2):
            assert rel(u[d], uo[d]) <= TOL_STEP, (step, d, rel(u[d], uo[d]))
        assert relp(p, po) <= TOL_STEP, (step, relp(p, po))
        assert sg["div_after"] <= 1e-9


def test_free_running_matches_golden(gpu_lib):
    """The shipped inputs physics, 11 free-running steps, against the committed fixture."""
    import os

    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "cavity32_exec_inputs.npz"))
    p = ns.default_params(n_cell=32, precision=ns.PREC_FP64_EXACT, poisson_tol_rel=1e-13)
    s = ns.Solver(p)
    s.init(ns.INIT_CAVITY)
    for step in range(1, 12):
        st = s.step()
        assert st["pseudo_iters"] == int(g["K"][step - 1])
        u, _, pp, _ = s.get_state()
        assert rel(u[0], g["u_%d" % step]) <= TOL_STEP
        assert rel(u[1], g["v_%d" % step]) <= TOL_STEP
        assert relp(pp, g["p_%d" % step]) <= TOL_STEP


@pytest.mark.parametrize("name", ["cavity128_4boxes", "tgv64_parity", "tgv64_fixed", "cavity40_partial_tiles",
                                  "tgv40_partial_tiles"])
def test_mixed_predictor_matches_fp64(gpu_lib, name):
    """Float-float anchor + FP32 increments reproduce the FP64 iterates.

    Both solvers start from the same state; the mixed predictor must take the
    same number of pseudo-iterations and give u, v, p within 1e-11 (relative
    L2) of the FP64 predictor (both with the FP64 Poisson solve).
    """
    n, okw, gkw, case = CASES[name]
    sol = {}
    for prec in (ns.PREC_FP64_EXACT, ns.PREC_MIXED):
        p = ns.default_params(n_cell=n, iter_num=100, precision=prec, poisson_tol_rel=1e-13, **gkw)
        s = ns.Solver(p)
        s.init(case)
        sol[prec] = s
    ref = sol[ns.PREC_FP64_EXACT]
    for _ in range(2):
        ref.step()
    u, up, pp, _ = ref.get_state()
    for s in sol.values():
        s.set_state(u, up, pp)
    for step in range(3):
        st = {k: s.step() for k, s in sol.items()}
        assert st[ns.PREC_MIXED]["pseudo_iters"] == st[ns.PREC_FP64_EXACT]["pseudo_iters"], st
        a = sol[ns.PREC_MIXED].get_state()
        b = ref.get_state()
        for d in range(2):
            assert rel(a[0][d], b[0][d]) <= 1e-11, (step, d, rel(a[0][d], b[0][d]))
        assert relp(a[2], b[2]) <= 1e-11, (step, relp(a[2], b[2]))


@pytest.mark.parametrize("precision", [ns.PREC_FP64, ns.PREC_MIXED])
def test_fast_modes_track_oracle(gpu_lib, oracle_lib, precision):
    o, s = make_pair("cavity128_4boxes", precision=precision)
    for step in range(4):
        sync_state(o, s)
        so = o.step()
        sg = s.step()
        u, _, p, _ = s.get_state()
        uo, _, po, _ = o.get_state()
        for d in range(2):
            assert rel(u[d], uo[d]) <= 1e-9, (step, d)
        assert relp(p, po) <= 1e-9
        assert abs(sg["pseudo_iters"] - so["pseudo_iters"]) <= 1


BC_CASES = {
    # name: (bc_lo, bc_hi, fix_quirks)
    "south_slip": ((135, -135, 135), (135, 165, 135), 0),
    "west_slip": ((-135, 135, 135), (135, 165, 135), 0),
    "east_slip_code1": ((135, 135, 135), (1, 165, 135), 0),       # quirk Q5: east slip is tested as == 1
    "east_slip_fixed": ((135, 135, 135), (-135, 165, 135), 1),
    "west_inlet_165": ((165, 135, 135), (135, 165, 135), 0),
    "west_inlet_m165": ((-165, 135, 135), (135, 135, 135), 0),
    "south_inlet": ((135, 165, 135), (135, 135, 135), 0),
}


@pytest.mark.parametrize("precision", [ns.PREC_FP64_EXACT, ns.PREC_MIXED])
@pytest.mark.parametrize("name", sorted(BC_CASES))
def test_bc_codes_resynced(gpu_lib, oracle_lib, name, precision):
    """Wall, slip and inlet codes of utilities.cpp:62-349 on every side: per-step
    parity with the oracle (both sides start each step from the oracle's state)."""
    lo, hi, fq = BC_CASES[name]
    n = 48
    o = Oracle(n, ren=100.0, dt=2e-3, iter_num=100, poisson_tol=1e-13, max_grid_size=(n, n, n), bc_lo=lo, bc_hi=hi,
               fix_quirks=fq)
    o.init(0)
    p = ns.default_params(n_cell=n, ren=100.0, fixed_dt=2e-3, iter_num=100, precision=precision, poisson_tol_rel=1e-12,
                          max_grid_size=(n, n, n), bc_lo=lo, bc_hi=hi, fix_quirks=fq)
    s = ns.Solver(p)
    s.init(ns.INIT_CAVITY)
    tol = TOL_STEP if precision == ns.PREC_FP64_EXACT else 1e-9
    for step in range(4):
        if step > 0:
            sync_state(o, s)
        so = o.step()
        sg = s.step()
        assert sg["pseudo_iters"] == so["pseudo_iters"], (name, step, sg["pseudo_iters"], so["pseudo_iters"])
        u, _, pg, _ = s.get_state()
        uo, _, po, _ = o.get_state()
        for d in range(2):
            assert rel(u[d], uo[d]) <= tol, (name, step, d, rel(u[d], uo[d]))
        assert relp(pg, po) <= tol, (name, step, relp(pg, po))
    o.close()
    s.close()


def test_east_slip_code_m135_unsupported_in_parity_mode(gpu_lib):
    """The reference leaves stale ghosts for an east -135 wall (it tests slip as
    == 1, quirk Q5); the parity mode refuses it instead of guessing."""
    p = ns.default_params(n_cell=32, bc_lo=(135, 135, 135), bc_hi=(-135, 165, 135), fix_quirks=0)
    with pytest.raises(ns.NsError):
        ns.Solver(p)


@pytest.mark.parametrize("name", ["cavity32", "cavity128_4boxes", "tgv64_parity", "tgv64_fixed"])
def test_gmres_option_resynced(gpu_lib, oracle_lib, name):
    """The GMRES option of the Poisson solve (GMRES_Poisson.cpp:56-131, here
    with one V-cycle as the right preconditioner) reaches the same discrete
    solution: per-step parity with the oracle, like the V-cycle solver."""
    o, s = make_pair(name, poisson_solver=1, gmres_restart=20)
    for step in range(3):
        sync_state(o, s)
        so = o.step()
        sg = s.step()
        assert sg["pseudo_iters"] == so["pseudo_iters"]
        assert sg["poisson_res"] <= 1e-12 and sg["poisson_cycles"] >= 1
        u, _, p, _ = s.get_state()
        uo, _, po, _ = o.get_state()
        for d in range(2):
            assert rel(u[d], uo[d]) <= TOL_STEP, (step, d, rel(u[d], uo[d]))
        assert relp(p, po) <= TOL_STEP


def test_gmres_matches_vcycles(gpu_lib):
    sols = {}
    for solver in (0, 1):
        p = ns.default_params(n_cell=128, ren=100.0, fixed_dt=0.5 / 128, precision=ns.PREC_FP64, poisson_tol_rel=1e-13,
                              poisson_solver=solver, gmres_restart=8)
        s = ns.Solver(p)
        s.init(ns.INIT_CAVITY)
        for _ in range(2):
            st = s.step()
        sols[solver] = (s.get_state(), st)
    (ua, _, pa, _), sta = sols[0]
    (ub, _, pb, _), stb = sols[1]
    for d in range(2):
        assert rel(ub[d], ua[d]) <= 1e-11
    assert relp(pb, pa) <= 1e-11
    # restarts of 8 vectors: more Krylov iterations than 8 are possible, and fine
    assert stb["poisson_cycles"] <= 4 * max(sta["poisson_cycles"], 1)


@pytest.mark.parametrize("name,precision", [("cavity32", ns.PREC_FP64_EXACT), ("cavity32", ns.PREC_MIXED),
                                            ("tgv64_fixed", ns.PREC_FP64_EXACT), ("tgv64_parity", ns.PREC_MIXED)])
def test_explicit_steps_resynced(gpu_lib, oracle_lib, name, precision):
    """PSEUDO_TIMESTEPPING = 0 (main.cpp:902-925): whole steps per step against
    the oracle, K = 1 on both sides, u and p within 1e-10 (the velocity over
    both components, relative to the whole field), the post-step max|div u|,
    which the explicit mode's missing reflection (quirk Q3) keeps above
    round-off on the cavity, within 1e-8. The mixed mode runs this predictor
    in FP64 and its Poisson solve in FP32 V-cycles inside the defect
    correction."""
    n, okw, gkw, case = CASES[name]
    o = Oracle(n, iter_num=100, poisson_tol=1e-13, pseudo_timestepping=0, **okw)
    o.init(case)
    p = ns.default_params(n_cell=n, iter_num=100, precision=precision, poisson_tol_rel=1e-12, pseudo_timestepping=0,
                          **gkw)
    s = ns.Solver(p)
    s.init(case)
    for step in range(4):
        sync_state(o, s)
        so = o.step()
        sg = s.step()
        assert sg["pseudo_iters"] == so["pseudo_iters"] == 1
        u, _, pg, _ = s.get_state()
        uo, _, po, _ = o.get_state()
        ru = math.sqrt(sum(np.linalg.norm(u[d] - uo[d]) ** 2 for d in range(2)) /
                       sum(np.linalg.norm(uo[d]) ** 2 for d in range(2)))
        assert ru <= 1e-10, (step, ru)
        assert relp(pg, po) <= 1e-10, (step, relp(pg, po))
        assert abs(sg["div_after"] - so["div_after"]) <= 1e-8 * so["div_after"] + 1e-12, \
            (step, sg["div_after"], so["div_after"])
