"""The 3D advance (dim = 3): per-step parity with the oracle's 3D restatement
(lid cavity with walls on every side; perturbed periodic Taylor-Green in the
reference's parity mode and in the physical mode), the mixed-precision
predictor (FP64 anchor, FP32 increment stages) and Poisson solve (FP32
V-cycles inside FP64 defect correction) against the FP64 ones, and the
discrete divergence after every step.

Tolerances: relative L2 <= 1e-10 per step in u, v, w and p (p modulo its
constant), identical pseudo-iteration counts; mixed vs FP64 <= 1e-10."""
import math

import numpy as np
import pytest

import amressif_gb300 as ns
from amressif_gb300 import workloads as wl

pytestmark = pytest.mark.gpu


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


def relp(a, b):
    return rel(a - a.mean(), b - b.mean())


L2PI = 2 * math.pi
CASES3 = {
    # name: (n, kwargs shared by the oracle and the GPU, periodic TGV input)
    "cavity16": (16, dict(ren=100.0, bc_lo=(135, 135, 135), bc_hi=(135, 165, 135)), False),
    # a west inlet (-165), slip walls south, bottom and top, the east code 1 that the reference
    # reads as slip, and the lid: every ghost rule of cont2cart (utilities.cpp:62-349) in 3D
    "walls16": (16, dict(ren=100.0, bc_lo=(-165, -135, -135), bc_hi=(1, 165, -135)), False),
    "tgv16_parity": (16, dict(ren=1600.0, prob_hi=(L2PI,) * 3, bc_lo=(111,) * 3, bc_hi=(111,) * 3), True),
    "tgv24_fixed": (24, dict(ren=1600.0, prob_hi=(L2PI,) * 3, bc_lo=(111,) * 3, bc_hi=(111,) * 3, fix_quirks=1), True),
}


def state3(n, tgv):
    if tgv:
        return wl.tgv3d_perturbed_state(n, amp=1e-3, seed=0)
    z = [np.zeros((n, n, n + 1)), np.zeros((n, n + 1, n)), np.zeros((n + 1, n, n))]
    return z, [a.copy() for a in z], np.zeros((n, n, n))


def dt_of(n, kw):
    h = kw.get("prob_hi", (1.0,))[0] / n
    return 0.4 * h


@pytest.mark.parametrize("name", sorted(CASES3))
def test_3d_steps_resynced(gpu_lib, oracle_lib, name):
    from oracle.orc import Oracle

    n, kw, tgv = CASES3[name]
    dt = dt_of(n, kw)
    o = Oracle(n, dim=3, dt=dt, iter_num=100, poisson_tol=1e-13, max_grid_size=(n, n, n), **kw)
    p = ns.default_params(dim=3, n_cell=n, fixed_dt=dt, iter_num=100, precision=ns.PREC_FP64, poisson_tol_rel=1e-12,
                          max_grid_size=(n, n, n), **kw)
    s = ns.Solver(p)
    u, up, pp = state3(n, tgv)
    o.set_state(u, up, pp)
    for step in range(3):
        uo, upo, po, _ = o.get_state()
        s.set_state(uo, upo, po)
        so = o.step()
        sg = s.step()
        assert sg["pseudo_iters"] == so["pseudo_iters"], (step, sg["pseudo_iters"], so["pseudo_iters"])
        ug, _, pg, _ = s.get_state()
        uo, _, po, _ = o.get_state()
        for d in range(3):
            assert rel(ug[d], uo[d]) <= 1e-10, (step, d, rel(ug[d], uo[d]))
        assert relp(pg, po) <= 1e-10, (step, relp(pg, po))
        if kw.get("fix_quirks") or not tgv:
            assert sg["div_after"] <= 1e-10
    o.close()


@pytest.mark.parametrize("dc_residual", [0, 1])
def test_3d_mixed_poisson_matches_fp64(gpu_lib, dc_residual):
    """The mixed solve (FP32 V-cycles inside the defect correction; its
    residual and phi in float-float, dc_residual 0, or FP64, 1) against the
    FP64 solver over three steps: the same pseudo-iteration counts, u and p
    within 1e-10."""
    n = 32
    kw = dict(ren=1600.0, prob_hi=(L2PI,) * 3, bc_lo=(111,) * 3, bc_hi=(111,) * 3, fix_quirks=1)
    dt = dt_of(n, kw)
    out = {}
    for prec in (ns.PREC_FP64, ns.PREC_MIXED):
        p = ns.default_params(dim=3, n_cell=n, fixed_dt=dt, iter_num=100, precision=prec, poisson_tol_rel=1e-12,
                              poisson_tol_div=1e-10, max_grid_size=(n, n, n), dc_residual=dc_residual, **kw)
        s = ns.Solver(p)
        s.set_state(*wl.tgv3d_perturbed_state(n, amp=1e-3, seed=0))
        ks = [s.step()["pseudo_iters"] for _ in range(3)]
        out[prec] = (ks, s.get_state())
    assert out[ns.PREC_FP64][0] == out[ns.PREC_MIXED][0]
    (ua, _, pa, _), (ub, _, pb, _) = out[ns.PREC_FP64][1], out[ns.PREC_MIXED][1]
    for d in range(3):
        assert rel(ub[d], ua[d]) <= 1e-10
    assert relp(pb, pa) <= 1e-10


# the fused increment stage works on 32 x 8 column tiles and 16-plane chunks:
# these add two x tiles with a partial one (40, walls) and face N at the
# start of a further x tile (32 and 64, periodic)
CASES3_MIXED = dict(CASES3)
CASES3_MIXED.update({
    "cavity40": (40, dict(ren=100.0, bc_lo=(135, 135, 135), bc_hi=(135, 165, 135)), False),
    "tgv32_fixed": (32, dict(ren=1600.0, prob_hi=(L2PI,) * 3, bc_lo=(111,) * 3, bc_hi=(111,) * 3, fix_quirks=1), True),
    "tgv64_parity": (64, dict(ren=1600.0, prob_hi=(L2PI,) * 3, bc_lo=(111,) * 3, bc_hi=(111,) * 3), True),
})


@pytest.mark.parametrize("name", sorted(CASES3_MIXED))
def test_3d_mixed_predictor_matches_fp64(gpu_lib, name):
    """FP64 anchor + FP32 increment stages against the FP64 predictor on the
    same steps (both with FP64-accurate Poisson solves): identical
    pseudo-iteration counts and u, p within 1e-11 (relative L2)."""
    n, kw, tgv = CASES3_MIXED[name]
    dt = dt_of(n, kw)
    out = {}
    tol = 1e-13 if n < 64 else 1e-12  # at 64^3 the mixed solve's floor is above 1e-13
    for prec in (ns.PREC_FP64, ns.PREC_MIXED):
        p = ns.default_params(dim=3, n_cell=n, fixed_dt=dt, iter_num=100, precision=prec, poisson_tol_rel=tol,
                              max_grid_size=(n, n, n), **kw)
        s = ns.Solver(p)
        s.set_state(*state3(n, tgv))
        ks = [s.step()["pseudo_iters"] for _ in range(4)]
        out[prec] = (ks, s.get_state())
        s.close()
    assert out[ns.PREC_FP64][0] == out[ns.PREC_MIXED][0]
    (ua, _, pa, _), (ub, _, pb, _) = out[ns.PREC_FP64][1], out[ns.PREC_MIXED][1]
    for d in range(3):
        assert rel(ub[d], ua[d]) <= 1e-11, (d, rel(ub[d], ua[d]))
    assert relp(pb, pa) <= 1e-11, relp(pb, pa)


@pytest.mark.parametrize("name", sorted(CASES3))
def test_3d_building_blocks(gpu_lib, oracle_lib, name):
    """The per-call-site entry points on a 3D context (main.cpp:879-1180):
    the RK stages against the oracle's 3D stages (the GPU's FP64 stage uses
    FMA, so agreement is to round-off, 1e-13 relative), the pseudo-norm, the
    Poisson right-hand side, solve and projection against the oracle's
    (1e-10); and a step assembled from the blocks equal, bit for bit, to
    ns_step on another context from the same state."""
    from oracle.orc import FIELD_PRHS, FIELD_STAR, Oracle

    n, kw, tgv = CASES3[name]
    dt = dt_of(n, kw)
    o = Oracle(n, dim=3, dt=dt, iter_num=100, poisson_tol=1e-13, max_grid_size=(n, n, n), **kw)
    mk = lambda: ns.Solver(ns.default_params(dim=3, n_cell=n, fixed_dt=dt, iter_num=100, precision=ns.PREC_FP64,
                                             poisson_tol_rel=1e-13, max_grid_size=(n, n, n), **kw))
    s, t = mk(), mk()
    u, up, pp = state3(n, tgv)
    o.set_state(u, up, pp)
    o.step()
    uo, upo, po, _ = o.get_state()
    for x in (o, s, t):
        x.set_state(uo, upo, po)
    o.step_begin()
    s.step_begin()
    # the pseudo-increments near convergence (norm ~1e-11) carry the round-off of
    # the velocities, which the GPU's FMA and the oracle's separate roundings make
    # differently: the norms agree to 1e-9 relative or to eps max|u| absolute
    floor = 2.2e-16 * max(float(np.abs(a).max()) for a in uo)
    K = 0
    while True:
        for sub in range(4):
            o.rk_stage(sub)
            s.rk_stage(sub)
        if K == 0:
            for d in range(3):
                assert rel(s.get_field(ns.FIELD_VEL_STAR, d), o.field(FIELD_STAR, d)) <= 1e-13
        eo, eg = o.pseudo_norm(), s.pseudo_norm()
        assert abs(eg - eo) <= 1e-9 * eo + floor, (K, eg, eo)
        K += 1
        if eo <= 1e-10 or K > 100:
            break
    assert eg <= 1e-10
    do, so_ = o.poisson_rhs()
    dg, sg = s.poisson_rhs()
    assert abs(dg - do) <= 1e-10 * abs(do)
    assert rel(s.get_field(ns.FIELD_POISSON_RHS), o.field(FIELD_PRHS)) <= 1e-10
    o.poisson_solve()
    cyc, res = s.poisson_solve(ns.PREC_FP64)
    assert res <= 1e-13 and cyc >= 1
    o.project()
    dag = s.project()
    ug, _, pg, _ = s.get_state()
    uo, _, po, _ = o.get_state()
    for d in range(3):
        assert rel(ug[d], uo[d]) <= 1e-10, (d, rel(ug[d], uo[d]))
    assert relp(pg, po) <= 1e-10
    if kw.get("fix_quirks") or not tgv:
        assert dag <= 1e-10
    # the same step through ns_step
    st = t.step()
    assert st["pseudo_iters"] == K
    ut, _, pt, _ = t.get_state()
    for d in range(3):
        np.testing.assert_array_equal(ug[d], ut[d])
    np.testing.assert_array_equal(pg, pt)
    o.close()


EXPLICIT3 = [(name, ns.PREC_FP64) for name in sorted(CASES3)] + \
    [("cavity16", ns.PREC_MIXED), ("tgv24_fixed", ns.PREC_MIXED)]


@pytest.mark.parametrize("name,precision", EXPLICIT3)
def test_3d_explicit_steps_resynced(gpu_lib, oracle_lib, name, precision):
    """PSEUDO_TIMESTEPPING = 0 in the AMREX_SPACEDIM = 3 build
    (explicit_time_marching, momentum.cpp:96-192, main.cpp:902-925): one
    predictor pass a step (K = 1), no flux reflection at walls (quirk Q3).
    Per-step parity with the oracle's 3D restatement: the velocity (all three
    components, relative to the whole field: the first cavity step from rest
    sees only the lid ghost, so u* is uniform in z and w is round-off on both
    sides) and p within 1e-10, and max|div u| after the projection, which Q3
    (cavity) and Q1/Q2 (the periodic box in parity mode) keep well above
    round-off, within 1e-8 of the oracle's. The mixed mode runs this
    predictor in FP64 and its Poisson solve in FP32 V-cycles inside the
    float-float defect correction."""
    from oracle.orc import Oracle

    n, kw, tgv = CASES3[name]
    dt = dt_of(n, kw)
    o = Oracle(n, dim=3, dt=dt, iter_num=100, poisson_tol=1e-13, max_grid_size=(n, n, n), pseudo_timestepping=0,
               **kw)
    p = ns.default_params(dim=3, n_cell=n, fixed_dt=dt, iter_num=100, precision=precision, poisson_tol_rel=1e-12,
                          max_grid_size=(n, n, n), pseudo_timestepping=0, **kw)
    s = ns.Solver(p)
    o.set_state(*state3(n, tgv))
    for step in range(4):
        uo, upo, po, _ = o.get_state()
        s.set_state(uo, upo, po)
        so = o.step()
        sg = s.step()
        assert sg["pseudo_iters"] == so["pseudo_iters"] == 1
        assert abs(sg["norm_error"] - so["norm_error"]) <= 1e-9 * so["norm_error"], (step, sg["norm_error"])
        ug, _, pg, _ = s.get_state()
        uo, _, po, _ = o.get_state()
        ru = math.sqrt(sum(np.linalg.norm(ug[d] - uo[d]) ** 2 for d in range(3)) /
                       sum(np.linalg.norm(uo[d]) ** 2 for d in range(3)))
        assert ru <= 1e-10, (step, ru)
        assert relp(pg, po) <= 1e-10, (step, relp(pg, po))
        assert abs(sg["div_after"] - so["div_after"]) <= 1e-8 * so["div_after"] + 1e-12, \
            (step, sg["div_after"], so["div_after"])
    o.close()


def test_3d_explicit_predictor_building_block(gpu_lib, oracle_lib):
    """ns_explicit_predictor on a 3D context against the oracle's: u* within
    round-off (the GPU's FP64 passes use FMA; 1e-13 relative) and the
    pseudo-increment norm within 1e-9."""
    from oracle.orc import FIELD_STAR, Oracle

    n, kw, tgv = CASES3["cavity16"]
    dt = dt_of(n, kw)
    o = Oracle(n, dim=3, dt=dt, iter_num=100, poisson_tol=1e-13, max_grid_size=(n, n, n), pseudo_timestepping=0,
               **kw)
    s = ns.Solver(ns.default_params(dim=3, n_cell=n, fixed_dt=dt, iter_num=100, precision=ns.PREC_FP64,
                                    max_grid_size=(n, n, n), pseudo_timestepping=0, **kw))
    o.set_state(*state3(n, tgv))
    o.step()
    o.step()
    uo, upo, po, _ = o.get_state()
    o.set_state(uo, upo, po)
    s.set_state(uo, upo, po)
    o.step_begin()
    s.step_begin()
    eo = o.explicit_predictor()
    eg = s.explicit_predictor()
    for d in range(3):
        assert rel(s.get_field(ns.FIELD_VEL_STAR, d), o.field(FIELD_STAR, d)) <= 1e-13
    assert abs(eg - eo) <= 1e-9 * eo, (eg, eo)
    o.close()


TGV3_INIT = {
    # the reference's Taylor-Green init in the 3D build: the 2D vortex in every z plane
    "tgv16_init_parity": (16, dict(ren=100.0, prob_hi=(L2PI,) * 3, bc_lo=(111,) * 3, bc_hi=(111,) * 3)),
    "tgv16_init_fixed": (16, dict(ren=100.0, prob_hi=(L2PI,) * 3, bc_lo=(111,) * 3, bc_hi=(111,) * 3, fix_quirks=1)),
}


@pytest.mark.parametrize("name", sorted(TGV3_INIT))
def test_3d_tgv_init_first_stage_and_steps(gpu_lib, oracle_lib, name):
    """ns_init_fields(NS_INIT_TGV) on a 3D context against the oracle's
    hybrid_grid_init (fn_init.cpp:61-229): the same initial state, the first
    stage on the analytic cell velocity (w = 0) within 1e-13, and three
    free-running FP64 steps within 1e-10 with the same pseudo-iteration
    counts."""
    from oracle.orc import FIELD_STAR, Oracle

    n, kw = TGV3_INIT[name]
    dt = dt_of(n, kw)
    mk_o = lambda: Oracle(n, dim=3, dt=dt, iter_num=100, poisson_tol=1e-13, max_grid_size=(n, n, n), **kw)
    mk_s = lambda: ns.Solver(ns.default_params(dim=3, n_cell=n, fixed_dt=dt, iter_num=100, precision=ns.PREC_FP64,
                                               poisson_tol_rel=1e-12, max_grid_size=(n, n, n), **kw))
    o, s = mk_o(), mk_s()
    o.init(1)
    s.init(ns.INIT_TGV)
    ug, upg, pg, _ = s.get_state()
    uo, upo, po, _ = o.get_state()
    for d in range(3):
        np.testing.assert_array_equal(ug[d], uo[d])
        np.testing.assert_array_equal(upg[d], upo[d])
    np.testing.assert_array_equal(pg, po)
    o.step_begin()
    s.step_begin()
    o.rk_stage(0)
    s.rk_stage(0)
    for d in range(3):
        assert rel(s.get_field(ns.FIELD_VEL_STAR, d), o.field(FIELD_STAR, d)) <= 1e-13 if d < 2 else \
            np.abs(s.get_field(ns.FIELD_VEL_STAR, d)).max() <= 1e-14
    o.close()
    s.close()
    o, s = mk_o(), mk_s()
    o.init(1)
    s.init(ns.INIT_TGV)
    for step in range(3):
        so = o.step()
        sg = s.step()
        assert sg["pseudo_iters"] == so["pseudo_iters"], (step, sg["pseudo_iters"], so["pseudo_iters"])
        ug, _, pg, _ = s.get_state()
        uo, _, po, _ = o.get_state()
        ru = math.sqrt(sum(np.linalg.norm(ug[d] - uo[d]) ** 2 for d in range(3)) /
                       sum(np.linalg.norm(uo[d]) ** 2 for d in range(3)))
        assert ru <= 1e-10, (step, ru)
        assert relp(pg, po) <= 1e-10, (step, relp(pg, po))
    o.close()


def test_3d_tgv_init_mixed_matches_fp64(gpu_lib):
    """The mixed predictor after ns_init_fields(NS_INIT_TGV): its first
    pseudo-iteration runs in FP64 on the analytic cell velocity, the rest in
    mixed precision; three steps against the FP64 solver (same
    pseudo-iteration counts, u and p within 1e-11)."""
    n, kw = TGV3_INIT["tgv16_init_fixed"]
    dt = dt_of(n, kw)
    out = []
    for prec in (ns.PREC_FP64, ns.PREC_MIXED):
        s = ns.Solver(ns.default_params(dim=3, n_cell=n, fixed_dt=dt, iter_num=100, precision=prec,
                                        poisson_tol_rel=1e-12, max_grid_size=(n, n, n), **kw))
        s.init(ns.INIT_TGV)
        ks = [s.step()["pseudo_iters"] for _ in range(3)]
        u, _, p, _ = s.get_state()
        out.append((ks, u, p))
        s.close()
    assert out[0][0] == out[1][0]
    ru = math.sqrt(sum(np.linalg.norm(out[1][1][d] - out[0][1][d]) ** 2 for d in range(3)) /
                   sum(np.linalg.norm(out[0][1][d]) ** 2 for d in range(3)))
    assert ru <= 1e-11, ru
    assert relp(out[1][2], out[0][2]) <= 1e-11


@pytest.mark.parametrize("name", sorted(CASES3))
def test_3d_gmres_option_resynced(gpu_lib, oracle_lib, name):
    """poisson_solver = 1 in the 3D build (the GMRES option of
    GMRES_Poisson.cpp:56-131, whose operator has a 7-point branch): restarted
    GMRES with one FP64 V-cycle as right preconditioner, per step against the
    oracle's exact solve (u, p within 1e-10, identical pseudo-iteration
    counts), and against the V-cycle solver on the same state."""
    from oracle.orc import Oracle

    n, kw, tgv = CASES3[name]
    dt = dt_of(n, kw)
    o = Oracle(n, dim=3, dt=dt, iter_num=100, poisson_tol=1e-13, max_grid_size=(n, n, n), **kw)
    mk = lambda solver: ns.Solver(ns.default_params(dim=3, n_cell=n, fixed_dt=dt, iter_num=100, precision=ns.PREC_FP64,
                                                    poisson_tol_rel=1e-12, max_grid_size=(n, n, n),
                                                    poisson_solver=solver, **kw))
    s, t = mk(1), mk(0)
    o.set_state(*state3(n, tgv))
    for step in range(3):
        uo, upo, po, _ = o.get_state()
        s.set_state(uo, upo, po)
        t.set_state(uo, upo, po)
        so = o.step()
        sg = s.step()
        st = t.step()
        assert sg["pseudo_iters"] == so["pseudo_iters"], (step, sg["pseudo_iters"], so["pseudo_iters"])
        assert sg["poisson_cycles"] >= 1 and sg["poisson_res"] <= 1e-12
        ug, _, pg, _ = s.get_state()
        ut, _, pt, _ = t.get_state()
        uo, _, po, _ = o.get_state()
        for d in range(3):
            assert rel(ug[d], uo[d]) <= 1e-10, (step, d, rel(ug[d], uo[d]))
            assert rel(ug[d], ut[d]) <= 1e-10, (step, d, rel(ug[d], ut[d]))
        assert relp(pg, po) <= 1e-10, (step, relp(pg, po))
        if kw.get("fix_quirks") or not tgv:
            assert sg["div_after"] <= 1e-10
    o.close()



def test_3d_free_running_matches_golden(gpu_lib):
    """The committed 3D fixture (the oracle's 16^3 lid cavity, 5 free-running
    steps from rest) against the FP64 3D path: the same pseudo-iteration
    counts, the final velocity (all components) and p within 1e-10."""
    import os

    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "cavity16_3d.npz"))
    n = 16
    s = ns.Solver(ns.default_params(dim=3, n_cell=n, fixed_dt=0.4 / n, iter_num=100, precision=ns.PREC_FP64,
                                    poisson_tol_rel=1e-13, max_grid_size=(n, n, n), ren=100.0,
                                    bc_lo=(135, 135, 135), bc_hi=(135, 165, 135)))
    s.init(ns.INIT_CAVITY)
    for step in range(int(g["nsteps"])):
        st = s.step()
        assert st["pseudo_iters"] == int(g["K"][step]), (step, st["pseudo_iters"])
    u, _, p, _ = s.get_state()
    ru = math.sqrt(sum(np.linalg.norm(u[d] - g[k]) ** 2 for d, k in enumerate("uvw")) /
                   sum(np.linalg.norm(g[k]) ** 2 for k in "uvw"))
    assert ru <= 1e-10, ru
    assert relp(p, g["p"]) <= 1e-10
