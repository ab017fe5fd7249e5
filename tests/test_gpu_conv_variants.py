"""The reference's two alternative convective routines on the CUDA path,
against the oracle: convective_flux_calc_quick (NS_CONV_QUICK,
fn_flux_calc.cpp:204-393; 2D, one box) and convective_flux_calc
(NS_CONV_UMIST_FORM, fn_flux_calc.cpp:395-692, which leaves the total flux
without a convective term; 2D and 3D).

Tolerances as for the default QUICK routine: the FP64 exact mode reproduces
the oracle's pseudo-stages bit for bit; whole steps agree to a relative L2 of
1e-10 in u, v and p (modulo its constant) with identical pseudo-iteration
counts; the FP64 mode with reciprocal multiplies to 1e-9. Without a convective
term the periodic Taylor-Green box carries almost no pressure (max|p - mean p|
about 1e-4, against 0.3-0.5 with QUICK, for max|u| about 1): both solves meet
their tolerance relative to the Poisson right-hand side, so p (modulo its
constant) is compared relative to the larger of its own norm and the
dynamic-pressure scale max|u|^2 per cell.
"""
import math

import numpy as np
import pytest

import amressif_gb300 as ns
from oracle.orc import FIELD_STAR, Oracle

pytestmark = pytest.mark.gpu

L2PI = 2 * math.pi
CASES = {
    # name: (n, shared kwargs, oracle dt / gpu fixed_dt, init case); one box each
    # 48 = one and a half 32-column stage tiles: partial tiles at the east wall and the wrap
    "cavity48": (48, dict(ren=100.0), 2e-3, 0),
    "walls40": (40, dict(ren=100.0, bc_lo=(-165, -135, 135), bc_hi=(1, 165, 135)), 2e-3, 0),
    # Re 100 at dt = dx / 4: at Re 1000, dt = dx / 2 the inconsistent convective term of
    # convective_flux_calc_quick blows up within a few steps. Its pseudo-iteration does not
    # converge on this machine either (K reaches IterNum + 1 = 101), which the step parity then covers
    "tgv64_parity": (64, dict(ren=100.0, prob_hi=(L2PI,) * 3, bc_lo=(111,) * 3, bc_hi=(111,) * 3), 0.25 * L2PI / 64, 1),
    "tgv64_fixed": (64, dict(ren=100.0, prob_hi=(L2PI,) * 3, bc_lo=(111,) * 3, bc_hi=(111,) * 3, fix_quirks=1),
                    0.25 * L2PI / 64, 1),
}
SCHEMES = [ns.CONV_QUICK, ns.CONV_UMIST_FORM]


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


def relp(a, b, u):
    a0, b0 = a - a.mean(), b - b.mean()
    scale = max(float(np.abs(x).max()) for x in u) ** 2 * math.sqrt(b.size)
    return np.linalg.norm(a0 - b0) / max(np.linalg.norm(b0), scale)


def make_pair(name, scheme, precision=ns.PREC_FP64_EXACT, **extra):
    n, kw, dt, case = CASES[name]
    o = Oracle(n, iter_num=100, poisson_tol=1e-13, dt=dt, max_grid_size=(n, n, n), conv_scheme=scheme, **kw, **extra)
    o.init(case)
    p = ns.default_params(n_cell=n, iter_num=100, precision=precision, poisson_tol_rel=1e-12, fixed_dt=dt,
                          max_grid_size=(n, n, n), conv_scheme=scheme, **kw, **extra)
    s = ns.Solver(p)
    s.init(case)
    return o, s


def sync_state(o, s):
    u, up, p, _ = o.get_state()
    s.set_state(u, up, p)
    o.set_state(u, up, p)


@pytest.mark.parametrize("scheme", SCHEMES)
@pytest.mark.parametrize("name", sorted(CASES))
def test_conv_variant_stages_bit_exact(gpu_lib, oracle_lib, name, scheme):
    o, s = make_pair(name, scheme)
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
                                              err_msg="iteration %d stage %d comp %d" % (it, sub, d))
        eo = o.pseudo_norm()
        eg = s.pseudo_norm()
        assert abs(eg - eo) <= 1e-13 * abs(eo), (eg, eo)
    o.close()


def test_conv_variant_first_stage_uses_analytic_cell_velocity(gpu_lib, oracle_lib):
    """hybrid_grid_init's analytic velCart feeds convective_flux_calc_quick's
    face values in the first stage of a run."""
    o, s = make_pair("tgv64_parity", ns.CONV_QUICK)
    o.step_begin()
    s.step_begin()
    o.rk_stage(0)
    s.rk_stage(0)
    for d in range(2):
        np.testing.assert_array_equal(s.get_field(ns.FIELD_VEL_STAR, d), o.field(FIELD_STAR, d))
    o.close()


@pytest.mark.parametrize("scheme", SCHEMES)
@pytest.mark.parametrize("name", ["cavity48", "walls40", "tgv64_fixed"])
def test_conv_variant_steps_resynced(gpu_lib, oracle_lib, name, scheme):
    o, s = make_pair(name, scheme)
    for step in range(4):
        sync_state(o, s)
        so = o.step()
        sg = s.step()
        assert sg["pseudo_iters"] == so["pseudo_iters"], (step, sg["pseudo_iters"], so["pseudo_iters"])
        u, _, p, _ = s.get_state()
        uo, _, po, _ = o.get_state()
        for d in range(2):
            assert rel(u[d], uo[d]) <= 1e-10, (step, d, rel(u[d], uo[d]))
        assert relp(p, po, uo) <= 1e-10, (step, relp(p, po, uo))
        assert sg["div_after"] <= 1e-9
    o.close()


@pytest.mark.parametrize("scheme", SCHEMES)
def test_conv_variant_explicit_predictor_bit_exact(gpu_lib, oracle_lib, scheme):
    o, s = make_pair("cavity48", scheme, pseudo_timestepping=0)
    for _ in range(2):
        o.step()
    sync_state(o, s)
    o.step_begin()
    s.step_begin()
    eo = o.explicit_predictor()
    eg = s.explicit_predictor()
    for d in range(2):
        np.testing.assert_array_equal(s.get_field(ns.FIELD_VEL_STAR, d), o.field(FIELD_STAR, d))
    assert abs(eg - eo) <= 1e-13 * abs(eo)
    o.close()


@pytest.mark.parametrize("scheme", SCHEMES)
def test_conv_variant_fp64_mode_tracks_oracle(gpu_lib, oracle_lib, scheme):
    o, s = make_pair("cavity48", scheme, precision=ns.PREC_FP64)
    for step in range(4):
        sync_state(o, s)
        so = o.step()
        sg = s.step()
        u, _, p, _ = s.get_state()
        uo, _, po, _ = o.get_state()
        for d in range(2):
            assert rel(u[d], uo[d]) <= 1e-9, (step, d)
        assert relp(p, po, uo) <= 1e-9
        assert abs(sg["pseudo_iters"] - so["pseudo_iters"]) <= 1
    o.close()


def test_conv_variants_change_the_step(gpu_lib):
    """The three routines give three different steps from the same state."""
    out = []
    for scheme in (ns.CONV_NEW_QUICK, ns.CONV_QUICK, ns.CONV_UMIST_FORM):
        n, kw, dt, case = CASES["cavity48"]
        s = ns.Solver(ns.default_params(n_cell=n, fixed_dt=dt, max_grid_size=(n, n, n), conv_scheme=scheme, **kw))
        s.init(case)
        for _ in range(3):
            s.step()
        out.append(s.get_state()[0][0])
    assert np.abs(out[1] - out[0]).max() > 1e-6
    assert np.abs(out[2] - out[0]).max() > 1e-6
    assert np.abs(out[2] - out[1]).max() > 1e-6


def test_conv_variants_not_in_the_adjoint(gpu_lib):
    n, kw, dt, case = CASES["cavity48"]
    s = ns.Solver(ns.default_params(n_cell=n, fixed_dt=dt, max_grid_size=(n, n, n), conv_scheme=ns.CONV_UMIST_FORM,
                                    **kw))
    s.init(case)
    with pytest.raises(ns.NsError) as e:
        s.adjoint_fwd(np.zeros(0), nsteps=2)
    assert e.value.code == ns.NS_ERR_UNSUPPORTED


@pytest.mark.parametrize("name", ["cavity16", "tgv16_fixed"])
def test_conv_umist_form_3d_steps_resynced(gpu_lib, oracle_lib, name):
    """convective_flux_calc in the AMREX_SPACEDIM = 3 build: per-step parity
    of the FP64 3D path with the oracle's 3D restatement."""
    from amressif_gb300 import workloads as wl

    n = 16
    if name == "cavity16":
        kw = dict(ren=100.0, bc_lo=(135, 135, 135), bc_hi=(135, 165, 135))
        z = [np.zeros((n, n, n + 1)), np.zeros((n, n + 1, n)), np.zeros((n + 1, n, n))]
        st = (z, [a.copy() for a in z], np.zeros((n, n, n)))
        dt = 0.4 / n
    else:
        kw = dict(ren=1600.0, prob_hi=(L2PI,) * 3, bc_lo=(111,) * 3, bc_hi=(111,) * 3, fix_quirks=1)
        st = wl.tgv3d_perturbed_state(n, amp=1e-3, seed=0)
        dt = 0.4 * L2PI / n
    o = Oracle(n, dim=3, dt=dt, iter_num=100, poisson_tol=1e-13, max_grid_size=(n, n, n),
               conv_scheme=ns.CONV_UMIST_FORM, **kw)
    p = ns.default_params(dim=3, n_cell=n, fixed_dt=dt, iter_num=100, precision=ns.PREC_FP64, poisson_tol_rel=1e-12,
                          max_grid_size=(n, n, n), conv_scheme=ns.CONV_UMIST_FORM, **kw)
    s = ns.Solver(p)
    o.set_state(*st)
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
        assert relp(pg, po, uo) <= 1e-10, (step, relp(pg, po, uo))
        assert sg["div_after"] <= 1e-10
    o.close()
