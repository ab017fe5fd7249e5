"""Failure paths of the time step, driven from the host (no GPU fault).

The reference warns and carries on when the pseudo-iteration exceeds IterNum
(main.cpp:1030-1033) or its norm exceeds 1e2 (main.cpp:1035-1038); the
library returns those as the positive warnings NS_WARN_PSEUDO_MAXITER and
NS_WARN_PSEUDO_DIVERGED with the step completed. A Poisson solve capped
before its tolerance returns NS_ERR_MG_STALL, again with the step completed;
NaN in the input fields returns NS_ERR_NONFINITE. Each case is compared with
the oracle where the oracle defines the outcome (the same pseudo-iteration
count and the same completed step).
"""
import ctypes

import numpy as np
import pytest

import amressif_gb300 as ns
from oracle.orc import Oracle

pytestmark = pytest.mark.gpu


def raw_step(s):
    st = ns.NsStepStats()
    rc = ns.lib().ns_step(s.h, ctypes.byref(st))
    return rc, ns.stats_dict(st)


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def pair(n=32, dt=1e-3, iter_num=100, dtau_clip=0, precision=ns.PREC_FP64_EXACT, **gkw):
    o = Oracle(n, ren=100.0, dt=dt, iter_num=iter_num, dtau_clip=dtau_clip, poisson_tol=1e-13,
               max_grid_size=(n, n, n))
    o.init(0)
    p = ns.default_params(n_cell=n, ren=100.0, fixed_dt=dt, iter_num=iter_num, dtau_clip=dtau_clip,
                          precision=precision, poisson_tol_rel=1e-12, max_grid_size=(n, n, n), **gkw)
    s = ns.Solver(p)
    s.init(ns.INIT_CAVITY)
    return o, s


def same_state(o, s, tol=1e-10):
    ug, _, pg, _ = s.get_state()
    uo, _, po, _ = o.get_state()
    for d in range(2):
        assert rel(ug[d], uo[d]) <= tol, (d, rel(ug[d], uo[d]))
    assert rel(pg - pg.mean(), po - po.mean()) <= tol


@pytest.mark.parametrize("precision", [ns.PREC_FP64_EXACT, ns.PREC_MIXED])
def test_iter_num_cap_warns_and_completes_the_step(gpu_lib, oracle_lib, precision):
    o, s = pair(iter_num=1, precision=precision)
    for step in range(3):
        so = o.step()
        rc, sg = raw_step(s)
        assert rc == ns.NS_WARN_PSEUDO_MAXITER and sg["status"] == ns.NS_WARN_PSEUDO_MAXITER, (step, rc)
        assert so["status"] == 1 and sg["pseudo_iters"] == so["pseudo_iters"] == 2, (sg, so)
        assert sg["div_after"] <= 1e-9  # Poisson and projection ran
    same_state(o, s, tol=1e-10 if precision == ns.PREC_FP64_EXACT else 1e-6)


def test_unstable_pseudo_step_warns_diverged(gpu_lib, oracle_lib):
    # dt = 0.2 on 32^2 at Re 100 without the clip: the pseudo-time step
    # 0.4 dt is outside the RK4 stability interval of the stiff viscous modes
    # (8 nu 0.4 dt / dx^2 = 6.6 against the limit 2.785), and the pseudo-norm
    # passes 1e2 on the third iteration (the oracle: K = 3, norm 1.8e7). At
    # dt = 0.1 the same estimate gives 3.3, yet the step converges in 30
    # iterations.
    o, s = pair(dt=0.2)
    so = o.step()
    rc, sg = raw_step(s)
    assert rc == ns.NS_WARN_PSEUDO_DIVERGED == sg["status"] and so["status"] == 2, (rc, sg, so)
    assert sg["pseudo_iters"] == so["pseudo_iters"] and sg["norm_error"] > 1e2
    assert abs(sg["norm_error"] - so["norm_error"]) <= 1e-12 * so["norm_error"]
    same_state(o, s, tol=1e-9)


@pytest.mark.parametrize("precision", [ns.PREC_FP64, ns.PREC_MIXED])
def test_poisson_cycle_cap_returns_stall_after_the_step(gpu_lib, precision):
    p = ns.default_params(n_cell=64, ren=100.0, fixed_dt=2e-3, precision=precision, poisson_tol_rel=1e-12,
                          poisson_max_cycles=1)
    s = ns.Solver(p)
    s.init(ns.INIT_CAVITY)
    rc, st = raw_step(s)
    assert rc == ns.NS_ERR_MG_STALL, rc
    assert st["poisson_cycles"] == 1 and st["poisson_res"] > 1e-12
    assert s.step_count == 1 and np.isfinite(st["div_after"])  # projected with the capped phi
    assert "stalled" in ns.lib().ns_last_error(s.h).decode()
    s.close()


@pytest.mark.parametrize("dim,precision", [(2, ns.PREC_FP64_EXACT), (2, ns.PREC_MIXED), (3, ns.PREC_FP64),
                                           (3, ns.PREC_MIXED)])
def test_nan_in_initial_data_is_reported(gpu_lib, dim, precision):
    n = 32 if dim == 2 else 16
    p = ns.default_params(dim=dim, n_cell=n, ren=100.0, fixed_dt=1e-3, precision=precision, poisson_tol_rel=1e-12)
    s = ns.Solver(p)
    u = [np.zeros(s.face_shape(d)) for d in range(dim)]
    u[0].flat[u[0].size // 2 + 3] = np.nan
    s.set_state(u, [a.copy() for a in u], np.zeros(s.cell_shape()))
    rc, _ = raw_step(s)
    assert rc == ns.NS_ERR_NONFINITE, rc
    assert "NaN" in ns.lib().ns_last_error(s.h).decode() or "finite" in ns.lib().ns_last_error(s.h).decode()
    # a clean state afterwards steps normally
    z = [np.zeros(s.face_shape(d)) for d in range(dim)]
    s.set_state(z, z, np.zeros(s.cell_shape()))
    rc, st = raw_step(s)
    assert rc == ns.NS_OK and st["div_after"] <= 1e-9
    s.close()
