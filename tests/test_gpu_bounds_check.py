"""The bounds-check build (libamressif_gb300_check.so, -DNS_BOUNDS_CHECK; the
counterpart of the reference's DEBUG=TRUE build): the column-marching
predictor kernels and the multigrid smoothers test every index they form by
hand against the array it addresses and record a failure in status words
instead of trapping. Grids whose width is not a multiple of the strips (40,
48: partial column strips and row strips, the east ghost lanes, the wrap of
a periodic box inside a strip) and the 4096^2 grid of the warp-marching
smoother must run with no failure, and give the normal build's steps (same
pseudo-iteration counts, states within 1e-12 relative).
"""
import math

import numpy as np
import pytest

import amressif_gb300 as ns
from amressif_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

PER = dict(prob_hi=(2 * math.pi,) * 3, bc_lo=(111,) * 3, bc_hi=(111,) * 3)
CASES = {
    "cavity40": (40, dict(ren=100.0, fixed_dt=0.5 / 40), False),
    "cavity48_lid_controls": (48, dict(ren=400.0, fixed_dt=0.5 / 48), False),
    "tgv40_periodic_fixed": (40, dict(ren=1000.0, fixed_dt=0.5 * 2 * math.pi / 40, fix_quirks=1, **PER), True),
    "tgv48_periodic_parity": (48, dict(ren=1000.0, fixed_dt=0.5 * 2 * math.pi / 48, **PER), True),
    "cavity4096": (4096, dict(ren=1000.0, fixed_dt=0.5 / 4096, dtau_clip=1), False),
}


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


@pytest.mark.parametrize("precision", [ns.PREC_MIXED, ns.PREC_FP64])
@pytest.mark.parametrize("name", sorted(CASES))
def test_checked_build_finds_no_out_of_range_index(gpu_lib, name, precision):
    n, kw, tgv = CASES[name]
    if n == 4096 and precision == ns.PREC_FP64:
        pytest.skip("the warp-marching smoother runs in the FP32 V-cycles only")
    steps = 1 if n == 4096 else 3
    out = []
    for checked in (False, True):
        p = ns.default_params(n_cell=n, iter_num=100, precision=precision, poisson_tol_rel=1e-12,
                              max_grid_size=(n, n, n), **kw)
        s = ns.Solver(p, checked=checked)
        if tgv:
            s.set_state(*wl.tgv_perturbed_state(n, amp=1e-3, seed=0))
        else:
            s.init(ns.INIT_CAVITY)
        if "lid_controls" in name:
            s.set_controls(wl.lid_controls(8, seed=1))
        ks = [s.step()["pseudo_iters"] for _ in range(steps)]
        if checked:
            count, first, site = s.bounds_check()
            assert count == 0, "out-of-range index %d at site %d (%d failures)" % (first, site, count)
        else:
            with pytest.raises(ns.NsError):
                s.bounds_check()  # the normal build has no status words
        u, _, pp, _ = s.get_state()
        out.append((ks, u, pp))
        s.close()
    assert out[0][0] == out[1][0]
    for a, b in zip(out[0][1], out[1][1]):
        assert rel(b, a) <= 1e-12
    assert rel(out[1][2] - out[1][2].mean(), out[0][2] - out[0][2].mean()) <= 1e-12


@pytest.mark.parametrize("periodic", [False, True])
def test_checked_build_conv_quick_variant(gpu_lib, periodic):
    """convective_flux_calc_quick's cell kernel reads the y-face fab through its
    flat layout at the last column, element (0, j+1) (site 61): no failure on a
    40^2 cavity or periodic box, and the normal build's steps."""
    n = 40
    kw = dict(ren=100.0, fixed_dt=0.25 * 2 * math.pi / n, fix_quirks=1, **PER) if periodic else \
        dict(ren=100.0, fixed_dt=0.5 / n)
    out = []
    for checked in (False, True):
        p = ns.default_params(n_cell=n, iter_num=100, precision=ns.PREC_FP64_EXACT, poisson_tol_rel=1e-12,
                              max_grid_size=(n, n, n), conv_scheme=ns.CONV_QUICK, **kw)
        s = ns.Solver(p, checked=checked)
        if periodic:
            s.set_state(*wl.tgv_perturbed_state(n, amp=1e-3, seed=0))
        else:
            s.init(ns.INIT_CAVITY)
        ks = [s.step()["pseudo_iters"] for _ in range(2)]
        if checked:
            count, first, site = s.bounds_check()
            assert count == 0, "out-of-range index %d at site %d (%d failures)" % (first, site, count)
        u, _, pp, _ = s.get_state()
        out.append((ks, u))
        s.close()
    assert out[0][0] == out[1][0]
    for a, b in zip(out[0][1], out[1][1]):
        assert rel(b, a) <= 1e-12



@pytest.mark.parametrize("name", ["cavity40_3d", "tgv24_3d_periodic"])
def test_checked_build_3d_mixed_predictor(gpu_lib, name):
    """The 3D tiled flux pass of the mixed predictor (k3i_fluxtot: halo tiles
    of 36 x 12 cells, the z window of each column, the face loads; sites
    71-73): no failure on a 40^3 cavity (two x tiles, one partial) and a 24^3
    periodic box, and the normal build's steps."""
    n = 40 if name == "cavity40_3d" else 24
    if name == "cavity40_3d":
        kw = dict(ren=100.0, fixed_dt=0.4 / n)
    else:
        kw = dict(ren=1600.0, fixed_dt=0.4 * 2 * math.pi / n, fix_quirks=1, **PER)
    out = []
    for checked in (False, True):
        p = ns.default_params(dim=3, n_cell=n, iter_num=100, precision=ns.PREC_MIXED, poisson_tol_rel=1e-12,
                              max_grid_size=(n, n, n), **kw)
        s = ns.Solver(p, checked=checked)
        if name == "cavity40_3d":
            s.init(ns.INIT_CAVITY)
        else:
            s.set_state(*wl.tgv3d_perturbed_state(n, amp=1e-3, seed=0))
        ks = [s.step()["pseudo_iters"] for _ in range(2)]
        if checked:
            count, first, site = s.bounds_check()
            assert count == 0, "out-of-range index %d at site %d (%d failures)" % (first, site, count)
        u, _, _, _ = s.get_state()
        out.append((ks, u))
        s.close()
    assert out[0][0] == out[1][0]
    for a, b in zip(out[0][1], out[1][1]):
        assert rel(b, a) <= 1e-12
