"""ns_ctx_create rejects parameters the reference aborts on, or that this
library does not take, before it touches the GPU (CPU test through the C
ABI): the returned status, and no context."""
import ctypes

import pytest

import amressif_gb300 as ns


def create(gpu_lib, **kw):
    p = ns.default_params(**kw)
    h = ctypes.c_void_p(0)
    rc = gpu_lib.ns_ctx_create(ctypes.byref(p), None, ctypes.byref(h))
    return rc, h.value


@pytest.mark.parametrize("kw,code", [
    (dict(n_cell=20), ns.NS_ERR_ARG),                 # not a multiple of 8
    (dict(n_cell=4), ns.NS_ERR_ARG),                  # too small for the box layout
    # multiple of 8, but the hierarchy stops at 202 (808 -> 404 -> 202): too large for the bottom block
    (dict(n_cell=808), ns.NS_ERR_UNSUPPORTED),
    (dict(dim=3, n_cell=104), ns.NS_ERR_UNSUPPORTED),  # 104 -> 52 -> 26 > 24
    (dict(ren=0.0), ns.NS_ERR_ARG),
    (dict(ren=float("nan")), ns.NS_ERR_ARG),
    (dict(dc_residual=2), ns.NS_ERR_ARG),
    (dict(dim=4), ns.NS_ERR_UNSUPPORTED),
    # periodic on one side only: the reference makes a direction periodic only when both
    # codes are 111 (main.cpp:160-162) yet gives the 111 side an interior BC type
    # (main.cpp:815-816); not a valid box
    (dict(bc_lo=(111, 135, 135), bc_hi=(135, 165, 135)), ns.NS_ERR_BC),
    # a code the reference does not know ("Invalid bc_lo", main.cpp:815-822)
    (dict(bc_lo=(135, 999, 135), bc_hi=(135, 165, 135)), ns.NS_ERR_BC),
    # the outlet code 195: "Not yet implemented" in the reference's ghost fill
    # (utilities.cpp:176-179 for the east side)
    (dict(bc_lo=(135, 135, 135), bc_hi=(195, 165, 135)), ns.NS_ERR_BC),
    # east -135 in parity mode: the reference tests east slip as == 1 (quirk Q5)
    (dict(bc_lo=(135, 135, 135), bc_hi=(-135, 165, 135), fix_quirks=0), ns.NS_ERR_UNSUPPORTED),
    # the convective routine: an unknown one; the alternatives with the mixed predictor;
    # convective_flux_calc_quick with two boxes (the defaults split 32 x 32 into 32 x 16 boxes)
    # and in 3D, where it reads and writes outside its fabs
    (dict(conv_scheme=3), ns.NS_ERR_ARG),
    (dict(conv_scheme=-1), ns.NS_ERR_ARG),
    (dict(conv_scheme=ns.CONV_QUICK, precision=ns.PREC_MIXED, max_grid_size=(32, 32, 32)), ns.NS_ERR_UNSUPPORTED),
    (dict(conv_scheme=ns.CONV_UMIST_FORM, precision=ns.PREC_MIXED), ns.NS_ERR_UNSUPPORTED),
    (dict(conv_scheme=ns.CONV_QUICK), ns.NS_ERR_UNSUPPORTED),
    (dict(dim=3, n_cell=16, conv_scheme=ns.CONV_QUICK, max_grid_size=(16, 16, 16)), ns.NS_ERR_UNSUPPORTED),
])
def test_rejected_before_any_device_work(gpu_lib, kw, code):
    rc, h = create(gpu_lib, **kw)
    assert rc == code, (kw, rc)
    assert not h


def test_null_arguments(gpu_lib):
    h = ctypes.c_void_p(0)
    assert gpu_lib.ns_ctx_create(None, None, ctypes.byref(h)) == ns.NS_ERR_ARG
    p = ns.default_params()
    assert gpu_lib.ns_ctx_create(ctypes.byref(p), None, None) == ns.NS_ERR_ARG
