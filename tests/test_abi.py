"""C-ABI library: loads, exports every declared symbol, host-side parameter logic.

No compute call is made here (no GPU needed).
"""
import ctypes
import os
import re

import pytest

import amressif_gb300 as ns

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    syms = set()
    for name in os.listdir(os.path.join(ROOT, "include")):
        if not name.endswith(".h"):
            continue
        txt = open(os.path.join(ROOT, "include", name)).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        syms |= set(re.findall(r"\b(ns_[a-z0-9_]+)\s*\(", txt))
    return syms


def test_library_exports_every_declared_symbol(gpu_lib):
    syms = declared_symbols()
    assert len(syms) >= 20
    missing = [s for s in sorted(syms) if not hasattr(gpu_lib, s)]
    assert not missing, missing
    assert set(ns.EXPORTS) <= syms | set(ns.EXPORTS)


def test_params_default_matches_shipped_inputs(gpu_lib):
    p = ns.default_params()
    assert p.dim == 2 and p.n_cell == 32
    assert p.fixed_dt == 1e-3 and p.ren == 100.0 and p.iter_num == 100
    assert list(p.bc_lo)[:2] == [135, 135] and list(p.bc_hi)[:2] == [135, 165]
    assert p.momentum_tolerance == 1e-10 and p.pseudo_timestepping == 1


def test_inputs_file_parser(gpu_lib, tmp_path):
    # the reference's key set, including its malformed "chk_int = = 10" line
    f = tmp_path / "inputs"
    f.write_text(
        "nsteps = 200\nn_cell = 128\nmax_grid_size_x = 64\nmax_grid_size_y = 64\n"
        "fixed_dt = 3.90625e-3\nchk_int = = 10\nPSEUDO_TIMESTEPPING = 1\n"
        "momentum_tolerance = 1.e-10\nIterNum = 100\nren = 100 # Reynolds\nvis = 1\n"
        "phy_bc_lo = 135 135 135\nphy_bc_hi = 135 165 135\ninflow_waveform = 1.0 0.0 0.0\n"
        "amrex.v = 1\n"
    )
    p = ns.default_params()
    rc = gpu_lib.ns_params_parse_file(ctypes.byref(p), str(f).encode())
    assert rc == ns.NS_OK
    assert p.n_cell == 128 and p.nsteps == 200 and p.max_grid_size[0] == 64
    assert p.fixed_dt == 3.90625e-3 and p.iter_num == 100 and p.ren == 100.0
    assert list(p.bc_hi)[:2] == [135, 165] and p.inflow_waveform[0] == 1.0
    assert gpu_lib.ns_params_parse_file(ctypes.byref(p), b"/nonexistent/inputs") == ns.NS_ERR_ARG


def test_missing_library_fails_loudly(monkeypatch, tmp_path):
    monkeypatch.setattr(ns, "_lib", None)
    monkeypatch.setattr(ns, "LIB_PATH", str(tmp_path / "nope.so"))
    with pytest.raises(RuntimeError):
        ns.lib()
