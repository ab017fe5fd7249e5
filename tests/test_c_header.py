"""The C ABI as a C host sees it (CPU test): include/amressif_gpu.h compiles as
C99 with warnings as errors, a C program links the library and calls the
entry points that do no device work (defaults, the inputs-file parser, a
rejected ns_ctx_create), and the layouts of the structs it shares with the
ctypes binding (sizes and the offsets of the last fields) agree."""
import ctypes
import os
import shutil
import subprocess

import pytest

import amressif_gb300 as ns

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROGRAM = r"""
#include <stddef.h>
#include <stdio.h>
#include "amressif_gpu.h"

int main(int argc, char** argv) {
  ns_params p;
  ns_params_default(&p);
  if (p.conv_scheme != NS_CONV_NEW_QUICK || p.precision != NS_PREC_FP64_EXACT) return 2;
  if (argc > 1 && ns_params_parse_file(&p, argv[1]) != NS_OK) return 3;
  ns_ctx* c = NULL;
  ns_params bad = p;
  bad.n_cell = 20; /* not a multiple of 8: rejected before any device work */
  const int rc = ns_ctx_create(&bad, NULL, &c);
  printf("%d %d %d %f %d\n", p.n_cell, p.max_grid_size[0], p.max_grid_size[1], p.ren, rc);
  printf("%zu %zu %zu %zu %zu\n", sizeof(ns_params), offsetof(ns_params, conv_scheme), sizeof(ns_step_stats),
         sizeof(ns_adjoint_opts), sizeof(ns_adjoint_stats));
  return c == NULL ? 0 : 4;
}
"""


@pytest.fixture(scope="module")
def c_program(tmp_path_factory, gpu_lib):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    d = tmp_path_factory.mktemp("cabi")
    src = d / "host.c"
    src.write_text(PROGRAM)
    exe = d / "host"
    libdir = os.path.dirname(ns.LIB_PATH)
    cmd = [cc, "-std=c99", "-Wall", "-Wextra", "-Werror", "-pedantic", "-I", os.path.join(ROOT, "include"), str(src),
           "-L", libdir, "-lamressif_gb300", "-Wl,-rpath," + libdir, "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe, d


def test_header_compiles_as_c_and_host_entry_points_run(c_program):
    exe, d = c_program
    inputs = d / "inputs"
    inputs.write_text("n_cell = 64\nmax_grid_size_x = 32\nmax_grid_size_y = 16\nren = 400.0\n")
    r = subprocess.run([str(exe), str(inputs)], capture_output=True, text=True)
    assert r.returncode == 0, (r.returncode, r.stdout, r.stderr)
    first = r.stdout.split("\n")[0].split()
    assert first[:3] == ["64", "32", "16"] and float(first[3]) == 400.0
    assert int(first[4]) == ns.NS_ERR_ARG


def test_struct_layouts_match_the_ctypes_binding(c_program):
    exe, _ = c_program
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    sizes = [int(x) for x in r.stdout.split("\n")[1].split()]
    assert sizes[0] == ctypes.sizeof(ns.NsParams)
    assert sizes[1] == ns.NsParams.conv_scheme.offset
    assert sizes[2] == ctypes.sizeof(ns.NsStepStats)
    assert sizes[3] == ctypes.sizeof(ns.NsAdjointOpts)
    assert sizes[4] == ctypes.sizeof(ns.NsAdjointStats)
