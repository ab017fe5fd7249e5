"""The allocation-free Poisson right-hand side, checked against ns_poisson_rhs.

ns_poisson_rhs_noalloc serves callers that cannot call cudaMalloc (a host
whose device memory all belongs to its own arena, or a job with a fixed memory
budget): it reads caller-owned device arrays and keeps its reduction scratch in
a fixed array inside the library. This test allocates the caller's arrays
itself (through the CUDA runtime), runs two calls in a row on two different
velocity fields, and requires the same f, max|div u| and sum f as the context
entry point, bit for bit: with the context's own row pitch, with a wider
pitch that is not a multiple of 32, and at the largest size the fixed scratch
holds (4096^2). An odd grid (37^2), which the context does not accept, is
checked against the oracle's restatement of poisson_righthand_side_calc
instead. The file sorts last so that a failure here cannot hide the results of
the other GPU tests.
"""
import ctypes
import ctypes.util
import os

import numpy as np
import pytest

import amressif_gb300 as ns

pytestmark = pytest.mark.gpu


def cudart():
    names = ["libcudart.so", "libcudart.so.13", "/usr/local/cuda/lib64/libcudart.so",
             "/usr/local/cuda/lib64/libcudart.so.13"]
    found = ctypes.util.find_library("cudart")
    if found:
        names.insert(0, found)
    for n in names:
        try:
            lib = ctypes.CDLL(n)
        except OSError:
            continue
        lib.cudaMalloc.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_size_t]
        lib.cudaFree.argtypes = [ctypes.c_void_p]
        lib.cudaMemcpy.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int]
        lib.cudaDeviceSynchronize.argtypes = []
        return lib
    pytest.skip("CUDA runtime library not found")


class DevArray:
    def __init__(self, rt, host):
        self.rt = rt
        self.nbytes = host.nbytes
        self.ptr = ctypes.c_void_p()
        assert rt.cudaMalloc(ctypes.byref(self.ptr), self.nbytes) == 0
        assert rt.cudaMemcpy(self.ptr, host.ctypes.data_as(ctypes.c_void_p), self.nbytes, 1) == 0

    def get(self, shape):
        out = np.empty(shape)
        assert self.rt.cudaMemcpy(out.ctypes.data_as(ctypes.c_void_p), self.ptr, self.nbytes, 2) == 0
        return out

    def free(self):
        self.rt.cudaFree(self.ptr)


def pitched(a, pitch, rows):
    out = np.zeros((rows, pitch))
    out[: a.shape[0], : a.shape[1]] = a
    return out


def run_noalloc(gpu_lib, rt, u, v, n, pitch, dx, dt):
    du = DevArray(rt, pitched(u, pitch, n + 1))
    dv = DevArray(rt, pitched(v, pitch, n + 1))
    df = DevArray(rt, np.full((n + 1, pitch), np.nan))
    out = (ctypes.c_double * 2)()
    rc = gpu_lib.ns_poisson_rhs_noalloc(du.ptr, dv.ptr, df.ptr, n, pitch, dx, dx, dt, out, None)
    f = df.get((n + 1, pitch))[:n, :n] if rc == ns.NS_OK else None
    # sizes beyond the fixed scratch, too small a pitch and non-finite or
    # non-positive spacings are rejected before any device work
    bad = [gpu_lib.ns_poisson_rhs_noalloc(du.ptr, dv.ptr, df.ptr, 8192, 8224, dx, dx, dt, out, None),
           gpu_lib.ns_poisson_rhs_noalloc(du.ptr, dv.ptr, df.ptr, n, n, dx, dx, dt, out, None),
           gpu_lib.ns_poisson_rhs_noalloc(du.ptr, dv.ptr, df.ptr, n, pitch, float("nan"), dx, dt, out, None),
           gpu_lib.ns_poisson_rhs_noalloc(du.ptr, dv.ptr, df.ptr, n, pitch, dx, dx, float("inf"), out, None),
           gpu_lib.ns_poisson_rhs_noalloc(du.ptr, dv.ptr, df.ptr, n, pitch, dx, -dx, dt, out, None)]
    res = (rc, f, out[0], out[1])
    for d in (du, dv, df):
        d.free()
    assert bad == [ns.NS_ERR_UNSUPPORTED] + [ns.NS_ERR_ARG] * 4, bad
    return res


def context_rhs(n, dt, u, up, pr):
    p = ns.default_params(n_cell=n, ren=100.0, fixed_dt=dt, precision=ns.PREC_FP64_EXACT, poisson_tol_rel=1e-12)
    s = ns.Solver(p)
    s.set_state(u, up, pr)
    s.step_begin()
    dmax, fsum = s.poisson_rhs()
    f = s.get_field(ns.FIELD_POISSON_RHS)
    s.close()
    return f, dmax, fsum


def random_state(n, seed):
    rng = np.random.default_rng(seed)
    u = [rng.standard_normal((n, n + 1)), rng.standard_normal((n + 1, n))]
    return u, [a.copy() for a in u], rng.standard_normal((n, n))


def test_noalloc_poisson_rhs_matches_context_path(gpu_lib):
    rt = cudart()
    n = 64
    dt = 2e-3
    p = ns.default_params(n_cell=n, ren=100.0, fixed_dt=dt, precision=ns.PREC_FP64_EXACT, poisson_tol_rel=1e-12)
    s = ns.Solver(p)
    s.init(ns.INIT_CAVITY)
    states = []
    for _ in range(2):
        s.step()
        u, up, pr, _ = s.get_state()
        states.append((u, up, pr))
    s.close()
    dx = 1.0 / n
    # two calls in a row on two velocity fields, at the context's own pitch and
    # at a wider one (100 elements: rows not on 256-byte boundaries)
    for pitch in ((n + 1 + 31) // 32 * 32, 100):
        for call, (u, up, pr) in enumerate(states):
            f_ref, dmax_ref, sum_ref = context_rhs(n, dt, u, up, pr)
            rc, f, dmax, fsum = run_noalloc(gpu_lib, rt, u[0], u[1], n, pitch, dx, dt)
            assert rc == ns.NS_OK, (pitch, call, rc)
            np.testing.assert_array_equal(f, f_ref, err_msg="pitch %d call %d" % (pitch, call))
            assert dmax == dmax_ref and fsum == sum_ref, (pitch, call, dmax, fsum, dmax_ref, sum_ref)


def test_noalloc_poisson_rhs_largest_grid(gpu_lib):
    """n = 4096, the most blocks (8192) whose partials the scratch holds."""
    rt = cudart()
    n, dt = 4096, 0.5 / 4096
    for seed in (1, 2):
        u, up, pr = random_state(n, seed)
        f_ref, dmax_ref, sum_ref = context_rhs(n, dt, u, up, pr)
        rc, f, dmax, fsum = run_noalloc(gpu_lib, rt, u[0], u[1], n, 4128, 1.0 / n, dt)
        assert rc == ns.NS_OK
        np.testing.assert_array_equal(f, f_ref)
        assert dmax == dmax_ref and fsum == sum_ref, (dmax, fsum, dmax_ref, sum_ref)


def test_noalloc_poisson_rhs_odd_grid_against_oracle(gpu_lib, oracle_lib):
    """n = 37: not a multiple of the 32-column warps nor of the 64-row blocks.
    f and max|div u| must equal the oracle's bit for bit (same operation order,
    no contraction); sum f is reduced in another order."""
    from oracle.orc import FIELD_PRHS, Oracle

    rt = cudart()
    n, dt = 37, 1e-3
    for seed in (3, 4):
        u, up, pr = random_state(n, seed)
        o = Oracle(n, ren=100.0, dt=dt, max_grid_size=(n, n, n))
        o.set_state(u, up, pr)
        o.step_begin()
        dmax_o, sum_o = o.poisson_rhs()
        f_o = o.field(FIELD_PRHS)
        o.close()
        rc, f, dmax, fsum = run_noalloc(gpu_lib, rt, u[0], u[1], n, 41, 1.0 / n, dt)
        assert rc == ns.NS_OK
        np.testing.assert_array_equal(f, f_o)
        assert dmax == dmax_o
        assert abs(fsum - sum_o) <= 1e-13 * np.abs(f_o).sum(), (fsum, sum_o)
