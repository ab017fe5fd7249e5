"""The allocation-free Poisson right-hand side, checked against ns_poisson_rhs.

ns_poisson_rhs_noalloc serves callers that cannot call cudaMalloc (a host
whose device memory all belongs to its own arena, or a job with a fixed memory
budget): it reads caller-owned device arrays and keeps its reduction scratch in
a fixed array inside the library. This test allocates the caller's arrays
itself (through the CUDA runtime), runs two calls in a row on two different
velocity fields, and requires the same f, max|div u| and sum f as the context
entry point, bit for bit. The file sorts last so that a failure here cannot
hide the results of the other GPU tests.
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


def test_noalloc_poisson_rhs_matches_context_path(gpu_lib):
    rt = cudart()
    n = 64
    pitch = (n + 1 + 31) // 32 * 32  # the context's own row pitch
    p = ns.default_params(n_cell=n, ren=100.0, fixed_dt=2e-3, precision=ns.PREC_FP64_EXACT, poisson_tol_rel=1e-12)
    s = ns.Solver(p)
    s.init(ns.INIT_CAVITY)
    states = []
    for _ in range(2):
        s.step()
        u, up, pr, _ = s.get_state()
        states.append((u, up, pr))
    dx = dy = 1.0 / n
    for call, (u, up, pr) in enumerate(states):
        # context entry point on the same velocity
        s.set_state(u, up, pr)
        s.step_begin()
        dmax_ref, sum_ref = s.poisson_rhs()
        f_ref = s.get_field(ns.FIELD_POISSON_RHS)
        # caller-owned device arrays, pitch `pitch`, n+1 rows each
        du = DevArray(rt, pitched(u[0], pitch, n + 1))
        dv = DevArray(rt, pitched(u[1], pitch, n + 1))
        df = DevArray(rt, np.full((n + 1, pitch), np.nan))
        out = (ctypes.c_double * 2)()
        rc = gpu_lib.ns_poisson_rhs_noalloc(du.ptr, dv.ptr, df.ptr, n, pitch, dx, dy, 2e-3, out, None)
        assert rc == ns.NS_OK, (call, rc)
        f = df.get((n + 1, pitch))[:n, :n]
        np.testing.assert_array_equal(f, f_ref, err_msg="call %d" % call)
        assert out[0] == dmax_ref and out[1] == sum_ref, (call, list(out), dmax_ref, sum_ref)
        # sizes beyond the fixed scratch are rejected before any device work
        assert gpu_lib.ns_poisson_rhs_noalloc(du.ptr, dv.ptr, df.ptr, 8192, 8224, dx, dy, 2e-3, out, None) == \
            ns.NS_ERR_UNSUPPORTED
        for d in (du, dv, df):
            d.free()
    s.close()
