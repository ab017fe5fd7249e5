"""ctypes binding of the CPU oracle (test infrastructure only).

Only tests/, __graft_entry__.smoke() and the CPU-baseline leg of bench.py use
this module, as the checker of the CUDA path. Arrays are numpy float64, dense,
x fastest: a face array of direction d has extent N+1 along d.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libns_oracle.so")

FIELD_STAR, FIELD_BASE, FIELD_PREV, FIELD_DIFF, FIELD_MRHS = 0, 1, 2, 3, 4
FIELD_P, FIELD_PHI, FIELD_PRHS, FIELD_CART, FIELD_TOTAL = 10, 11, 12, 13, 20


class OrcParams(ctypes.Structure):
    _fields_ = [
        ("dim", ctypes.c_int),
        ("n_cell", ctypes.c_int),
        ("max_grid_size", ctypes.c_int * 3),
        ("prob_lo", ctypes.c_double * 3),
        ("prob_hi", ctypes.c_double * 3),
        ("ren", ctypes.c_double),
        ("dt", ctypes.c_double),
        ("iter_num", ctypes.c_int),
        ("momentum_tolerance", ctypes.c_double),
        ("pseudo_timestepping", ctypes.c_int),
        ("bc_lo", ctypes.c_int * 3),
        ("bc_hi", ctypes.c_int * 3),
        ("inflow", ctypes.c_double * 3),
        ("fix_quirks", ctypes.c_int),
        ("poisson_tol", ctypes.c_double),
        ("nthreads", ctypes.c_int),
        ("dtau_clip", ctypes.c_int),
        ("conv_scheme", ctypes.c_int),
    ]


class OrcStepStats(ctypes.Structure):
    _fields_ = [
        ("pseudo_iters", ctypes.c_int),
        ("norm_error", ctypes.c_double),
        ("div_before", ctypes.c_double),
        ("rhs_sum", ctypes.c_double),
        ("poisson_iters", ctypes.c_int),
        ("poisson_res", ctypes.c_double),
        ("div_after", ctypes.c_double),
        ("status", ctypes.c_int),
    ]


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("oracle library not built: run __graft_entry__.build() (expects %s)" % LIB_PATH)
        L = ctypes.CDLL(LIB_PATH)
        P = ctypes.POINTER
        dp = P(ctypes.c_double)
        L.orc_create.argtypes = [P(OrcParams), P(ctypes.c_void_p)]
        L.orc_destroy.argtypes = [ctypes.c_void_p]
        L.orc_init.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.orc_set_state.argtypes = [ctypes.c_void_p, P(dp), P(dp), dp, ctypes.c_double]
        L.orc_get_state.argtypes = [ctypes.c_void_p, P(dp), P(dp), dp, dp]
        L.orc_set_cart.argtypes = [ctypes.c_void_p, P(dp)]
        L.orc_step.argtypes = [ctypes.c_void_p, P(OrcStepStats)]
        L.orc_step_begin.argtypes = [ctypes.c_void_p]
        L.orc_rk_stage.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.orc_pseudo_norm.argtypes = [ctypes.c_void_p]
        L.orc_pseudo_norm.restype = ctypes.c_double
        L.orc_explicit_predictor.argtypes = [ctypes.c_void_p, dp]
        L.orc_poisson_rhs.argtypes = [ctypes.c_void_p, dp, dp]
        L.orc_poisson_solve.argtypes = [ctypes.c_void_p, P(ctypes.c_int), dp]
        L.orc_project.argtypes = [ctypes.c_void_p, dp]
        L.orc_get_field.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, dp]
        L.orc_put_field.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, dp]
        L.orc_solve_poisson_array.argtypes = [ctypes.c_void_p, dp, dp, P(ctypes.c_int), dp]
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def face_shape(dim, n, d):
    """numpy shape (slowest first) of the face array of direction d."""
    ext = [n + (1 if e == d else 0) for e in range(dim)]
    return tuple(reversed(ext))


def cell_shape(dim, n):
    return (n,) * dim


class Oracle:
    """One oracle context. Parameters follow the reference inputs-file keys."""

    def __init__(self, n_cell, dim=2, max_grid_size=None, prob_lo=(0.0, 0.0, 0.0), prob_hi=(1.0, 1.0, 1.0),
                 ren=100.0, dt=1e-3, iter_num=100, momentum_tolerance=1e-10, pseudo_timestepping=1,
                 bc_lo=(135, 135, 135), bc_hi=(135, 165, 135), inflow=(1.0, 0.0, 0.0), fix_quirks=0,
                 poisson_tol=1e-13, nthreads=0, dtau_clip=0, conv_scheme=0):
        p = OrcParams()
        p.dim, p.n_cell = dim, n_cell
        mgs = max_grid_size or (n_cell, n_cell, n_cell)
        for i in range(3):
            p.max_grid_size[i] = mgs[i]
            p.prob_lo[i], p.prob_hi[i] = prob_lo[i], prob_hi[i]
            p.bc_lo[i], p.bc_hi[i] = bc_lo[i], bc_hi[i]
            p.inflow[i] = inflow[i]
        p.ren, p.dt, p.iter_num = ren, dt, iter_num
        p.momentum_tolerance, p.pseudo_timestepping = momentum_tolerance, pseudo_timestepping
        p.fix_quirks, p.poisson_tol, p.nthreads = fix_quirks, poisson_tol, nthreads
        p.dtau_clip = dtau_clip
        p.conv_scheme = conv_scheme
        self.params = p
        self.dim, self.n = dim, n_cell
        h = ctypes.c_void_p()
        rc = lib().orc_create(ctypes.byref(p), ctypes.byref(h))
        if rc != 0:
            raise ValueError("orc_create failed with code %d" % rc)
        self.h = h

    def close(self):
        if self.h:
            lib().orc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- state ---------------------------------------------------------------
    def init(self, case):
        rc = lib().orc_init(self.h, case)
        if rc != 0:
            raise ValueError("orc_init failed %d" % rc)

    def _faces(self):
        return [np.zeros(face_shape(self.dim, self.n, d)) for d in range(self.dim)]

    def set_state(self, u, u_prev, p, time=0.0):
        u = [np.ascontiguousarray(a, dtype=np.float64) for a in u]
        up = [np.ascontiguousarray(a, dtype=np.float64) for a in u_prev]
        p = np.ascontiguousarray(p, dtype=np.float64)
        arr_u = (ctypes.POINTER(ctypes.c_double) * self.dim)(*[_dp(a) for a in u])
        arr_up = (ctypes.POINTER(ctypes.c_double) * self.dim)(*[_dp(a) for a in up])
        rc = lib().orc_set_state(self.h, arr_u, arr_up, _dp(p), time)
        if rc != 0:
            raise ValueError("orc_set_state failed %d" % rc)

    def set_cart(self, cart):
        cart = [np.ascontiguousarray(a, dtype=np.float64) for a in cart]
        arr = (ctypes.POINTER(ctypes.c_double) * self.dim)(*[_dp(a) for a in cart])
        rc = lib().orc_set_cart(self.h, arr)
        if rc != 0:
            raise ValueError("orc_set_cart failed %d" % rc)

    def get_state(self):
        u, up = self._faces(), self._faces()
        p = np.zeros(cell_shape(self.dim, self.n))
        phi = np.zeros(cell_shape(self.dim, self.n))
        arr_u = (ctypes.POINTER(ctypes.c_double) * self.dim)(*[_dp(a) for a in u])
        arr_up = (ctypes.POINTER(ctypes.c_double) * self.dim)(*[_dp(a) for a in up])
        lib().orc_get_state(self.h, arr_u, arr_up, _dp(p), _dp(phi))
        return u, up, p, phi

    def field(self, which, comp=0):
        if which <= FIELD_MRHS:
            out = np.zeros(face_shape(self.dim, self.n, comp))
        else:
            out = np.zeros(cell_shape(self.dim, self.n))
        rc = lib().orc_get_field(self.h, which, comp, _dp(out))
        if rc != 0:
            raise ValueError("orc_get_field failed")
        return out

    def put_field(self, which, comp, arr):
        arr = np.ascontiguousarray(arr, dtype=np.float64)
        rc = lib().orc_put_field(self.h, which, comp, _dp(arr))
        if rc != 0:
            raise ValueError("orc_put_field failed")

    # -- stepping ------------------------------------------------------------
    def step(self):
        st = OrcStepStats()
        rc = lib().orc_step(self.h, ctypes.byref(st))
        if rc != 0:
            raise ValueError("orc_step failed %d" % rc)
        return {k: getattr(st, k) for k, _ in OrcStepStats._fields_}

    def step_begin(self):
        lib().orc_step_begin(self.h)

    def rk_stage(self, sub):
        rc = lib().orc_rk_stage(self.h, sub)
        if rc != 0:
            raise ValueError("orc_rk_stage failed")

    def pseudo_norm(self):
        return lib().orc_pseudo_norm(self.h)

    def explicit_predictor(self):
        v = ctypes.c_double()
        lib().orc_explicit_predictor(self.h, ctypes.byref(v))
        return v.value

    def poisson_rhs(self):
        a, b = ctypes.c_double(), ctypes.c_double()
        lib().orc_poisson_rhs(self.h, ctypes.byref(a), ctypes.byref(b))
        return a.value, b.value

    def poisson_solve(self):
        it, res = ctypes.c_int(), ctypes.c_double()
        lib().orc_poisson_solve(self.h, ctypes.byref(it), ctypes.byref(res))
        return it.value, res.value

    def project(self):
        v = ctypes.c_double()
        lib().orc_project(self.h, ctypes.byref(v))
        return v.value

    def solve_poisson(self, f):
        f = np.ascontiguousarray(f, dtype=np.float64)
        phi = np.zeros_like(f)
        it, res = ctypes.c_int(), ctypes.c_double()
        lib().orc_solve_poisson_array(self.h, _dp(f), _dp(phi), ctypes.byref(it), ctypes.byref(res))
        return phi, it.value, res.value
