"""Python binding of the amressif_gb300 C ABI (include/amressif_gpu.h).

The solver itself is C++/CUDA; this module only loads the in-tree shared
library with ctypes and mirrors the entry points, for the tests and bench.py.
Loading fails loudly when the library has not been built: there is no CPU
fallback.
"""
import ctypes
import os

import numpy as np

from . import workloads  # noqa: F401  (host-side inputs of the benchmark configurations)

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libamressif_gb300.so")
# the bounds-check build (the same entry points, compiled with -DNS_BOUNDS_CHECK)
LIB_CHECK_PATH = os.path.join(PKG, "libamressif_gb300_check.so")

NS_OK = 0
NS_WARN_PSEUDO_MAXITER = 1
NS_WARN_PSEUDO_DIVERGED = 2
NS_ERR_ARG = -1
NS_ERR_BC = -2
NS_ERR_CUDA = -3
NS_ERR_MG_STALL = -4
NS_ERR_NOMEM = -5
NS_ERR_STATE = -6
NS_ERR_UNSUPPORTED = -7
NS_ERR_NONFINITE = -8

PREC_FP64_EXACT, PREC_FP64, PREC_MIXED = 0, 1, 2
CONV_NEW_QUICK, CONV_QUICK, CONV_UMIST_FORM = 0, 1, 2  # ns_params.conv_scheme
INIT_CAVITY, INIT_TGV = 0, 1
FIELD_VEL, FIELD_VEL_PREV, FIELD_PRESSURE, FIELD_PHI, FIELD_VEL_STAR, FIELD_POISSON_RHS, FIELD_CART = range(7)

# every symbol declared in include/amressif_gpu.h
EXPORTS = [
    "ns_params_default", "ns_params_parse_file", "ns_ctx_create", "ns_ctx_destroy", "ns_last_error",
    "ns_get_dt", "ns_get_time", "ns_init_fields", "ns_put_box", "ns_get_box", "ns_set_state",
    "ns_get_state", "ns_step_begin", "ns_rk_stage", "ns_pseudo_norm", "ns_explicit_predictor",
    "ns_poisson_rhs", "ns_poisson_solve", "ns_project", "ns_step", "ns_step_host", "ns_sync",
    "ns_profile_enable", "ns_profile_read", "ns_launch_count", "ns_host_alloc", "ns_host_free",
    "ns_poisson_rhs_noalloc",
    "ns_adjoint_opts_default", "ns_set_controls", "ns_step_adjoint_fwd", "ns_step_adjoint_bwd",
    "ns_adjoint_get_state_grad", "ns_step_jvp", "ns_step_vjp", "ns_adjoint_op",
    "ns_checkpoint_get", "ns_checkpoint_put", "ns_get_step", "ns_get_cell_velocity", "ns_bounds_check_read",
]


class PinnedArray:
    """numpy float64 array over page-locked host memory (ns_host_alloc)."""

    def __init__(self, shape):
        n = int(np.prod(shape))
        self.ptr = lib().ns_host_alloc(n * 8)
        if not self.ptr:
            raise MemoryError("ns_host_alloc failed")
        buf = (ctypes.c_double * n).from_address(self.ptr)
        self.a = np.frombuffer(buf, dtype=np.float64).reshape(shape)

    def free(self):
        if self.ptr:
            self.a = None
            lib().ns_host_free(self.ptr)
            self.ptr = None

PROF_KINDS = ["stage_exact", "stage_fast", "anchor", "increment", "explicit", "step_begin", "poisson_rhs",
              "project", "mg_smooth0", "mg_smooth", "mg_restrict0", "mg_restrict", "mg_bottom", "mg_resnorm",
              "dc_update", "other", "mg_cycle"]


class NsError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s (status %d)" % (msg, code))
        self.code = code


class NsParams(ctypes.Structure):
    _fields_ = [
        ("dim", ctypes.c_int),
        ("n_cell", ctypes.c_int),
        ("max_grid_size", ctypes.c_int * 3),
        ("prob_lo", ctypes.c_double * 3),
        ("prob_hi", ctypes.c_double * 3),
        ("ren", ctypes.c_double),
        ("vis", ctypes.c_double),
        ("cfl", ctypes.c_double),
        ("fixed_dt", ctypes.c_double),
        ("iter_num", ctypes.c_int),
        ("momentum_tolerance", ctypes.c_double),
        ("pseudo_timestepping", ctypes.c_int),
        ("bc_lo", ctypes.c_int * 3),
        ("bc_hi", ctypes.c_int * 3),
        ("inflow_waveform", ctypes.c_double * 3),
        ("nsteps", ctypes.c_int),
        ("precision", ctypes.c_int),
        ("fix_quirks", ctypes.c_int),
        ("poisson_tol_rel", ctypes.c_double),
        ("poisson_tol_div", ctypes.c_double),
        ("poisson_max_cycles", ctypes.c_int),
        ("dtau_clip", ctypes.c_int),
        ("poisson_solver", ctypes.c_int),
        ("gmres_restart", ctypes.c_int),
        ("dc_residual", ctypes.c_int),
        ("poisson_warm_start", ctypes.c_int),
        ("conv_scheme", ctypes.c_int),
    ]


class NsStepStats(ctypes.Structure):
    _fields_ = [
        ("pseudo_iters", ctypes.c_int),
        ("norm_error", ctypes.c_double),
        ("div_before", ctypes.c_double),
        ("rhs_sum", ctypes.c_double),
        ("poisson_cycles", ctypes.c_int),
        ("poisson_res", ctypes.c_double),
        ("div_after", ctypes.c_double),
        ("status", ctypes.c_int),
        ("ms_predictor", ctypes.c_double),
        ("ms_poisson", ctypes.c_double),
        ("ms_project", ctypes.c_double),
        ("poisson_fp64_fallback", ctypes.c_int),
        ("ms_h2d", ctypes.c_double),
        ("ms_d2h", ctypes.c_double),
    ]


class NsAdjointOpts(ctypes.Structure):
    _fields_ = [
        ("nsteps", ctypes.c_int),
        ("nsnap", ctypes.c_int),
        ("lin_tol", ctypes.c_double),
        ("lin_max_iters", ctypes.c_int),
    ]


class NsAdjointStats(ctypes.Structure):
    _fields_ = [
        ("J", ctypes.c_double),
        ("nsteps", ctypes.c_int),
        ("nsnap", ctypes.c_int),
        ("steps_advanced", ctypes.c_longlong),
        ("predictor_runs", ctypes.c_longlong),
        ("adjoint_steps", ctypes.c_longlong),
        ("lin_iters", ctypes.c_longlong),
        ("lin_max_iters_seen", ctypes.c_int),
        ("lin_max_res", ctypes.c_double),
        ("poisson_cycles", ctypes.c_longlong),
        ("ms_forward", ctypes.c_double),
        ("ms_backward", ctypes.c_double),
        ("status", ctypes.c_int),
    ]


_lib = None
_lib_check = None


def lib(checked=False):
    """Load the CUDA library (raises if it is missing: no CPU fallback);
    checked=True loads the bounds-check build."""
    global _lib, _lib_check
    if checked:
        if _lib_check is None:
            if not os.path.exists(LIB_CHECK_PATH):
                raise RuntimeError("libamressif_gb300_check.so is not built; run __graft_entry__.build()")
            _lib_check = _declare(ctypes.CDLL(LIB_CHECK_PATH))
        return _lib_check
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("libamressif_gb300.so is not built; run __graft_entry__.build()")
        _lib = _declare(ctypes.CDLL(LIB_PATH))
    return _lib


def _declare(L):
    """argument and result types of the C ABI on a loaded library"""
    P = ctypes.POINTER
    dp = P(ctypes.c_double)
    vp = ctypes.c_void_p
    i3 = P(ctypes.c_int)
    L.ns_params_default.argtypes = [P(NsParams)]
    L.ns_params_default.restype = None
    L.ns_params_parse_file.argtypes = [P(NsParams), ctypes.c_char_p]
    L.ns_ctx_create.argtypes = [P(NsParams), vp, P(vp)]
    L.ns_ctx_destroy.argtypes = [vp]
    L.ns_ctx_destroy.restype = None
    L.ns_last_error.argtypes = [vp]
    L.ns_last_error.restype = ctypes.c_char_p
    L.ns_get_dt.argtypes = [vp]
    L.ns_get_dt.restype = ctypes.c_double
    L.ns_get_time.argtypes = [vp]
    L.ns_get_time.restype = ctypes.c_double
    L.ns_init_fields.argtypes = [vp, ctypes.c_int]
    L.ns_put_box.argtypes = [vp, ctypes.c_int, ctypes.c_int, dp, i3, i3, ctypes.c_longlong, ctypes.c_longlong, ctypes.c_int]
    L.ns_get_box.argtypes = [vp, ctypes.c_int, ctypes.c_int, dp, i3, i3, ctypes.c_longlong, ctypes.c_longlong, ctypes.c_int]
    L.ns_set_state.argtypes = [vp, P(dp), P(dp), dp, ctypes.c_double]
    L.ns_get_state.argtypes = [vp, P(dp), P(dp), dp, dp]
    L.ns_step_begin.argtypes = [vp]
    L.ns_rk_stage.argtypes = [vp, ctypes.c_int]
    L.ns_pseudo_norm.argtypes = [vp, dp]
    L.ns_explicit_predictor.argtypes = [vp, dp]
    L.ns_poisson_rhs.argtypes = [vp, dp, dp]
    L.ns_poisson_solve.argtypes = [vp, ctypes.c_int, P(ctypes.c_int), dp]
    L.ns_project.argtypes = [vp, dp]
    L.ns_step.argtypes = [vp, P(NsStepStats)]
    L.ns_step_host.argtypes = [vp, P(dp), P(dp), dp, P(NsStepStats)]
    L.ns_sync.argtypes = [vp]
    L.ns_profile_enable.argtypes = [vp, ctypes.c_int]
    L.ns_profile_read.argtypes = [vp, dp, P(ctypes.c_longlong), ctypes.c_int, ctypes.c_int]
    L.ns_launch_count.argtypes = [vp]
    L.ns_launch_count.restype = ctypes.c_longlong
    L.ns_host_alloc.argtypes = [ctypes.c_ulonglong]
    L.ns_host_alloc.restype = ctypes.c_void_p
    L.ns_host_free.argtypes = [ctypes.c_void_p]
    L.ns_host_free.restype = None
    L.ns_poisson_rhs_noalloc.argtypes = [vp, vp, vp, ctypes.c_int, ctypes.c_longlong, ctypes.c_double,
                                         ctypes.c_double, ctypes.c_double, dp, vp]
    L.ns_adjoint_opts_default.argtypes = [P(NsAdjointOpts)]
    L.ns_adjoint_opts_default.restype = None
    L.ns_set_controls.argtypes = [vp, ctypes.c_int, dp]
    L.ns_step_adjoint_fwd.argtypes = [vp, P(NsAdjointOpts), ctypes.c_int, dp, dp, P(NsAdjointStats)]
    L.ns_step_adjoint_bwd.argtypes = [vp, dp, P(NsAdjointStats)]
    L.ns_adjoint_get_state_grad.argtypes = [vp, P(dp), P(dp), dp]
    L.ns_step_jvp.argtypes = [vp, P(dp), P(dp), dp, dp, P(dp), P(dp), dp]
    L.ns_step_vjp.argtypes = [vp, P(dp), P(dp), dp, P(dp), P(dp), dp, dp]
    L.ns_adjoint_op.argtypes = [vp, ctypes.c_int, P(dp), dp, P(dp), dp]
    L.ns_checkpoint_get.argtypes = [vp, P(dp), P(dp), dp, dp, P(ctypes.c_longlong)]
    L.ns_checkpoint_put.argtypes = [vp, P(dp), P(dp), dp, ctypes.c_double, ctypes.c_longlong]
    L.ns_get_cell_velocity.argtypes = [vp, P(dp)]
    L.ns_get_step.argtypes = [vp]
    L.ns_get_step.restype = ctypes.c_longlong
    L.ns_bounds_check_read.argtypes = [vp, P(ctypes.c_ulonglong), ctypes.c_int]
    return L


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def default_params(**kw):
    p = NsParams()
    lib().ns_params_default(ctypes.byref(p))
    for k, v in kw.items():
        f = getattr(p, k)
        if isinstance(f, ctypes.Array):
            for i, x in enumerate(v):
                f[i] = x
        else:
            setattr(p, k, v)
    return p


def stats_dict(st):
    return {k: getattr(st, k) for k, _ in type(st)._fields_}


def adjoint_opts(**kw):
    o = NsAdjointOpts()
    lib().ns_adjoint_opts_default(ctypes.byref(o))
    for k, v in kw.items():
        setattr(o, k, v)
    return o


def _pair(arrs):
    return (ctypes.POINTER(ctypes.c_double) * 2)(*[_dp(a) for a in arrs])


def _opt(a):
    return None if a is None else _dp(a)


class Solver:
    """One device context (ns_ctx). Arrays are dense float64, x fastest."""

    def __init__(self, params, stream=None, checked=False):
        """checked=True: a context of the bounds-check build"""
        self.L = lib(checked)
        self.params = params
        self.n = params.n_cell
        self.dim = params.dim
        h = ctypes.c_void_p()
        rc = self.L.ns_ctx_create(ctypes.byref(params), stream, ctypes.byref(h))
        if rc != NS_OK:
            raise NsError(rc, "ns_ctx_create failed")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.L.ns_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc, what, allow_warn=False):
        if rc < 0 or (rc > 0 and not allow_warn):
            msg = self.L.ns_last_error(self.h)
            raise NsError(rc, "%s: %s" % (what, msg.decode() if msg else ""))
        return rc

    @property
    def dt(self):
        return self.L.ns_get_dt(self.h)

    @property
    def time(self):
        return self.L.ns_get_time(self.h)

    def face_shape(self, d):
        n = self.n
        if self.dim == 3:
            return (n + (d == 2), n + (d == 1), n + (d == 0))
        return (n + (1 if d == 1 else 0), n + (1 if d == 0 else 0))

    def cell_shape(self):
        return (self.n,) * self.dim

    def init(self, case):
        self._check(self.L.ns_init_fields(self.h, case), "ns_init_fields")

    def set_state(self, u, u_prev, p, time=0.0):
        u = [np.ascontiguousarray(a, dtype=np.float64) for a in u]
        up = [np.ascontiguousarray(a, dtype=np.float64) for a in u_prev]
        p = np.ascontiguousarray(p, dtype=np.float64)
        au = (ctypes.POINTER(ctypes.c_double) * self.dim)(*[_dp(a) for a in u])
        aup = (ctypes.POINTER(ctypes.c_double) * self.dim)(*[_dp(a) for a in up])
        self._check(self.L.ns_set_state(self.h, au, aup, _dp(p), time), "ns_set_state")

    def get_state(self):
        u = [np.zeros(self.face_shape(d)) for d in range(self.dim)]
        up = [np.zeros(self.face_shape(d)) for d in range(self.dim)]
        p = np.zeros(self.cell_shape())
        phi = np.zeros(self.cell_shape())
        au = (ctypes.POINTER(ctypes.c_double) * self.dim)(*[_dp(a) for a in u])
        aup = (ctypes.POINTER(ctypes.c_double) * self.dim)(*[_dp(a) for a in up])
        self._check(self.L.ns_get_state(self.h, au, aup, _dp(p), _dp(phi)), "ns_get_state")
        return u, up, p, phi

    @staticmethod
    def _box(arr):
        """(lo, hi, jstride, kstride) of a whole dense array (x fastest)."""
        sh = arr.shape
        lo = (ctypes.c_int * 3)(0, 0, 0)
        hi = (ctypes.c_int * 3)(sh[-1] - 1, sh[-2] - 1, sh[-3] - 1 if arr.ndim == 3 else 0)
        return lo, hi, sh[-1], sh[-1] * sh[-2] if arr.ndim == 3 else 0

    def put_field(self, field, comp, arr):
        arr = np.ascontiguousarray(arr, dtype=np.float64)
        lo, hi, js, ks = self._box(arr)
        self._check(self.L.ns_put_box(self.h, field, comp, _dp(arr), lo, hi, js, ks, 0), "ns_put_box")

    def get_field(self, field, comp=0):
        if field in (FIELD_VEL, FIELD_VEL_PREV, FIELD_VEL_STAR):
            out = np.zeros(self.face_shape(comp))
        else:
            out = np.zeros(self.cell_shape())
        lo, hi, js, ks = self._box(out)
        self._check(self.L.ns_get_box(self.h, field, comp, _dp(out), lo, hi, js, ks, 0), "ns_get_box")
        return out

    def step(self, allow_warn=True):
        st = NsStepStats()
        rc = self.L.ns_step(self.h, ctypes.byref(st))
        self._check(rc, "ns_step", allow_warn=allow_warn)
        d = stats_dict(st)
        d["rc"] = rc
        return d

    def step_host(self, u, u_prev, p):
        """End-to-end step from/to host arrays (modified in place)."""
        st = NsStepStats()
        rc = self.L.ns_step_host(self.h, self._vec(u), self._vec(u_prev), _dp(p), ctypes.byref(st))
        self._check(rc, "ns_step_host", allow_warn=True)
        return stats_dict(st)

    def step_begin(self):
        self._check(self.L.ns_step_begin(self.h), "ns_step_begin")

    def rk_stage(self, sub):
        self._check(self.L.ns_rk_stage(self.h, sub), "ns_rk_stage")

    def pseudo_norm(self):
        v = ctypes.c_double()
        self._check(self.L.ns_pseudo_norm(self.h, ctypes.byref(v)), "ns_pseudo_norm")
        return v.value

    def explicit_predictor(self):
        v = ctypes.c_double()
        self._check(self.L.ns_explicit_predictor(self.h, ctypes.byref(v)), "ns_explicit_predictor")
        return v.value

    def poisson_rhs(self):
        a, b = ctypes.c_double(), ctypes.c_double()
        self._check(self.L.ns_poisson_rhs(self.h, ctypes.byref(a), ctypes.byref(b)), "ns_poisson_rhs")
        return a.value, b.value

    def poisson_solve(self, precision=PREC_FP64):
        it, res = ctypes.c_int(), ctypes.c_double()
        self._check(self.L.ns_poisson_solve(self.h, precision, ctypes.byref(it), ctypes.byref(res)), "ns_poisson_solve")
        return it.value, res.value

    def project(self):
        v = ctypes.c_double()
        self._check(self.L.ns_project(self.h, ctypes.byref(v)), "ns_project")
        return v.value

    def sync(self):
        self._check(self.L.ns_sync(self.h), "ns_sync")

    def profile(self, on=True):
        self._check(self.L.ns_profile_enable(self.h, 1 if on else 0), "ns_profile_enable")

    def profile_read(self, reset=False):
        """{kind: (launches, total device ms)} from the per-launch CUDA events."""
        k = len(PROF_KINDS)
        ms = (ctypes.c_double * k)()
        cnt = (ctypes.c_longlong * k)()
        self._check(self.L.ns_profile_read(self.h, ms, cnt, k, 1 if reset else 0), "ns_profile_read")
        return {PROF_KINDS[i]: (int(cnt[i]), float(ms[i])) for i in range(k)}

    def bounds_check(self, reset=False):
        """(failed tests, first failing index, its site) of the bounds-check
        build; NsError(NS_ERR_UNSUPPORTED) on the normal build"""
        st = (ctypes.c_ulonglong * 3)()
        self._check(self.L.ns_bounds_check_read(self.h, st, 1 if reset else 0), "ns_bounds_check_read")
        return int(st[0]), int(st[1]), int(st[2])

    def launch_count(self):
        return int(self.L.ns_launch_count(self.h))

    @property
    def step_count(self):
        return int(self.L.ns_get_step(self.h))

    def checkpoint_get(self):
        """(u, u_prev, p, time, step): the restart state of SaveCheckpoint"""
        u = [np.zeros(self.face_shape(d)) for d in range(self.dim)]
        up = [np.zeros(self.face_shape(d)) for d in range(self.dim)]
        p = np.zeros(self.cell_shape())
        t, k = ctypes.c_double(), ctypes.c_longlong()
        self._check(self.L.ns_checkpoint_get(self.h, self._vec(u), self._vec(up), _dp(p), ctypes.byref(t), ctypes.byref(k)),
                    "ns_checkpoint_get")
        return u, up, p, t.value, k.value

    def cell_velocity(self):
        """velCart (the face averages of u^n) from the device, one cell array per component"""
        out = [np.zeros(self.cell_shape()) for _ in range(self.dim)]
        self._check(self.L.ns_get_cell_velocity(self.h, self._vec(out)), "ns_get_cell_velocity")
        return out

    def checkpoint_put(self, u, u_prev, p, time, step):
        u = [np.ascontiguousarray(a, dtype=np.float64) for a in u]
        up = [np.ascontiguousarray(a, dtype=np.float64) for a in u_prev]
        p = np.ascontiguousarray(p, dtype=np.float64)
        self._check(self.L.ns_checkpoint_put(self.h, self._vec(u), self._vec(up), _dp(p), time, step), "ns_checkpoint_put")

    # ---- discrete adjoint (ns_step_adjoint_fwd / ns_step_adjoint_bwd pair) ----
    def _vec(self, arrs):
        return (ctypes.POINTER(ctypes.c_double) * self.dim)(*[_dp(a) for a in arrs])

    def set_controls(self, controls):
        """Piecewise-constant lid profile (len divides n_cell); None: uniform lid."""
        if controls is None:
            self._check(self.L.ns_set_controls(self.h, 0, None), "ns_set_controls")
            self.nseg = 0
            return
        c = np.ascontiguousarray(controls, dtype=np.float64)
        self._check(self.L.ns_set_controls(self.h, c.size, _dp(c)), "ns_set_controls")
        self.nseg = c.size

    def adjoint_fwd(self, controls, **opts):
        """Forward run with binomial snapshots; returns (J, stats dict)."""
        o = adjoint_opts(**opts)
        c = np.ascontiguousarray(controls, dtype=np.float64)
        J = ctypes.c_double()
        st = NsAdjointStats()
        self._check(self.L.ns_step_adjoint_fwd(self.h, ctypes.byref(o), c.size, _dp(c), ctypes.byref(J), ctypes.byref(st)),
                    "ns_step_adjoint_fwd", allow_warn=True)
        self.nseg = c.size
        return J.value, stats_dict(st)

    def adjoint_bwd(self):
        """Reverse sweep of the last adjoint_fwd; returns (dJ/dcontrols, stats dict)."""
        g = np.zeros(max(1, getattr(self, "nseg", 0)))
        st = NsAdjointStats()
        self._check(self.L.ns_step_adjoint_bwd(self.h, _dp(g), ctypes.byref(st)), "ns_step_adjoint_bwd", allow_warn=True)
        return g[: getattr(self, "nseg", 0)], stats_dict(st)

    def adjoint_state_grad(self):
        ub = [np.zeros(self.face_shape(d)) for d in range(self.dim)]
        upb = [np.zeros(self.face_shape(d)) for d in range(self.dim)]
        pb = np.zeros(self.cell_shape())
        self._check(self.L.ns_adjoint_get_state_grad(self.h, self._vec(ub), self._vec(upb), _dp(pb)), "ns_adjoint_get_state_grad")
        return ub, upb, pb

    def step_jvp(self, du, duprev, dp, dc=None):
        du = [np.ascontiguousarray(a, dtype=np.float64) for a in du]
        dup = [np.ascontiguousarray(a, dtype=np.float64) for a in duprev]
        dp = np.ascontiguousarray(dp, dtype=np.float64)
        dc = None if dc is None else np.ascontiguousarray(dc, dtype=np.float64)
        o = [np.zeros(self.face_shape(d)) for d in range(self.dim)]
        op = [np.zeros(self.face_shape(d)) for d in range(self.dim)]
        odp = np.zeros(self.cell_shape())
        self._check(self.L.ns_step_jvp(self.h, self._vec(du), self._vec(dup), _dp(dp), _opt(dc), self._vec(o), self._vec(op), _dp(odp)),
                    "ns_step_jvp")
        return o, op, odp

    def step_vjp(self, ubar, uprevbar, pbar):
        ub = [np.ascontiguousarray(a, dtype=np.float64) for a in ubar]
        upb = [np.ascontiguousarray(a, dtype=np.float64) for a in uprevbar]
        pb = np.ascontiguousarray(pbar, dtype=np.float64)
        o = [np.zeros(self.face_shape(d)) for d in range(self.dim)]
        op = [np.zeros(self.face_shape(d)) for d in range(self.dim)]
        opb = np.zeros(self.cell_shape())
        cb = np.zeros(max(1, getattr(self, "nseg", 0)))
        self._check(self.L.ns_step_vjp(self.h, self._vec(ub), self._vec(upb), _dp(pb), self._vec(o), self._vec(op), _dp(opb), _dp(cb)),
                    "ns_step_vjp")
        return o, op, opb, cb[: getattr(self, "nseg", 0)]

    def adjoint_op(self, x, transpose=False, dc=None):
        """J x (+ dA/dc dc) or (J^T x, dA/dc^T x) at the current state's u*."""
        x = [np.ascontiguousarray(a, dtype=np.float64) for a in x]
        y = [np.zeros(self.face_shape(d)) for d in range(self.dim)]
        cb = np.zeros(max(1, getattr(self, "nseg", 0)))
        dcv = None if dc is None else np.ascontiguousarray(dc, dtype=np.float64)
        self._check(self.L.ns_adjoint_op(self.h, 1 if transpose else 0, self._vec(x), _opt(dcv), self._vec(y), _dp(cb)),
                    "ns_adjoint_op")
        return (y, cb[: getattr(self, "nseg", 0)]) if transpose else y
