"""The Array4 box interface (ns_put_box / ns_get_box) as an AMReX host uses it.

The reference splits the domain into boxes of max_grid_size (main.cpp:317-324)
and keeps every field in ghosted FArrayBoxes (main.cpp:330-383); a host hands
the library each valid box through MultiFab::array(mfi), i.e. a pointer to
the box's lo corner inside a ghosted buffer, with the buffer's own jstride
and kstride. These tests place the four 64^2 boxes of a 128^2 cavity
(and eight 8^3 boxes of a 16^3 cavity) in ghosted host buffers whose ghost
cells hold NaN, move them in box by box, and require the next step to be
bitwise identical to the one of a context filled with ns_set_state; ns_get_box
must return each box bit for bit and leave the ghost cells untouched.
"""
import ctypes

import numpy as np
import pytest

import amressif_gb300 as ns

pytestmark = pytest.mark.gpu

NG = 2  # ghost layers of the host buffers (velCart's count, main.cpp:347)


class GhostedBox:
    """A ghosted host FArrayBox over [lo, hi] (x fastest), ghosts NaN."""

    def __init__(self, lo, hi, dim):
        self.lo, self.hi, self.dim = list(lo), list(hi), dim
        ext = [hi[d] - lo[d] + 1 + 2 * NG if d < dim else 1 for d in range(3)]
        self.buf = np.full(tuple(reversed(ext)), np.nan)
        self.jstride = ext[0]
        self.kstride = ext[0] * ext[1]

    def valid(self):
        s = tuple(slice(NG, NG + self.hi[d] - self.lo[d] + 1) for d in reversed(range(self.dim)))
        return self.buf[(0,) + s] if self.dim == 2 else self.buf[s]

    def ptr(self):
        off = NG + NG * self.jstride + (NG * self.kstride if self.dim == 3 else 0)
        return ctypes.cast(self.buf.ctypes.data + 8 * off, ctypes.POINTER(ctypes.c_double))


def lohi(lo, hi):
    return (ctypes.c_int * 3)(*lo), (ctypes.c_int * 3)(*hi)


def put(s, field, comp, box):
    lo, hi = lohi(box.lo, box.hi)
    return ns.lib().ns_put_box(s.h, field, comp, box.ptr(), lo, hi, box.jstride, box.kstride, 0)


def get(s, field, comp, box):
    lo, hi = lohi(box.lo, box.hi)
    return ns.lib().ns_get_box(s.h, field, comp, box.ptr(), lo, hi, box.jstride, box.kstride, 0)


def boxes(n, m, dim, face_dir=None):
    """The boxes of max_grid_size m (face fields extend to n along face_dir)."""
    out = []
    for idx in np.ndindex(*([n // m] * dim)):
        lo = [idx[d] * m for d in range(dim)] + [0] * (3 - dim)
        hi = [lo[d] + m - 1 + (1 if d == face_dir else 0) for d in range(dim)] + [0] * (3 - dim)
        out.append((lo, hi))
    return out


def sl(a, lo, hi, dim):
    return a[tuple(slice(lo[d], hi[d] + 1) for d in reversed(range(dim)))]


def fill_by_boxes(s, state, n, m, dim):
    u, up, p = state
    for comp in range(dim):
        for field, arr in ((ns.FIELD_VEL, u[comp]), (ns.FIELD_VEL_PREV, up[comp])):
            for lo, hi in boxes(n, m, dim, comp):
                b = GhostedBox(lo, hi, dim)
                b.valid()[...] = sl(arr, lo, hi, dim)
                assert put(s, field, comp, b) == ns.NS_OK
    for lo, hi in boxes(n, m, dim):
        b = GhostedBox(lo, hi, dim)
        b.valid()[...] = sl(p, lo, hi, dim)
        assert put(s, ns.FIELD_PRESSURE, 0, b) == ns.NS_OK


def check_round_trip(s, state, n, m, dim):
    u, up, p = state
    for comp in range(dim):
        for field, arr in ((ns.FIELD_VEL, u[comp]), (ns.FIELD_VEL_PREV, up[comp])):
            for lo, hi in boxes(n, m, dim, comp):
                b = GhostedBox(lo, hi, dim)
                assert get(s, field, comp, b) == ns.NS_OK
                np.testing.assert_array_equal(b.valid(), sl(arr, lo, hi, dim))
                assert np.isnan(b.buf).sum() == b.buf.size - b.valid().size  # ghosts untouched
    for lo, hi in boxes(n, m, dim):
        b = GhostedBox(lo, hi, dim)
        assert get(s, ns.FIELD_PRESSURE, 0, b) == ns.NS_OK
        np.testing.assert_array_equal(b.valid(), sl(p, lo, hi, dim))


def params(dim, n, m):
    kw = dict(dim=dim, n_cell=n, ren=100.0, fixed_dt=0.5 / n, iter_num=100, precision=ns.PREC_FP64_EXACT,
              poisson_tol_rel=1e-12, max_grid_size=(m, m, m))
    return ns.default_params(**kw)


@pytest.mark.parametrize("dim,n,m,steps", [(2, 128, 64, 3), (3, 16, 8, 2)])
def test_boxes_match_whole_state(gpu_lib, dim, n, m, steps):
    a = ns.Solver(params(dim, n, m))
    a.init(ns.INIT_CAVITY)
    for _ in range(steps):
        a.step()
    u, up, p, _ = a.get_state()
    state = (u, up, p)
    b = ns.Solver(params(dim, n, m))
    zf = [np.zeros(b.face_shape(d)) for d in range(dim)]
    b.set_state(zf, zf, np.zeros(b.cell_shape()), time=a.time)
    fill_by_boxes(b, state, n, m, dim)
    check_round_trip(b, state, n, m, dim)
    sa, sb = a.step(), b.step()
    assert sa["pseudo_iters"] == sb["pseudo_iters"]
    ua, upa, pa, _ = a.get_state()
    ub, upb, pb, _ = b.get_state()
    for d in range(dim):
        np.testing.assert_array_equal(ua[d], ub[d])
        np.testing.assert_array_equal(upa[d], upb[d])
    np.testing.assert_array_equal(pa, pb)
    a.close()
    b.close()


def test_box_arguments_are_validated(gpu_lib):
    s2 = ns.Solver(params(2, 32, 16))
    s3 = ns.Solver(params(3, 16, 8))
    L = ns.lib()
    buf = np.zeros(40 * 40 * 40)
    ptr = buf.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    cases = [
        (s2, ns.FIELD_VEL, 0, (0, 0, 0), (16, 15, 0), 16, 0, ns.NS_ERR_ARG),   # jstride below the width 17
        (s2, ns.FIELD_VEL, 0, (0, 0, 0), (33, 15, 0), 40, 0, ns.NS_ERR_ARG),   # face box beyond x face 32
        (s2, ns.FIELD_PRESSURE, 0, (0, 0, 0), (32, 0, 0), 40, 0, ns.NS_ERR_ARG),  # cell box beyond cell 31
        (s2, ns.FIELD_VEL, 0, (0, 0, 1), (8, 8, 1), 40, 0, ns.NS_ERR_ARG),     # 2D takes only the plane k = 0
        (s2, ns.FIELD_VEL, 2, (0, 0, 0), (8, 8, 0), 40, 0, ns.NS_ERR_ARG),     # no z component in 2D
        (s2, 99, 0, (0, 0, 0), (8, 8, 0), 40, 0, ns.NS_ERR_ARG),               # unknown field
        (s3, ns.FIELD_VEL, 2, (0, 0, 0), (7, 7, 8), 8, 60, ns.NS_ERR_ARG),     # kstride below a plane (8 x 8)
        (s3, ns.FIELD_VEL, 2, (0, 0, 0), (7, 7, 17), 8, 64, ns.NS_ERR_ARG),    # z face box beyond face 16
        (s3, ns.FIELD_CART, 0, (0, 0, 0), (7, 7, 7), 8, 64, ns.NS_ERR_ARG),    # the cell-velocity override is put only
        (s3, ns.FIELD_VEL, 2, (0, 0, 0), (7, 7, 16), 8, 64, ns.NS_OK),         # the whole z extent of a box
        (s2, ns.FIELD_VEL, 1, (0, 0, 0), (31, 32, 0), 32, 0, ns.NS_OK),        # the whole v field
    ]
    for s, field, comp, lo, hi, js, ks, want in cases:
        l, h = lohi(lo, hi)
        assert L.ns_get_box(s.h, field, comp, ptr, l, h, js, ks, 0) == want, (field, comp, lo, hi, js, ks)
    s2.close()
    s3.close()
