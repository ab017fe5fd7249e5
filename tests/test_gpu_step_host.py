"""ns_step_host, the end-to-end host-buffer step (the path bench.py times as
e2e): (u, u_prev, p) in from pinned host memory, one step, (u, u_prev, p)
out, updated in place. Two calls in a row must equal, bit for bit, ns_step on
a device-resident context from the same state; the outgoing u_prev (copied
back on a second stream while the step runs, in 2D) is the incoming u."""
import numpy as np
import pytest

import amressif_gb300 as ns

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dim,precision", [(2, ns.PREC_FP64), (2, ns.PREC_MIXED), (3, ns.PREC_MIXED)])
def test_step_host_matches_device_steps(gpu_lib, dim, precision):
    n = 64 if dim == 2 else 16
    mk = lambda: ns.Solver(ns.default_params(dim=dim, n_cell=n, ren=400.0, fixed_dt=0.5 / n, iter_num=100,
                                             precision=precision, poisson_tol_rel=1e-12))
    a, b = mk(), mk()
    a.init(ns.INIT_CAVITY)
    for _ in range(2):
        a.step()
    u, up, p, _ = a.get_state()
    b.set_state(u, up, p, time=a.time)
    shp = [a.face_shape(d) for d in range(dim)]
    bufs = [ns.PinnedArray(s) for s in shp] + [ns.PinnedArray(s) for s in shp] + [ns.PinnedArray(a.cell_shape())]
    for buf, arr in zip(bufs, u + up + [p]):
        buf.a[...] = arr
    uh, uph, ph = [x.a for x in bufs[:dim]], [x.a for x in bufs[dim:2 * dim]], bufs[-1].a
    for call in range(2):
        u_in = [x.copy() for x in uh]
        st_h = a.step_host(uh, uph, ph)
        st_d = b.step()
        assert st_h["pseudo_iters"] == st_d["pseudo_iters"], call
        assert st_h["ms_h2d"] > 0 and st_h["ms_d2h"] > 0
        ub, upb, pb, _ = b.get_state()
        for d in range(dim):
            np.testing.assert_array_equal(uh[d], ub[d], err_msg="call %d u" % call)
            np.testing.assert_array_equal(uph[d], upb[d], err_msg="call %d u_prev" % call)
            np.testing.assert_array_equal(uph[d], u_in[d])
        np.testing.assert_array_equal(ph, pb)
    for x in bufs:
        x.free()
    a.close()
    b.close()
