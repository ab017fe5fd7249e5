"""Checkpoint / restart (ns_checkpoint_get / ns_checkpoint_put): a run that is
checkpointed, written to the reference's directory layout, read back into a
fresh context and continued must reproduce the uninterrupted run bit for bit
(the pseudo-iteration counts included), in the FP64 and mixed modes."""
import numpy as np
import pytest

import amressif_gb300 as ns
from amressif_gb300 import checkpoint as ck

pytestmark = pytest.mark.gpu


def params(precision):
    return ns.default_params(n_cell=64, ren=400.0, fixed_dt=0.5 / 64, iter_num=100, precision=precision,
                             poisson_tol_rel=1e-12, max_grid_size=(32, 32, 32))


@pytest.mark.parametrize("precision", [ns.PREC_FP64_EXACT, ns.PREC_MIXED])
def test_restart_is_bit_exact(gpu_lib, tmp_path, precision):
    a = ns.Solver(params(precision))
    a.init(ns.INIT_CAVITY)
    for _ in range(4):
        a.step()
    u, up, p, t, k = a.checkpoint_get()
    assert k == 4 and t == pytest.approx(4 * 0.5 / 64)
    path = ck.write_checkpoint(str(tmp_path), k, u, up, p, t, (32, 32))
    ka = [a.step()["pseudo_iters"] for _ in range(3)]
    ua, upa, pa, ta, kka = a.checkpoint_get()

    u2, up2, p2, t2 = ck.read_checkpoint(path)
    b = ns.Solver(params(precision))
    b.checkpoint_put(u2, up2, p2, t2, k)
    kb = [b.step()["pseudo_iters"] for _ in range(3)]
    ub, upb, pb, tb, kkb = b.checkpoint_get()
    assert ka == kb and kka == kkb == 7
    assert ta == tb
    for x, y in zip(ua + upa, ub + upb):
        np.testing.assert_array_equal(x, y)
    np.testing.assert_array_equal(pa, pb)


@pytest.mark.parametrize("precision", [ns.PREC_FP64, ns.PREC_MIXED])
def test_restart_is_bit_exact_3d(gpu_lib, tmp_path, precision):
    """3D: the reference's vel_zCont / vel_zContPrev files included"""
    kw = dict(dim=3, n_cell=16, ren=100.0, fixed_dt=0.4 / 16, iter_num=100, precision=precision,
              poisson_tol_rel=1e-12, max_grid_size=(8, 8, 8))
    a = ns.Solver(ns.default_params(**kw))
    a.init(ns.INIT_CAVITY)
    for _ in range(3):
        a.step()
    u, up, p, t, k = a.checkpoint_get()
    path = ck.write_checkpoint(str(tmp_path), k, u, up, p, t, (8, 8, 8))
    ka = [a.step()["pseudo_iters"] for _ in range(2)]
    ua, upa, pa, _, _ = a.checkpoint_get()
    u2, up2, p2, t2 = ck.read_checkpoint(path)
    b = ns.Solver(ns.default_params(**kw))
    b.checkpoint_put(u2, up2, p2, t2, k)
    kb = [b.step()["pseudo_iters"] for _ in range(2)]
    ub, upb, pb, _, kkb = b.checkpoint_get()
    assert ka == kb and kkb == 5
    for x, y in zip(ua + upa, ub + upb):
        np.testing.assert_array_equal(x, y)
    np.testing.assert_array_equal(pa, pb)


@pytest.mark.parametrize("dim", [2, 3])
def test_plotfile_from_device_cell_velocity(gpu_lib, tmp_path, dim):
    """Export_Flow_Field's velCart from the device (ns_get_cell_velocity)
    equals the face averages of the state, bit for bit, and lands in the
    plotfile's U, V (, W) components"""
    n = 32 if dim == 2 else 16
    s = ns.Solver(ns.default_params(dim=dim, n_cell=n, ren=100.0, fixed_dt=0.4 / n, poisson_tol_rel=1e-12,
                                    precision=ns.PREC_FP64))
    s.init(ns.INIT_CAVITY)
    for _ in range(2):
        s.step()
    u, _, p, _ = s.get_state()
    cart = s.cell_velocity()
    ref = ck.cell_velocity(u)
    for a, b in zip(cart, ref):
        np.testing.assert_array_equal(a, b)
    path = ck.write_plotfile(str(tmp_path), "plt", s.step_count, u, p, s.time, (8,) * dim, cart=cart)
    f, t, step = ck.read_plotfile(path)
    assert step == 2 and t == s.time
    for name, c in zip("UVW", cart):
        np.testing.assert_array_equal(f[name], c)
