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
