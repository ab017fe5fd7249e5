"""Generate the golden fixtures of the CPU oracle.

The reference ships no golden vectors, so these fixtures pin the oracle's own
output (checked in tests/test_oracle.py against known answers) so that every
build of it (x86 here, Arm on the GPU host) and the CUDA path are compared to
the same numbers.

cavity32_exec_inputs.npz: the shipped inputs-file physics (n_cell 32, boxes
32x16, Re 100, fixed_dt 1e-3, 11 steps, lid u = 1), every step: u, v, p
(mean removed) and the pseudo-iteration count K.

cavity16_3d.npz: the lid cavity in the AMREX_SPACEDIM = 3 build (16^3 cells,
one box, Re 100, fixed_dt 0.4 dx, lid u = 1), 5 steps from rest: K of each
step, the kinetic energy of each step, and the final u, v, w and p (mean
removed).

Run: python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle.orc import Oracle  # noqa: E402


def cavity32():
    o = Oracle(32, max_grid_size=(32, 16, 16), ren=100.0, dt=1e-3, iter_num=100, poisson_tol=1e-13)
    o.init(0)
    out = {"nsteps": 11}
    K = []
    for step in range(1, 12):
        s = o.step()
        K.append(s["pseudo_iters"])
        u, _, p, _ = o.get_state()
        out["u_%d" % step] = u[0]
        out["v_%d" % step] = u[1]
        out["p_%d" % step] = p - p.mean()
    out["K"] = np.array(K)
    np.savez_compressed(os.path.join(HERE, "cavity32_exec_inputs.npz"), **out)


def cavity16_3d():
    n = 16
    o = Oracle(n, dim=3, max_grid_size=(n, n, n), ren=100.0, dt=0.4 / n, iter_num=100, poisson_tol=1e-13,
               bc_lo=(135, 135, 135), bc_hi=(135, 165, 135))
    o.init(0)
    K, E = [], []
    for _ in range(5):
        s = o.step()
        K.append(s["pseudo_iters"])
        u, _, p, _ = o.get_state()
        E.append(0.5 * sum(float((a * a).sum()) for a in u) / n ** 3)
    out = {"nsteps": 5, "K": np.array(K), "energy": np.array(E), "u": u[0], "v": u[1], "w": u[2], "p": p - p.mean()}
    np.savez_compressed(os.path.join(HERE, "cavity16_3d.npz"), **out)


if __name__ == "__main__":
    cavity32()
    cavity16_3d()
    print("ok")
