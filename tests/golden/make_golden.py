"""Generate the golden fixtures of the CPU oracle.

The reference ships no golden vectors, so these fixtures pin the oracle's own
output (checked in tests/test_oracle.py against known answers) so that every
build of it (x86 here, Arm on the GPU host) and the CUDA path are compared to
the same numbers.

cavity32_exec_inputs.npz: the shipped inputs-file physics (n_cell 32, boxes
32x16, Re 100, fixed_dt 1e-3, 11 steps, lid u = 1), every step: u, v, p
(mean removed) and the pseudo-iteration count K.

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


if __name__ == "__main__":
    cavity32()
    print("ok")
