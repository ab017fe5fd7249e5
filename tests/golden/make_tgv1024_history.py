"""Per-step history of the oracle over the full 500 steps of the perturbed
Taylor-Green run at 1024^2 (doubly periodic [0, 2 pi]^2, Re = 1000,
dt = 0.5 dx, the seeded 1e-3 divergence-free perturbation of
amressif_gb300.workloads, the reference's parity mode with quirks Q1/Q2).

The oracle takes seconds per step at this size, so the GPU test compares its
own 500-step run with this fixture instead of running the oracle beside it.
Recorded per step: the pseudo-iteration count K, max|div u| after the
projection, the kinetic energy 1/2 h^2 (sum u^2 + sum v^2) over the faces
0..n-1 of each direction, the projection of (u, v) on the initial
Taylor-Green mode, and the 2-norms of u, v and p (p with its mean removed).

Run: python tests/golden/make_tgv1024_history.py   (about 35 min on 8 cores)
"""
import json
import math
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from amressif_gb300 import workloads as wl  # noqa: E402
from oracle.orc import Oracle  # noqa: E402

N = 1024
NSTEPS = 500
OUT = os.path.join(HERE, "tgv1024_parity_history.json")


def scalars(u, v, p, h):
    n = u.shape[0]
    return {"ke": 0.5 * h * h * float((u[:, :n] ** 2).sum() + (v[:n, :] ** 2).sum()),
            "amp": wl.tgv_amplitude(u, v), "norm_u": float(np.linalg.norm(u)), "norm_v": float(np.linalg.norm(v)),
            "norm_p": float(np.linalg.norm(p - p.mean()))}


def main():
    h = 2 * math.pi / N
    o = Oracle(N, ren=1000.0, dt=0.5 * h, iter_num=100, poisson_tol=1e-13, max_grid_size=(N, N, N),
               prob_hi=(2 * math.pi,) * 3, bc_lo=(111,) * 3, bc_hi=(111,) * 3)
    u, up, p = wl.tgv_perturbed_state(N, amp=1e-3, seed=0)
    o.set_state(u, up, p)
    hist = []
    t0 = time.time()
    for step in range(1, NSTEPS + 1):
        st = o.step()
        ug, _, pg, _ = o.get_state()
        rec = {"step": step, "K": st["pseudo_iters"], "div_after": st["div_after"]}
        rec.update(scalars(ug[0], ug[1], pg, h))
        hist.append(rec)
        if step % 25 == 0:
            print("step %d K=%d %.0f s" % (step, rec["K"], time.time() - t0), flush=True)
    o.close()
    out = {"workload": "Taylor-Green 1024^2, [0,2pi]^2 periodic, Re=1000, dt=0.5dx, seeded 1e-3 perturbation "
                       "(seed 0), parity mode (Q1/Q2), oracle Poisson tolerance 1e-13",
           "nsteps": NSTEPS, "history": hist}
    with open(OUT, "w") as f:
        json.dump(out, f, indent=0)


if __name__ == "__main__":
    main()
