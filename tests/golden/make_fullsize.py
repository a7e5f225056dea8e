"""Writes the full-size oracle fixtures used by tests/test_gpu_fullsize_oracle.py.

The oracle (the CPU restatement of the reference's numerics, OpenMP build,
bitwise equal to the strict build) runs two of the benchmark configurations
at their stated size and step count:

  tg256   256^3 periodic 5-species Taylor-Green, WENO5, CFL 0.4, 100 steps of
          the flow step (no chemistry: the mixture does not react), dt from
          ComputeDt each step, the flow residual norm recorded every step.
  ib256   256^3 sphere pack (solid fraction 0.4), pressure-driven air, order 2,
          CFL 0.1, 500 steps, dt from ComputeDt each step, the Darcy
          permeability recorded every 50 steps.

Each fixture stores the dt sequence (so the GPU run replays exactly the same
steps), the per-step residual norms, per-component sums and L2 norms of the
final state, the final state at 4096 seeded sample cells, and for ib256 the
permeability history.  Several CPU hours on 8 cores:

    OMP_NUM_THREADS=8 python tests/golden/make_fullsize.py tg256
    OMP_NUM_THREADS=8 python tests/golden/make_fullsize.py ib256
"""
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for p in (ROOT, os.path.dirname(HERE)):
    if p not in sys.path:
        sys.path.insert(0, p)

from mesoflow_gb300 import cases  # noqa: E402
from oracle_run import OracleLevel  # noqa: E402

NSAMPLE = 4096


def sample_index(n, seed=7):
    return np.sort(np.random.default_rng(seed).choice(n ** 3, NSAMPLE, replace=False))


def config(name):
    if name == "tg256":
        return cases.taylor_green_mix(n=256, order=5, max_grid=64), 100, True, 0
    if name == "ib256":
        return cases.porous_ib(n=256, order=2, max_grid=64), 500, False, 50
    raise SystemExit("unknown fixture " + name)


def run(name):
    case, nsteps, only_flow, perm_every = config(name)
    o = OracleLevel(case, variant="omp")
    dts, norms, perms = [], [], []
    t0 = time.time()
    for s in range(nsteps):
        dt = o.compute_dt()
        norms.append(o.advance(dt, only_flow=only_flow))
        dts.append(dt)
        if perm_every and (s + 1) % perm_every == 0:
            perms.append(cases.permeability(case, o.state()))
        print(f"{name} step {s + 1}/{nsteps} dt {dt:.6e} {time.time() - t0:.0f} s", flush=True)
    S = o.state()
    flat = S.reshape(S.shape[0], -1)
    idx = sample_index(case.n_cell[0])
    out = os.path.join(HERE, f"{name}.npz")
    np.savez_compressed(out, dts=np.array(dts), norms=np.array(norms), sums=flat.sum(axis=1, dtype=np.float64),
                        l2=np.sqrt((flat * flat).sum(axis=1, dtype=np.float64)), absmax=np.abs(flat).max(axis=1),
                        idx=idx, sample=flat[:, idx], perms=np.array(perms), perm_every=perm_every)
    print("wrote", out, flush=True)


if __name__ == "__main__":
    for a in sys.argv[1:]:
        run(a)
