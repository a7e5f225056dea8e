"""The GPU against the oracle at the benchmark configurations' full size.

* The 256^3 immersed-boundary benchmark workload exactly as bench.py runs it
  (sphere pack, order 2, 64^3 boxes, the cut-cell cache and the compacted face
  lists on): after three warm-up steps on the GPU, one more step of
  mfg_advance_level equals one oracle step (OpenMP build, run here on the
  host) from the same state per cell and component to 1e-12 of the
  component's domain maximum.
* 256^3 5-species Taylor-Green, WENO5, CFL 0.4, 100 steps of the flow step:
  the GPU replays the dt sequence of the oracle's own 100-step run
  (tests/golden/tg256.npz, made by tests/golden/make_fullsize.py) and
  matches the oracle's residual norm at every step (to 1e-9 of the norm plus
  the one-step tolerance carried through (U_n+1 - U_n)/dt) and its final state
  at 4096 seeded sample cells (relative L2 per component <= 1e-10).
* 256^3 sphere pack, order 2, 500 steps toward steady state: the GPU replays
  the oracle's dt sequence (tests/golden/ib256.npz) and matches its Darcy
  permeability every 50 steps to 1e-9 relative, and its final state at the
  sample cells (relative L2 <= 1e-10).
"""
import os

import numpy as np
import pytest

from mesoflow_gb300 import abi, cases
from mesoflow_gb300.driver import Mflo
from helpers import rel_err
from oracle_run import OracleLevel

torch = pytest.importorskip("torch")
pytestmark = [pytest.mark.gpu, pytest.mark.slow]

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
TOL_STEP = 1e-12
TOL_L2 = 1e-10


def fixture(name):
    p = os.path.join(GOLDEN, name + ".npz")
    if not os.path.exists(p):
        pytest.skip(f"{name}.npz not generated (tests/golden/make_fullsize.py)")
    return np.load(p)


def test_bench_workload_one_step_matches_oracle():
    c = cases.porous_ib(n=256, order=2, max_grid=64)
    g = Mflo(c, device="cuda")
    dt = g.est_timestep()
    for _ in range(3):  # warm-up as the benchmark: the cut-cell cache is built and in use
        g.advance(dt, norms=False)
    o = OracleLevel(c, variant="omp")
    o.level.set_state(g.state())  # one step of each from the same state
    ro = o.advance(dt)
    g.advance(dt, norms=True)
    err, comp = rel_err(g.state(), o.state())
    print(f"bench workload, one step: max per-cell error / component max {err:.3e} (component {comp})")
    assert err <= TOL_STEP, (err, comp)
    so = o.state()
    scale = np.array([np.linalg.norm(so[q]) for q in range(c.ncomp)]) / dt
    assert np.all(np.abs(g.resnorms - ro) <= 1e-9 * np.abs(ro) + TOL_STEP * scale)


def sample_l2(state, F, what):
    flat = state.reshape(state.shape[0], -1)[:, F["idx"]]
    ref = F["sample"]
    worst = 0.0
    for q in range(ref.shape[0]):
        den = np.linalg.norm(ref[q])
        if den > 0:
            e = np.linalg.norm(flat[q] - ref[q]) / den
            worst = max(worst, e)
            assert e <= TOL_L2, q
    print(f"{what}: worst relative L2 over the sample cells {worst:.3e}")


def test_taylor_green_256_100_steps_matches_oracle():
    F = fixture("tg256")
    c = cases.taylor_green_mix(n=256, order=5, max_grid=64)
    g = Mflo(c, device="cuda", only_flow=True)
    norms = []
    for dt in F["dts"]:
        g.advance(float(dt), norms=True)
        norms.append(g.resnorms.copy())
    norms = np.array(norms)
    on = F["norms"]
    state_scale = F["l2"][None, :] / F["dts"][:, None]
    nz = on != 0
    print(f"taylor-green 100 steps: worst residual-norm relative difference "
          f"{np.max(np.abs(norms - on)[nz] / np.abs(on)[nz]):.3e}")
    assert np.all(np.abs(norms - on) <= 1e-9 * np.abs(on) + TOL_STEP * state_scale)
    sample_l2(g.state(), F, "taylor-green 100 steps")


def test_ib_256_500_steps_permeability_matches_oracle():
    F = fixture("ib256")
    c = cases.porous_ib(n=256, order=2, max_grid=64)
    g = Mflo(c, device="cuda")
    every = int(F["perm_every"])
    perms = []
    for s, dt in enumerate(F["dts"]):
        g.advance(float(dt), norms=False)
        if (s + 1) % every == 0:
            perms.append(cases.permeability(c, g.state()))
    perms = np.array(perms)
    print(f"sphere pack 500 steps: permeability GPU {perms[-1]:.12e} oracle {F['perms'][-1]:.12e}, worst relative "
          f"difference {np.max(np.abs(perms - F['perms']) / np.abs(F['perms'])):.3e}")
    assert np.all(np.abs(perms - F["perms"]) <= 1e-9 * np.abs(F["perms"])), (perms, F["perms"])
    sample_l2(g.state(), F, "sphere pack 500 steps")
