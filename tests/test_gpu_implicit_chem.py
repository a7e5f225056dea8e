"""Implicit (ROS2) chemistry sub-step on the GPU (mfg_set_chem_integrator
kind 1), which stands in for the reference's SUNDIALS CVODE option: stiff
decay (L-stable where explicit RK3 diverges, linear invariants kept),
accuracy against exp(-k dt), and the catalyst reactions against the oracle's
restatement and against many small explicit RK3 steps."""
import ctypes as C

import numpy as np
import pytest

from mesoflow_gb300 import abi, cases
from mesoflow_gb300.level import Level
from oracle_run import OracleLevel

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _decay(k):
    c = cases.catalyst(n=8, order=5, max_grid=8)
    P = c.params
    P.nreact = 1
    for s in range(abi.MAX_SPECIES):
        P.nu[0][s] = 0.0
        P.order[0][s] = 0.0
    P.nu[0][0], P.nu[0][1], P.order[0][0] = -1.0, 1.0, 1.0
    P.A[0], P.Ea[0] = k, 0.0
    return c


def _run(c, dt, kind, rtol=1e-8, atol=1e-12, maxsub=2000, nsub=1):
    lib = abi.load()
    abi.check("init", lib.mfg_init(C.byref(c.params)))
    abi.check("integrator", lib.mfg_set_chem_integrator(kind, rtol, atol, maxsub))
    try:
        lev = Level(c.boxes, c.ncomp, backend="torch", device="cuda")
        lev.set_state(c.state)
        st = C.c_void_p(torch.cuda.current_stream().cuda_stream)
        n = len(c.boxes)
        for q in range(nsub):
            for a, b in zip(lev.s_old, lev.s_new):
                a.copy_(b)
            abi.check("chem", lib.mfg_chem_substep(lev.descriptors(), n, C.byref(c.geom), 0.0, dt / nsub, st))
        torch.cuda.synchronize()
        v = C.c_uint32()
        abi.check("status", lib.mfg_status(C.byref(v), 1))
        assert not (v.value & abi.STATUS_CHEM_STEPS), "implicit chemistry ran out of substeps"
        return lev.get_state(c.shape_zyx)
    finally:
        abi.check("integrator", lib.mfg_set_chem_integrator(0, 1e-8, 1e-12, 1000))


def _oracle(c, dt, rtol, atol, maxsub=2000):
    o = OracleLevel(c)
    for a, b in zip(o.level.s_old, o.level.s_new):
        a[...] = b
    assert o.lib.oracle_chem_substep_ros2(C.byref(c.params), o.desc, len(c.boxes), dt, rtol, atol, maxsub) == 0
    return o.state()


def test_ros2_stiff_decay():
    c = _decay(1e10)  # k dt = 1e4
    A, B = abi.FLO_NVARS, abi.FLO_NVARS + 1
    a0, b0 = c.state[A], c.state[B]
    g = _run(c, 1e-6, 1, rtol=1e-3, atol=1e-6)
    assert np.all(np.abs(g[A]) <= 1e-6 * a0.max())
    assert np.allclose(g[A] + g[B], a0 + b0, rtol=1e-13, atol=0)
    o = _oracle(c, 1e-6, 1e-3, 1e-6)
    assert np.allclose(g[B], o[B], rtol=1e-12, atol=0)
    # the explicit SSP-RK3 sub-step is unstable at this k dt
    e = _run(c, 1e-6, 0)
    assert not np.all(np.abs(e[A]) <= 1e3 * a0.max())


def test_ros2_accuracy_and_oracle():
    c = _decay(5e5)  # k dt = 0.5
    A = abi.FLO_NVARS
    g = _run(c, 1e-6, 1, rtol=1e-6, atol=1e-12)
    assert np.allclose(g[A], c.state[A] * np.exp(-0.5), rtol=2e-5, atol=0)
    o = _oracle(c, 1e-6, 1e-6, 1e-12)
    assert np.allclose(g[A], o[A], rtol=1e-9, atol=0)


def test_ros2_catalyst_matches_fine_explicit_and_oracle():
    """The catalyst's surface reactions over dt = 2e-5 s (k c dt up to ~4: a
    few e-folds of the fastest pathway), ROS2 at rtol 1e-5 against 200 explicit
    RK3 sub-steps (errors ~1e-8) and against the oracle's ROS2."""
    c = cases.catalyst(n=8, order=5, max_grid=8)
    dt = 2e-5
    sp = slice(abi.FLO_NVARS, abi.FLO_NVARS + c.params.nspec)
    g = _run(c, dt, 1, rtol=1e-5, atol=1e-10, maxsub=5000)
    ref = _run(c, dt, 0, nsub=200)
    scale = np.abs(ref[sp]).max(axis=(1, 2, 3), keepdims=True)
    assert np.max(np.abs(g[sp] - ref[sp]) / scale) < 1e-4
    o = _oracle(c, dt, 1e-5, 1e-10, maxsub=5000)
    assert np.max(np.abs(g[sp] - o[sp]) / scale) < 1e-7
    # the non-species components are untouched
    assert np.array_equal(g[:abi.FLO_NVARS], c.state[:abi.FLO_NVARS])
