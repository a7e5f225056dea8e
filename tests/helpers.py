"""Shared helpers of the parity tests."""
import numpy as np

from mesoflow_gb300 import abi


def rel_err(g, o, axis_comp=0):
    """Per-component max |g - o| / s_c with s_c = max over the domain of |o_c|
    (the floor keeps near-zero fields, e.g. resting velocities, out of a
    relative test).  Returns the worst component's value and its index."""
    g = np.asarray(g)
    o = np.asarray(o)
    worst, wc = 0.0, -1
    for c in range(o.shape[axis_comp]):
        oc = np.take(o, c, axis=axis_comp)
        gc = np.take(g, c, axis=axis_comp)
        s = np.abs(oc).max()
        if s == 0.0:
            e = np.abs(gc).max()
        else:
            e = np.abs(gc - oc).max() / s
        if e > worst or wc < 0:
            worst, wc = e, c
    return worst, wc


def perturb(case, seed, amp=1e-3, vel_amp=None):
    """Seeded perturbation of a case's conserved and primitive fields, so that
    parity is tested on non-uniform states."""
    rng = np.random.default_rng(seed)
    S = case.state.copy()
    shp = S.shape[1:]
    for c in (abi.RHO, abi.RHOE, abi.DENS, abi.PRES, abi.TEMP):
        S[c] *= 1.0 + amp * rng.standard_normal(shp)
    va = vel_amp if vel_amp is not None else amp * 10.0
    for c in (abi.RHOU, abi.RHOV, abi.RHOW):
        S[c] += va * S[abi.RHO] * rng.standard_normal(shp)
    for c in (abi.VELX, abi.VELY, abi.VELZ):
        S[c] += va * rng.standard_normal(shp)
    for s in range(case.params.nspec):
        S[abi.FLO_NVARS + s] *= 1.0 + amp * rng.standard_normal(shp)
    case.state = S
    return case
