"""Adjoint form: gradients of the integrated surface reaction rate after n
steps from mfg_adjoint_objective, against central finite differences of the
GPU forward and of the oracle's forward (the CPU restatement of the
reference's step), on a perturbed 16^3 catalyst case (8 gas + 2 site
species, 8 Arrhenius surface reactions, velocity inlet, WENO5).

Two parameter sets: the case's seeded Arrhenius table (one reaction carries
almost all of J) and a balanced table whose rate constants are all 1e3 at the
initial 500 K, so that every log A_r has a gradient of order J/8.

Tolerance: |g_adj - g_fd| <= 1e-6 |g_fd| + 2e-9 |J|, with central differences
of step h = 1e-5 in log A and in u_in (FD truncation O(h^2) and rounding
~eps |J| / h, both far below the bound)."""
import copy
import ctypes as C
import math

import numpy as np
import pytest

from mesoflow_gb300 import abi, cases
from mesoflow_gb300.adjoint import ReactionProblem, reaction_objective
from mesoflow_gb300.level import Level
from helpers import perturb
from oracle_run import OracleLevel

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

NSTEPS = 4
H = 1e-5
RTOL = 1e-6
ATOL_J = 2e-9


@pytest.fixture(scope="module", params=["arrhenius", "balanced"])
def setup(request):
    case = perturb(cases.catalyst(n=16, order=5, max_grid=8), 8, vel_amp=1e-2)
    if request.param == "balanced":
        for r in range(case.params.nreact):
            case.params.A[r] = 1e3 * math.exp(case.params.Ea[r] / (cases.RU * 500.0))
    o = OracleLevel(case)
    dt = o.est_timestep()
    logA = np.array([math.log(case.params.A[r]) for r in range(case.params.nreact)])
    u_in = case.meta["u_in"]
    return case, dt, logA, u_in


def oracle_J(case, P, dt, nsteps=NSTEPS, variant="strict"):
    c2 = copy.copy(case)
    c2.params = P
    o = OracleLevel(c2, variant=variant)
    for _ in range(nsteps):
        o.advance(dt)
    J = C.c_double()
    assert o.lib.oracle_objective(C.byref(P), C.byref(case.geom), o.desc, len(case.boxes), C.byref(J)) == 0
    return J.value


def fd(fun, logA, u_in, h=H):
    g = np.zeros(len(logA))
    for r in range(len(logA)):
        a, b = logA.copy(), logA.copy()
        a[r] += h
        b[r] -= h
        g[r] = (fun(a, u_in) - fun(b, u_in)) / (2 * h)
    hu = h * max(1.0, abs(u_in))
    gu = (fun(logA, u_in + hu) - fun(logA, u_in - hu)) / (2 * hu)
    return g, gu


def test_adjoint_configuration_gradient_matches_fd_of_oracle_h1e6():
    """The adjoint configuration's check at a size the oracle finishes in
    seconds: the catalyst block with its seeded sphere pack (seed 5), 32^3 in
    16^3 boxes, 10 steps with checkpoints every 5 steps (the bounded-memory
    path), central differences of the oracle's forward (OpenMP build, bitwise
    the strict one) with h = 1e-6, as in the adjoint benchmark's specification
    (there 128^3 and 50 steps, beyond what the CPU finishes 18 times).

    Tolerance for dJ/dlog A_r: 1e-6 |g| + 3e-8 |J|: with h = 1e-6 the central
    difference carries the rounding noise of J between the perturbed runs
    divided by h, about 1e-8 |J|; the gradients of the reactions that carry J
    agree to 1e-6 relative.  dJ/du_in is 4 orders of magnitude below J/u_in
    here (in 10 steps the inlet's influence has not reached the catalyst), and
    its central differences scatter by about 1% between step sizes (8.07e-15,
    8.15e-15, 8.19e-15 for h = 1e-4, 1e-5, 1e-6): the adjoint value must lie
    within the range of those three."""
    case = cases.catalyst(n=32, order=5, max_grid=16, seed=5)
    nsteps = 10
    dt = OracleLevel(case, variant="omp").est_timestep()
    logA = np.array([math.log(case.params.A[r]) for r in range(case.params.nreact)])
    u_in = case.meta["u_in"]
    p = ReactionProblem(case, nsteps, dt, checkpoint_every=5)
    J, gA, gu = p.gradient(logA, u_in)
    Jo = oracle_J(case, p.params_for(logA, u_in), dt, nsteps, "omp")
    assert abs(J - Jo) <= 1e-10 * abs(Jo)
    fA, fu = fd(lambda a, u: oracle_J(case, p.params_for(a, u), dt, nsteps, "omp"), logA, u_in, h=1e-6)
    print("J", J, "adjoint", gA, gu, "fd", fA, fu)
    print("worst |adjoint - fd| / |J| over log A", np.max(np.abs(gA - fA)) / abs(J))
    assert close(gA, fA, J, 3e-8), (gA, fA)
    fus = [fu]
    for h in (1e-5, 1e-4):
        Pp, Pm = p.params_for(logA, u_in + h), p.params_for(logA, u_in - h)
        fus.append((oracle_J(case, Pp, dt, nsteps, "omp") - oracle_J(case, Pm, dt, nsteps, "omp")) / (2 * h))
    print("dJ/du_in adjoint", gu, "fd over h = 1e-6, 1e-5, 1e-4", fus)
    assert min(fus) * (1 - 1e-6) <= gu <= max(fus) * (1 + 1e-6), (gu, fus)


def close(adj, ref, J, atol_j=ATOL_J):
    return np.all(np.abs(np.asarray(adj) - np.asarray(ref)) <= RTOL * np.abs(ref) + atol_j * abs(J))


def test_adjoint_forward_is_the_plain_step(setup):
    case, dt, logA, u_in = setup
    p = ReactionProblem(case, NSTEPS, dt, checkpoint_every=3)
    J0 = p.objective(logA, u_in)
    plain = p.level.get_state(case.shape_zyx)
    J, gA, gu = p.gradient(logA, u_in)
    after = p.level.get_state(case.shape_zyx)
    assert np.array_equal(plain, after)
    assert abs(J - J0) <= 1e-13 * abs(J0)
    assert J0 > 0 and np.all(np.isfinite(gA)) and np.isfinite(gu)


def test_adjoint_matches_fd_of_gpu_forward(setup):
    case, dt, logA, u_in = setup
    p = ReactionProblem(case, NSTEPS, dt, checkpoint_every=3)
    J, gA, gu = p.gradient(logA, u_in)
    fA, fu = fd(p.objective, logA, u_in)
    print("J", J, "adjoint dJ/dlogA", gA, "fd", fA, "dJ/du_in", gu, fu)
    assert close(gA, fA, J), (gA, fA)
    assert close(gu, fu, J), (gu, fu)


def test_adjoint_matches_fd_of_oracle(setup):
    case, dt, logA, u_in = setup
    p = ReactionProblem(case, NSTEPS, dt, checkpoint_every=2)
    J, gA, gu = p.gradient(logA, u_in)
    Jo = oracle_J(case, p.params_for(logA, u_in), dt)
    assert abs(J - Jo) <= 1e-10 * abs(Jo)
    fA, fu = fd(lambda a, u: oracle_J(case, p.params_for(a, u), dt), logA, u_in)
    assert close(gA, fA, J), (gA, fA)
    assert close(gu, fu, J), (gu, fu)


def test_checkpoint_interval_does_not_change_gradients(setup):
    case, dt, logA, u_in = setup
    ref = ReactionProblem(case, NSTEPS, dt, checkpoint_every=1).gradient(logA, u_in)
    for ce in (0, 2, 3, 10):
        J, gA, gu = ReactionProblem(case, NSTEPS, dt, checkpoint_every=ce).gradient(logA, u_in)
        assert abs(J - ref[0]) <= 1e-13 * abs(ref[0])
        assert np.allclose(gA, ref[1], rtol=1e-11, atol=1e-13 * np.abs(ref[1]).max())
        assert abs(gu - ref[2]) <= 1e-11 * abs(ref[2]) + 1e-13 * np.abs(ref[1]).max()


def test_autograd_function(setup):
    case, dt, logA, u_in = setup
    p = ReactionProblem(case, 2, dt)
    la = torch.tensor(logA, dtype=torch.float64, requires_grad=True)
    u = torch.tensor(u_in, dtype=torch.float64, requires_grad=True)
    J = reaction_objective(la, u, p)
    (2.0 * J).backward()
    J2, gA, gu = p.gradient(logA, u_in)
    assert abs(J.item() - J2) <= 1e-13 * abs(J2)
    assert np.allclose(la.grad.numpy(), 2.0 * gA, rtol=1e-11, atol=1e-13 * np.abs(gA).max())
    assert abs(u.grad.item() - 2.0 * gu) <= 1e-11 * abs(gu) + 1e-13 * np.abs(gA).max()


def test_adjoint_rejects_unsupported_configuration():
    case = cases.porous_ib(n=16, order=2, max_grid=8)
    lib = abi.load()
    abi.check("mfg_init", lib.mfg_init(C.byref(case.params)))
    lev = Level(case.boxes, case.ncomp, backend="torch", device="cuda", with_dsdt=False)
    lev.set_state(case.state)
    J = C.c_double()
    rc = lib.mfg_adjoint_objective(lev.descriptors(), len(case.boxes), C.byref(case.geom), 1, 1e-9, 1, C.byref(J),
                                   None, None, C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == abi.ERR_STATE


def test_flux_sweep_equals_per_face_form(setup):
    """The column-sweep adjoint flux kernel (default) and its per-face form
    sum the same edge adjoints in a different order: the gradients agree to
    rounding."""
    case, dt, logA, u_in = setup
    ref = ReactionProblem(case, NSTEPS, dt, checkpoint_every=0).gradient(logA, u_in)
    lib = abi.load()
    abi.check("form", lib.mfg_set_adjoint_flux_form(0))
    try:
        J, gA, gu = ReactionProblem(case, NSTEPS, dt, checkpoint_every=0).gradient(logA, u_in)
    finally:
        abi.check("form", lib.mfg_set_adjoint_flux_form(1))
    assert abs(J - ref[0]) <= 1e-13 * abs(ref[0])  # J is an atomic sum
    assert np.allclose(gA, ref[1], rtol=1e-11, atol=1e-13 * np.abs(ref[1]).max())
    assert abs(gu - ref[2]) <= 1e-11 * abs(ref[2]) + 1e-13 * np.abs(ref[1]).max()
