"""Gradients of the integrated surface reaction rate through the library's
hand-written discrete adjoint of the RK3 step (mfg_adjoint_objective), and a
torch.autograd.Function over it.

The objective is J = dx dy dz * sum_cells sum_r k_r(T) prod_s c_s^o_rs on the
state after n steps of mfg_advance_level (chemistry and clipping on) from a
fixed initial state; the parameters are the log pre-exponentials log A_r of
the reaction table and the normal velocity u_in of the velocity-inlet
boundaries.  The reference solver has no adjoint: this follows its forward
step (Source/mflo_evolve.cpp:251-318) and its rate law (chemistry.H
compute_spec_source).
"""
import ctypes as C
import math

import numpy as np

from . import abi
from .level import Level


def _copy_params(p):
    return abi.Params.from_buffer_copy(p)


class ReactionProblem:
    """A case advanced nsteps steps of dt from its initial state on the GPU."""

    def __init__(self, case, nsteps, dt, checkpoint_every=10, device="cuda"):
        import torch
        self.lib = abi.load()
        self.case = case
        self.nsteps = int(nsteps)
        self.dt = float(dt)
        self.checkpoint_every = int(checkpoint_every)
        self.nreact = case.params.nreact
        self.level = Level(case.boxes, case.ncomp, backend="torch", device=device, with_dsdt=False)
        self.desc = self.level.descriptors()
        self.stream = torch.cuda.current_stream().cuda_stream

    def params_for(self, logA, u_in):
        """The case's parameter table with A_r = exp(log A_r) and the inlet velocity set."""
        P = _copy_params(self.case.params)
        for r in range(self.nreact):
            P.A[r] = math.exp(float(logA[r]))
        for d in range(3):
            for kind, ext in ((P.bc_lo[d], P.ext_lo[d]), (P.bc_hi[d], P.ext_hi[d])):
                if kind == abi.BC_EXT_DIR and ext.kind == abi.EXT_VELOCITY_INLET:
                    ext.vel[d] = float(u_in)
        return P

    def reset(self, logA, u_in):
        """Uploads the parameter table for (log A, u_in) and restores the initial state."""
        P = self.params_for(logA, u_in)
        abi.check("mfg_init", self.lib.mfg_init(C.byref(P)))
        self.level.set_state(self.case.state)

    def objective(self, logA, u_in):
        """J after nsteps plain steps (no adjoint)."""
        self.reset(logA, u_in)
        n = len(self.case.boxes)
        g = C.byref(self.case.geom)
        st = C.c_void_p(self.stream)
        for i in range(self.nsteps):
            abi.check("mfg_advance_level", self.lib.mfg_advance_level(self.desc, n, g, i * self.dt, self.dt, 0, 1,
                                                                      None, st))
        J = C.c_double()
        abi.check("mfg_reaction_objective", self.lib.mfg_reaction_objective(self.desc, n, g, C.byref(J), st))
        return J.value

    def gradient(self, logA, u_in):
        """(J, dJ/dlog A (nreact), dJ/du_in) from one adjoint run."""
        self.reset(logA, u_in)
        J = C.c_double()
        gA = (C.c_double * max(self.nreact, 1))()
        gu = C.c_double()
        abi.check("mfg_adjoint_objective",
                  self.lib.mfg_adjoint_objective(self.desc, len(self.case.boxes), C.byref(self.case.geom),
                                                 self.nsteps, self.dt, self.checkpoint_every, C.byref(J), gA,
                                                 C.byref(gu), C.c_void_p(self.stream)))
        return J.value, np.array(gA[:self.nreact]), gu.value


def _function():
    import torch

    class ReactionObjective(torch.autograd.Function):
        """J(log A, u_in) with the adjoint gradients in backward."""

        @staticmethod
        def forward(ctx, logA, u_in, problem):
            J, gA, gu = problem.gradient(logA.detach().cpu().numpy(), float(u_in.detach().cpu()))
            ctx.save_for_backward(torch.as_tensor(gA, dtype=logA.dtype, device=logA.device),
                                  torch.as_tensor(gu, dtype=u_in.dtype, device=u_in.device))
            return torch.as_tensor(J, dtype=logA.dtype, device=logA.device)

        @staticmethod
        def backward(ctx, gJ):
            gA, gu = ctx.saved_tensors
            return gJ * gA, gJ * gu, None

    return ReactionObjective


_FN = None


def reaction_objective(logA, u_in, problem):
    """Differentiable J(log A, u_in) (torch tensors) for a ReactionProblem."""
    global _FN
    if _FN is None:
        _FN = _function()
    return _FN.apply(logA, u_in, problem)
