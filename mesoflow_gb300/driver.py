"""Single-level time stepping through the C ABI (the host loop of
mflo::EvolveAMR, Source/mflo_evolve.cpp:18-89, for one level).
"""
import ctypes as C

import numpy as np

from . import abi
from .level import Level


class Mflo:
    """Owns the device state of one level and advances it with
    mfg_advance_level.  Mirrors mflo's single-level step: ComputeDt
    (EstTimeStep, change_max = 1.1, stop_time clamp), Advance_coupled_strang,
    update_primitive_vars, clip_neg_speciesconc, compute_residual_norms."""

    def __init__(self, case, device="cuda", stream=None, with_dsdt=False, only_flow=False, clip=True):
        import torch
        self.lib = abi.load()
        self.case = case
        self.only_flow = only_flow
        self.clip = clip
        abi.check("mfg_init", self.lib.mfg_init(C.byref(case.params)))
        self.level = Level(case.boxes, case.ncomp, backend="torch", device=device, with_dsdt=with_dsdt)
        self.level.set_state(case.state)
        self.desc = self.level.descriptors()
        self.stream = stream if stream is not None else torch.cuda.current_stream().cuda_stream
        self.time = 0.0
        self.dt = 1e100
        self.istep = 0
        self.resnorms = np.zeros(case.ncomp)

    def est_timestep(self):
        out = C.c_double()
        abi.check("mfg_est_timestep", self.lib.mfg_est_timestep(self.desc, len(self.case.boxes),
                                                                 C.byref(self.case.geom), self.time,
                                                                 C.byref(out), C.c_void_p(self.stream)))
        return out.value

    def compute_dt(self, stop_time=1e300):
        """ComputeDt for one level (Source/mflo_timestep.cpp:18-50)."""
        dt_new = min(self.est_timestep(), 1.1 * self.dt)
        eps = 1e-3 * dt_new
        if self.time + dt_new > stop_time - eps:
            dt_new = stop_time - self.time
        self.dt = dt_new
        return dt_new

    def advance(self, dt=None, norms=True, only_flow=None):
        if dt is None:
            dt = self.compute_dt()
        of = self.only_flow if only_flow is None else only_flow
        rn = (C.c_double * self.case.ncomp)()
        abi.check("mfg_advance_level",
                  self.lib.mfg_advance_level(self.desc, len(self.case.boxes), C.byref(self.case.geom), self.time,
                                             dt, int(of), int(self.clip), rn if norms else None,
                                             C.c_void_p(self.stream)))
        if norms:
            self.resnorms = np.array(rn[:])
        self.time += dt
        self.istep += 1
        return dt

    def evolve(self, final_time, only_flow=None, stop_time=1e300, max_step=10 ** 9, norms=False):
        """mflo::EvolveAMR's loop (Source/mflo_evolve.cpp:18-89) for one level:
        steps of ComputeDt + advance while time < final_time."""
        while self.istep < max_step and self.time < final_time:
            dt = self.compute_dt(stop_time)
            self.advance(dt, norms=norms, only_flow=only_flow)
            if self.time >= stop_time - 1e-6 * dt:
                break

    def evolve_split(self, t_ss, t_react, dt_react, dt_react_rk, dt_ss, bg_inertgas=False, stop_time=1e300,
                     max_step=10 ** 9):
        """mflo::Evolve_split (Source/mflo_splitchem.cpp:24-72), for slow
        chemistry: the flow to t_ss (no chemistry), then until react_time
        reaches t_react: chemistry sub-steps of dt_react_rk over dt_react on the
        frozen flow (Advance_chemistry), the flow variables brought to the new
        concentrations (update_vars_after_chemsolve), and dt_ss more of flow."""
        st = C.c_void_p(self.stream)
        n = len(self.case.boxes)
        self.evolve(t_ss, only_flow=True, stop_time=stop_time, max_step=max_step)
        flow_time, react_time = t_ss, 0.0
        while react_time < t_react:
            if bg_inertgas:
                abi.check("mfg_store_inertgas_conc", self.lib.mfg_store_inertgas_conc(self.desc, n, st))
            tchem = 0.0
            while tchem < dt_react:
                abi.check("mfg_chem_advance_rk2",
                          self.lib.mfg_chem_advance_rk2(self.desc, n, react_time + tchem, dt_react_rk, st))
                tchem += dt_react_rk
            abi.check("mfg_update_vars_after_chemsolve",
                      self.lib.mfg_update_vars_after_chemsolve(self.desc, n, int(bg_inertgas), st))
            self.evolve(flow_time + dt_ss, only_flow=True, stop_time=stop_time, max_step=max_step)
            react_time += dt_react
            flow_time += dt_ss

    def state(self):
        return self.level.get_state(self.case.shape_zyx)

    def _level_arrays(self):
        import torch
        torch.cuda.synchronize()
        boxes = [(tuple(lo), tuple(hi)) for lo, hi in self.case.boxes]
        return boxes, [a.detach().cpu().numpy() for a in self.level.s_new]

    def write_plotfile(self, path, specnames=None):
        """mflo::WritePlotFile (Source/mflo_plot.cpp:44-55) of this level."""
        from . import plotfile
        boxes, arrays = self._level_arrays()
        plotfile.write_plotfile(path, [self.case.geom], [boxes], [arrays],
                                plotfile.varnames(self.case.params.nspec, specnames), self.time, [self.istep])

    def write_checkpoint(self, path, specnames=None):
        """mflo::WriteCheckpointFile (Source/mflo_plot.cpp:57-145) of this level."""
        from . import plotfile
        boxes, arrays = self._level_arrays()
        plotfile.write_checkpoint(path, [boxes], [arrays], plotfile.varnames(self.case.params.nspec, specnames),
                                  [self.istep], [self.dt if self.dt < 1e100 else 0.0], [self.time])

    def read_checkpoint(self, path, specnames=None):
        """mflo::ReadCheckpointFile (Source/mflo_plot.cpp:147-240): restores the
        state, time, step count and dt of a checkpoint of this box layout."""
        import torch
        from . import plotfile
        r = plotfile.read_checkpoint(path, plotfile.varnames(self.case.params.nspec, specnames))
        if r["finest_level"] != 0 or r["boxes"][0] != [(tuple(lo), tuple(hi)) for lo, hi in self.case.boxes]:
            raise ValueError("checkpoint box layout differs from this level's")
        for dst, src in zip(self.level.s_new, r["arrays"][0]):
            dst.copy_(torch.as_tensor(src, device=dst.device))
        self.istep, self.dt, self.time = r["istep"][0], r["dt"][0], r["t_new"][0]

    def status(self, clear=False):
        v = C.c_uint32()
        abi.check("mfg_status", self.lib.mfg_status(C.byref(v), int(clear)))
        return v.value
