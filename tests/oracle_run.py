"""Single-level runs of the oracle (test infrastructure only)."""
import ctypes as C

import numpy as np

from mesoflow_gb300 import abi
from mesoflow_gb300.level import Level

import oracle_lib


class OracleLevel:
    def __init__(self, case, variant="strict", with_flux=False):
        self.lib = oracle_lib.load(variant)
        self.case = case
        self.level = Level(case.boxes, case.ncomp, backend="numpy", with_flux=with_flux)
        self.level.set_state(case.state)
        self.desc = self.level.descriptors()
        self.time = 0.0
        self.dt = 1e100

    def est_timestep(self):
        out = C.c_double()
        self.lib.oracle_est_timestep(C.byref(self.case.params), C.byref(self.case.geom), self.desc,
                                     len(self.case.boxes), C.byref(out))
        return out.value

    def compute_dt(self, stop_time=1e300):
        dt_new = min(self.est_timestep(), 1.1 * self.dt)
        if self.time + dt_new > stop_time - 1e-3 * dt_new:
            dt_new = stop_time - self.time
        self.dt = dt_new
        return dt_new

    def advance(self, dt, only_flow=False, clip=True):
        rn = (C.c_double * self.case.ncomp)()
        rc = self.lib.oracle_advance(C.byref(self.case.params), C.byref(self.case.geom), self.desc,
                                     len(self.case.boxes), self.time, dt, int(only_flow), int(clip), rn)
        if rc != 0:
            raise abi.MfloError("oracle_advance", rc)
        self.time += dt
        return np.array(rn[:])

    def state(self):
        return self.level.get_state(self.case.shape_zyx)

    # the loops of mflo::EvolveAMR and mflo::Evolve_split, as the driver runs them
    def evolve(self, final_time, only_flow=False, stop_time=1e300):
        while self.time < final_time:
            dt = self.compute_dt(stop_time)
            self.advance(dt, only_flow=only_flow)
            if self.time >= stop_time - 1e-6 * dt:
                break

    def evolve_split(self, t_ss, t_react, dt_react, dt_react_rk, dt_ss, bg_inertgas=False):
        P, n = C.byref(self.case.params), len(self.case.boxes)
        self.evolve(t_ss, only_flow=True)
        flow_time, react_time = t_ss, 0.0
        while react_time < t_react:
            if bg_inertgas:
                assert self.lib.oracle_store_inertgas_conc(P, self.desc, n) == 0
            tchem = 0.0
            while tchem < dt_react:
                assert self.lib.oracle_chem_advance_rk2(P, self.desc, n, dt_react_rk) == 0
                tchem += dt_react_rk
            rc = self.lib.oracle_update_vars_after_chemsolve(P, self.desc, n, int(bg_inertgas))
            if rc != 0:
                raise abi.MfloError("oracle_update_vars_after_chemsolve", rc)
            self.evolve(flow_time + dt_ss, only_flow=True)
            react_time += dt_react
            flow_time += dt_ss


class OracleAmr:
    """Multi-level runs of the oracle (subcycled coarse steps with flux
    registers, reflux and average-down) on an AmrCase, in host memory."""

    def __init__(self, amr, variant="strict"):
        from mesoflow_gb300.level import MultiLevel
        self.lib = oracle_lib.load(variant)
        self.amr = amr
        self.ml = MultiLevel(amr, backend="numpy", with_dsdt=True)
        self.desc = self.ml.descriptors()
        self.geoms = self.ml.geoms()
        self.time = 0.0

    def advance(self, dt0, only_flow=False, clip=True):
        rc = self.lib.oracle_advance_amr(C.byref(self.amr.params), self.geoms, self.desc, len(self.amr.boxes),
                                         len(self.amr.geoms), self.time, dt0, int(only_flow), int(clip))
        if rc != 0:
            raise abi.MfloError("oracle_advance_amr", rc)
        self.time += dt0

    def box_state(self, g):
        return self.ml.box_state(g)

    def composite_totals(self, comps):
        """Sum over the finest data covering each point: level-l cells covered
        by level l+1 are left out; each level weighted by its cell volume."""
        amr = self.amr
        tot = np.zeros(len(comps))
        mag = np.zeros(len(comps))
        nlev = len(amr.geoms)
        for g, (lo, hi, lv) in enumerate(amr.boxes):
            s = self.box_state(g)
            mask = np.ones(s.shape[1:], dtype=bool)
            if lv + 1 < nlev:
                r = int(round(amr.geoms[lv].dx[0] / amr.geoms[lv + 1].dx[0]))
                for flo, fhi, fl in amr.boxes:
                    if fl != lv + 1:
                        continue
                    a = [max(lo[d], flo[d] // r) for d in range(3)]
                    b = [min(hi[d], (fhi[d] + 1) // r - 1) for d in range(3)]
                    if all(a[d] <= b[d] for d in range(3)):
                        mask[a[2] - lo[2]:b[2] - lo[2] + 1, a[1] - lo[1]:b[1] - lo[1] + 1,
                             a[0] - lo[0]:b[0] - lo[0] + 1] = False
            gm = amr.geoms[lv]
            vol = gm.dx[0] * gm.dx[1] * gm.dx[2]
            for q, c in enumerate(comps):
                tot[q] += s[c][mask].sum(dtype=np.float64) * vol
                mag[q] += np.abs(s[c][mask]).sum(dtype=np.float64) * vol
        return tot, mag
