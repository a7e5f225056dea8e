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
