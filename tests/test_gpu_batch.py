"""Batched AMR form (mfg_boxlist_*): the batched launches and the CUDA-graph
replay give the states of the plain per-box launches of the same kernel
bodies, on one level (where the per-box path is itself parity-tested against
the oracle) and on a multi-level hierarchy of uneven boxes: bitwise on the
catalyst configurations, to the parity tolerance on the porous one (the
batched and per-box kernels are compiled separately and the compiler may
contract a multiply and an add differently in each)."""
import ctypes as C

import numpy as np
import pytest

from mesoflow_gb300 import abi, cases
from mesoflow_gb300.level import Level, MultiLevel
from helpers import perturb

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _boxlist(lib, desc, n, geoms, nlev):
    h = C.c_void_p()
    abi.check("mfg_boxlist_create", lib.mfg_boxlist_create(desc, n, geoms, nlev, C.byref(h)))
    return h


def test_batched_single_level_equals_per_box_step():
    c = perturb(cases.catalyst(n=24, order=5, max_grid=12), 21, vel_amp=1e-2)
    lib = abi.load()
    abi.check("mfg_init", lib.mfg_init(C.byref(c.params)))
    a = Level(c.boxes, c.ncomp, backend="torch", device="cuda")
    b = Level(c.boxes, c.ncomp, backend="torch", device="cuda")
    a.set_state(c.state)
    b.set_state(c.state)
    s = torch.cuda.Stream()
    st = C.c_void_p(s.cuda_stream)
    geoms = (abi.Geom * 1)(c.geom)
    h = _boxlist(lib, b.descriptors(), len(c.boxes), geoms, 1)
    dt = 2e-9
    with torch.cuda.stream(s):
        for step in range(2):
            abi.check("mfg_advance_level", lib.mfg_advance_level(a.descriptors(), len(c.boxes), C.byref(c.geom),
                                                                 0.0, dt, 0, 1, None, st))
            abi.check("mfg_boxlist_step", lib.mfg_boxlist_step(h, 0.0, dt, 1, st))
    s.synchronize()
    lib.mfg_boxlist_destroy(h)
    assert np.array_equal(a.get_state(c.shape_zyx), b.get_state(c.shape_zyx))


@pytest.mark.parametrize("order", [2, 5])
def test_batched_porous_matches_per_box_step(order):
    """Pressure inlet/outlet, single-gas thermo: the batched step equals the
    per-box step to the parity tolerance (1e-12 of each component's domain
    maximum; the two are separate kernels, whose multiply-add contraction the
    compiler chooses independently, so equality is to the last bits)."""
    from helpers import rel_err
    c = perturb(cases.porous_ib(n=32, order=order, max_grid=16), 31, vel_amp=1e-2)
    lib = abi.load()
    abi.check("mfg_init", lib.mfg_init(C.byref(c.params)))
    a = Level(c.boxes, c.ncomp, backend="torch", device="cuda")
    b = Level(c.boxes, c.ncomp, backend="torch", device="cuda")
    a.set_state(c.state)
    b.set_state(c.state)
    s = torch.cuda.Stream()
    st = C.c_void_p(s.cuda_stream)
    geoms = (abi.Geom * 1)(c.geom)
    h = _boxlist(lib, b.descriptors(), len(c.boxes), geoms, 1)
    dt = 5e-10
    with torch.cuda.stream(s):
        for _ in range(2):
            abi.check("mfg_advance_level", lib.mfg_advance_level(a.descriptors(), len(c.boxes), C.byref(c.geom),
                                                                 0.0, dt, 0, 1, None, st))
            abi.check("mfg_boxlist_step", lib.mfg_boxlist_step(h, 0.0, dt, 1, st))
    s.synchronize()
    lib.mfg_boxlist_destroy(h)
    err, comp = rel_err(b.get_state(c.shape_zyx), a.get_state(c.shape_zyx))
    assert err <= 1e-12, (err, comp)


@pytest.mark.parametrize("order", [5, 2])
def test_multilevel_plain_batched_graph_bitwise(order):
    amr = cases.catalyst_amr(n0=32, nlev=2, order=order, blocking=8, max_grid=16, base_grid=16, nspheres=6)
    lib = abi.load()
    abi.check("mfg_init", lib.mfg_init(C.byref(amr.params)))
    s = torch.cuda.Stream()
    st = C.c_void_p(s.cuda_stream)
    dt = 2e-9
    out = []
    for mode in (0, 1, 2):
        ml = MultiLevel(amr, backend="torch", device="cuda")
        geoms = ml.geoms()
        h = _boxlist(lib, ml.descriptors(), len(amr.boxes), geoms, len(amr.geoms))
        with torch.cuda.stream(s):
            for step in range(2):
                abi.check("mfg_boxlist_step", lib.mfg_boxlist_step(h, 0.0, dt, mode, st))
        s.synchronize()
        lib.mfg_boxlist_destroy(h)
        out.append([ml.box_state(g) for g in range(len(amr.boxes))])
    for g in range(len(amr.boxes)):
        assert np.all(np.isfinite(out[0][g]))
        assert np.array_equal(out[0][g], out[1][g]), g
        assert np.array_equal(out[0][g], out[2][g]), g


def test_autotune_keeps_results():
    amr = cases.catalyst_amr(n0=32, nlev=2, order=5, blocking=8, max_grid=16, base_grid=16, nspheres=6)
    lib = abi.load()
    abi.check("mfg_init", lib.mfg_init(C.byref(amr.params)))
    s = torch.cuda.Stream()
    st = C.c_void_p(s.cuda_stream)
    dt = 2e-9
    res = []
    for tune in (False, True):
        ml = MultiLevel(amr, backend="torch", device="cuda")
        h = _boxlist(lib, ml.descriptors(), len(amr.boxes), ml.geoms(), len(amr.geoms))
        if tune:
            r = (C.c_double * 16)()
            with torch.cuda.stream(s):
                abi.check("mfg_boxlist_autotune", lib.mfg_boxlist_autotune(h, dt, r, st))
            assert all(r[3 * p + 1] >= 1 for p in (0, 1, 2, 4))
            ml.set_states(amr.states)  # the search ran phases on the state
        with torch.cuda.stream(s):
            abi.check("mfg_boxlist_step", lib.mfg_boxlist_step(h, 0.0, dt, 2, st))
        s.synchronize()
        lib.mfg_boxlist_destroy(h)
        res.append([ml.box_state(g) for g in range(len(amr.boxes))])
    for g in range(len(amr.boxes)):
        assert np.array_equal(res[0][g], res[1][g]), g


def _amr_gpu(lib, amr, mode, steps, dt, s):
    st = C.c_void_p(s.cuda_stream)
    ml = MultiLevel(amr, backend="torch", device="cuda")
    h = _boxlist(lib, ml.descriptors(), len(amr.boxes), ml.geoms(), len(amr.geoms))
    with torch.cuda.stream(s):
        for step in range(steps):
            abi.check("mfg_boxlist_step_amr", lib.mfg_boxlist_step_amr(h, step * dt, dt, mode, st))
    s.synchronize()
    lib.mfg_boxlist_destroy(h)
    return [ml.box_state(g) for g in range(len(amr.boxes))]


def _amr_rel_err(gs, os_):
    """Worst component of max |g - o| / s_c over all boxes of all levels, s_c
    the maximum of |o_c| or, for a momentum or velocity component, of the
    vector's three components (the transverse momenta of this x-driven flow
    are small differences of large pressure fluxes)."""
    groups = {c: (abi.RHOU, abi.RHOV, abi.RHOW) for c in (abi.RHOU, abi.RHOV, abi.RHOW)}
    groups.update({c: (abi.VELX, abi.VELY, abi.VELZ) for c in (abi.VELX, abi.VELY, abi.VELZ)})
    worst, wc = 0.0, -1
    for c in range(os_[0].shape[0]):
        sc = max(np.abs(o[q]).max() for o in os_ for q in groups.get(c, (c,)))
        e = max(np.abs(g[c] - o[c]).max() for g, o in zip(gs, os_))
        e = e / sc if sc > 0 else e
        if e > worst or wc < 0:
            worst, wc = e, c
    return worst, wc


@pytest.mark.parametrize("nlev", [2, 3])
def test_amr_step_matches_oracle(nlev):
    """The reference's multi-level step (subcycled levels, two-level fill with
    time-interpolated conservative interpolation, flux registers, reflux,
    average-down, chemistry per substep) on a properly nested catalyst
    hierarchy: one coarse step equals the oracle's to the one-step parity
    tolerance (1e-12 of each component's scale), two steps to 1e-11."""
    from oracle_run import OracleAmr
    amr = cases.catalyst_amr(n0=32, nlev=nlev, order=5, blocking=8, max_grid=16, base_grid=16, nspheres=6)
    lib = abi.load()
    abi.check("mfg_init", lib.mfg_init(C.byref(amr.params)))
    s = torch.cuda.Stream()
    dt = 2e-9
    o = OracleAmr(amr)
    for steps, tol in ((1, 1e-12), (2, 1e-11)):
        g = _amr_gpu(lib, amr, 1, steps, dt, s)
        o.advance(dt)
        ob = [o.box_state(b) for b in range(len(amr.boxes))]
        assert all(np.all(np.isfinite(x)) for x in g)
        err, comp = _amr_rel_err(g, ob)
        assert err <= tol, (steps, err, comp)


def test_amr_plain_batched_graph_bitwise():
    amr = cases.catalyst_amr(n0=32, nlev=3, order=5, blocking=8, max_grid=16, base_grid=16, nspheres=6)
    lib = abi.load()
    abi.check("mfg_init", lib.mfg_init(C.byref(amr.params)))
    s = torch.cuda.Stream()
    out = [_amr_gpu(lib, amr, mode, 2, 2e-9, s) for mode in (0, 1, 2)]
    for g in range(len(amr.boxes)):
        assert np.array_equal(out[0][g], out[1][g]), g
        assert np.array_equal(out[0][g], out[2][g]), g


def test_amr_rejects_unnested_hierarchy():
    amr = cases.catalyst_amr(n0=32, nlev=3, order=5, blocking=8, max_grid=16, base_grid=16, nspheres=6,
                             nested=False)
    lib = abi.load()
    abi.check("mfg_init", lib.mfg_init(C.byref(amr.params)))
    ml = MultiLevel(amr, backend="torch", device="cuda")
    h = _boxlist(lib, ml.descriptors(), len(amr.boxes), ml.geoms(), len(amr.geoms))
    s = torch.cuda.Stream()
    assert lib.mfg_boxlist_step_amr(h, 0.0, 2e-9, 1, C.c_void_p(s.cuda_stream)) == abi.ERR_ARG
    lib.mfg_boxlist_destroy(h)


@pytest.mark.parametrize("name", ["cat5", "porous2"])
def test_device_time_loop_equals_host_loop(name):
    """mfg_boxlist_evolve (ComputeDt, step and loop condition on the device, one
    graph launch) gives bitwise the states, time, dt and step count of the host
    loop of ComputeDt (mfg_est_timestep, change_max 1.1, stop-time clamp) and
    batched steps, including the final step clamped to the stop time."""
    from helpers import perturb as _p
    c = _p(cases.catalyst(n=24, order=5, max_grid=12), 31, vel_amp=1e-2) if name == "cat5" else \
        _p(cases.porous_ib(n=24, order=2, max_grid=12), 32, vel_amp=1e-2)
    lib = abi.load()
    abi.check("mfg_init", lib.mfg_init(C.byref(c.params)))
    s = torch.cuda.Stream()
    st = C.c_void_p(s.cuda_stream)
    geoms = (abi.Geom * 1)(c.geom)
    a = Level(c.boxes, c.ncomp, backend="torch", device="cuda")
    b = Level(c.boxes, c.ncomp, backend="torch", device="cuda")
    a.set_state(c.state)
    b.set_state(c.state)
    ha = _boxlist(lib, a.descriptors(), len(c.boxes), geoms, 1)
    hb = _boxlist(lib, b.descriptors(), len(c.boxes), geoms, 1)
    # host loop
    t, dtp, n = 0.0, 1e100, 0
    with torch.cuda.stream(s):
        est = C.c_double()
        abi.check("est", lib.mfg_est_timestep(a.descriptors(), len(c.boxes), C.byref(c.geom), t, C.byref(est), st))
    stop = 4.5 * est.value
    with torch.cuda.stream(s):
        while n < 10 and t < stop:
            abi.check("est", lib.mfg_est_timestep(a.descriptors(), len(c.boxes), C.byref(c.geom), t,
                                                  C.byref(est), st))
            dt = min(est.value, 1.1 * dtp)
            if t + dt > stop - 1e-3 * dt:
                dt = stop - t
            abi.check("step", lib.mfg_boxlist_step(ha, t, dt, 1, st))
            t += dt
            n += 1
            dtp = dt
            if t >= stop - 1e-6 * dt:
                break
    s.synchronize()
    # device loop
    tt, dd, nn = C.c_double(0.0), C.c_double(1e100), C.c_int(0)
    with torch.cuda.stream(s):
        abi.check("evolve", lib.mfg_boxlist_evolve(hb, 1e300, stop, 10, C.byref(tt), C.byref(dd), C.byref(nn), st))
    s.synchronize()
    lib.mfg_boxlist_destroy(ha)
    lib.mfg_boxlist_destroy(hb)
    assert nn.value == n and tt.value == t and dd.value == dtp, (nn.value, n, tt.value, t)
    assert n >= 5
    assert np.array_equal(a.get_state(c.shape_zyx), b.get_state(c.shape_zyx))


def test_device_amr_loop_equals_host_loop():
    """mfg_boxlist_evolve_amr (subcycled ComputeDt and the coarse step's fill
    coefficients on the device, one graph launch) gives bitwise the states,
    time, per-level dt and step count of the host loop of per-level
    mfg_est_timestep, ComputeDt with subcycling (Source/mflo_timestep.cpp:18-50)
    and mfg_boxlist_step_amr, including a last step clamped to the stop time."""
    amr = cases.catalyst_amr(n0=32, nlev=3, order=5, blocking=8, max_grid=16, base_grid=16, nspheres=6)
    lib = abi.load()
    abi.check("mfg_init", lib.mfg_init(C.byref(amr.params)))
    s = torch.cuda.Stream()
    st = C.c_void_p(s.cuda_stream)
    nlev = len(amr.geoms)
    ratio = [1] + [int(round(amr.geoms[l - 1].dx[0] / amr.geoms[l].dx[0])) for l in range(1, nlev)]
    ma, mb = MultiLevel(amr, backend="torch", device="cuda"), MultiLevel(amr, backend="torch", device="cuda")
    ha = _boxlist(lib, ma.descriptors(), len(amr.boxes), ma.geoms(), nlev)
    hb = _boxlist(lib, mb.descriptors(), len(amr.boxes), mb.geoms(), nlev)
    est = C.c_double()

    def est_levels():
        out = []
        for l in range(nlev):
            lv = ma.levels[l]
            abi.check("est", lib.mfg_est_timestep(lv.descriptors(), len(lv.s_new), C.byref(amr.geoms[l]), 0.0,
                                                  C.byref(est), st))
            out.append(est.value)
        return out

    with torch.cuda.stream(s):
        stop = 2.5 * 4 * est_levels()[-1]
        t, n, dtp = 0.0, 0, [1e100] * nlev
        while n < 6 and t < stop:
            tmp = est_levels()
            dt0, nf = tmp[0], 1
            for l in range(nlev):
                tmp[l] = min(tmp[l], 1.1 * dtp[l])
                nf *= ratio[l]
                dt0 = min(dt0, nf * tmp[l])
            if t + dt0 > stop - 1e-3 * dt0:
                dt0 = stop - t
            dts = [dt0]
            for l in range(1, nlev):
                dts.append(dts[-1] / ratio[l])
            abi.check("amr", lib.mfg_boxlist_step_amr(ha, t, dt0, 1, st))
            t += dt0
            n += 1
            dtp = dts
            if t >= stop - 1e-6 * dt0:
                break
    s.synchronize()
    tt, nn = C.c_double(0.0), C.c_int(0)
    dd = (C.c_double * nlev)(*([1e100] * nlev))
    with torch.cuda.stream(s):
        abi.check("evolve_amr", lib.mfg_boxlist_evolve_amr(hb, 1e300, stop, 6, C.byref(tt), dd, C.byref(nn), st))
    s.synchronize()
    lib.mfg_boxlist_destroy(ha)
    lib.mfg_boxlist_destroy(hb)
    assert nn.value == n and tt.value == t and list(dd) == dtp, (nn.value, n, tt.value, t, list(dd), dtp)
    assert n >= 3
    for g in range(len(amr.boxes)):
        assert np.array_equal(ma.box_state(g), mb.box_state(g)), g
