"""Host views of the host-buffer level step (Level.host_views, the h_state
argument of mfg_advance_level_host): each view has the layout of its box's
phi_new descriptor over the host array, and arrays of another shape or not
C-contiguous are refused before any library call."""
import numpy as np
import pytest

from mesoflow_gb300 import cases
from mesoflow_gb300.level import Level


def level():
    c = cases.porous_ib(n=16, order=2, max_grid=8)
    return c, Level(c.boxes, c.ncomp, backend="numpy")


def test_views_mirror_phi_new_layout():
    c, lev = level()
    host = [np.zeros_like(a) for a in lev.s_new]
    views = lev.host_views(host)
    desc = lev.descriptors()
    assert len(views) == len(c.boxes)
    for b, (v, h) in enumerate(zip(views, host)):
        d = desc[b].s_new
        assert v.p == h.ctypes.data and v.p != d.p
        assert (v.jstride, v.kstride, v.nstride, v.ncomp) == (d.jstride, d.kstride, d.nstride, d.ncomp)
        assert tuple(v.begin) == tuple(d.begin) and tuple(v.end) == tuple(d.end)


def test_views_refuse_other_shapes_and_strided_arrays():
    c, lev = level()
    host = [np.zeros_like(a) for a in lev.s_new]
    bad = list(host)
    bad[1] = np.zeros(host[1].shape[:-1] + (host[1].shape[-1] + 1,))
    with pytest.raises(ValueError, match="shape"):
        lev.host_views(bad)
    bad = list(host)
    big = np.zeros(host[0].shape[:-1] + (2 * host[0].shape[-1],))
    bad[0] = big[..., ::2]
    with pytest.raises(ValueError, match="contiguous"):
        lev.host_views(bad)
