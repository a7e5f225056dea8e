"""Restart through the reference's checkpoint layout: a run checkpointed
after two steps and resumed from the files gives bitwise the states of the
uninterrupted run; the plotfile of the GPU state reads back unchanged."""
import numpy as np
import pytest

from mesoflow_gb300 import cases, plotfile
from mesoflow_gb300.driver import Mflo
from helpers import perturb

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def test_checkpoint_restart_bitwise(tmp_path):
    c = perturb(cases.catalyst(n=16, order=5, max_grid=8), 5, vel_amp=1e-2)
    a = Mflo(c, device="cuda")
    for _ in range(2):
        a.advance()
    a.write_checkpoint(str(tmp_path / "chk00002"))
    a.write_plotfile(str(tmp_path / "plt00002"))
    ref2, t2, dt2 = a.state(), a.time, a.dt
    for _ in range(2):
        a.advance()
    b = Mflo(c, device="cuda")
    b.read_checkpoint(str(tmp_path / "chk00002"))
    assert b.istep == 2 and b.time == t2 and b.dt == dt2
    assert np.array_equal(b.state(), ref2)
    for _ in range(2):
        b.advance()
    assert b.time == a.time
    assert np.array_equal(b.state(), a.state())
    r = plotfile.read_plotfile(str(tmp_path / "plt00002"))
    assert r["steps"] == [2] and r["names"][0] == "rho"
    got = np.zeros_like(ref2)
    for (lo, hi), arr in zip(r["boxes"][0], r["arrays"][0]):
        got[:, lo[2]:hi[2] + 1, lo[1]:hi[1] + 1, lo[0]:hi[0] + 1] = arr
    assert np.array_equal(got, ref2)
