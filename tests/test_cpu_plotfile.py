"""AMReX plotfile and checkpoint layouts (mesoflow_gb300.plotfile): a
two-level hierarchy written and read back gives the same doubles, boxes,
times and steps, and the text headers carry the fields the reference's
WriteMultiLevelPlotfile / WriteCheckpointFile put there."""
import os

import numpy as np

from mesoflow_gb300 import abi, cases, plotfile


def _hierarchy():
    c = cases.taylor_green_mix(n=8, order=5, max_grid=4)
    amr = cases.two_level(c, [((4, 4, 4), (11, 7, 7))])
    return amr, plotfile.hierarchy_arrays(amr, lambda g: amr.states[g])


def test_plotfile_round_trip(tmp_path):
    amr, (lb, la) = _hierarchy()
    names = plotfile.varnames(amr.params.nspec)
    path = str(tmp_path / "plt00010")
    plotfile.write_plotfile(path, amr.geoms, lb, la, names, time=1.25e-6, level_steps=[10, 20])
    r = plotfile.read_plotfile(path)
    assert r["names"] == names and r["finest_level"] == 1 and r["time"] == 1.25e-6
    assert r["ratios"] == [2] and r["steps"] == [10, 20]
    assert r["domains"] == [((0, 0, 0), (7, 7, 7)), ((0, 0, 0), (15, 15, 15))]
    g0 = amr.geoms[0]
    assert r["dx"][1] == [amr.geoms[1].dx[d] for d in range(3)]
    assert r["prob_lo"] == [g0.prob_lo[d] for d in range(3)]
    for l in range(2):
        assert r["boxes"][l] == lb[l]
        for a, b in zip(r["arrays"][l], la[l]):
            assert np.array_equal(a, b)
    head = open(os.path.join(path, "Header")).read().split("\n")
    assert head[0] == "HyperCLaw-V1.1" and head[1] == str(abi.FLO_NVARS + amr.params.nspec)
    assert head[2:4] == ["rho", "rhou"] and "Level_1/Cell" in head
    cell_h = open(os.path.join(path, "Level_0", "Cell_H")).read().split("\n")
    assert cell_h[:4] == ["1", "0", str(len(names)), "0"]
    # per-box minima of the first box, as written in the header
    i = cell_h.index("%d,%d" % (len(lb[0]), len(names)))
    mins = [float(x) for x in cell_h[i + 1].rstrip(",").split(",")]
    assert mins == [la[0][0][c].min() for c in range(len(names))]
    with open(os.path.join(path, "Level_0", "Cell_D_00000"), "rb") as f:
        first = f.readline().decode()
    assert first.startswith("FAB ((8, (64 11 52 0 1 12 0 1023)),(8, (8 7 6 5 4 3 2 1)))((0,0,0) (3,3,3) (0,0,0)) ")


def test_checkpoint_round_trip(tmp_path):
    amr, (lb, la) = _hierarchy()
    names = plotfile.varnames(amr.params.nspec)
    path = str(tmp_path / "chk00010")
    plotfile.write_checkpoint(path, lb, la, names, istep=[10, 20], dt=[2e-9, 1e-9], t_new=[2e-8, 2e-8])
    r = plotfile.read_checkpoint(path, names)
    assert r["finest_level"] == 1 and r["istep"] == [10, 20] and r["dt"] == [2e-9, 1e-9]
    assert r["t_new"] == [2e-8, 2e-8]
    for l in range(2):
        assert r["boxes"][l] == lb[l]
        for a, b in zip(r["arrays"][l], la[l]):
            assert np.array_equal(a, b)
    assert os.path.exists(os.path.join(path, "Level_1", "rho_H"))
    head = open(os.path.join(path, "Header")).read().split("\n")
    assert head[:2] == ["Checkpoint file for mflo", "1"]
