"""AMReX plotfile and checkpoint formats for the state of a level hierarchy.

The reference writes its output with amrex::WriteMultiLevelPlotfile
(mflo::WritePlotFile, Source/mflo_plot.cpp:44-55: phi_new of every level,
the variable names of Source/mflo.cpp:34-53, t_new[0], istep, the refinement
ratios) and its restart files with mflo::WriteCheckpointFile /
ReadCheckpointFile (Source/mflo_plot.cpp:57-240: a text Header with
finest_level, istep, dt, t_new and each level's BoxArray, then phi_new of
each level through VisMF under Level_<l>/<first variable name>).  This module
writes and reads both layouts from host arrays, so that states computed on
the GPU can be visualised, compared and restarted like the reference's.

Layouts (restated from AMReX's documented plotfile format; AMReX is not
vendored in the reference, so the byte layout is not pinned by a reference
file):

* plotfile ``<dir>/Header``: "HyperCLaw-V1.1", the variable count and names,
  the dimension, time, finest level, prob_lo, prob_hi, the ratios, each
  level's domain box, the level steps, each level's cell size, the coordinate
  system (0) and boundary width (0); then per level "lev nboxes time", the
  level step, each box's physical extent per direction and the path
  "Level_<l>/Cell".
* VisMF MultiFab ``<prefix>_H``: version 1, organisation 0, ncomp, ngrow, the
  BoxArray, the FabOnDisk list (data file, byte offset), per-box minima and
  maxima of every component; data ``<prefix>_D_00000``: per box a text line
  "FAB ((8, (64 11 52 0 1 12 0 1023)),(8, (8 7 6 5 4 3 2 1)))<box> <ncomp>"
  followed by the box's doubles, little-endian, component-major with x
  fastest (the order of the state arrays here).

Floating-point header values are printed with 17 significant digits, so a
file read back gives the same doubles.
"""
import os
import re

import numpy as np

from . import abi

REAL_DESC = "((8, (64 11 52 0 1 12 0 1023)),(8, (8 7 6 5 4 3 2 1)))"
PLOT_VERSION = "HyperCLaw-V1.1"

_BASE_NAMES = ["rho", "rhou", "rhov", "rhow", "rhoe", "density", "velx", "vely", "velz", "pressure",
               "temperature", "volfrac"]


def varnames(nspec, specnames=None):
    """Component names of Source/mflo.cpp:37-53 (species names from the case's
    species list, S0..S<n-1> when none is given)."""
    names = list(_BASE_NAMES)
    assert len(names) == abi.FLO_NVARS
    names += list(specnames) if specnames is not None else [f"S{s}" for s in range(nspec)]
    return names


def _g(x):
    return format(float(x), ".17g")


def _box_str(lo, hi):
    return "((%d,%d,%d) (%d,%d,%d) (0,0,0))" % (lo[0], lo[1], lo[2], hi[0], hi[1], hi[2])


def _boxarray_str(boxes):
    return "(%d 0\n" % len(boxes) + "".join(_box_str(lo, hi) + "\n" for lo, hi in boxes) + ")"


def write_multifab(prefix, boxes, arrays):
    """VisMF::Write of one level: prefix_H and prefix_D_00000.  boxes: list of
    (lo, hi); arrays: per box (ncomp, nz, ny, nx) float64."""
    ncomp = arrays[0].shape[0]
    offsets = []
    dname = os.path.basename(prefix) + "_D_00000"
    with open(prefix + "_D_00000", "wb") as f:
        for (lo, hi), a in zip(boxes, arrays):
            a = np.ascontiguousarray(a, dtype="<f8")
            assert a.shape == (ncomp, hi[2] - lo[2] + 1, hi[1] - lo[1] + 1, hi[0] - lo[0] + 1)
            offsets.append(f.tell())
            f.write(("FAB " + REAL_DESC + _box_str(lo, hi) + " %d\n" % ncomp).encode())
            f.write(a.tobytes())
    lines = ["1", "0", str(ncomp), "0", _boxarray_str(boxes), str(len(boxes))]
    lines += ["FabOnDisk: %s %d" % (dname, o) for o in offsets]
    lines.append("")
    for stat in (np.min, np.max):
        lines.append("%d,%d" % (len(boxes), ncomp))
        for a in arrays:
            lines.append("".join(_g(stat(a[c])) + "," for c in range(ncomp)))
        lines.append("")
    with open(prefix + "_H", "w") as f:
        f.write("\n".join(lines) + "\n")


def _parse_boxes(text):
    return [((int(a), int(b), int(c)), (int(d), int(e), int(g))) for a, b, c, d, e, g in
            re.findall(r"\(\((-?\d+),(-?\d+),(-?\d+)\) \((-?\d+),(-?\d+),(-?\d+)\) \(\d+,\d+,\d+\)\)", text)]


def read_multifab(prefix):
    """Inverse of write_multifab: (boxes, arrays)."""
    with open(prefix + "_H") as f:
        head = f.read()
    lines = head.split("\n")
    ncomp = int(lines[2])
    nb = int(lines[4].lstrip("(").split()[0])
    boxes = _parse_boxes("\n".join(lines[5:5 + nb]))
    fods = re.findall(r"FabOnDisk: (\S+) (\d+)", head)
    arrays = []
    d = os.path.dirname(prefix)
    for (lo, hi), (name, off) in zip(boxes, fods):
        with open(os.path.join(d, name), "rb") as f:
            f.seek(int(off))
            hdr = f.readline().decode()
            m = re.match(r"FAB \(\(8, \(64 11 52 0 1 12 0 1023\)\),\(8, \(8 7 6 5 4 3 2 1\)\)\)(.*) (\d+)\s*$", hdr)
            if not m:
                raise ValueError("unsupported FAB header: " + hdr.strip())
            blo, bhi = _parse_boxes(m.group(1))[0]
            nc = int(m.group(2))
            if (blo, bhi) != (lo, hi) or nc != ncomp:
                raise ValueError("FAB header does not match the MultiFab header")
            shape = (nc, hi[2] - lo[2] + 1, hi[1] - lo[1] + 1, hi[0] - lo[0] + 1)
            arrays.append(np.frombuffer(f.read(8 * int(np.prod(shape))), dtype="<f8").reshape(shape).copy())
    return boxes, arrays


def write_plotfile(path, geoms, level_boxes, level_arrays, names, time=0.0, level_steps=None):
    """amrex::WriteMultiLevelPlotfile: geoms one abi.Geom per level;
    level_boxes[l] list of (lo, hi); level_arrays[l] per-box arrays
    (ncomp, nz, ny, nx)."""
    nlev = len(geoms)
    steps = list(level_steps) if level_steps is not None else [0] * nlev
    os.makedirs(path, exist_ok=True)
    g0 = geoms[0]
    n0 = [g0.domain_hi[d] - g0.domain_lo[d] + 1 for d in range(3)]
    prob_lo = [g0.prob_lo[d] for d in range(3)]
    prob_hi = [g0.prob_lo[d] + n0[d] * g0.dx[d] for d in range(3)]
    ratios = [int(round(geoms[l].dx[0] / geoms[l + 1].dx[0])) for l in range(nlev - 1)]
    out = [PLOT_VERSION, str(len(names))] + list(names)
    out += ["3", _g(time), str(nlev - 1)]
    out.append("".join(_g(x) + " " for x in prob_lo))
    out.append("".join(_g(x) + " " for x in prob_hi))
    out.append("".join("%d " % r for r in ratios))
    out.append("".join(_box_str(g.domain_lo, g.domain_hi) + " " for g in geoms))
    out.append("".join("%d " % s for s in steps))
    for g in geoms:
        out.append("".join(_g(g.dx[d]) + " " for d in range(3)))
    out += ["0", "0"]
    for l, g in enumerate(geoms):
        out.append("%d %d %s" % (l, len(level_boxes[l]), _g(time)))
        out.append(str(steps[l]))
        for lo, hi in level_boxes[l]:
            for d in range(3):
                a = g.prob_lo[d] + (lo[d] - g.domain_lo[d]) * g.dx[d]
                b = g.prob_lo[d] + (hi[d] + 1 - g.domain_lo[d]) * g.dx[d]
                out.append(_g(a) + " " + _g(b))
        out.append("Level_%d/Cell" % l)
    with open(os.path.join(path, "Header"), "w") as f:
        f.write("\n".join(out) + "\n")
    for l in range(nlev):
        d = os.path.join(path, "Level_%d" % l)
        os.makedirs(d, exist_ok=True)
        write_multifab(os.path.join(d, "Cell"), level_boxes[l], level_arrays[l])


def read_plotfile(path):
    """Returns dict(names, time, finest_level, prob_lo, prob_hi, ratios,
    domains, steps, dx, boxes[l], arrays[l])."""
    with open(os.path.join(path, "Header")) as f:
        lines = f.read().split("\n")
    if lines[0] != PLOT_VERSION:
        raise ValueError("not a %s plotfile" % PLOT_VERSION)
    nv = int(lines[1])
    names = lines[2:2 + nv]
    p = 2 + nv
    dim = int(lines[p]); time = float(lines[p + 1]); finest = int(lines[p + 2])
    if dim != 3:
        raise ValueError("3D plotfiles only")
    prob_lo = [float(x) for x in lines[p + 3].split()]
    prob_hi = [float(x) for x in lines[p + 4].split()]
    ratios = [int(x) for x in lines[p + 5].split()]
    domains = _parse_boxes(lines[p + 6])
    steps = [int(x) for x in lines[p + 7].split()]
    dx = [[float(x) for x in lines[p + 8 + l].split()] for l in range(finest + 1)]
    boxes, arrays = [], []
    for l in range(finest + 1):
        b, a = read_multifab(os.path.join(path, "Level_%d" % l, "Cell"))
        boxes.append(b)
        arrays.append(a)
    return dict(names=names, time=time, finest_level=finest, prob_lo=prob_lo, prob_hi=prob_hi, ratios=ratios,
                domains=domains, steps=steps, dx=dx, boxes=boxes, arrays=arrays)


def write_checkpoint(path, level_boxes, level_arrays, names, istep, dt, t_new):
    """mflo::WriteCheckpointFile: Header (title, finest_level, istep, dt,
    t_new, each level's BoxArray) and Level_<l>/<names[0]> VisMF data."""
    nlev = len(level_boxes)
    os.makedirs(path, exist_ok=True)
    out = ["Checkpoint file for mflo", str(nlev - 1)]
    out.append("".join("%d " % s for s in istep))
    out.append("".join(_g(x) + " " for x in dt))
    out.append("".join(_g(x) + " " for x in t_new))
    for l in range(nlev):
        out.append(_boxarray_str(level_boxes[l]))
    with open(os.path.join(path, "Header"), "w") as f:
        f.write("\n".join(out) + "\n")
    for l in range(nlev):
        d = os.path.join(path, "Level_%d" % l)
        os.makedirs(d, exist_ok=True)
        write_multifab(os.path.join(d, names[0]), level_boxes[l], level_arrays[l])


def read_checkpoint(path, names):
    """mflo::ReadCheckpointFile: dict(finest_level, istep, dt, t_new, boxes[l], arrays[l])."""
    with open(os.path.join(path, "Header")) as f:
        text = f.read()
    lines = text.split("\n")
    finest = int(lines[1])
    istep = [int(x) for x in lines[2].split()]
    dt = [float(x) for x in lines[3].split()]
    t_new = [float(x) for x in lines[4].split()]
    rest = "\n".join(lines[5:])
    bas = re.findall(r"\(\d+ 0\n(?:\(\([^\n]*\)\n)*\)", rest)
    boxes, arrays = [], []
    for l in range(finest + 1):
        bl = _parse_boxes(bas[l])
        b, a = read_multifab(os.path.join(path, "Level_%d" % l, names[0]))
        if b != bl:
            raise ValueError("level %d: BoxArray of the Header and of the data differ" % l)
        boxes.append(b)
        arrays.append(a)
    return dict(finest_level=finest, istep=istep, dt=dt, t_new=t_new, boxes=boxes, arrays=arrays)


def hierarchy_arrays(amr, box_state):
    """Group an AmrCase's per-box states by level: (level_boxes, level_arrays).
    box_state(g) returns box g's array."""
    nlev = len(amr.geoms)
    lb = [[] for _ in range(nlev)]
    la = [[] for _ in range(nlev)]
    for g, (lo, hi, lv) in enumerate(amr.boxes):
        lb[lv].append((tuple(lo), tuple(hi)))
        la[lv].append(np.asarray(box_state(g), dtype=np.float64))
    return lb, la
