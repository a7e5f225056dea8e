"""Box layouts and per-box state storage of one AMR level.

A level is a list of AMReX-style boxes (valid cell ranges) covering part or
all of an index domain.  Each box holds component-major FP64 arrays shaped
(ncomp, nz, ny, nx) -- the amrex::Array4 layout -- for the ghosted state
(Sborder, grown by 3), phi_old, phi_new and optionally dsdt and face fluxes.
Storage is numpy (host) or torch (device); the C ABI sees only pointers and
strides.
"""
import ctypes as C

import numpy as np

from . import abi


def chop(domain_lo, domain_hi, max_size):
    """Splits [domain_lo, domain_hi] into boxes of at most max_size cells per side
    (as amr.max_grid_size does for a single level)."""
    ms = [max_size] * 3 if np.isscalar(max_size) else list(max_size)
    ranges = []
    for d in range(3):
        r, a = [], domain_lo[d]
        while a <= domain_hi[d]:
            b = min(a + ms[d] - 1, domain_hi[d])
            r.append((a, b))
            a = b + 1
        ranges.append(r)
    boxes = []
    for (z0, z1) in ranges[2]:
        for (y0, y1) in ranges[1]:
            for (x0, x1) in ranges[0]:
                boxes.append(((x0, y0, z0), (x1, y1, z1)))
    return boxes


def _array4(arr, begin, ncomp, ptr):
    nz, ny, nx = arr.shape[1], arr.shape[2], arr.shape[3]
    a = abi.Array4()
    a.p = ptr
    a.jstride = nx
    a.kstride = nx * ny
    a.nstride = nx * ny * nz
    for d in range(3):
        a.begin[d] = begin[d]
    a.end[0], a.end[1], a.end[2] = begin[0] + nx, begin[1] + ny, begin[2] + nz
    a.ncomp = ncomp
    return a


class Level:
    """Per-box arrays of one level.  backend: 'numpy' or 'torch' (device)."""

    def __init__(self, boxes, ncomp, backend="numpy", device=None, with_dsdt=True, with_flux=False,
                 with_sborder=True):
        self.boxes = [(tuple(lo), tuple(hi)) for lo, hi in boxes]
        self.ncomp = ncomp
        self.backend = backend
        self.device = device
        self.sborder, self.s_old, self.s_new, self.dsdt, self.flux = [], [], [], [], []
        g = abi.NGROW
        for lo, hi in self.boxes:
            n = [hi[d] - lo[d] + 1 for d in range(3)]
            self.sborder.append(self._zeros((ncomp, n[2] + 2 * g, n[1] + 2 * g, n[0] + 2 * g))
                                if with_sborder else None)
            self.s_old.append(self._zeros((ncomp, n[2], n[1], n[0])))
            self.s_new.append(self._zeros((ncomp, n[2], n[1], n[0])))
            self.dsdt.append(self._zeros((ncomp, n[2], n[1], n[0])) if with_dsdt else None)
            if with_flux:
                self.flux.append([self._zeros((ncomp, n[2] + (d == 2), n[1] + (d == 1), n[0] + (d == 0)))
                                  for d in range(3)])
            else:
                self.flux.append([None, None, None])
        self._desc = None

    # -- storage backend ---------------------------------------------------
    def _zeros(self, shape):
        if self.backend == "numpy":
            return np.zeros(shape, dtype=np.float64)
        import torch
        return torch.zeros(shape, dtype=torch.float64, device=self.device)

    def _ptr(self, a):
        if a is None:
            return None
        return a.ctypes.data if self.backend == "numpy" else a.data_ptr()

    # -- C ABI descriptors ---------------------------------------------------
    def descriptors(self):
        """ctypes array of mfg_box for every box (cached)."""
        if self._desc is not None:
            return self._desc
        arr = (abi.Box * len(self.boxes))()
        g = abi.NGROW
        for b, (lo, hi) in enumerate(self.boxes):
            d = arr[b]
            for q in range(3):
                d.lo[q], d.hi[q] = lo[q], hi[q]
            glo = tuple(lo[q] - g for q in range(3))
            if self.sborder[b] is not None:
                d.sborder = _array4(self.sborder[b], glo, self.ncomp, self._ptr(self.sborder[b]))
            d.s_old = _array4(self.s_old[b], lo, self.ncomp, self._ptr(self.s_old[b]))
            d.s_new = _array4(self.s_new[b], lo, self.ncomp, self._ptr(self.s_new[b]))
            if self.dsdt[b] is not None:
                d.dsdt = _array4(self.dsdt[b], lo, self.ncomp, self._ptr(self.dsdt[b]))
            for q in range(3):
                f = self.flux[b][q]
                if f is not None:
                    d.flux[q] = _array4(f, lo, self.ncomp, self._ptr(f))
        self._desc = arr
        return arr

    def host_views(self, host):
        """ctypes array of mfg_array4: each box's phi_new layout over the host
        array host[b] (same shape as s_new[b], C-contiguous; pinned for link
        speed), for mfg_advance_level_host."""
        desc = self.descriptors()
        arr = (abi.Array4 * len(self.boxes))()
        for b, h in enumerate(host):
            if tuple(h.shape) != tuple(self.s_new[b].shape):
                raise ValueError(f"host array {b}: shape {tuple(h.shape)}, phi_new {tuple(self.s_new[b].shape)}")
            contiguous = h.flags.c_contiguous if isinstance(h, np.ndarray) else h.is_contiguous()
            if not contiguous:
                raise ValueError(f"host array {b} is not C-contiguous")
            arr[b] = desc[b].s_new
            arr[b].p = h.ctypes.data if isinstance(h, np.ndarray) else h.data_ptr()
        return arr

    # -- whole-level state -----------------------------------------------------
    def set_state(self, full, domain_lo=(0, 0, 0), which="new"):
        """Copies a domain array (ncomp, Z, Y, X) into every box's phi_new (or phi_old)."""
        dst = self.s_new if which == "new" else self.s_old
        for b, (lo, hi) in enumerate(self.boxes):
            sl = tuple(slice(lo[q] - domain_lo[q], hi[q] - domain_lo[q] + 1) for q in (2, 1, 0))
            part = full[(slice(None),) + sl]
            if self.backend == "numpy":
                dst[b][...] = part
            else:
                import torch
                dst[b].copy_(torch.as_tensor(np.ascontiguousarray(part), device=self.device))

    def get_state(self, shape_zyx, domain_lo=(0, 0, 0), which="new", comps=None):
        src = {"new": self.s_new, "old": self.s_old, "dsdt": self.dsdt}[which]
        nc = self.ncomp if comps is None else len(comps)
        out = np.zeros((nc,) + tuple(shape_zyx))
        for b, (lo, hi) in enumerate(self.boxes):
            sl = tuple(slice(lo[q] - domain_lo[q], hi[q] - domain_lo[q] + 1) for q in (2, 1, 0))
            a = src[b] if self.backend == "numpy" else src[b].detach().cpu().numpy()
            out[(slice(None),) + sl] = a if comps is None else a[list(comps)]
        return out

    def sborder_host(self, b):
        a = self.sborder[b]
        return a if self.backend == "numpy" else a.detach().cpu().numpy()

    def set_sborder(self, b, arr):
        if self.backend == "numpy":
            self.sborder[b][...] = arr
        else:
            import torch
            self.sborder[b].copy_(torch.as_tensor(np.ascontiguousarray(arr), device=self.device))

    def cells(self):
        return sum(int(np.prod([hi[q] - lo[q] + 1 for q in range(3)])) for lo, hi in self.boxes)


def geometry(domain_lo, domain_hi, prob_lo, prob_hi, periodic):
    g = abi.Geom()
    for d in range(3):
        n = domain_hi[d] - domain_lo[d] + 1
        g.dx[d] = (prob_hi[d] - prob_lo[d]) / n
        g.prob_lo[d] = prob_lo[d]
        g.domain_lo[d] = domain_lo[d]
        g.domain_hi[d] = domain_hi[d]
        g.is_periodic[d] = 1 if periodic[d] else 0
    return g


class MultiLevel:
    """Boxes of several levels in one descriptor array (mfg_box.level set), for
    the batched entry points.  backend: 'numpy' or 'torch'."""

    def __init__(self, amr, backend="torch", device=None, with_dsdt=False):
        self.amr = amr
        self.ncomp = amr.ncomp
        self.levels = []
        self.index = []  # global box -> (level, local box)
        for l in range(len(amr.geoms)):
            bl = [(lo, hi) for lo, hi, lv in amr.boxes if lv == l]
            self.levels.append(Level(bl, amr.ncomp, backend=backend, device=device, with_dsdt=with_dsdt))
        counters = [0] * len(amr.geoms)
        for lo, hi, lv in amr.boxes:
            self.index.append((lv, counters[lv]))
            counters[lv] += 1
        self.set_states(amr.states)
        self._desc = None

    def set_states(self, states):
        for (lv, b), s in zip(self.index, states):
            lev = self.levels[lv]
            if lev.backend == "numpy":
                lev.s_new[b][...] = s
            else:
                import torch
                lev.s_new[b].copy_(torch.as_tensor(np.ascontiguousarray(s), device=lev.device))

    def descriptors(self):
        if self._desc is not None:
            return self._desc
        per = [lev.descriptors() for lev in self.levels]
        arr = (abi.Box * len(self.index))()
        for g, (lv, b) in enumerate(self.index):
            arr[g] = per[lv][b]
            arr[g].level = lv
        self._desc = arr
        return arr

    def geoms(self):
        arr = (abi.Geom * len(self.amr.geoms))()
        for l, g in enumerate(self.amr.geoms):
            arr[l] = g
        return arr

    def box_state(self, g, which="new"):
        lv, b = self.index[g]
        lev = self.levels[lv]
        a = (lev.s_new if which == "new" else lev.s_old)[b]
        return a if lev.backend == "numpy" else a.detach().cpu().numpy()
