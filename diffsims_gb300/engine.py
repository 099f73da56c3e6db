"""Device-side engine: per-phase candidate tables and the batched
orientation simulation, all through the C ABI.

``PhaseTable`` = ReciprocalLatticeVector.from_min_dspacing + the structure
factor table of one phase (diffsims/crystallography/reciprocal_lattice_vector.py:1077-1142,
diffsims/utils/sim_utils.py:256-304).  ``simulate_phase`` = the orientation
loop of SimulationGenerator.calculate_diffraction2d
(diffsims/generators/simulation_generator.py:198-241) for one phase.
"""
from __future__ import annotations

import ctypes as C
import json
import os
import time
import weakref
from dataclasses import dataclass

import numpy as np
import torch

from . import _native as N
from .crystal import lattice_params, lattice_base, sites_of, structure_of
from .sim_utils import PackedAtoms, debye_waller_per_atom

FORMS = {"mixed": N.DS_FORM_MIXED, "fp64": N.DS_FORM_FP64}


def _device(device=None):
    if device is None:
        return torch.device("cuda", torch.cuda.current_device())
    return torch.device(device)


def reciprocal_basis(lattice) -> np.ndarray:
    """Rows a*, b*, c* (1/Angstrom, no 2 pi) in the x || a, z || c* frame."""
    return np.ascontiguousarray(np.linalg.inv(lattice_base(*lattice_params(lattice))).T)


def box_extent(recip: np.ndarray, min_dspacing: float) -> np.ndarray:
    lib = N.load_library(require_cuda=False)
    r = (C.c_double * 9)(*recip.reshape(-1).tolist())
    out = (C.c_int32 * 3)()
    N.check(lib.ds_box_extent(r, float(min_dspacing), out), "box_extent")
    return np.array(list(out), dtype=np.int64)


class PhaseTable:
    """Ordered candidate rows of one phase on the device: hkl (int32), |g|^2
    (FP64) and |F|^2 (FP32 for the mixed form, FP64 for the FP64 form)."""

    def __init__(self, phase, reciprocal_radius=1.0, with_direct_beam=True, scattering_params="lobato",
                 debye_waller_factors=None, form="mixed", device=None, stream=None, build=True):
        dev = _device(device)
        structure = structure_of(phase)
        els, xyz, occ = sites_of(structure)
        B = debye_waller_per_atom(els, debye_waller_factors)
        atoms = PackedAtoms(els, xyz, occ, B, scattering_params, dev)
        self._setup(reciprocal_basis(structure.lattice), atoms, reciprocal_radius, with_direct_beam, form, dev)
        if build:
            self.build(stream)

    @classmethod
    def from_parts(cls, recip, atoms: PackedAtoms, reciprocal_radius=1.0, with_direct_beam=True, form="mixed",
                   device=None, stream=None, build=True):
        """A table from a reciprocal basis (rows a*, b*, c*, 1/Angstrom) and
        packed atoms, without a phase object (the differentiable path)."""
        obj = cls.__new__(cls)
        obj._setup(np.ascontiguousarray(np.asarray(recip, dtype=np.float64).reshape(3, 3)), atoms, reciprocal_radius,
                   with_direct_beam, form, _device(device))
        if build:
            obj.build(stream)
        return obj

    @classmethod
    def sphere(cls, recip, atoms: PackedAtoms, reciprocal_radius, form="mixed", device=None, stream=None,
               build=True):
        """The candidate rows of the legacy ``DiffractionGenerator``:
        get_points_in_sphere (diffsims/utils/sim_utils.py:436-474) -- the box
        of half-widths floor(r / |a*|), ... in itertools.product order, 000 in
        place, |g| < r.  ``recip``: rows a*, b*, c* in the structure's frame."""
        obj = cls.__new__(cls)
        recip = np.ascontiguousarray(np.asarray(recip, dtype=np.float64).reshape(3, 3))
        hmax = np.floor(float(reciprocal_radius) / np.linalg.norm(recip, axis=1)).astype(np.int64)
        obj._setup(recip, atoms, reciprocal_radius, False, form, _device(device), sphere_hmax=hmax)
        if build:
            obj.build(stream)
        return obj

    def _setup(self, recip, atoms, reciprocal_radius, with_direct_beam, form, dev, sphere_hmax=None):
        lib = N.load_library()
        self.device = dev
        self.form = form
        self.recip = recip
        self.dmin = 1.0 / float(reciprocal_radius)
        self.radius = float(reciprocal_radius)
        self.sphere_rule = sphere_hmax is not None
        self.hmax = box_extent(self.recip, self.dmin) if sphere_hmax is None else sphere_hmax
        self.n_zero = 2 if with_direct_beam else 0
        box = int(np.prod(2 * self.hmax + 1))
        self.cap = box + self.n_zero
        self._hkl = torch.empty((self.cap, 3), dtype=torch.int32, device=dev)
        self._g2 = torch.empty(self.cap, dtype=torch.float64, device=dev)
        self._count = torch.zeros(1, dtype=torch.int64, device=dev)
        self._status = torch.zeros(1, dtype=torch.int32, device=dev)
        self._hm = (C.c_int32 * 3)(*self.hmax.tolist())
        self._rb = (C.c_double * 9)(*self.recip.reshape(-1).tolist())
        self._enum_bytes = lib.ds_enumerate_scratch_bytes(self._hm)
        self.atoms = atoms
        self._sf_bytes = lib.ds_structure_factor_scratch_bytes(self.cap, self.atoms.n_atoms)
        self._scratch = torch.empty(max(self._enum_bytes, self._sf_bytes), dtype=torch.uint8, device=dev)
        self._F2 = torch.empty(self.cap, dtype=torch.float32, device=dev)
        self._F2d = torch.empty(self.cap, dtype=torch.float64, device=dev) if form == "fp64" else None
        self.n = 0

    def build(self, stream=None):
        """Enumerate the hkl rows and compute |F|^2 on the device (inputs
        already resident).  Synchronises once to read the row count."""
        lib = N.load_library()
        st = N.stream_handle(stream)
        self._status.zero_()
        if self.sphere_rule:
            N.check(lib.ds_enumerate_sphere(self._rb, self._hm, self.radius, N.ptr(self._hkl), N.ptr(self._g2),
                                            self.cap, N.ptr(self._count), N.ptr(self._scratch), self._enum_bytes,
                                            N.ptr(self._status), st), "enumerate_sphere")
        else:
            N.check(lib.ds_enumerate_hkl(self._rb, self._hm, self.dmin, self.n_zero, N.ptr(self._hkl),
                                         N.ptr(self._g2), self.cap, N.ptr(self._count), N.ptr(self._scratch),
                                         self._enum_bytes, N.ptr(self._status), st), "enumerate_hkl")
        n = int(self._count.item())
        N.check_device_status(self._status, "enumerate_hkl")
        self.n = n
        self.hkl = self._hkl[:n]
        self.g2 = self._g2[:n]
        self.F2 = self._F2[:max(n, 1)]
        self.F2d = self._F2d[:max(n, 1)] if self._F2d is not None else None
        if n:
            a = self.atoms.cstruct()
            N.check(lib.ds_structure_factors(a, N.ptr(self.hkl), None, N.ptr(self.g2), n, FORMS[self.form],
                                             N.ptr(self.F2), N.ptr(self.F2d), None, N.ptr(self._scratch),
                                             self._scratch.numel(), N.ptr(self._status), st), "structure_factors")
        return self

    def hkl_host(self) -> np.ndarray:
        if getattr(self, "_hkl_host", None) is None or self._hkl_host.shape[0] != self.n:
            self._hkl_host = self.hkl.cpu().numpy()
        return self._hkl_host

    def cstruct(self) -> N.ds_phase_table:
        t = N.ds_phase_table()
        t.n_hkl = self.n
        t.hkl = self.hkl.data_ptr() if self.n else None
        t.g2 = self.g2.data_ptr() if self.n else None
        t.F2 = self.F2.data_ptr()
        t.F2d = self.F2d.data_ptr() if self.F2d is not None else None
        for i, v in enumerate(self.recip.reshape(-1)):
            t.recip[i] = float(v)
        for i, v in enumerate(self.hmax):
            t.hmax[i] = int(v)
        return t


@dataclass
class SimSettings:
    """The per-call simulation constants (the generator's settings)."""
    k0: float
    max_excitation_error: float
    shape_width: float
    shape_model: str
    precession_angle_rad: float = 0.0
    precession_mode: int = N.DS_PRECESSION_NONE
    minimum_intensity: float = 1e-20
    minima_number: float = 5.0
    form: str = "mixed"
    orient_tile: int = 0
    stage_cap: int = 0
    screen: str = "auto"
    refine_parts: int = 0   # word ranges per orientation in the refine / write passes (0: library choice)

    def cstruct(self) -> N.ds_sim_params:
        return N.ds_sim_params(self.k0, self.max_excitation_error, self.shape_width, self.precession_angle_rad,
                               self.minimum_intensity, self.minima_number, N.DS_SHAPE[self.shape_model],
                               self.precession_mode, FORMS[self.form], self.orient_tile, self.stage_cap,
                               N.DS_SCREEN[self.screen], self.refine_parts, 0)


class PhaseSpots:
    """CSR spots of one phase on the device: ``offsets`` (n_orient + 1),
    ``hkl_index`` (rows of the phase table), ``xyzi`` (x, y, z, intensity)."""

    def __init__(self, table: PhaseTable, offsets, hkl_index, xyzi, total, excitation_error=None):
        self.table = table
        self.offsets = offsets
        self.hkl_index = hkl_index[:total]
        self.xyzi = xyzi[:total]
        self.excitation_error = None if excitation_error is None else excitation_error[:total]
        self.total = total
        self._host = None

    @property
    def n_orient(self):
        return self.offsets.shape[0] - 1

    def host(self, pinned=False):
        """Host copies of the CSR arrays: (offsets int64, hkl_index int32
        (row of the phase table), xyzi (total, 4) float32: x, y, z, I).  With
        ``pinned`` the copies go through page-locked memory.  Miller indices
        are gathered per pattern on access (``hkl_of``)."""
        if self._host is None:
            if pinned:
                off, idx, xyzi = _fetch_pinned((self.offsets, self.hkl_index, self.xyzi))
            else:
                off, idx, xyzi = self.offsets.cpu(), self.hkl_index.cpu(), self.xyzi.cpu()
            torch.cuda.current_stream().synchronize()
            self._host = (off.numpy(), idx.numpy(), xyzi.numpy())
        return self._host

    @classmethod
    def from_vectors(cls, vectors, device=None):
        """Device CSR spots from host spot vectors (objects with ``data``
        (n, 3) and ``intensity`` (n,), and optionally ``hkl``), one per
        pattern: the form ``Simulation2D`` takes for user-built coordinates."""
        dev = _device(device)
        counts = [np.asarray(v.data).reshape(-1, 3).shape[0] for v in vectors]
        off = np.zeros(len(vectors) + 1, dtype=np.int64)
        off[1:] = np.cumsum(counts)
        total = int(off[-1])
        xyzi = np.zeros((max(total, 1), 4), dtype=np.float32)
        hkl = np.zeros((max(total, 1), 3), dtype=np.float64)
        for v, a, b in zip(vectors, off[:-1], off[1:]):
            xyzi[a:b, :3] = np.asarray(v.data, dtype=np.float64).reshape(-1, 3)
            inten = getattr(v, "intensity", None)
            xyzi[a:b, 3] = np.nan if inten is None else np.asarray(inten, dtype=np.float64)
            h = getattr(v, "hkl", None)
            if h is not None:
                hkl[a:b] = np.asarray(h, dtype=np.float64).reshape(-1, 3)
        obj = cls(None, torch.as_tensor(off).to(dev), torch.arange(max(total, 1), dtype=torch.int32).to(dev),
                  torch.as_tensor(xyzi).to(dev), total)
        obj._hkl_rows = hkl[:total]
        return obj

    def pattern(self, i):
        """(hkl (n, 3) int, xyz (n, 3) float64, intensity (n,) float64) of orientation i."""
        off, idx, xyzi = self.host()
        a, b = off[i], off[i + 1]
        if self.table is None:
            hkl = self._hkl_rows[idx[a:b]]
        else:
            hkl = self.table.hkl_host()[idx[a:b]] if b > a else np.zeros((0, 3), np.int32)
        rec = xyzi[a:b].astype(np.float64)
        return hkl, rec[:, :3], rec[:, 3]

    def nbytes(self):
        return self.offsets.numel() * 8 + self.total * (4 + 16)

    def select(self, index) -> "PhaseSpots":
        """The patterns ``index`` (an int, a slice or an integer array) as a
        new ``PhaseSpots``: their CSR rows gathered on the device, the table
        shared."""
        n = self.n_orient
        pick = np.atleast_1d(np.arange(n)[index]).astype(np.int64)
        dev = self.offsets.device
        sel = torch.as_tensor(pick, device=dev)
        starts = self.offsets[sel]
        counts = self.offsets[sel + 1] - starts
        off = torch.zeros(pick.shape[0] + 1, dtype=torch.int64, device=dev)
        off[1:] = torch.cumsum(counts, 0)
        total = int(off[-1].item())
        which = torch.repeat_interleave(torch.arange(pick.shape[0], device=dev), counts)
        src = starts[which] + (torch.arange(total, device=dev) - off[:-1][which])
        s = None if self.excitation_error is None else self.excitation_error[src]
        out = PhaseSpots(self.table, off, self.hkl_index[src], self.xyzi[src], total, s)
        if self.table is None:
            out._hkl_rows = self._hkl_rows
        return out

    def __deepcopy__(self, memo):
        """Copies of the device arrays; the phase table (read-only) is shared."""
        s = None if self.excitation_error is None else self.excitation_error.clone()
        out = PhaseSpots(self.table, self.offsets.clone(), self.hkl_index.clone(), self.xyzi.clone(), self.total, s)
        if self.table is None:
            out._hkl_rows = self._hkl_rows.copy()
        return out


def _fetch_pinned(tensors):
    """Device -> page-locked host copies (torch's caching host allocator
    reuses freed pinned blocks, so repeated calls do not pay for pinning)."""
    out = []
    for t in tensors:
        h = torch.empty(t.shape, dtype=t.dtype, pin_memory=True)
        h.copy_(t, non_blocking=True)
        out.append(h)
    return out


class SpotBuffers:
    """Reusable device buffers for ``simulate_phase`` (grown on demand)."""

    def __init__(self, device, with_excitation_error=False):
        self.device = device
        self.capacity = 0
        self.idx = self.xyzi = self.s = None
        self.with_s = with_excitation_error
        self.scratch = None
        self.status = torch.zeros(1, dtype=torch.int32, device=device)
        self.total = torch.zeros(1, dtype=torch.int64, device=device)

    def ensure(self, capacity, scratch_bytes):
        if capacity > self.capacity:
            self.capacity = int(capacity)
            self.idx = torch.empty(self.capacity, dtype=torch.int32, device=self.device)
            self.xyzi = torch.empty((self.capacity, 4), dtype=torch.float32, device=self.device)
            if self.with_s:
                self.s = torch.empty(self.capacity, dtype=torch.float64, device=self.device)
        if self.scratch is None or self.scratch.numel() < scratch_bytes:
            self.scratch = torch.empty(int(scratch_bytes), dtype=torch.uint8, device=self.device)


def estimate_spots(table: PhaseTable, settings: SimSettings, radius: float) -> int:
    """Expected spots per orientation: rows inside the |s| < s_max shell (area
    pi r^2 times thickness 2 s_max out of the 4/3 pi r^3 sphere), widened for
    precession."""
    band = 2 * settings.max_excitation_error + 2 * radius * np.sin(settings.precession_angle_rad)
    frac = min(1.0, 1.5 * band / max(radius, 1e-9))
    return int(table.n * frac) + 8


def simulate_phase(table: PhaseTable, quats: torch.Tensor, settings: SimSettings, radius: float,
                   buffers: SpotBuffers | None = None, stream=None, sync=True):
    """Run ds_simulate for one phase; returns PhaseSpots (device CSR).

    quats: (N, 4) float64 on the device.  On output-capacity overflow the call
    is repeated once with the exact size the first run reported.
    """
    lib = N.load_library()
    dev = table.device
    n_orient = int(quats.shape[0])
    buffers = buffers or SpotBuffers(dev)
    p = settings.cstruct()
    t = table.cstruct()
    sbytes = lib.ds_simulate_scratch_bytes(p, t, n_orient)
    cap = max(1024, n_orient * estimate_spots(table, settings, radius) * 5 // 4)
    offsets = torch.empty(n_orient + 1, dtype=torch.int64, device=dev)
    st = N.stream_handle(stream)
    for attempt in range(2):
        buffers.ensure(cap, sbytes)
        buffers.status.zero_()
        out = N.ds_spots(offsets.data_ptr(), buffers.idx.data_ptr(), buffers.xyzi.data_ptr(), buffers.capacity,
                         buffers.total.data_ptr(), buffers.s.data_ptr() if buffers.s is not None else None)
        N.check(lib.ds_simulate(p, t, N.ptr(quats), n_orient, out, N.ptr(buffers.scratch), sbytes,
                                N.ptr(buffers.status), st), "simulate")
        if not sync:
            return None
        v = N.check_device_status(buffers.status, "simulate", allow=N.DS_ERR_CAPACITY)
        N.check_device_status(table._status, "structure_factors")
        total = int(buffers.total.item())
        if not (v & N.DS_ERR_CAPACITY):
            return PhaseSpots(table, offsets, buffers.idx, buffers.xyzi, total, buffers.s)
        cap = total + 1024
    raise N.NativeError("simulate: output capacity still exceeded after resizing")


class HostSpotPool:
    """Page-locked host arrays for streamed results, kept across calls.

    Allocating (pinning) gigabytes of host memory costs far more than the
    copies that fill it, so a generator keeps the sets it has made and hands
    one out again once the result that used it has been garbage-collected
    (each set remembers its owner through a weak reference).  A caller that
    keeps every result alive gets a new set per call; one that drops the
    previous result (the usual loop) alternates between two.  The numpy
    arrays a result's ``host()`` returns guard the set too: while any of
    them (or a view of one) lives, the set is not handed out again.  At most
    ``max_sets`` idle sets are kept."""

    def __init__(self, max_sets=2, headroom=1.25):
        self.max_sets = int(max_sets)
        self.headroom = float(headroom)
        # [offsets int64, hkl_index int32, xyzi float32 (n, 4), owner weakref or None, guards
        #  (, addressable by kernels)]
        self._sets = []
        self.allocated_bytes = 0
        # spots per orientation of earlier calls, by (table rows, settings, radius):
        # sizes the next call's arrays when the kernel writes into them directly
        self.density = {}

    @staticmethod
    def mapped(s):
        """Whether set ``s`` is addressable by kernels at its host addresses
        (``ds_host_mapped``; asked once per set)."""
        if len(s) < 6:
            s.append(all(N.host_mapped(t.data_ptr()) for t in s[:3]))
        return s[5]

    @staticmethod
    def _free(s):
        return (s[3] is None or s[3]() is None) and all(g() is None for g in s[4])

    def acquire(self, n_orient, n_spots, index_dtype=torch.int32):
        """A free set with room for ``n_orient`` orientations and ``n_spots``
        spots (the smallest that fits) whose row array has ``index_dtype``
        (int32, or int16 holding the uint16 rows of small tables), or a new
        one."""
        fits = [s for s in self._sets if self._free(s) and s[0].shape[0] >= n_orient + 1 and s[1].shape[0] >= n_spots
                and s[1].dtype == index_dtype]
        if fits:
            s = min(fits, key=lambda s: s[1].shape[0])
            s[3] = None
            s[4] = []
            return s
        idle = [s for s in self._sets if self._free(s)]
        while idle and len(idle) >= self.max_sets:  # drop the smallest idle sets first
            victim = min(idle, key=lambda s: s[1].shape[0])
            idle.remove(victim)
            self._sets.remove(victim)
        n_o = int((n_orient + 1) * self.headroom) + 1
        n_s = max(int(n_spots * self.headroom), 1024)
        s = [torch.empty(n_o, dtype=torch.int64, pin_memory=True),
             torch.empty(n_s, dtype=index_dtype, pin_memory=True),
             torch.empty((n_s, 4), dtype=torch.float32, pin_memory=True), None, []]
        self.allocated_bytes += n_o * 8 + n_s * (16 + torch.empty(0, dtype=index_dtype).element_size())
        self._sets.append(s)
        return s

    def bind(self, s, owner):
        s[3] = weakref.ref(owner)

    @staticmethod
    def guard(s, array):
        """Keep set ``s`` from reuse while ``array`` (a numpy view of it) or
        any view derived from it lives: numpy views share the base object,
        here the tensor alias that ``Tensor.numpy()`` creates."""
        base = array.base if array.base is not None else array
        s[4].append(weakref.ref(base))


def _row_index_dtype(table) -> torch.dtype:
    """Storage of the spots' table rows on their way to the host: uint16 rows
    (kept in int16 tensors) when the table has at most 65536 rows, else int32."""
    return torch.int16 if table.n <= 65536 else torch.int32


def _rows_int32(idx: torch.Tensor) -> torch.Tensor:
    """Device rows as int32 (uint16 rows held in an int16 tensor widened)."""
    return idx if idx.dtype == torch.int32 else idx.to(torch.int32) & 0xFFFF


def _rows_numpy(idx: torch.Tensor) -> np.ndarray:
    """Host rows as numpy: int32, or the uint16 view of int16 storage."""
    a = idx.numpy()
    return a.view(np.uint16) if a.dtype == np.int16 else a


class StreamedSpots(PhaseSpots):
    """Spots of one phase simulated in orientation chunks, each chunk's CSR
    copied to page-locked host memory on a side stream while the later
    chunks compute.  For a result wanted on the host the device-to-host link
    (about 190 GB/s against 20 bytes per spot) bounds the call, not the
    kernel, so the copies start as soon as the first chunk is done.

    ``host()`` waits for the copies in flight.  The device CSR (``offsets``
    is global; ``hkl_index``, ``xyzi``, ``excitation_error``) is assembled
    from the chunks' regions on first access.  ``timings()`` gives the time
    split of the call once the copies are done."""

    def __init__(self, table, chunks, regions, host_bufs, done, total, timing=None, status_h=None,
                 off_stage=None):
        self.table = table
        self._status_h = status_h    # chunks' status words, complete at ``done`` (None: checked already)
        self._off_stage = off_stage  # page-locked copy of the chunks' offsets (chunk k at a + k), at ``done``
        self._chunks = chunks        # per chunk: (first orientation, chunk offsets on the device, spot base, k)
        self._regions = regions      # per chunk: (idx, xyzi, s, n_spots)
        self._host_bufs = host_bufs  # page-locked (offsets, hkl_index, xyzi) (pool set)
        self._done = done            # event after the last copy
        self.total = total
        self._n = sum(c[1].shape[0] - 1 for c in chunks)
        self._host = None
        self._dev = None
        self._off = None
        self._timing = timing or {}

    @property
    def n_orient(self):
        return self._n

    def _check_status(self):
        """Raise on a condition any chunk's kernel reported (waits for the
        copies, behind which the status words travel)."""
        if self._status_h is not None:
            self._done.synchronize()
            for v in self._status_h.tolist():
                N.check_status_value(int(v), "simulate")
            self._status_h = None

    def _device_csr(self):
        if self._dev is None:
            self._check_status()
            regs = [r for r in self._regions if r[3] > 0] or self._regions[:1]
            idx = _rows_int32(torch.cat([r[0][:r[3]] for r in regs]))
            xyzi = torch.cat([r[1][:r[3]] for r in regs])
            s = torch.cat([r[2][:r[3]] for r in regs]) if regs[0][2] is not None else None
            self._dev = (idx, xyzi, s)
            self._regions = None  # the chunk regions are no longer needed
        return self._dev

    @property
    def offsets(self):
        if self._off is None:
            self._check_status()
            parts = [o[:-1] + base for _, o, base, _ in self._chunks]
            parts.append(torch.full((1,), self.total, dtype=torch.int64, device=self._chunks[0][1].device))
            self._off = torch.cat(parts)
        return self._off

    @property
    def hkl_index(self):
        return self._device_csr()[0]

    @property
    def xyzi(self):
        return self._device_csr()[1]

    @property
    def excitation_error(self):
        return self._device_csr()[2]

    def host(self, pinned=False):
        if self._host is None:
            t0 = time.perf_counter()
            self._done.synchronize()
            t1 = time.perf_counter()
            self._check_status()
            hb = self._host_bufs
            off = hb[0][:self._n + 1].numpy()
            stage = self._off_stage.numpy()
            for a, o, base, k in self._chunks:  # chunk-relative offsets made global
                m = o.shape[0] - 1
                np.add(stage[a + k:a + k + m], base, out=off[a:a + m])
            off[self._n] = self.total
            self._host = (off, _rows_numpy(hb[1][:self.total]), hb[2][:self.total].numpy())
            for arr in self._host:
                HostSpotPool.guard(hb, arr)
            self._timing["host_wait_ms"] = (t1 - t0) * 1e3
            self._timing["host_wrap_ms"] = (time.perf_counter() - t1) * 1e3
        return self._host

    def nbytes(self):
        """Bytes of the host CSR (what the call copied to the host)."""
        row = self._host_bufs[1].element_size() if self._host_bufs is not None else 4
        return (self._n + 1) * 8 + self.total * (row + 16)

    def timings(self):
        """Time split of the call (milliseconds), complete after ``host()``:
        host set-up before the first launch, host time blocked on chunk
        counts, pinned-memory allocation, the chunks' device span (first
        launch to last chunk end) and the copies' span (first copy to the
        last), the wait in ``host()`` and the offsets fix-up."""
        t = dict(self._timing)
        ev = t.pop("_events", None)
        if ev is not None:
            self._done.synchronize()
            k0, k1, c0 = ev
            t["kernel_span_ms"] = k0.elapsed_time(k1)
            t["copy_span_ms"] = c0.elapsed_time(self._done) if c0 is not None else 0.0
            t["first_copy_after_launch_ms"] = k0.elapsed_time(c0) if c0 is not None else 0.0
        return t


def simulate_phase_streamed(table: PhaseTable, quats: torch.Tensor, settings: SimSettings, radius: float,
                            chunk=32768, first_chunk=1024, with_excitation_error=False,
                            host_pool: HostSpotPool | None = None, timing=False) -> StreamedSpots:
    """``simulate_phase`` for a result wanted on the host: the orientations
    run in chunks on the current stream, each into its own device region,
    and each chunk's spots are copied to page-locked host memory on a side
    stream as soon as its count is known, while the next chunks compute.
    Chunk sizes grow by 7/4 from ``first_chunk`` up to ``chunk``: the copies
    start early, and the copy of a chunk (at about 1.8 times the kernel's
    time per orientation) lasts as long as the next chunk's kernel, so the
    link does not wait for the kernel (with doubling it would).  The kernel
    stores each chunk's spot count into page-locked memory itself, so the
    compute stream holds no copy; the status words follow the spots and are
    checked when the result is read.  Table rows travel as uint16 for tables
    of at most 65536 rows.  A chunk whose spots overflow its region is re-run
    alone with the exact size.  The host arrays come from ``host_pool``
    (reused across calls) or are allocated; they are sized from the first
    chunk's spot count.  With ``timing`` the result records CUDA events for
    ``StreamedSpots.timings``."""
    t_start = time.perf_counter()
    lib = N.load_library()
    dev = table.device
    n = int(quats.shape[0])
    comp = torch.cuda.current_stream(dev)
    copy = torch.cuda.Stream(dev)
    host_pool = host_pool or HostSpotPool(max_sets=0)
    bounds = [0]
    size = max(1, min(first_chunk, chunk))
    while bounds[-1] < n:
        bounds.append(min(n, bounds[-1] + size))
        size = min(chunk, size * 7 // 4)
    if len(bounds) == 1:
        bounds.append(0)
    n_chunks = len(bounds) - 1
    p = settings.cstruct()
    t = table.cstruct()
    longest = max(b - a for a, b in zip(bounds[:-1], bounds[1:]))
    sbytes = lib.ds_simulate_scratch_bytes(p, t, longest)
    idt = _row_index_dtype(table)  # uint16 rows: 18 instead of 20 bytes per spot over the link
    per = estimate_spots(table, settings, radius)
    scratch = torch.empty(max(int(sbytes), 16), dtype=torch.uint8, device=dev)
    status = torch.zeros(n_chunks, dtype=torch.int32, device=dev)
    totals = torch.zeros(n_chunks, dtype=torch.int64, device=dev)
    totals_h = torch.zeros(n_chunks, dtype=torch.int64, pin_memory=True)
    status_h = torch.empty(n_chunks, dtype=torch.int32, pin_memory=True)
    # Each chunk's spot count goes straight to page-locked host memory in the
    # kernel's own store: a copy of it on the compute stream would queue in
    # the copy engine behind the spot copies and hold the next chunk's kernel
    # (and, through the host, the next copy) back.  The status words are
    # copied once after the last chunk.
    direct_totals = n > 0 and N.host_mapped(totals_h.data_ptr())
    # the chunks' offsets side by side in one array (chunk k at a + k), copied
    # to the host in one piece after the last chunk
    all_off = torch.empty(n + n_chunks, dtype=torch.int64, device=dev)
    off_stage = torch.empty(n + n_chunks, dtype=torch.int64, pin_memory=True)
    chunk_off = [all_off[a + k:b + k + 1] for k, (a, b) in enumerate(zip(bounds[:-1], bounds[1:]))]
    sf_status_h = torch.empty(1, dtype=torch.int32, pin_memory=True)
    sf_status_h.copy_(table._status, non_blocking=True)  # read after the first chunk, without a stall
    k_start = k_end = c_start = None
    if timing:
        k_start = torch.cuda.Event(enable_timing=True)
        k_end = torch.cuda.Event(enable_timing=True)
        c_start = torch.cuda.Event(enable_timing=True)
        k_start.record(comp)

    def launch(k, cap):
        a, b = bounds[k], bounds[k + 1]
        idx = torch.empty(cap, dtype=idt, device=dev)
        xyzi = torch.empty((cap, 4), dtype=torch.float32, device=dev)
        s = torch.empty(cap, dtype=torch.float64, device=dev) if with_excitation_error else None
        total_ptr = totals_h[k:].data_ptr() if direct_totals else totals[k:].data_ptr()
        out = N.ds_spots(chunk_off[k].data_ptr(), idx.data_ptr(), xyzi.data_ptr(), cap, total_ptr,
                         s.data_ptr() if s is not None else None, idx.element_size(), 0)
        N.check(lib.ds_simulate(p, t, N.ptr(quats[a:b]) if b > a else N.ptr(quats), b - a, out, N.ptr(scratch),
                                sbytes, N.ptr(status[k:]), N.stream_handle(comp)), "simulate")
        if not direct_totals:
            totals_h[k:k + 1].copy_(totals[k:k + 1], non_blocking=True)
            status_h[k:k + 1].copy_(status[k:k + 1], non_blocking=True)
        ev = torch.cuda.Event(enable_timing=timing)
        ev.record(comp)
        return [idx, xyzi, s, ev, cap]

    caps = [max(1024, (b - a) * per * 5 // 4) for a, b in zip(bounds[:-1], bounds[1:])]
    regions = [launch(k, caps[k]) for k in range(min(2, n_chunks))]
    t_launched = time.perf_counter()
    wait_s = alloc_s = 0.0
    hb = None
    h_idx = h_xyzi = None
    base = 0
    out_regions, chunks = [], []
    for k in range(n_chunks):
        idx, xyzi, s, ev, cap = regions[k]
        tw = time.perf_counter()
        ev.synchronize()
        wait_s += time.perf_counter() - tw
        if k == 0:
            N.check_status_value(int(sf_status_h[0]), "structure_factors")
        if not direct_totals:
            N.check_status_value(int(status_h[k]), "simulate", allow=N.DS_ERR_CAPACITY)
        cnt = int(totals_h[k])
        if cnt > cap:
            # the region overflowed (the count is exact): re-run the chunk alone
            status[k:k + 1].zero_()
            idx, xyzi, s, ev, cap = launch(k, cnt + 1024)
            ev.synchronize()
            if not direct_totals:
                N.check_status_value(int(status_h[k]), "simulate")
            cnt = int(totals_h[k])
        a, b = bounds[k], bounds[k + 1]
        if hb is None:
            # host arrays sized from the first chunk's spots per orientation
            need = int(np.ceil(cnt / max(b - a, 1) * n * 1.1)) + 4096
            ta = time.perf_counter()
            hb = host_pool.acquire(n, need, idt)
            alloc_s += time.perf_counter() - ta
            h_idx, h_xyzi = hb[1], hb[2]
        if base + cnt > h_idx.shape[0]:
            # the host arrays outgrew the estimate: a larger set (waits for the copies so far)
            copy.synchronize()
            ta = time.perf_counter()
            nb = host_pool.acquire(n, max(base + cnt, h_idx.shape[0] * 3 // 2), idt)
            alloc_s += time.perf_counter() - ta
            nb[1][:base].copy_(h_idx[:base])
            nb[2][:base].copy_(h_xyzi[:base])
            hb[3] = None
            hb[4] = []
            hb = nb
            h_idx, h_xyzi = hb[1], hb[2]
        copy.wait_event(ev)
        # copies only on the side stream: a kernel there would wait for an
        # SM behind the persistent simulation kernel, and the copies behind it
        with torch.cuda.stream(copy):
            if k == 0 and c_start is not None:
                c_start.record(copy)
            if cnt:
                h_idx[base:base + cnt].copy_(idx[:cnt], non_blocking=True)
                h_xyzi[base:base + cnt].copy_(xyzi[:cnt], non_blocking=True)
        out_regions.append((idx, xyzi, s, cnt))
        chunks.append((a, chunk_off[k], base, k))
        base += cnt
        if k + 2 < n_chunks:
            # chunk k + 1 is queued already: this launch follows the issue of
            # chunk k's copies, so the first copy starts one launch earlier
            regions.append(launch(k + 2, caps[k + 2]))
    # the offsets and (with the counts stored directly) every chunk's status
    # word, copied behind the spots on the copy stream; the status words are
    # checked before the result is read (a re-run chunk's word was cleared
    # first, so only real conditions remain)
    copy.wait_stream(comp)
    with torch.cuda.stream(copy):
        off_stage.copy_(all_off, non_blocking=True)
        if direct_totals:
            status_h.copy_(status, non_blocking=True)
    done = torch.cuda.Event(enable_timing=timing)
    done.record(copy)
    if k_end is not None:
        k_end.record(comp)
    # the chunk buffers were read on the copy stream as well
    for r in out_regions + [(all_off, None, None, 0)]:
        for x in r[:3]:
            if x is not None:
                x.record_stream(copy)
    rec = {"launch_ms": (t_launched - t_start) * 1e3, "chunk_wait_ms": wait_s * 1e3, "pinned_alloc_ms": alloc_s * 1e3,
           "streamed_call_ms": (time.perf_counter() - t_start) * 1e3, "chunks": n_chunks}
    if timing:
        rec["_events"] = (k_start, k_end, c_start)
    res = StreamedSpots(table, chunks, out_regions, hb, done, base, rec, status_h if direct_totals else None,
                        off_stage)
    host_pool.bind(hb, res)
    return res


class HostSpots(PhaseSpots):
    """Spots of one phase that the orientation kernel stored straight into
    page-locked host memory (``simulate_phase_to_host``).  ``host()`` returns
    views of those arrays (complete when the call returns); the device CSR
    (``offsets``, ``hkl_index``, ``xyzi``) is uploaded on first access.
    ``timings()`` gives the time split of the call."""

    def __init__(self, table, host_set, n_orient, total, timing=None):
        self.table = table
        self._set = host_set         # page-locked (offsets, hkl_index, xyzi) (pool set)
        self._n = int(n_orient)
        self.total = int(total)
        self.excitation_error = None
        self._host = None
        self._dev = None
        self._timing = timing or {}

    @property
    def n_orient(self):
        return self._n

    def _device_csr(self):
        if self._dev is None:
            hb, dev = self._set, self.table.device
            self._dev = (hb[0][:self._n + 1].to(dev), _rows_int32(hb[1][:self.total].to(dev)),
                         hb[2][:self.total].to(dev))
        return self._dev

    @property
    def offsets(self):
        return self._device_csr()[0]

    @property
    def hkl_index(self):
        return self._device_csr()[1]

    @property
    def xyzi(self):
        return self._device_csr()[2]

    def host(self, pinned=False):
        if self._host is None:
            t0 = time.perf_counter()
            hb = self._set
            self._host = (hb[0][:self._n + 1].numpy(), _rows_numpy(hb[1][:self.total]), hb[2][:self.total].numpy())
            for arr in self._host:
                HostSpotPool.guard(hb, arr)
            self._timing["host_wrap_ms"] = (time.perf_counter() - t0) * 1e3
        return self._host

    def nbytes(self):
        return (self._n + 1) * 8 + self.total * (self._set[1].element_size() + 16)

    def timings(self):
        """Time split of the call (milliseconds): host set-up before the
        launch, the host's wait for the kernel, page-locked allocation, and
        the kernel's device time, which is also the transfer's (its stores
        are the transfer; ``copy_span_ms`` repeats it)."""
        t = dict(self._timing)
        ev = t.pop("_events", None)
        if ev is not None:
            k0, k1 = ev
            k1.synchronize()
            t["kernel_span_ms"] = t["copy_span_ms"] = k0.elapsed_time(k1)
            t["first_copy_after_launch_ms"] = 0.0
        return t


def simulate_phase_to_host(table: PhaseTable, quats: torch.Tensor, settings: SimSettings, radius: float,
                           host_pool: HostSpotPool | None = None, timing=False) -> HostSpots | None:
    """``simulate_phase`` for a result wanted on the host, as one launch whose
    output arrays are page-locked host memory: the orientation kernel's own
    coalesced stores carry the spots over the host link while it computes.
    The link (about 190 GB/s against 20 bytes per spot) bounds the call; the
    kernel's work hides under it entirely, with no device staging of the
    spots and no separate copy.  The host arrays come from ``host_pool``,
    sized from the spots per orientation of an earlier call with the same
    table size and settings, else from ``estimate_spots``; a launch that
    overflows them is re-run once with the exact size.  Returns None, having
    launched nothing, when there are no orientations or the pool's memory is
    not addressable by kernels (the caller then copies instead:
    ``simulate_phase_streamed``).  Returns once the spots are on the host."""
    t_start = time.perf_counter()
    n = int(quats.shape[0])
    if n == 0:
        return None
    lib = N.load_library()
    dev = table.device
    host_pool = host_pool or HostSpotPool(max_sets=0)
    p = settings.cstruct()
    t = table.cstruct()
    sbytes = int(lib.ds_simulate_scratch_bytes(p, t, n))
    key = (int(table.n), float(settings.max_excitation_error), float(settings.shape_width),
           float(settings.precession_angle_rad), int(settings.precession_mode), float(radius))
    per = host_pool.density.get(key)
    need = int(n * per * 1.05) + 1024 if per is not None else n * estimate_spots(table, settings, radius)
    scratch = torch.empty(max(sbytes, 16), dtype=torch.uint8, device=dev)
    status = torch.zeros(1, dtype=torch.int32, device=dev)
    total = torch.zeros(1, dtype=torch.int64, device=dev)
    comp = torch.cuda.current_stream(dev)
    alloc_s = wait_s = 0.0
    events = None
    idt = _row_index_dtype(table)
    for attempt in range(2):
        ta = time.perf_counter()
        hb = host_pool.acquire(n, need, idt)
        alloc_s += time.perf_counter() - ta
        if not host_pool.mapped(hb):
            return None
        if attempt:
            status.zero_()
        if timing:
            events = (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
            events[0].record(comp)
        out = N.ds_spots(hb[0].data_ptr(), hb[1].data_ptr(), hb[2].data_ptr(), int(hb[1].shape[0]),
                         total.data_ptr(), None, hb[1].element_size(), 0)
        N.check(lib.ds_simulate(p, t, N.ptr(quats), n, out, N.ptr(scratch), sbytes, N.ptr(status),
                                N.stream_handle(comp)), "simulate")
        if timing:
            events[1].record(comp)
        tw = time.perf_counter()
        if attempt == 0:
            t_launched = tw
        v = N.check_device_status(status, "simulate", allow=N.DS_ERR_CAPACITY)  # waits for the kernel
        wait_s += time.perf_counter() - tw
        N.check_device_status(table._status, "structure_factors")
        cnt = int(total.item())
        if not (v & N.DS_ERR_CAPACITY):
            break
        need = cnt
    else:
        raise N.NativeError("simulate: output capacity still exceeded after resizing")
    host_pool.density[key] = cnt / n
    rec = {"launch_ms": (t_launched - t_start) * 1e3, "chunk_wait_ms": wait_s * 1e3,
           "pinned_alloc_ms": alloc_s * 1e3, "streamed_call_ms": (time.perf_counter() - t_start) * 1e3,
           "chunks": 1, "host_wait_ms": 0.0}
    if timing:
        rec["_events"] = events
    res = HostSpots(table, hb, n, cnt, rec)
    host_pool.bind(hb, res)
    return res


def apply_shape_factors(spots: PhaseSpots, F2: torch.Tensor, shape_factors: torch.Tensor, minimum_intensity: float,
                        stream=None) -> PhaseSpots:
    """The spots of ``spots`` (one phase, the model switched off) finished
    with per-spot shape factors ``shape_factors`` (float64): I = sf |F|^2,
    the per-pattern mask I > max I * minimum_intensity and ordered
    compaction (``ds_apply_shape_factors``)."""
    lib = N.load_library()
    dev = spots.offsets.device
    n = spots.n_orient
    total_in = int(spots.total)
    sf = shape_factors.to(dev, torch.float64).contiguous()
    if sf.numel() != total_in:
        raise ValueError(f"{sf.numel()} shape factors for {total_in} spots")
    nbytes = lib.ds_apply_shape_factors_scratch_bytes(n)
    scratch = torch.empty(max(int(nbytes), 16), dtype=torch.uint8, device=dev)
    status = torch.zeros(1, dtype=torch.int32, device=dev)
    total = torch.zeros(1, dtype=torch.int64, device=dev)
    offsets = torch.empty(n + 1, dtype=torch.int64, device=dev)
    cap = max(total_in, 1)
    idx = torch.empty(cap, dtype=torch.int32, device=dev)
    xyzi = torch.empty((cap, 4), dtype=torch.float32, device=dev)
    xin = spots.xyzi if total_in else torch.zeros((1, 4), dtype=torch.float32, device=dev)
    iin = spots.hkl_index if total_in else torch.zeros(1, dtype=torch.int32, device=dev)
    out = N.ds_spots(offsets.data_ptr(), idx.data_ptr(), xyzi.data_ptr(), cap, total.data_ptr(), None)
    N.check(lib.ds_apply_shape_factors(N.ptr(spots.offsets), N.ptr(iin), N.ptr(xin), N.ptr(sf) if total_in else None,
                                       N.ptr(F2), n, float(minimum_intensity), out, N.ptr(scratch), scratch.numel(),
                                       N.ptr(status), N.stream_handle(stream)), "apply_shape_factors")
    N.check_device_status(status, "apply_shape_factors")
    return PhaseSpots(spots.table, offsets, idx, xyzi, int(total.item()))


def custom_shape_spots(table: PhaseTable, quats: torch.Tensor, settings: SimSettings, radius: float, model,
                       kwargs: dict) -> PhaseSpots:
    """One phase's spots with a shape-factor function of the caller's
    (diffsims/generators/simulation_generator.py:387-411): the orientation
    kernel selects the spots with the model switched off and returns their
    excitation errors; ``model(s, width, **kwargs)`` is evaluated on each
    pattern's array on the host (with precession and
    ``approximate_precession=False``, its average over the precession circle,
    (1/2 pi) int_0^2pi model(s + r phi cos t) dt by adaptive quadrature per
    spot, diffsims/utils/shape_factor_models.py:222-268); the kernel
    ``ds_apply_shape_factors`` finishes the intensities, the mask and the
    compaction."""
    select = SimSettings(**{**settings.__dict__, "shape_model": "binary", "minimum_intensity": -1.0})
    first = simulate_phase(table, quats, select, radius, SpotBuffers(table.device, with_excitation_error=True))
    off, _, xyzi = first.host()
    s_all = first.excitation_error.cpu().numpy() if first.total else np.zeros(0)
    w = settings.shape_width
    sf = np.zeros(first.total, dtype=np.float64)
    phi = settings.precession_angle_rad
    if settings.precession_mode == N.DS_PRECESSION_INTEGRAL:
        from scipy.integrate import quad
        r_all = np.hypot(xyzi[:, 0].astype(np.float64), xyzi[:, 1].astype(np.float64))
        for k in range(first.total):
            s0, a = float(s_all[k]), float(r_all[k]) * phi
            sf[k] = quad(lambda t: model(s0 + a * np.cos(t), w, **kwargs), 0, 2 * np.pi)[0] / (2 * np.pi)
    else:
        for i in range(first.n_orient):
            a, b = int(off[i]), int(off[i + 1])
            if b > a:
                sf[a:b] = np.broadcast_to(np.asarray(model(s_all[a:b], w, **kwargs), dtype=np.float64), (b - a,))
    return apply_shape_factors(first, table.F2, torch.from_numpy(sf), settings.minimum_intensity)


@dataclass
class RasterSettings:
    """Arguments of Simulation2D.get_diffraction_pattern
    (diffsims/simulations/simulation2d.py:357-368) for ``rasterize``;
    ``truncate`` is scipy.ndimage.gaussian_filter's (4.0) and ``pixel_snap``
    moves positions within that many pixels of a whole pixel onto it (0: the
    reference's exact truncation)."""
    shape: tuple
    sigma: float = 10.0
    direct_beam_position: tuple | None = None
    in_plane_angle: float = 0.0
    calibration: float = 0.01
    mirrored: bool = False
    fast: bool = True
    normalize: bool = True
    clip_threshold: float = 1.0
    truncate: float = 4.0
    pixel_snap: float = 0.0

    def cstruct(self):
        if self.shape is None or len(self.shape) != 2:
            raise ValueError("shape must be (rows, columns)")
        H, W = int(self.shape[0]), int(self.shape[1])
        if self.direct_beam_position is None:
            # simulation2d.py:404-411: whole-pixel centre in fast mode, the
            # sub-pixel centre otherwise (spot coordinates are floats)
            cx, cy = (W // 2, H // 2) if self.fast else ((W - 1) / 2, (H - 1) / 2)
        else:
            cx, cy = self.direct_beam_position
        return N.ds_raster_params(H, W, int(bool(self.mirrored)), int(bool(self.fast)), int(bool(self.normalize)), 0,
                                  float(self.sigma), float(self.calibration), float(cx), float(cy),
                                  float(self.in_plane_angle), float(self.clip_threshold), float(self.truncate),
                                  float(self.pixel_snap))


class RasterBuffers:
    """Reusable scratch and status words for ``rasterize``."""

    def __init__(self, device):
        self.device = device
        self.status = torch.zeros(1, dtype=torch.int32, device=device)
        self.scratch = None

    def ensure(self, nbytes):
        if nbytes and (self.scratch is None or self.scratch.numel() < nbytes):
            self.scratch = torch.empty(nbytes, dtype=torch.uint8, device=self.device)


def rasterize(spots: PhaseSpots, settings: RasterSettings, start=0, stop=None, out=None, max_spots=None,
              buffers: RasterBuffers | None = None, stream=None, sync=True) -> torch.Tensor:
    """Detector images (stop - start, rows, columns) float32 on the device of
    patterns ``start:stop`` of one phase, one ds_rasterize launch.
    ``max_spots`` (spots of the largest pattern) is measured when not given."""
    lib = N.load_library()
    n_all = spots.n_orient
    stop = n_all if stop is None else stop
    if not 0 <= start <= stop <= n_all:
        raise IndexError(f"patterns {start}:{stop} of {n_all}")
    n = stop - start
    p = settings.cstruct()
    dev = spots.offsets.device
    if out is None:
        out = torch.empty((n, p.height, p.width), dtype=torch.float32, device=dev)
    elif (tuple(out.shape) != (n, p.height, p.width) or out.dtype != torch.float32 or not out.is_contiguous()
          or out.device != dev):
        raise ValueError(f"out must be a contiguous float32 ({n}, {p.height}, {p.width}) tensor on {dev}")
    if n == 0:
        return out
    off = spots.offsets[start:stop + 1]
    if max_spots is None:
        max_spots = int((off[1:] - off[:-1]).max().item())
    buffers = buffers or RasterBuffers(dev)
    sbytes = lib.ds_rasterize_scratch_bytes(p, max_spots)
    N.check(0 if sbytes or lib.ds_last_error() == b"" else N.DS_ERR_INVALID_ARGUMENT, "rasterize")
    buffers.ensure(sbytes)
    buffers.status.zero_()
    xyzi = spots.xyzi if spots.total > 0 else None
    N.check(lib.ds_rasterize(p, N.ptr(off), N.ptr(xyzi), n, max_spots, N.ptr(out), N.ptr(buffers.scratch), sbytes,
                             N.ptr(buffers.status), N.stream_handle(stream)), "rasterize")
    if sync:
        N.check_device_status(buffers.status, "rasterize")
    return out


# ---------------------------------------------------------------- batches ----
BATCH_MAX = 96  # phases per launch (include/diffsims_gb300.h)


class PhaseBatch:
    """Many phases simulated in one persistent launch per group of up to 96
    phases (``ds_simulate_batch``): one CSR output over all phases'
    orientations.  ``run`` launches; ``capture`` records the launch sequence
    in a CUDA graph that ``replay`` re-issues (inputs and outputs stay at
    the same addresses); ``spots`` gives one ``PhaseSpots`` per phase.

    The orientation tile is chosen by ``Autotuner`` unless ``orient_tile``
    is given."""

    def __init__(self, tables, quats, settings: SimSettings, radius: float, orient_tile=None, autotuner=None,
                 device=None):
        if len(tables) != len(quats) or not tables:
            raise ValueError("one quaternion set per phase table is needed")
        self.device = tables[0].device if device is None else torch.device(device)
        self.tables = list(tables)
        self.quats = [q.to(self.device, torch.float64).contiguous() for q in quats]
        self.settings = settings
        self.radius = float(radius)
        self.n_orient = [int(q.shape[0]) for q in self.quats]
        self.groups = [list(range(i, min(i + BATCH_MAX, len(tables)))) for i in range(0, len(tables), BATCH_MAX)]
        self._items = [self._items_of(g) for g in self.groups]
        self.status = torch.zeros(len(self.groups), dtype=torch.int32, device=self.device)
        self.totals = torch.zeros(len(self.groups), dtype=torch.int64, device=self.device)
        self.offsets = [torch.zeros(sum(self.n_orient[i] for i in g) + 1, dtype=torch.int64, device=self.device)
                        for g in self.groups]
        self.graph = None
        self.stage_cap = int(settings.stage_cap)
        self.refine_parts = int(settings.refine_parts)
        self.orient_tile = 0
        if orient_tile is None:
            orient_tile = (autotuner or AUTOTUNER).tile_for(self)
        self.orient_tile = int(orient_tile)
        self._plan()

    def _items_of(self, group):
        arr = (N.ds_batch_phase * len(group))()
        for k, i in enumerate(group):
            arr[k].table = self.tables[i].cstruct()
            arr[k].quats = self.quats[i].data_ptr() if self.n_orient[i] else None
            arr[k].n_orient = self.n_orient[i]
        return arr

    def cparams(self, orient_tile=None):
        p = self.settings.cstruct()
        p.orient_tile = int(self.orient_tile if orient_tile is None else orient_tile)
        p.stage_cap = int(self.stage_cap)
        if self.refine_parts:
            p.refine_parts = int(self.refine_parts)
        return p

    def _plan(self, capacity=None):
        lib = N.load_library()
        p = self.cparams()
        self.scratch_bytes = [lib.ds_simulate_batch_scratch_bytes(p, it, len(it)) for it in self._items]
        if any(b == 0 for b, g in zip(self.scratch_bytes, self.groups) if sum(self.n_orient[i] for i in g)):
            N.check(N.DS_ERR_INVALID_ARGUMENT, "simulate_batch")
        self.scratch = [torch.empty(max(int(b), 16), dtype=torch.uint8, device=self.device) for b in self.scratch_bytes]
        if capacity is None:
            capacity = [max(1024, sum(self.n_orient[i] * estimate_spots(self.tables[i], self.settings, self.radius)
                                      for i in g) * 5 // 4) for g in self.groups]
        self.capacity = [int(c) for c in capacity]
        self.idx = [torch.empty(c, dtype=torch.int32, device=self.device) for c in self.capacity]
        self.xyzi = [torch.empty((c, 4), dtype=torch.float32, device=self.device) for c in self.capacity]
        self.graph = None

    def _launch(self, stream=None, orient_tile=None):
        lib = N.load_library()
        st = N.stream_handle(stream)
        p = self.cparams(orient_tile)
        self.status.zero_()
        for gi, it in enumerate(self._items):
            out = N.ds_spots(self.offsets[gi].data_ptr(), self.idx[gi].data_ptr(), self.xyzi[gi].data_ptr(),
                             self.capacity[gi], self.totals[gi:gi + 1].data_ptr(), None)
            N.check(lib.ds_simulate_batch(p, it, len(it), out, N.ptr(self.scratch[gi]), self.scratch[gi].numel(),
                                          N.ptr(self.status[gi:gi + 1]), st), "simulate_batch")

    def run(self, stream=None, sync=True):
        """Launch (or replay the captured graph); with ``sync`` check the status
        words and, on output overflow, grow the outputs and run again."""
        for attempt in range(2):
            if self.graph is not None:
                self.graph.replay()
            else:
                self._launch(stream)
            if not sync:
                return self
            st = [int(v) for v in self.status.cpu().numpy()]
            for t in self.tables:
                N.check_device_status(t._status, "structure_factors")
            for v in st:
                N.check_status_value(v, "simulate_batch", allow=N.DS_ERR_CAPACITY)
            if not any(v & N.DS_ERR_CAPACITY for v in st):
                return self
            totals = self.totals.cpu().numpy()
            self._plan([int(t) + 1024 for t in totals])  # drops the graph: outputs moved
        raise N.NativeError("simulate_batch: output capacity still exceeded after resizing")

    def capture(self, warmup=True):
        """Record the launch sequence in a CUDA graph (after a checked run that
        sizes the outputs)."""
        if warmup:
            self.run()
        s = torch.cuda.Stream(device=self.device)
        s.wait_stream(torch.cuda.current_stream(self.device))
        g = torch.cuda.CUDAGraph()
        with torch.cuda.stream(s):
            with torch.cuda.graph(g, stream=s, capture_error_mode="relaxed"):
                self._launch(stream=s)
        torch.cuda.current_stream(self.device).wait_stream(s)
        self.graph = g
        return self

    def replay(self):
        self.graph.replay()
        return self

    def spots(self):
        """One ``PhaseSpots`` per phase (views into the batch outputs)."""
        out = []
        for gi, g in enumerate(self.groups):
            off = self.offsets[gi]
            bounds = np.cumsum([0] + [self.n_orient[i] for i in g])
            starts = off[torch.as_tensor(bounds, device=self.device)].cpu().numpy()
            for k, i in enumerate(g):
                a, b = int(starts[k]), int(starts[k + 1])
                o = off[bounds[k]:bounds[k + 1] + 1] - a
                out.append(PhaseSpots(self.tables[i], o, self.idx[gi][a:b], self.xyzi[gi][a:b], b - a))
        return out


class Autotuner:
    """Picks the tile shape of a batched launch by timing the feasible
    candidates on the batch itself (CUDA events, best of a few launches):
    orientations per tile (the largest any phase may use; bigger tables get
    smaller tiles so their bitmap fits shared memory), the per-CTA candidate
    staging (screened reflections held per tile before the ordered writes),
    then, at the best of those, the reflections per work unit of the refine
    and write passes (each orientation's candidate bitmap cut into 1, 2, 4 or
    8 word ranges that the CTA's warps take from a shared counter).
    Remembers the choice per problem class (phases, orientations and table
    sizes in powers of two, shape model, precession, form); with a ``path``
    (or the environment variable ``DS_AUTOTUNE_CACHE``) the choices also
    persist in a JSON file keyed by GPU name, so a later process on the same
    kind of GPU skips the timing runs."""

    TILES = (4, 8, 16, 32)
    STAGE_PER_ORIENT = (384, 1536, 4096)  # staging capacity = tile x this
    PARTS = (1, 2, 4, 8)                  # word ranges per orientation (refine / write units)
    CANDIDATES = TILES

    def __init__(self, repeats=3, path=None):
        self.repeats = repeats
        self.cache = {}
        self.timings = {}
        self.path = path

    @staticmethod
    def _key_str(k) -> str:
        return "|".join(str(v) for v in k)

    def _load(self) -> dict:
        try:
            with open(self.path) as f:
                data = json.load(f)
            return data if isinstance(data, dict) else {}
        except (OSError, ValueError):
            return {}

    def lookup(self, device_name: str, k):
        """A stored (orient_tile, stage_cap, refine_parts) for this GPU and
        problem class, or None (entries without the parts read as 0: the
        library's choice)."""
        if not self.path:
            return None
        v = self._load().get(device_name, {}).get(self._key_str(k))
        if not isinstance(v, list) or len(v) not in (2, 3):
            return None
        return (int(v[0]), int(v[1]), int(v[2]) if len(v) == 3 else 0)

    def store(self, device_name: str, k, choice):
        """Add one choice to the file (read, update, write a temporary file, rename)."""
        if not self.path:
            return
        data = self._load()
        data.setdefault(device_name, {})[self._key_str(k)] = [int(v) for v in choice]
        tmp = f"{self.path}.{os.getpid()}.tmp"
        with open(tmp, "w") as f:
            json.dump(data, f, indent=1, sort_keys=True)
        os.replace(tmp, self.path)

    @staticmethod
    def key(batch: "PhaseBatch"):
        lg = lambda v: int(np.ceil(np.log2(max(int(v), 1))))
        s = batch.settings
        return (len(batch.tables), lg(sum(batch.n_orient)), lg(max(t.n for t in batch.tables)),
                s.shape_model, int(s.precession_mode), s.form)

    def tune(self, batch: "PhaseBatch"):
        """(orient_tile, stage_cap, refine_parts) for this batch (cached per class)."""
        k = self.key(batch)
        if k in self.cache:
            return self.cache[k]
        device_name = torch.cuda.get_device_name(batch.device) if self.path else None
        stored = self.lookup(device_name, k) if self.path else None
        if stored is not None:
            self.cache[k] = stored
            return stored
        lib = N.load_library()
        fp64 = batch.settings.form == "fp64"
        integ = batch.settings.precession_mode == N.DS_PRECESSION_INTEGRAL
        tiles = [c for c in self.TILES if c <= (8 if fp64 else 16 if integ else 32)]
        best, best_ms, times = None, None, {}

        def trial(c, sc, parts):
            batch.orient_tile, batch.stage_cap, batch.refine_parts = c, sc, parts
            p = batch.cparams()
            if any(lib.ds_simulate_batch_scratch_bytes(p, it, len(it)) == 0 for it in batch._items):
                return None  # infeasible (tile does not fit shared memory)
            try:
                batch._plan()
                batch.run()  # sizes the outputs, checks the status
            except (ValueError, N.NativeError):
                return None
            ms = []
            for _ in range(self.repeats):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                batch._launch()
                e1.record()
                e1.synchronize()
                ms.append(e0.elapsed_time(e1))
            return min(ms)

        for c in tiles:
            for sc in (c * spo for spo in self.STAGE_PER_ORIENT):
                t = trial(c, sc, 0)
                if t is None:
                    continue
                times[f"tile{c}_stage{sc}"] = t
                if best_ms is None or t < best_ms:
                    best, best_ms = (c, sc, 0), t
        if best is not None:
            c, sc, _ = best
            default_parts = 2 if c >= 2 else 8
            for parts in self.PARTS:
                if parts == default_parts:
                    continue
                t = trial(c, sc, parts)
                if t is None:
                    continue
                times[f"tile{c}_stage{sc}_parts{parts}"] = t
                if t < best_ms:
                    best, best_ms = (c, sc, parts), t
        if best is None:
            best = (4, 0, 0)
        self.cache[k] = best
        self.timings[k] = times
        if self.path and times:
            self.store(device_name, k, best)
        return best

    def tile_for(self, batch: "PhaseBatch") -> int:
        tile, stage, parts = self.tune(batch)
        batch.stage_cap = stage
        batch.refine_parts = parts
        return tile


AUTOTUNER = Autotuner(path=os.environ.get("DS_AUTOTUNE_CACHE") or None)


def simulate_batch(tables, quats, settings: SimSettings, radius: float, orient_tile=None):
    """Spots of many phases (one quaternion set each) from batched launches;
    returns one ``PhaseSpots`` per phase."""
    return PhaseBatch(tables, quats, settings, radius, orient_tile=orient_tile).run().spots()


def polar_flatten(spots_list, radial_axes=None, azimuthal_axes=None, precision="fp64"):
    """Padded (r, theta, intensity) templates of every pattern of the given
    phases in order (``ds_polar_flatten``): three float64 device tensors of
    shape (patterns, max spots per pattern); with both axes, r and theta
    hold closest-axis indices and out-of-range spots are dropped.
    ``precision`` 'fp64' (default) computes r and theta in FP64 from the
    float32 positions, as the reference does; 'fp32' in FP32 with float
    axes (``ds_polar_flatten_f32``: ~2e-7 relative, bound by HBM instead of
    the FP64 pipe)."""
    lib = N.load_library()
    if not spots_list:
        raise ValueError("no patterns")
    if precision not in ("fp64", "fp32"):
        raise ValueError("precision must be 'fp64' or 'fp32'")
    f32 = precision == "fp32"
    axis_np, axis_t = (np.float32, torch.float32) if f32 else (np.float64, torch.float64)
    entry = lib.ds_polar_flatten_f32 if f32 else lib.ds_polar_flatten
    dev = spots_list[0].offsets.device
    counts = [int(s.n_orient) for s in spots_list]
    maxes = [int((s.offsets[1:] - s.offsets[:-1]).max().item()) if s.n_orient else 0 for s in spots_list]
    n, m = sum(counts), max(maxes)
    # the kernel writes every slot of every pattern (zero padding included)
    r = torch.empty((n, m), dtype=torch.float64, device=dev)
    t = torch.empty((n, m), dtype=torch.float64, device=dev)
    i = torch.empty((n, m), dtype=torch.float64, device=dev)
    binned = radial_axes is not None and azimuthal_axes is not None
    rax = torch.as_tensor(np.asarray(radial_axes, dtype=axis_np)).to(dev, axis_t) if binned else None
    aax = torch.as_tensor(np.asarray(azimuthal_axes, dtype=axis_np)).to(dev, axis_t) if binned else None
    row = 0
    for s, c in zip(spots_list, counts):
        if c and m:
            xyzi = s.xyzi if s.total else torch.zeros((1, 4), dtype=torch.float32, device=dev)
            N.check(entry(N.ptr(s.offsets), N.ptr(xyzi), c, m, N.ptr(rax),
                                         0 if rax is None else rax.numel(), N.ptr(aax),
                                         0 if aax is None else aax.numel(), N.ptr(r[row:]), N.ptr(t[row:]),
                                         N.ptr(i[row:]), N.stream_handle()), "polar_flatten")
        row += c
    return r, t, i
