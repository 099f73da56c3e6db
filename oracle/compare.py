"""Spot-set comparison against the FP64 oracle -- TEST INFRASTRUCTURE.

The checker used by the GPU parity tests and by the error report of
``bench.py`` (outside its timed regions): the oracle's patterns
(``kinematic.simulate``, optionally computed by spawned worker processes)
against CSR spots given as host arrays.  Nothing here is imported by the
``diffsims_gb300`` package.

Differences are classified, never hidden:

* ``boundary_flips``: a row selected on one side only whose FP64 distance
  from the selection boundary is below ``flip_window`` (the excitation-error
  cutoff of generators/simulation_generator.py:363-375 decided on round-off);
* ``noise_spots``: rows whose |F|^2 is FP64 round-off of a systematic absence
  on the oracle's side (below 1e-24 of the largest possible |F|^2), which the
  reference's ``1e-20 * max`` mask (simulation_generator.py:237-240) keeps only
  when every spot of the pattern is such a row;
* ``unexplained``: anything else (the caller fails on it).
"""
from __future__ import annotations

import multiprocessing as mp
import os
import warnings

import numpy as np

from . import kinematic as ok


def _simulate_chunk(args):
    crystal, quats, p, return_s = args
    os.environ.setdefault("OMP_NUM_THREADS", "1")
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        return ok.simulate(crystal, quats, p, return_s=return_s)


def simulate_parallel(crystal, quats, p, return_s=True, workers=None, min_chunk=16):
    """``kinematic.simulate`` over contiguous orientation ranges in spawned
    worker processes (safe after CUDA initialisation in the caller); the
    patterns come back in orientation order."""
    quats = np.asarray(quats, dtype=np.float64).reshape(-1, 4)
    n = quats.shape[0]
    workers = int(workers or min(os.cpu_count() or 1, 32))
    workers = max(1, min(workers, n // min_chunk))
    if workers <= 1:
        return _simulate_chunk((crystal, quats, p, return_s))
    parts = np.array_split(quats, workers)
    with mp.get_context("spawn").Pool(workers) as pool:
        res = pool.map(_simulate_chunk, [(crystal, q, p, return_s) for q in parts])
    return [pat for chunk in res for pat in chunk]


def boundary_distance(p, k0, s, z, r):
    """FP64 distance of one (orientation, row) pair from the selection
    boundary, in 1/Angstrom (generators/simulation_generator.py:363-375)."""
    eps = p.max_excitation_error
    phi = np.deg2rad(abs(p.precession_angle))
    if phi == 0:
        return abs(abs(s) - eps)
    Pz, Pt = k0 * np.cos(phi), k0 * np.sin(phi)
    with np.errstate(invalid="ignore"):
        zup = Pz - np.sqrt(k0 ** 2 - (r + Pt) ** 2)
        zdo = Pz - np.sqrt(k0 ** 2 - (r - Pt) ** 2)
    return min(abs(zup - (z - eps)), abs((z + eps) - zdo))


def spot_errors(off, idx, xyzi, s_gpu, crystal, quats, p, ref, flip_window=1e-9, max_unexplained=20):
    """Statistics of CSR spots (host arrays: ``off`` (n+1), ``idx`` rows of the
    phase table, ``xyzi`` (x, y, z, I), ``s_gpu`` excitation errors or None)
    against the oracle's patterns ``ref``.

    Returns a dict: patterns, spots, boundary_flips, max_flip_distance,
    noise_spots, max_rel_I (relative intensity error over the spots both
    sides keep), max_abs_pos (position error / max(|g|, 1e-3)), max_abs_s,
    ordered (rows ascending in every pattern), unexplained (a list of
    (orientation, row, boundary distance) for the first differences that are
    neither flips nor noise)."""
    table = ok.phase_table(crystal, p)
    Rs = ok.quaternion_to_matrix(quats)
    k0 = 1 / ok.electron_wavelength(p.accelerating_voltage)
    off = np.asarray(off, dtype=np.int64)
    idx = np.asarray(idx, dtype=np.int64)
    xyzi = np.asarray(xyzi, dtype=np.float64)
    g = table[2]
    stats = dict(patterns=len(ref), spots=int(off[-1]), boundary_flips=0, noise_spots=0, max_rel_I=0.0,
                 max_abs_pos=0.0, max_abs_s=0.0, max_flip_distance=0.0, ordered=True, unexplained=[])
    # the largest |F|^2 the structure can have: (sum_j occ_j f_j(0))^2
    f2_scale = float(ok.kinematical_intensities([[0, 0, 0]], [0.0], crystal.elements, crystal.xyz,
                                                crystal.occupancy, np.zeros(len(crystal.elements)),
                                                p.scattering_params)[0]) or 1.0
    if off.shape[0] != len(ref) + 1 or off[0] != 0 or np.any(np.diff(off) < 0):
        stats["unexplained"].append((-1, -1, float("nan")))
        return stats
    for i, r in enumerate(ref):
        a, b = off[i], off[i + 1]
        gi = idx[a:b]
        if np.any(np.diff(gi) <= 0):
            stats["ordered"] = False
        common, ia, ib = np.intersect1d(gi, r.index, return_indices=True)
        diff = np.setxor1d(gi, r.index)
        if diff.size:
            rot, s_all = ok.excitation_errors(crystal, p, table, Rs[i])
        for j in diff:
            if j in r.index:
                I_ref = r.intensity[np.searchsorted(r.index, j)]
                if I_ref <= 1e-24 * f2_scale:
                    stats["noise_spots"] += 1
                    continue
            rr = np.hypot(rot[j, 0], rot[j, 1])
            dist = boundary_distance(p, k0, s_all[j], rot[j, 2], rr)
            if dist < flip_window:
                stats["boundary_flips"] += 1
                stats["max_flip_distance"] = max(stats["max_flip_distance"], float(dist))
                continue
            if len(stats["unexplained"]) < max_unexplained:
                stats["unexplained"].append((i, int(j), float(dist)))
        Ig, Ir = xyzi[a:b][ia, 3], r.intensity[ib]
        den = np.maximum(np.abs(Ir), 1e-300)
        rel = np.abs(Ig - Ir) / den
        rel = np.where((Ir == 0) & (Ig == 0), 0.0, rel)
        noise = (Ir <= 1e-24 * f2_scale) & (Ig <= 1e-24 * f2_scale)  # round-off on both sides
        stats["noise_spots"] += int(noise.sum())
        rel = np.where(noise, 0.0, rel)
        if rel.size:
            stats["max_rel_I"] = max(stats["max_rel_I"], float(rel.max()))
            pos = np.abs(xyzi[a:b][ia, :3] - r.xyz[ib]).max(axis=1) / np.maximum(g[common], 1e-3)
            stats["max_abs_pos"] = max(stats["max_abs_pos"], float(pos.max()))
            if s_gpu is not None and r.excitation_error is not None:
                ds = np.abs(np.asarray(s_gpu[a:b], dtype=np.float64)[ia] - r.excitation_error[ib])
                stats["max_abs_s"] = max(stats["max_abs_s"], float(ds.max()))
    return stats
