"""Shared helpers of the GPU parity tests: run the CUDA path on an oracle
``Crystal`` and compare its CSR spots with the FP64 oracle, counting
selection flips at the cutoff instead of hiding them."""
import warnings

import numpy as np

from oracle import kinematic as ok


def to_phase(crystal: ok.Crystal):
    import diffsims_gb300 as ds
    atoms = [ds.Atom(e, x, o) for e, x, o in zip(crystal.elements, crystal.xyz, crystal.occupancy)]
    return ds.Phase("test", ds.Structure(atoms, ds.Lattice(*crystal.lattice)))


def generator_for(p: ok.SimParams):
    import diffsims_gb300 as ds
    return ds.SimulationGenerator(p.accelerating_voltage, p.scattering_params, p.precession_angle,
                                  p.shape_factor_model, p.approximate_precession, p.minimum_intensity,
                                  **p.shape_kwargs)


def gpu_run(crystal, quats, p: ok.SimParams, form="mixed", orient_tile=0, with_s=True):
    import torch
    from diffsims_gb300.engine import PhaseTable, SpotBuffers, simulate_phase
    dev = torch.device("cuda", 0)
    gen = generator_for(p)
    table = PhaseTable(to_phase(crystal), p.reciprocal_radius, p.with_direct_beam, p.scattering_params,
                       list(crystal.B), form=form, device=dev)
    settings = gen.settings(p.max_excitation_error, p.shape_factor_width, form, orient_tile)
    q = torch.as_tensor(np.asarray(quats, dtype=np.float64)).to(dev)
    spots = simulate_phase(table, q, settings, p.reciprocal_radius, SpotBuffers(dev, with_s))
    return spots, table


def _boundary_distance(p, k0, s, z, r):
    """Distance of one (orientation, row) pair from the selection boundary,
    in the same units as the excitation error."""
    eps = p.max_excitation_error
    phi = np.deg2rad(abs(p.precession_angle))
    if phi == 0:
        return abs(abs(s) - eps)
    Pz, Pt = k0 * np.cos(phi), k0 * np.sin(phi)
    with np.errstate(invalid="ignore"):
        zup = Pz - np.sqrt(k0 ** 2 - (r + Pt) ** 2)
        zdo = Pz - np.sqrt(k0 ** 2 - (r - Pt) ** 2)
    return min(abs(zup - (z - eps)), abs((z + eps) - zdo))


def compare(spots, crystal, quats, p: ok.SimParams, rtol=1e-5, flip_window=1e-9, ref=None):
    """Statistics of the GPU spots against the oracle; raises on any
    difference not explained by a cutoff flip within ``flip_window``."""
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        ref = ref if ref is not None else ok.simulate(crystal, quats, p, return_s=True)
    table = ok.phase_table(crystal, p)
    Rs = ok.quaternion_to_matrix(quats)
    k0 = 1 / ok.electron_wavelength(p.accelerating_voltage)
    off = spots.offsets.cpu().numpy()
    idx = spots.hkl_index.cpu().numpy().astype(np.int64)
    xyzi = spots.xyzi.cpu().numpy().astype(np.float64)
    s_gpu = spots.excitation_error.cpu().numpy() if spots.excitation_error is not None else None
    g = table[2]
    stats = dict(patterns=len(ref), spots=int(off[-1]), boundary_flips=0, noise_spots=0, max_rel_I=0.0,
                 max_abs_pos=0.0, max_abs_s=0.0, max_flip_distance=0.0)
    # the largest |F|^2 the structure can have: (sum_j occ_j f_j(0))^2
    f2_scale = float(ok.kinematical_intensities([[0, 0, 0]], [0.0], crystal.elements, crystal.xyz,
                                                crystal.occupancy, np.zeros(len(crystal.elements)),
                                                p.scattering_params)[0]) or 1.0
    assert off.shape[0] == len(ref) + 1 and off[0] == 0 and np.all(np.diff(off) >= 0)
    for i, r in enumerate(ref):
        a, b = off[i], off[i + 1]
        gi = idx[a:b]
        assert np.all(np.diff(gi) > 0), f"orientation {i}: spots not in table order"
        common, ia, ib = np.intersect1d(gi, r.index, return_indices=True)
        for j in np.setxor1d(gi, r.index):
            if j in r.index:
                # a spot the reference keeps only through FP64 round-off: a
                # systematic absence (|F|^2 ~ 1e-32 of the strongest possible)
                # kept because every spot of this pattern is one, so the
                # 1e-20 * max mask compares noise with noise.  The CUDA path
                # computes those |F|^2 as exact zeros and drops them.
                I_ref = r.intensity[np.searchsorted(r.index, j)]
                if I_ref <= 1e-24 * f2_scale:
                    stats["noise_spots"] += 1
                    continue
            rot, s_all = ok.excitation_errors(crystal, p, table, Rs[i])
            rr = np.hypot(rot[j, 0], rot[j, 1])
            dist = _boundary_distance(p, k0, s_all[j], rot[j, 2], rr)
            if dist < flip_window:
                stats["boundary_flips"] += 1
                stats["max_flip_distance"] = max(stats["max_flip_distance"], dist)
                continue
            raise AssertionError(f"orientation {i}: row {j} hkl {table[0][j]} differs (in gpu: {j in gi}), "
                                 f"boundary distance {dist:.3e}")
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
            if s_gpu is not None:
                stats["max_abs_s"] = max(stats["max_abs_s"], float(np.abs(s_gpu[a:b][ia] - r.excitation_error[ib]).max()))
    assert stats["max_rel_I"] <= rtol, stats
    assert stats["max_abs_pos"] <= 1e-5, stats
    return stats
