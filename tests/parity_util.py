"""Shared helpers of the GPU parity tests: run the CUDA path on an oracle
``Crystal`` and compare its CSR spots with the FP64 oracle, counting
selection flips at the cutoff instead of hiding them."""
import warnings

import numpy as np

from oracle import compare as oc
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


def compare(spots, crystal, quats, p: ok.SimParams, rtol=1e-5, flip_window=1e-9, ref=None):
    """Statistics of the GPU spots against the oracle (``oracle.compare.spot_errors``);
    raises on any difference not explained by a cutoff flip within
    ``flip_window`` or by FP64 round-off of a systematic absence, on
    intensities beyond ``rtol`` relative and on positions beyond 1e-5 |g|."""
    if ref is None:
        with warnings.catch_warnings():
            warnings.simplefilter("ignore")
            ref = ok.simulate(crystal, quats, p, return_s=True)
    s_gpu = spots.excitation_error.cpu().numpy() if spots.excitation_error is not None else None
    stats = oc.spot_errors(spots.offsets.cpu().numpy(), spots.hkl_index.cpu().numpy(),
                           spots.xyzi.cpu().numpy(), s_gpu, crystal, quats, p, ref, flip_window)
    assert not stats["unexplained"], f"spots differ beyond the cutoff window: {stats}"
    assert stats["ordered"], "spots not in table order"
    assert stats["max_rel_I"] <= rtol, stats
    assert stats["max_abs_pos"] <= 1e-5, stats
    return stats
