"""GPU path of ``SimulationGenerator.calculate_diffraction1d`` (enumeration
and FP64 structure factors on the GPU, symmetry families on the host)
against the oracle: identical families in the same order, |g| to 1e-13,
intensities (0-100 scale) to 1e-9."""
import numpy as np
import pytest

from oracle import kinematic as ok
from tests.test_oracle_diffraction1d import _phase_of, crystals, rotations

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", list(crystals()))
def test_diffraction1d_matches_oracle(name):
    import diffsims_gb300 as ds
    phase, cr = _phase_of(name)
    dw = {e: b for e, b in zip(cr.elements, cr.B)}
    sim = ds.SimulationGenerator(300).calculate_diffraction1d(phase, 0.5, debye_waller_factors=dw)
    g, inten, idx = ok.diffraction1d(cr, rotations(crystals()[name][0]))
    np.testing.assert_array_equal(sim.hkl, idx)
    np.testing.assert_allclose(sim.reciprocal_spacing, g, rtol=1e-13)
    np.testing.assert_allclose(sim.intensities, inten, rtol=1e-9, atol=1e-9)
    assert isinstance(sim.reciprocal_spacing, np.ndarray) and len(sim.hkl) == len(sim.intensities)
