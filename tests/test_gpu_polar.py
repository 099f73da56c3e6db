"""Polar templates on the GPU (ds_polar_flatten) against the oracle's
restatement of Simulation2D.polar_flatten_simulations and the reference's own
shape / padding checks."""
import numpy as np
import pytest

from oracle import kinematic as ok
from tests import parity_util as pu

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import __graft_entry__
    __graft_entry__.build()
    torch.cuda.set_device(0)


def _single():
    import diffsims_gb300 as ds
    al = pu.to_phase(ok.Crystal((0.405,) * 3 + (90, 90, 90), ["Al"], [[0, 0, 0]]))
    v = ds.DiffractingVector(al, [[1, 0, 0], [2, 0, 0], [3, 3, 0], [-4, 0, 0], [-5, 0, 0], [-6, 0, 0], [-7, 0, 0],
                                  [-8, 0, 0]], intensity=[1, 2, 3, 4, 5, 6, 7, 8])
    return ds.Simulation2D(al, v, ds.Rotation.identity(), ds.SimulationGenerator(200)), v


def test_reference_polar_kats():
    # diffsims/tests/simulations/test_simulations2d.py:101-127
    sim, v = _single()
    r, t, i = sim.polar_flatten_simulations()
    assert r.shape == t.shape == i.shape == (1, 8)
    want = ok.polar_flatten([(v.data, v.intensity)])
    for a, b in zip((r, t, i), want):
        np.testing.assert_allclose(a, b, rtol=1e-15, atol=0)
    ra, ta = np.linspace(0, 7, 5), np.linspace(0, 2 * np.pi, 10)
    r, t, i = sim.polar_flatten_simulations(radial_axes=ra, azimuthal_axes=ta)
    assert r.shape == t.shape == i.shape == (1, 8) and r.dtype.kind == "i"
    np.testing.assert_array_equal(r[:, 6:], 0)
    np.testing.assert_array_equal(t[:, 6:], 0)
    np.testing.assert_array_equal(i[:, 6:], 0)
    for a, b in zip((r, t, i), ok.polar_flatten([(v.data, v.intensity)], ra, ta)):
        np.testing.assert_array_equal(a, b)


def test_polar_templates_of_simulated_phases():
    import diffsims_gb300 as ds
    from tests.test_gpu_batch import random_cell
    crystals = [random_cell(41, 6, edges=(4, 6)), random_cell(42, 20, edges=(7, 9))]
    rots = [ds.Rotation(ok.random_quaternions(30, seed=7)), ds.Rotation(ok.random_quaternions(11, seed=8))]
    gen = ds.SimulationGenerator(200, shape_factor_model="sinc")
    sim = gen.calculate_diffraction2d([pu.to_phase(c) for c in crystals], rots, reciprocal_radius=1.2)
    pats = [(v.data, v.intensity) for v in sim]
    r, t, i = sim.polar_flatten_simulations()
    want = ok.polar_flatten(pats)
    assert r.shape == want[0].shape
    np.testing.assert_allclose(r, want[0], rtol=1e-15, atol=0)
    np.testing.assert_allclose(t, want[1], rtol=0, atol=4e-16 * np.pi)  # atan2: last-place differences
    np.testing.assert_array_equal(i, want[2])
    ra, ta = np.linspace(0, 1.2, 64), np.linspace(-np.pi, np.pi, 181)
    r, t, i = sim.polar_flatten_simulations(radial_axes=ra, azimuthal_axes=ta)
    wr, wt, wi = ok.polar_flatten(pats, ra, ta)
    np.testing.assert_array_equal(r, wr)
    np.testing.assert_array_equal(t, wt)
    np.testing.assert_array_equal(i, wi)
