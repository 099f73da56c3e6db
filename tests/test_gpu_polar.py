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


def _near_boundary(v, axis, rel):
    """Whether v lies within rel (relative, floor 1e-12) of a closest-axis
    decision boundary: an entry (searchsorted) or a midpoint of two."""
    mids = 0.5 * (axis[1:] + axis[:-1])
    tol = rel * max(abs(v), 1.0) + 1e-12
    return np.min(np.abs(axis - v)) < tol or (mids.size and np.min(np.abs(mids - v)) < tol)


def test_polar_templates_fp32_mode():
    """ds_polar_flatten_f32: r within 3e-7 and theta within 3e-7 relative (+1e-12)
    of the FP64 restatement on the same float32 positions, intensities exact,
    the same padding; binned indices equal except in patterns with a spot
    whose FP64 value is within 1e-6 of a decision boundary."""
    import diffsims_gb300 as ds
    from tests.test_gpu_batch import random_cell
    crystals = [random_cell(43, 8, edges=(4, 7)), random_cell(44, 16, edges=(7, 10))]
    rots = [ds.Rotation(ok.random_quaternions(40, seed=9)), ds.Rotation(ok.random_quaternions(17, seed=10))]
    gen = ds.SimulationGenerator(200, shape_factor_model="lorentzian")
    sim = gen.calculate_diffraction2d([pu.to_phase(c) for c in crystals], rots, reciprocal_radius=1.3)
    pats = [(v.data, v.intensity) for v in sim]
    r, t, i = sim.polar_flatten_simulations(precision="fp32")
    wr, wt, wi = ok.polar_flatten(pats)
    assert r.shape == wr.shape and r.dtype == np.float64
    np.testing.assert_allclose(r, wr, rtol=3e-7, atol=1e-12)
    np.testing.assert_allclose(t, wt, rtol=3e-7, atol=1e-12)
    np.testing.assert_array_equal(i, wi)
    ra, ta = np.linspace(0, 1.3, 97), np.linspace(-np.pi, np.pi, 361)
    r, t, i = sim.polar_flatten_simulations(radial_axes=ra, azimuthal_axes=ta, precision="fp32")
    wr, wt, wi = ok.polar_flatten(pats, ra, ta)
    assert r.dtype.kind == "i" and r.shape == wr.shape
    diff = np.argwhere((r != wr) | (t != wt) | (i != wi))
    exact_r, exact_t, _ = ok.polar_flatten(pats)
    for p, k in diff:
        # a differing slot: some spot of that pattern sits on a boundary
        row_r, row_t = exact_r[p], exact_t[p]
        assert any(_near_boundary(v, ra, 1e-6) for v in row_r) or any(_near_boundary(v, ta, 1e-6) for v in row_t)
    with pytest.raises(ValueError):
        sim.polar_flatten_simulations(precision="fp16")


def test_polar_binned_nonuniform_axes():
    """Axes that are not evenly spaced (random sorted values with repeats and
    a geometric radial axis): the search from the uniform estimate falls back
    to bisection and the FP64 mode still equals the oracle exactly."""
    import diffsims_gb300 as ds
    from tests.test_gpu_batch import random_cell
    rng = np.random.default_rng(12)
    cr = random_cell(45, 10, edges=(5, 8))
    sim = ds.SimulationGenerator(200, shape_factor_model="linear").calculate_diffraction2d(
        pu.to_phase(cr), ds.Rotation(ok.random_quaternions(25, seed=13)), reciprocal_radius=1.1)
    pats = [(v.data, v.intensity) for v in sim]
    axes = [(np.geomspace(0.01, 1.1, 40), np.sort(rng.uniform(-np.pi, np.pi, 50))),
            (np.sort(np.concatenate([rng.uniform(0, 1.1, 30), [0.3] * 4])), np.linspace(-np.pi, np.pi, 7))]
    for ra, ta in axes:
        r, t, i = sim.polar_flatten_simulations(radial_axes=ra, azimuthal_axes=ta)
        wr, wt, wi = ok.polar_flatten(pats, ra, ta)
        np.testing.assert_array_equal(r, wr)
        np.testing.assert_array_equal(t, wt)
        np.testing.assert_array_equal(i, wi)
