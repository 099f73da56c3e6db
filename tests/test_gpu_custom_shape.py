"""Shape-factor functions of the caller's (diffsims/generators/simulation_generator.py:117-120,387-411):
the orientation kernel selects, the function runs on the host on each
pattern's excitation errors, ``ds_apply_shape_factors`` finishes the
intensities, the 1e-20 max mask and the ordered output.  Against the FP64
oracle, which calls the same function the reference's way; bars as in the
other parity tests (intensities 1e-5 relative, positions 1e-5 |g|, spot sets
equal except counted cutoff flips)."""
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


def gaussian_rod(excitation_error, maximum_excitation_error, scale=0.5):
    return np.exp(-(excitation_error / (scale * maximum_excitation_error)) ** 2)


def local_excite(excitation_error, maximum_excitation_error, t):
    # the reference's own test function (negative for negative s)
    return (np.sin(t) * excitation_error) / maximum_excitation_error


def _crystal():
    rng = np.random.default_rng(21)
    return ok.Crystal((7.3, 8.1, 6.6, 88.0, 95.0, 101.0), list(rng.choice(["Si", "O", "Fe"], 12)), rng.random((12, 3)),
                      B=rng.uniform(0.3, 1.2, 12))


@pytest.mark.parametrize("fn, kw, prec", [(gaussian_rod, {"scale": 0.5}, {}),
                                          (local_excite, {"t": 0.2}, {}),
                                          (gaussian_rod, {"scale": 0.7}, dict(precession_angle=0.5,
                                                                               approximate_precession=False)),
                                          (gaussian_rod, {"scale": 0.7}, dict(precession_angle=0.5))])
def test_custom_shape_function_matches_oracle(fn, kw, prec):
    import diffsims_gb300 as ds
    crystal = _crystal()
    q = ok.random_quaternions(48, seed=3)
    p = ok.SimParams(accelerating_voltage=200, shape_factor_model=fn, shape_kwargs=kw, reciprocal_radius=1.4,
                     max_excitation_error=0.02, **prec)
    gen = ds.SimulationGenerator(200, shape_factor_model=fn, **prec, **kw)
    sim = gen.calculate_diffraction2d(pu.to_phase(crystal), ds.Rotation(q), reciprocal_radius=1.4,
                                      max_excitation_error=0.02, debye_waller_factors=list(crystal.B))
    st = pu.compare(sim.spots(0), crystal, q, p, rtol=1e-5)
    print(fn.__name__, prec, {k: v for k, v in st.items() if k != "unexplained"})
    assert st["spots"] > 100


def test_custom_shape_function_in_the_legacy_generator():
    """DiffractionGenerator.calculate_ed_data with a function of the caller's:
    the same two-launch path, against the built-in model the function copies."""
    from diffsims_gb300.diffraction_generator import DiffractionGenerator
    from tests.test_gpu_legacy import structure_of

    def my_linear(excitation_error, maximum_excitation_error):
        return np.clip(1 - np.abs(excitation_error) / maximum_excitation_error, 0, None)

    eul = np.random.default_rng(4).uniform(-180, 180, (20, 3))
    a = DiffractionGenerator(200, shape_factor_model=my_linear).calculate_ed_data(structure_of("p1"), 1.5, eul)
    b = DiffractionGenerator(200, shape_factor_model="linear").calculate_ed_data(structure_of("p1"), 1.5, eul)
    for x, y in zip(a, b):
        assert np.array_equal(x._hkl, y._hkl)
        np.testing.assert_allclose(x._I, y._I, rtol=2e-5)
