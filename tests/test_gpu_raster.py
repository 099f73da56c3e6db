"""GPU parity of the detector rasteriser (ds_rasterize) against the oracle.

The oracle is the reference's own recipe (diffsims/simulations/simulation2d.py:357-442,
diffsims/pattern/detector_functions.py:251-359): truncation to whole pixels,
last write wins, ``scipy.ndimage.gaussian_filter``; or boxed sub-pixel
Gaussians.  Both are fed the GPU's own float32 spot positions, so pixel
positions must agree exactly; values agree to float32 rounding (1e-6 of the
image maximum).
"""
import os
import types
import warnings

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


def _vectors(patterns):
    return [types.SimpleNamespace(data=np.asarray(x, dtype=np.float64).reshape(-1, 3),
                                  intensity=np.asarray(i, dtype=np.float64), hkl=None) for x, i in patterns]


def _spots_of(patterns):
    from diffsims_gb300.engine import PhaseSpots
    return PhaseSpots.from_vectors(_vectors(patterns))


def _raster(spots, **kw):
    from diffsims_gb300.engine import RasterSettings, rasterize
    return rasterize(spots, RasterSettings(**kw)).cpu().numpy().astype(np.float64)


def _oracle(spots, **kw):
    off, _, xyzi = spots.host()
    kw = dict(kw)
    kw.pop("pixel_snap", None)
    kw.pop("truncate", None)
    out = []
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        for i in range(len(off) - 1):
            rec = xyzi[off[i]:off[i + 1]].astype(np.float64)
            out.append(ok.diffraction_pattern(rec[:, :3], rec[:, 3], **kw))
    return np.array(out)


def _assert_images(got, want, rel=2e-6):
    assert got.shape == want.shape
    for g, w in zip(got, want):
        scale = np.nanmax(np.abs(w)) if np.isfinite(w).any() else 1.0
        np.testing.assert_array_equal(np.isnan(g), np.isnan(w))
        np.testing.assert_allclose(np.nan_to_num(g), np.nan_to_num(w), rtol=0, atol=rel * max(scale, 1e-300))


def _sim_spots(n=48, seed=4):
    crystal = ok.Crystal((7.3, 8.1, 6.6, 88.0, 95.0, 101.0), ["Si", "O", "O", "Fe"],
                         [[0.1, 0.2, 0.3], [0.4, 0.1, 0.7], [0.8, 0.6, 0.2], [0.3, 0.9, 0.5]], B=[0.5] * 4)
    q = ok.random_quaternions(n, seed=seed)
    p = ok.SimParams(accelerating_voltage=200, shape_factor_model="linear", reciprocal_radius=1.2,
                     max_excitation_error=0.01, precession_angle=0.5)
    spots, _ = pu.gpu_run(crystal, q, p, "mixed", with_s=False)
    return spots


def test_library_shape_matches_oracle():
    """256 x 256 detector, sigma 1 px, r = 1.2 filling the frame: the
    template-library workload's raster settings."""
    spots = _sim_spots()
    kw = dict(shape=(256, 256), sigma=1.0, calibration=1.2 / 128)
    _assert_images(_raster(spots, **kw), _oracle(spots, **kw))


@pytest.mark.parametrize("kw", [
    dict(shape=(256, 256), sigma=1.0, calibration=1.2 / 128, normalize=False),
    dict(shape=(128, 160), sigma=2.0, calibration=0.012, in_plane_angle=33.0, mirrored=True),
    dict(shape=(37, 45), sigma=1.5, calibration=0.04),                     # width not a multiple of 4
    dict(shape=(6, 7), sigma=2.5, calibration=0.25, normalize=False),      # filter wider than the image
    dict(shape=(300, 520), sigma=3.0, calibration=0.006, direct_beam_position=(100.3, 120.7)),  # two row segments
    dict(shape=(64, 64), sigma=0.0, calibration=0.03, normalize=False),   # no filter
    dict(shape=(96, 96), sigma=1.2, calibration=0.02, fast=False, clip_threshold=0.01),
    dict(shape=(96, 100), sigma=3.0, calibration=0.02, fast=False, clip_threshold=1e-4, normalize=False,
         in_plane_angle=-71.0),
])
def test_variants_match_oracle(kw):
    spots = _sim_spots(24, seed=9)
    _assert_images(_raster(spots, **kw), _oracle(spots, **kw))


def test_last_write_wins_and_edges():
    # two spots on one pixel (the later one counts), one outside the frame,
    # one on each border row / column (reflect mode at the edges)
    pats = [([[0.0, 0.0, 0], [0.0004, 0.0003, 0], [0.5, 0, 0], [-0.05, 0, 0], [0.049, 0.049, 0]],
             [3.0, 7.0, 1.0, 2.0, 4.0]),
            ([[0.2, 0.2, 0]], [1.0]),           # out of frame: zeros, no normalisation
            ([[0.01, 0.0, 0]], [0.0]),          # in frame, zero intensity: 0 / 0
            ([], [])]
    spots = _spots_of(pats)
    for kw in (dict(shape=(11, 11), sigma=1.0, calibration=0.01),
               dict(shape=(11, 11), sigma=1.0, calibration=0.01, normalize=False)):
        got, want = _raster(spots, **kw), _oracle(spots, **kw)
        _assert_images(got, want)
    got = _raster(spots, shape=(11, 11), sigma=1.0, calibration=0.01)
    assert np.all(got[1] == 0) and np.all(np.isnan(got[2])) and np.all(got[3] == 0)


def test_reference_fast_vs_slow_kat():
    # diffsims/tests/simulations/test_simulations2d.py:133-181: one spot of
    # intensity 30 at the centre, calibration 1, clip 0.01, unnormalised
    spots = _spots_of([([[0.0, 0.0, 0.0]], [30.0])])
    kw = dict(shape=(11, 11), sigma=1, calibration=1, normalize=False, clip_threshold=0.01)
    fast = _raster(spots, fast=True, **kw)[0]
    slow = _raster(spots, fast=False, **kw)[0]
    _assert_images(fast[None], _oracle(spots, fast=True, **kw))
    _assert_images(slow[None], _oracle(spots, fast=False, **kw))
    assert np.all((slow - fast) < kw["clip_threshold"])
    kw["shape"] = (10, 10)
    assert not np.allclose(_raster(spots, fast=True, **kw)[0], _raster(spots, fast=False, **kw)[0])


def test_fast_mode_amplitude_cases():
    """The slice rasteriser's normalisation paths against the oracle: a
    dominant spot (the maximum pass builds only the slices that can hold the
    maximum), negative amplitudes (every slice built and read back), a NaN
    amplitude (numpy's max is NaN: a NaN image), equal amplitudes on an odd
    width, and spots on every border row and column."""
    rng = np.random.default_rng(17)
    pats = []
    xy = rng.uniform(-0.6, 0.6, size=(60, 2))
    amp = rng.uniform(0.01, 1.0, 60)
    amp[7] = 500.0
    pats.append((np.c_[xy, np.zeros(60)], amp))                       # dominant spot
    amp2 = amp.copy()
    amp2[::3] *= -1
    pats.append((np.c_[xy, np.zeros(60)], amp2))                      # negative amplitudes
    amp3 = amp.copy()
    amp3[11] = np.nan
    pats.append((np.c_[xy, np.zeros(60)], amp3))                      # a NaN amplitude
    pats.append((np.c_[xy, np.zeros(60)], np.ones(60)))               # equal amplitudes
    edge = np.array([[-0.64, -0.64, 0], [0.63, 0.63, 0], [-0.64, 0.2, 0], [0.1, 0.63, 0], [0.0, -0.64, 0]])
    pats.append((edge, np.array([1.0, 2.0, 3.0, 4.0, 5.0])))           # border rows and columns
    spots = _spots_of(pats)
    for kw in (dict(shape=(128, 128), sigma=1.0, calibration=0.01),
               dict(shape=(97, 131), sigma=1.3, calibration=0.01),
               dict(shape=(128, 128), sigma=2.0, calibration=0.01, normalize=False)):
        got, want = _raster(spots, **kw), _oracle(spots, **kw)
        _assert_images(got, want)
    got = _raster(spots, shape=(128, 128), sigma=1.0, calibration=0.01)
    assert np.all(np.isnan(got[2])) and got[0].max() == 1.0


def test_many_spots_use_global_arena():
    """A pattern whose per-pattern arena exceeds shared memory (5000 spots)
    runs from the global scratch arena: same images."""
    rng = np.random.default_rng(5)
    pats = []
    for n in (5000, 37, 4100):
        xy = rng.uniform(-0.6, 0.6, size=(n, 2))
        pats.append((np.c_[xy, np.zeros(n)], rng.uniform(0.01, 2.0, n)))
    spots = _spots_of(pats)
    from diffsims_gb300 import _native as N
    from diffsims_gb300.engine import RasterSettings
    lib = N.load_library()
    assert lib.ds_rasterize_scratch_bytes(RasterSettings((128, 128)).cstruct(), 5000) > 0
    for kw in (dict(shape=(128, 128), sigma=1.0, calibration=0.01),
               dict(shape=(128, 128), sigma=1.0, calibration=0.01, fast=False, clip_threshold=0.05)):
        _assert_images(_raster(spots, **kw), _oracle(spots, **kw))


def test_graphite_golden_through_gpu_raster(golden_dir):
    """The reference's golden image (diffsims/tests/generators/test_simulation_generator.py:320-345)
    from the GPU's spots and the GPU rasteriser.  Sixteen of its spots sit
    exactly on pixel boundaries in the reference's arithmetic; float32 spot
    positions put them within 1e-5 px of it, and pixel_snap puts them back."""
    import diffsims_gb300 as ds
    q = ok.euler_to_quaternion([0, 90, 90], degrees=True)
    p = ok.SimParams(accelerating_voltage=200, reciprocal_radius=1.6768, max_excitation_error=0.1,
                     with_direct_beam=False)
    from tests.test_gpu_parity import graphite
    spots, _ = pu.gpu_run(graphite(), q, p, "mixed", with_s=False)
    from diffsims_gb300.engine import RasterSettings, rasterize
    img = rasterize(spots, RasterSettings((128, 128), sigma=1.4, calibration=0.0262, pixel_snap=1e-4))
    old = np.load(os.path.join(golden_dir, "graphite_pattern_128.npy"))
    np.testing.assert_allclose(img[0].cpu().numpy().astype(np.float64), old, atol=2e-6)
    # the public per-pattern call gives the same image
    gen = pu.generator_for(p)
    sim = gen.calculate_diffraction2d(pu.to_phase(graphite()), ds.Rotation(q), reciprocal_radius=1.6768,
                                      max_excitation_error=0.1, with_direct_beam=False)
    one = sim.get_diffraction_pattern((128, 128), sigma=1.4, calibration=0.0262)
    assert one.shape == (128, 128) and one.dtype == np.float64 and one.max() == 1.0


def test_batched_chunks_and_api():
    """get_diffraction_patterns in chunks through one preallocated buffer equals
    one call over all patterns, and each equals get_diffraction_pattern."""
    import torch
    import diffsims_gb300 as ds
    crystal = ok.Crystal((4.05,) * 3 + (90, 90, 90), ["Al"] * 4,
                         [[0, 0, 0], [0, .5, .5], [.5, 0, .5], [.5, .5, 0]], B=[0.5] * 4)
    q = ok.random_quaternions(40, seed=1)
    gen = ds.SimulationGenerator(200, shape_factor_model="linear", precession_angle=0.5)
    sim = gen.calculate_diffraction2d(pu.to_phase(crystal), ds.Rotation(q), reciprocal_radius=1.2,
                                      debye_waller_factors={"Al": 0.5})
    kw = dict(shape=(256, 256), sigma=1.0, calibration=1.2 / 128)
    full = sim.get_diffraction_patterns(**kw)
    buf = torch.empty((16, 256, 256), dtype=torch.float32, device=full.device)
    for a in range(0, 40, 16):
        b = min(a + 16, 40)
        part = sim.get_diffraction_patterns(**kw, start=a, stop=b, out=buf[:b - a])
        assert torch.equal(part, full[a:b])
    for i in (0, 17, 39):
        sim.rotation_index = i
        np.testing.assert_array_equal(sim.get_diffraction_pattern(**kw), full[i].cpu().numpy().astype(np.float64))


def test_user_built_simulation2d():
    """Simulation2D built from DiffractingVector objects, as the reference's
    tests do (diffsims/tests/simulations/test_simulations2d.py:27-49)."""
    import diffsims_gb300 as ds
    al = pu.to_phase(ok.Crystal((4.05,) * 3 + (90, 90, 90), ["Al"], [[0, 0, 0]]))
    v = ds.DiffractingVector(al, [[1, 0, 0], [2, 0, 0], [3, 3, 0], [-4, 0, 0]], intensity=[1, 2, 3, 4])
    sim = ds.Simulation2D(al, v, ds.Rotation.identity(), ds.SimulationGenerator(200))
    assert np.array_equal(sim.coordinates.data, v.data)
    img = sim.get_diffraction_pattern((64, 64), sigma=1, calibration=0.2)
    want = ok.diffraction_pattern(v.data, v.intensity, (64, 64), sigma=1, calibration=0.2)
    _assert_images(img[None], want[None])
    with pytest.raises(ValueError):
        ds.Simulation2D(al, [v, v], ds.Rotation.identity(), ds.SimulationGenerator(200))
