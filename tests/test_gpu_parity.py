"""GPU parity: the CUDA path against the FP64 oracle on the same seeded inputs.

Bars: hkl sets and orders bit-exact; spot sets identical except counted
selection flips within 1e-9 1/Angstrom of the cutoff; intensities within
1e-5 relative (mixed form) / 1e-9 (FP64 form); positions within 1e-5 |g|.
"""
import os
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


def al_fcc(B=0.5):
    return ok.Crystal((4.05, 4.05, 4.05, 90, 90, 90), ["Al"] * 4,
                      [[0, 0, 0], [0, .5, .5], [.5, 0, .5], [.5, .5, 0]], B=[B] * 4)


def si_crystal(a=5.431):
    xyz = []
    for c in [[0, 0, 0], [0.5, 0, 0.5], [0, 0.5, 0.5], [0.5, 0.5, 0]]:
        xyz += [c, [c[0] + .25, c[1] + .25, c[2] + .25]]
    return ok.Crystal((a, a, a, 90, 90, 90), ["Si"] * 8, xyz)


def random_p1(n_atoms, seed, edges=(8, 15), angles=(70, 110), zs=("C", "N", "O", "Si", "Fe")):
    rng = np.random.default_rng(seed)
    lat = tuple(rng.uniform(*edges, 3)) + tuple(rng.uniform(*angles, 3))
    return ok.Crystal(lat, list(rng.choice(zs, n_atoms)), rng.random((n_atoms, 3)),
                      B=rng.uniform(0.3, 1.5, n_atoms))


def graphite():
    return ok.Crystal((2.464, 2.464, 6.711, 90, 90, 120), ["C"] * 4,
                      [[0, 0, .25], [0, 0, .75], [1 / 3, 2 / 3, .25], [2 / 3, 1 / 3, .75]])


# ------------------------------------------------------------------ A1/A2
@pytest.mark.parametrize("crystal, r", [
    (al_fcc(), 1.0), (al_fcc(), 1 / 0.7), (graphite(), 1.6768), (random_p1(4, 1), 2.0),
    (ok.Crystal((7.1, 9.3, 12.4, 90, 90, 90), ["O"], [[0, 0, 0]]), 1.5),
    (ok.Crystal((3.0, 20.0, 7.5, 85.0, 95.0, 100.0), ["O"], [[0, 0, 0]]), 1.5),
    (ok.Crystal((2.8665,) * 3 + (90, 90, 90), ["Fe"] * 2, [[0, 0, 0], [.5, .5, .5]]), 2.0),
])
@pytest.mark.parametrize("direct_beam", [True, False])
def test_enumeration_bit_exact(crystal, r, direct_beam):
    import torch
    from diffsims_gb300.engine import PhaseTable
    t = PhaseTable(pu.to_phase(crystal), r, direct_beam, "lobato", None, device=torch.device("cuda", 0))
    want = ok.enumerate_hkl(crystal.rbase, 1 / r, n_zero=2 if direct_beam else 0)
    np.testing.assert_array_equal(t.hkl.cpu().numpy(), want)
    g2 = ok.g_squared(ok.g_cartesian(want, crystal.rbase))
    np.testing.assert_array_equal(t.g2.cpu().numpy(), g2)  # bit for bit


def test_enumeration_kats():
    import torch
    from diffsims_gb300.engine import PhaseTable
    dev = torch.device("cuda", 0)
    al = ok.Crystal((4.04,) * 3 + (90, 90, 90), ["Al"], [[0, 0, 1]])
    t = PhaseTable(pu.to_phase(al), 1 / 0.7, False, device=dev)
    h = t.hkl.cpu().numpy()
    assert t.n == 798 and list(h[0]) == [5, 2, 2] and list(h[-1]) == [-5, -2, -2]
    fe = ok.Crystal((2.8665,) * 3 + (90, 90, 90), ["Fe"] * 2, [[0, 0, 0], [.5, .5, .5]])
    assert [PhaseTable(pu.to_phase(fe), 1 / d, False, device=dev).n for d in (2, 1, 0.5)] == [18, 92, 750]


# ------------------------------------------------------------------ A3
@pytest.mark.parametrize("name, crystal", [("al", al_fcc()), ("graphite", graphite()), ("si", si_crystal()),
                                           ("p1_200", random_p1(200, 5)), ("p1_500", random_p1(500, 6))])
@pytest.mark.parametrize("sp", ["lobato", "xtables", None])
def test_structure_factor_table(name, crystal, sp):
    import torch
    from diffsims_gb300.engine import PhaseTable
    dev = torch.device("cuda", 0)
    r = 1.5
    want_hkl = ok.enumerate_hkl(crystal.rbase, 1 / r, n_zero=2)
    gs = np.sqrt(ok.g_squared(ok.g_cartesian(want_hkl, crystal.rbase)))
    F = ok.structure_factor(want_hkl, gs, crystal.elements, crystal.xyz, crystal.occupancy, crystal.B, sp)
    F2 = (F * F.conjugate()).real
    tm = PhaseTable(pu.to_phase(crystal), r, True, sp, list(crystal.B), form="mixed", device=dev)
    tf = PhaseTable(pu.to_phase(crystal), r, True, sp, list(crystal.B), form="fp64", device=dev)
    got_m = tm.F2.cpu().numpy().astype(np.float64)
    got_f = tf.F2d.cpu().numpy()
    scale = F2.max()
    # FP64 form: FP64 throughout
    np.testing.assert_allclose(got_f, F2, rtol=1e-10, atol=1e-13 * scale)
    # mixed form: relative 1e-5 on every reflection above FP64 round-off of the largest one
    big = F2 > 1e-12 * scale
    rel = np.abs(got_m[big] - F2[big]) / F2[big]
    assert rel.max() <= 1e-5, (name, sp, rel.max())
    # near-zero |F|^2 (systematic absences) stay near-zero at FP64 size
    assert np.all(got_m[~big] <= 1e-10 * scale)


def test_kinematical_intensities_match_reference_golden(golden_dir):
    import diffsims_gb300 as ds
    from tests.golden.make_golden import structures
    ref = dict(np.load(os.path.join(golden_dir, "reference_numerics.npz")))
    for name, (lat, els, xyz, occ, dw) in structures().items():
        st = ds.Structure([ds.Atom(e, x, o) for e, x, o in zip(els, xyz, occ)], ds.Lattice(*lat))
        for sp in ("lobato", "xtables", None):
            with warnings.catch_warnings():
                warnings.simplefilter("ignore")
                got = ds.get_kinematical_intensities(st, ref[f"kin_{name}_hkl"], ref[f"kin_{name}_gspacing"], dw,
                                                     sp, prefactor=ref[f"kin_{name}_prefactor"])
            want = ref[f"kin_{name}_{sp}"]
            np.testing.assert_allclose(got, want, rtol=1e-11, atol=1e-11 * np.abs(want).max())


def test_kinematical_intensities_kats():
    # diffsims/tests/utils/test_sim_utils.py:330-394
    import diffsims_gb300 as ds
    ni = ds.Structure([ds.Atom("Ni", [0, 0, 0])], ds.Lattice(3, 3, 5, 90, 90, 120))
    np.testing.assert_almost_equal(ds.get_kinematical_intensities(ni, [[0, 0, 0]], [0.0], {"Al": 1})[0], 43.0979, 4)
    np.testing.assert_almost_equal(ds.get_kinematical_intensities(ni, [[0, 0, 0]], [0.0], None, None)[0], 1.0)
    unk = ds.Structure([ds.Atom("UnOb", [0, 0, 0])], ds.Lattice(3.5236, 3.5236, 3.5236))
    with pytest.warns(UserWarning, match="not found in scattering parameter library"):
        assert ds.get_kinematical_intensities(unk, [[0, 0, 0]], [0.0])[0] == 0.0


# ------------------------------------------------------------------ A4-A7
def test_config1_al_fcc_1000_orientations():
    """Al FCC, 200 kV, r = 1.0, s_max = 0.01, linear, Lobato, B = 0.5, 1000
    uniform SO(3) orientations from seed 0."""
    q = ok.random_quaternions(1000, seed=0)
    p = ok.SimParams(accelerating_voltage=200, shape_factor_model="linear", reciprocal_radius=1.0,
                     max_excitation_error=0.01)
    for form, rtol in (("mixed", 1e-5), ("fp64", 1e-6)):
        spots, _ = pu.gpu_run(al_fcc(), q, p, form)
        st = pu.compare(spots, al_fcc(), q, p, rtol=rtol)
        assert st["boundary_flips"] <= 2, st
        assert st["max_abs_s"] < 1e-9, st


@pytest.mark.parametrize("shape", ["linear", "lorentzian", "sinc", "sin2c", "atanc"])
@pytest.mark.parametrize("prec", [0.0, 0.5])
def test_shapes_and_precession_p1(shape, prec):
    crystal = random_p1(40, 11)
    q = ok.random_quaternions(96, seed=4)
    p = ok.SimParams(accelerating_voltage=200, shape_factor_model=shape, reciprocal_radius=1.5,
                     max_excitation_error=0.015, precession_angle=prec)
    spots, _ = pu.gpu_run(crystal, q, p, "mixed")
    st = pu.compare(spots, crystal, q, p, rtol=1e-5)
    assert st["spots"] > 100


_TIGHT_CACHE = {}


@pytest.mark.parametrize("form", ["mixed", "fp64"])
@pytest.mark.parametrize("shape", ["linear", "lorentzian", "sinc", "sin2c", "atanc"])
def test_precession_rotation_average(shape, form):
    """approximate_precession=False: the per-spot rotation average against the
    oracle's tight quadrature, 1e-5 relative on every intensity."""
    crystal = random_p1(30, 17)
    q = ok.random_quaternions(8, seed=6)
    p = ok.SimParams(accelerating_voltage=200, shape_factor_model=shape, reciprocal_radius=1.2,
                     max_excitation_error=0.015, precession_angle=1.0, approximate_precession=False,
                     precession_quadrature="tight")
    if shape not in _TIGHT_CACHE:
        with warnings.catch_warnings():
            warnings.simplefilter("ignore")
            _TIGHT_CACHE[shape] = ok.simulate(crystal, q, p, return_s=True)
    spots, _ = pu.gpu_run(crystal, q, p, form)
    st = pu.compare(spots, crystal, q, p, rtol=1e-5, ref=_TIGHT_CACHE[shape])
    assert st["spots"] > 100, st


@pytest.mark.parametrize("shape", ["linear", "sinc", "lorentzian"])
def test_precession_rotation_average_vs_reference_quadrature(shape):
    """Against the reference's own adaptive quadrature (default tolerances):
    the GPU value is within that quadrature's own error (its distance from
    the tight integral) plus 1e-5 relative."""
    crystal = al_fcc()
    q = ok.random_quaternions(16, seed=3)
    kw = dict(accelerating_voltage=200, shape_factor_model=shape, reciprocal_radius=2.0,
              max_excitation_error=0.01, precession_angle=0.5, approximate_precession=False)
    ref = ok.simulate(crystal, q, ok.SimParams(**kw), return_s=True)
    tight = ok.simulate(crystal, q, ok.SimParams(precession_quadrature="tight", **kw), return_s=True)
    spots, _ = pu.gpu_run(crystal, q, ok.SimParams(**kw), "mixed")
    off = spots.offsets.cpu().numpy()
    idx = spots.hkl_index.cpu().numpy()
    inten = spots.xyzi.cpu().numpy()[:, 3].astype(np.float64)
    n = 0
    for i, (r, t) in enumerate(zip(ref, tight)):
        assert np.array_equal(r.index, t.index)
        gi = idx[off[i]:off[i + 1]]
        common, ia, ib = np.intersect1d(gi, r.index, return_indices=True)
        assert len(common) == len(r.index), i
        got = inten[off[i]:off[i + 1]][ia]
        allowed = np.abs(r.intensity[ib] - t.intensity[ib]) + 1e-5 * t.intensity[ib] + 1e-30
        assert np.all(np.abs(got - r.intensity[ib]) <= allowed), i
        n += len(common)
    assert n > 50


@pytest.mark.parametrize("kw", [dict(with_direct_beam=False), dict(minimum_intensity=1e-3),
                                dict(shape_factor_width=0.03), dict(scattering_params="xtables"),
                                dict(scattering_params=None), dict(accelerating_voltage=300),
                                dict(shape_factor_model="sinc", shape_kwargs={"minima_number": 3})])
def test_generator_options(kw):
    crystal = random_p1(30, 21)
    q = ok.random_quaternions(64, seed=9)
    base = dict(accelerating_voltage=200, shape_factor_model="lorentzian", reciprocal_radius=1.5,
                max_excitation_error=0.02)
    base.update(kw)
    p = ok.SimParams(**base)
    spots, _ = pu.gpu_run(crystal, q, p, "mixed")
    pu.compare(spots, crystal, q, p, rtol=1e-5)


@pytest.mark.parametrize("kw, count", [(dict(), 70), (dict(precession_angle=0.5), 250),
                                       (dict(precession_angle=0.5, approximate_precession=False), 250)])
def test_spot_count_kats(kw, count):
    # diffsims/tests/generators/test_simulation_generator.py:137-161
    import diffsims_gb300 as ds
    gen = ds.SimulationGenerator(300, **kw)
    sim = gen.calculate_diffraction2d(pu.to_phase(si_crystal()), reciprocal_radius=5.0)
    assert sim.coordinates.size == count


def test_direct_beam_and_nesting():
    # diffsims/tests/generators/test_simulation_generator.py:188-265
    import diffsims_gb300 as ds
    gen = ds.SimulationGenerator(300)
    si = pu.to_phase(si_crystal())
    sim = gen.calculate_diffraction2d(si, reciprocal_radius=0.5, with_direct_beam=True)
    v = sim.coordinates
    i0 = [tuple(h) for h in v.hkl.astype(int)].index((0, 0, 0))
    assert np.all(v.intensity[i0] >= v.intensity)
    sim = gen.calculate_diffraction2d(si, reciprocal_radius=0.5, with_direct_beam=False)
    assert (0, 0, 0) not in [tuple(h) for h in sim.coordinates.hkl.astype(int)]
    big = pu.to_phase(si_crystal(10))
    r1 = ds.Rotation.from_euler([[0, 0, 0], [0.1, 0.1, 0.1]])
    r2 = ds.Rotation.from_euler([[0, 0, 0], [0.1, 0.1, 0.1], [0.2, 0.2, 0.2]])
    sim = gen.calculate_diffraction2d([si, big], rotation=[r1, r2])
    assert [len(c) for c in sim.coordinates] == [2, 3] and len(list(sim)) == 5
    with pytest.raises(ValueError):
        gen.calculate_diffraction2d([si, big], rotation=[r1])


def test_appropriate_scaling():
    # diffsims/tests/generators/test_simulation_generator.py:170-186
    import diffsims_gb300 as ds
    gen = ds.SimulationGenerator(300)
    a = gen.calculate_diffraction2d(pu.to_phase(si_crystal(5)), reciprocal_radius=5.0).coordinates
    b = gen.calculate_diffraction2d(pu.to_phase(si_crystal(10)), reciprocal_radius=5.0).coordinates
    ia = [tuple(h) for h in a.hkl.astype(int)].index((2, 2, 0))
    ib = [tuple(h) for h in b.hkl.astype(int)].index((2, 2, 0))
    np.testing.assert_allclose(a.data[ia], 2 * b.data[ib], rtol=1e-6)


def test_graphite_golden_through_gpu(golden_dir):
    """The reference's golden image, rasterised from the GPU's spots."""
    from scipy import ndimage as ndi
    q = ok.euler_to_quaternion([0, 90, 90], degrees=True)
    p = ok.SimParams(accelerating_voltage=200, reciprocal_radius=1.6768, max_excitation_error=0.1,
                     with_direct_beam=False)
    spots, _ = pu.gpu_run(graphite(), q, p, "mixed")
    xyzi = spots.xyzi.cpu().numpy().astype(np.float64)
    t = ok.transformed_pixel_coordinates(xyzi[:, :3], (128, 128), 0.0262)
    near = np.abs(t[:, :2] - np.round(t[:, :2])) < 1e-4
    t[:, :2][near] = np.round(t[:, :2])[near]
    inf = (t[:, 0] >= 0) & (t[:, 0] < 128) & (t[:, 1] >= 0) & (t[:, 1] < 128)
    co = t[inf].astype(int)
    img = np.zeros((128, 128))
    img[co[:, 1], co[:, 0]] = xyzi[inf, 3]
    img = ndi.gaussian_filter(img, 1.4)
    img /= img.max()
    old = np.load(os.path.join(golden_dir, "graphite_pattern_128.npy"))
    np.testing.assert_allclose(img, old, atol=1e-6)


@pytest.mark.parametrize("tile", [4, 8, 16, 32])
def test_orientation_tiles_agree(tile):
    crystal = random_p1(20, 3)
    q = ok.random_quaternions(333, seed=2)
    p = ok.SimParams(accelerating_voltage=200, shape_factor_model="lorentzian", reciprocal_radius=1.2,
                     max_excitation_error=0.02)
    a, _ = pu.gpu_run(crystal, q, p, "mixed", orient_tile=tile)
    b, _ = pu.gpu_run(crystal, q, p, "mixed", orient_tile=4)
    assert a.total == b.total
    assert np.array_equal(a.offsets.cpu().numpy(), b.offsets.cpu().numpy())
    assert np.array_equal(a.hkl_index.cpu().numpy(), b.hkl_index.cpu().numpy())
    assert np.array_equal(a.xyzi.cpu().numpy(), b.xyzi.cpu().numpy())  # deterministic, bit for bit


@pytest.mark.parametrize("stage_cap", [1, 64, 700])
def test_staging_fallback_agrees(stage_cap):
    """Orientation parts whose candidates do not fit the per-CTA staging walk
    the bitmap and re-evaluate: same spots, bit for bit."""
    import torch
    from diffsims_gb300.engine import PhaseTable, SpotBuffers, simulate_phase
    dev = torch.device("cuda", 0)
    crystal = random_p1(20, 13)
    q = ok.random_quaternions(100, seed=5)
    p = ok.SimParams(accelerating_voltage=200, shape_factor_model="sinc", reciprocal_radius=1.4,
                     max_excitation_error=0.02, minimum_intensity=1e-3)
    gen = pu.generator_for(p)
    table = PhaseTable(pu.to_phase(crystal), 1.4, True, "lobato", list(crystal.B), device=dev)
    qd = torch.as_tensor(q).to(dev)
    s0 = gen.settings(0.02)
    s1 = gen.settings(0.02)
    s1.stage_cap = stage_cap
    a = simulate_phase(table, qd, s0, 1.4, SpotBuffers(dev))
    b = simulate_phase(table, qd, s1, 1.4, SpotBuffers(dev))
    assert a.total == b.total
    assert np.array_equal(a.offsets.cpu().numpy(), b.offsets.cpu().numpy())
    assert np.array_equal(a.hkl_index.cpu().numpy(), b.hkl_index.cpu().numpy())
    xa, xb = a.xyzi.cpu().numpy(), b.xyzi.cpu().numpy()
    assert np.array_equal(xa[:, 3], xb[:, 3])
    np.testing.assert_allclose(xa[:, :3], xb[:, :3], atol=1e-6)  # z: FP32 in the staged path, double-float otherwise
    pu.compare(b, crystal, q, p)


@pytest.mark.parametrize("name, crystal, r, eps", [
    ("p1", random_p1(30, 17), 1.5, 0.02), ("al", al_fcc(), 1.0, 0.01), ("long_c", random_p1(8, 19, edges=(4, 20)), 1.8, 0.02),
    ("graphite", graphite(), 1.6768, 0.1), ("si_big", si_crystal(), 3.0, 0.01)])
def test_line_screen_matches_row_screen(name, crystal, r, eps):
    """The per-(orientation, hkl line) interval screen, the brick screen and
    the per-row screen keep different supersets (bricks: the same rows);
    after the exact selection the spots agree bit for bit."""
    import torch
    from diffsims_gb300.engine import PhaseTable, SpotBuffers, simulate_phase
    dev = torch.device("cuda", 0)
    q = np.vstack([ok.random_quaternions(300, seed=3), ok.euler_to_quaternion([[0, 0, 0], [0, 90, 0], [45, 54.7356, 0],
                                                                             [0, 90, 90], [10, 0.05, 3]], degrees=True)])
    p = ok.SimParams(accelerating_voltage=200, shape_factor_model="linear", reciprocal_radius=r, max_excitation_error=eps)
    gen = pu.generator_for(p)
    table = PhaseTable(pu.to_phase(crystal), r, True, "lobato", list(crystal.B), device=dev)
    qd = torch.as_tensor(q).to(dev)
    res = {}
    for screen in ("rows", "lines", "bricks"):
        st = gen.settings(eps)
        st.screen = screen
        res[screen] = simulate_phase(table, qd, st, r, SpotBuffers(dev, with_excitation_error=True))
    a = res["rows"]
    for other in ("lines", "bricks"):
        b = res[other]
        assert a.total == b.total, other
        assert np.array_equal(a.offsets.cpu().numpy(), b.offsets.cpu().numpy()), other
        assert np.array_equal(a.hkl_index.cpu().numpy(), b.hkl_index.cpu().numpy()), other
        assert np.array_equal(a.xyzi.cpu().numpy(), b.xyzi.cpu().numpy()), other
        assert np.array_equal(a.excitation_error.cpu().numpy(), b.excitation_error.cpu().numpy()), other
    pu.compare(res["bricks"], crystal, q, p)


@pytest.mark.parametrize("kw", [dict(precession_angle=0.5), dict(precession_angle=1.0, approximate_precession=False,
                                                                 shape_factor_model="sinc"),
                                dict(shape_factor_model="sinc", with_direct_beam=False)])
@pytest.mark.parametrize("tile", [0, 4, 32])
def test_brick_screen_matches_row_screen(kw, tile):
    """Bricks against rows with precession (the widened band), without the
    direct beam, and for several orientation tiles: bit for bit."""
    import torch
    from diffsims_gb300.engine import PhaseTable, SpotBuffers, simulate_phase
    dev = torch.device("cuda", 0)
    crystal = random_p1(60, 23)
    base = dict(accelerating_voltage=200, shape_factor_model="lorentzian", reciprocal_radius=1.6,
                max_excitation_error=0.015)
    base.update(kw)
    p = ok.SimParams(**base)
    gen = pu.generator_for(p)
    table = PhaseTable(pu.to_phase(crystal), p.reciprocal_radius, p.with_direct_beam, "lobato", list(crystal.B),
                       device=dev)
    q = ok.random_quaternions(700, seed=12)
    qd = torch.as_tensor(q).to(dev)
    res = {}
    for screen in ("rows", "bricks"):
        st = gen.settings(p.max_excitation_error, orient_tile=tile)
        st.screen = screen
        res[screen] = simulate_phase(table, qd, st, p.reciprocal_radius, SpotBuffers(dev))
    a, b = res["rows"], res["bricks"]
    assert a.total == b.total and a.total > 1000
    assert np.array_equal(a.offsets.cpu().numpy(), b.offsets.cpu().numpy())
    assert np.array_equal(a.hkl_index.cpu().numpy(), b.hkl_index.cpu().numpy())
    assert np.array_equal(a.xyzi.cpu().numpy(), b.xyzi.cpu().numpy())


def test_capacity_overflow_is_retried():
    import torch
    from diffsims_gb300 import engine
    crystal = random_p1(10, 8)
    q = ok.random_quaternions(50, seed=1)
    p = ok.SimParams(accelerating_voltage=200, reciprocal_radius=1.5, max_excitation_error=0.02)
    orig = engine.estimate_spots
    engine.estimate_spots = lambda *a, **k: 0  # force the first attempt to overflow
    try:
        spots, _ = pu.gpu_run(crystal, q, p, "mixed")
    finally:
        engine.estimate_spots = orig
    pu.compare(spots, crystal, q, p)


@pytest.mark.parametrize("screen", ["lines", "rows", "bricks"])
def test_empty_table_and_no_direct_beam(screen):
    """A radius below the first reflection and no direct beam: an empty
    candidate table, empty patterns; and small tables without 000 rows."""
    import torch
    from diffsims_gb300.engine import PhaseTable, SpotBuffers, simulate_phase
    dev = torch.device("cuda", 0)
    crystal = al_fcc()
    q = ok.random_quaternions(40, seed=2)
    for r, db in ((0.1, False), (0.1, True), (0.6, False)):
        p = ok.SimParams(accelerating_voltage=200, reciprocal_radius=r, with_direct_beam=db, max_excitation_error=0.05)
        gen = pu.generator_for(p)
        t = PhaseTable(pu.to_phase(crystal), r, db, "lobato", list(crystal.B), device=dev)
        st = gen.settings(0.05)
        st.screen = screen
        sp = simulate_phase(t, torch.as_tensor(q).to(dev), st, r, SpotBuffers(dev))
        assert sp.offsets.shape[0] == 41
        if t.n == 0:
            assert sp.total == 0
        else:
            pu.compare(sp, crystal, q, p)


def test_empty_and_single_orientation():
    import torch
    from diffsims_gb300.engine import PhaseTable, SpotBuffers, simulate_phase
    import diffsims_gb300 as ds
    dev = torch.device("cuda", 0)
    crystal = al_fcc()
    p = ok.SimParams(accelerating_voltage=200, reciprocal_radius=1.0)
    gen = pu.generator_for(p)
    t = PhaseTable(pu.to_phase(crystal), 1.0, True, device=dev)
    sp = simulate_phase(t, torch.zeros((0, 4), dtype=torch.float64, device=dev), gen.settings(), 1.0)
    assert sp.total == 0 and sp.offsets.cpu().tolist() == [0]
    # beam along a zone axis: the whole zero-order Laue zone is excited
    q = ok.euler_to_quaternion([0, 0, 0])
    spots, _ = pu.gpu_run(crystal, q, p, "mixed")
    pu.compare(spots, crystal, q, p)


def test_simulation2d_selectors_cursor_and_transforms():
    """iphase / irot selections (diffsims/simulations/simulation2d.py:43-106),
    the phase / rotation cursor and its iteration (:200-260), the current
    phase and rotation matrix, deepcopy, the in-plane transform (:261-311)
    and get_closest (:767-781) on a two-phase result."""
    import diffsims_gb300 as ds
    from diffsims_gb300.simulation2d import get_closest
    gen = ds.SimulationGenerator(300)
    si = pu.to_phase(si_crystal())
    big = pu.to_phase(si_crystal(10))
    big.name = "big"
    r1 = ds.Rotation.from_euler([[0, 0, 0], [0.1, 0.1, 0.1], [0.3, 0.2, 0.1]])
    r2 = ds.Rotation.from_euler([[0, 0, 0], [0.1, 0.1, 0.1], [0.2, 0.2, 0.2], [0.5, 0.1, 0.4]])
    sim = gen.calculate_diffraction2d([si, big], rotation=[r1, r2], reciprocal_radius=1.0)

    def same(a, b):
        np.testing.assert_array_equal(a.data, b.data)
        np.testing.assert_array_equal(a.intensity, b.intensity)
        np.testing.assert_array_equal(a.hkl, b.hkl)

    one = sim.iphase[0]
    assert one.phases is si and len(one) == 3 and not one.has_multiple_phases
    for i in range(3):
        same(one.coordinates[i], sim.coordinates[0][i])
    named = sim.iphase["big"]
    assert named.phases is big and len(named) == 4
    same(named.coordinates[3], sim.coordinates[1][3])
    both = sim.iphase[0:2]
    assert both.num_phases == 2 and len(both) == 7
    with pytest.raises(ValueError):
        one.iphase[0]
    with pytest.raises(ValueError):
        sim.iphase[1.5]
    sub = sim.irot[1:3]
    assert [len(c) for c in sub.coordinates] == [2, 2]
    same(sub.coordinates[0][0], sim.coordinates[0][1])
    same(sub.coordinates[1][1], sim.coordinates[1][2])
    np.testing.assert_allclose(sub.rotations[1].data, r2.data[1:3], rtol=0, atol=1e-15)
    single = one.irot[2]
    same(single.coordinates, sim.coordinates[0][2])
    with pytest.raises(ValueError):
        single.irot[0]
    # the cursor: iteration visits every pattern in order and ends at (0, 0)
    seen = list(sim)
    assert len(seen) == 7 and sim.phase_index == 0 and sim.rotation_index == 0
    same(seen[4], sim.coordinates[1][1])
    sim.phase_index, sim.rotation_index = 1, 2
    assert sim.current_phase is big and sim.current_size == 4
    np.testing.assert_allclose(sim.get_current_rotation_matrix(), r2.to_matrix()[2], rtol=0, atol=0)
    same(sim.get_current_coordinates(), sim.coordinates[1][2])
    # in-plane transform against the reference's polar form
    v = sim.get_current_coordinates()
    t = sim.rotate_shift_coordinates(30.0, center=(1.0, -2.0), mirrored=True)
    x, y = v.data[:, 0], v.data[:, 1]
    theta = -np.arctan2(y, x) + np.deg2rad(30.0)
    rd = np.sqrt(x ** 2 + y ** 2)
    np.testing.assert_allclose(t.data[:, 0], rd * np.cos(theta) + 1.0, rtol=0, atol=1e-12)
    np.testing.assert_allclose(t.data[:, 1], rd * np.sin(theta) - 2.0, rtol=0, atol=1e-12)
    np.testing.assert_array_equal(t.data[:, 2], v.data[:, 2])
    np.testing.assert_array_equal(t.intensity, v.intensity)
    # deepcopy: its own spot arrays
    d = sim.deepcopy()
    assert d.simulation_generator is gen and d is not sim
    d.spots(0).xyzi.zero_()
    assert np.any(sim.spots(0).xyzi.cpu().numpy() != 0)
    same(d.coordinates[1][3], sim.coordinates[1][3])
    np.testing.assert_array_equal(get_closest([0.0, 1.0, 2.0, 3.0], np.array([0.4, 1.6, 5.0, -1.0])), [0, 2, 3, 0])
