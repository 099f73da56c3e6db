"""Pin the FP64 oracle against the reference's own golden vectors and KATs.

CPU only.  The fixtures come from tests/golden/make_golden.py, which runs the
reference's own ``sim_utils`` / ``shape_factor_models`` functions and copies its
golden detector image.
"""
import os
import warnings

import numpy as np
import pytest

from oracle import kinematic as ok


@pytest.fixture(scope="module")
def ref(golden_dir):
    return dict(np.load(os.path.join(golden_dir, "reference_numerics.npz")))


def si_crystal(a=5.431):
    xyz = []
    for c in [[0, 0, 0], [0.5, 0, 0.5], [0, 0.5, 0.5], [0.5, 0.5, 0]]:
        xyz += [c, [c[0] + .25, c[1] + .25, c[2] + .25]]
    return ok.Crystal((a, a, a, 90, 90, 90), ["Si"] * 8, xyz)


# diffsims/tests/utils/test_sim_utils.py:49-60
@pytest.mark.parametrize("kv, lam", [(100, 0.0370143659), (200, 0.0250793403), (300, 0.0196874888), ("inf", 0)])
def test_wavelength_kat(kv, lam):
    np.testing.assert_almost_equal(ok.electron_wavelength(kv), lam)


def test_wavelength_matches_reference(ref):
    got = [ok.electron_wavelength(v) for v in ref["wavelength_kv"]]
    np.testing.assert_array_equal(got, ref["wavelength"])


@pytest.mark.parametrize("w", [0.01, 0.015, 0.02])
def test_shape_models_match_reference(ref, w):
    key = f"w{w}"
    s = ref[f"shape_s_{key}"]
    np.testing.assert_array_equal(ok.sf_linear(s.copy(), w), ref[f"shape_linear_{key}"])
    np.testing.assert_array_equal(ok.sf_sinc(s.copy(), w), ref[f"shape_sinc_{key}"])
    np.testing.assert_array_equal(ok.sf_sinc(s.copy(), w, 3), ref[f"shape_sinc3_{key}"])
    np.testing.assert_array_equal(ok.sf_sin2c(s.copy(), w), ref[f"shape_sin2c_{key}"])
    np.testing.assert_array_equal(ok.sf_atanc(s.copy(), w), ref[f"shape_atanc_{key}"])
    np.testing.assert_array_equal(ok.sf_lorentzian(s.copy(), w), ref[f"shape_lorentzian_{key}"])
    r = ref[f"shape_r_{key}"]
    for deg in (0.5, 1.0):
        np.testing.assert_array_equal(ok.sf_lorentzian_precession(s.copy(), w, r, np.deg2rad(deg)),
                                      ref[f"shape_lprec{deg}_{key}"])


def test_shape_quirks():
    # sinc(0) = 0 and atanc(0) = 1 (diffsims/utils/shape_factor_models.py:95-101,147-151)
    assert ok.sf_sinc(np.array([0.0]), 0.01)[0] == 0.0
    assert ok.sf_atanc(np.array([0.0]), 0.01)[0] == 1.0
    # diffsims/tests/generators/test_simulation_generator.py:106-110
    np.testing.assert_allclose(ok.sf_linear(np.array([-2, -1, -0.5, 0, 0.5, 1, 2.0]), 1),
                               [0, 0, 0.5, 1, 0.5, 0, 0])


def test_precession_quad_matches_reference(ref):
    s, r = ref["quad_s"], ref["quad_r"]
    for name in ("linear", "sinc", "sin2c", "atanc", "lorentzian", "binary"):
        fn = ok.ALL_SHAPE_MODELS[name]
        with warnings.catch_warnings():
            warnings.simplefilter("ignore")
            got = ok.sf_precession_integral(s, r, np.deg2rad(0.5), fn, 0.01)
        np.testing.assert_allclose(got, ref[f"quad_{name}"], rtol=1e-12, atol=1e-15)


@pytest.mark.parametrize("name", ["al_fcc", "si_fd3m", "p1_60", "graphite", "unknown"])
@pytest.mark.parametrize("sp", ["lobato", "xtables", None])
def test_kinematical_intensities_match_reference(ref, name, sp):
    from tests.golden.make_golden import structures
    lat, els, xyz, occ, dw = structures()[name]
    hkl = ref[f"kin_{name}_hkl"]
    B = [dw.get(ok.element_symbol(e), 0) for e in els]
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        got = ok.kinematical_intensities(hkl, ref[f"kin_{name}_gspacing"], els, xyz, occ, B, sp,
                                         prefactor=ref[f"kin_{name}_prefactor"])
    want = ref[f"kin_{name}_{sp}"]
    np.testing.assert_allclose(got, want, rtol=1e-12, atol=1e-12 * np.abs(want).max())


def test_unknown_element_warns():
    # diffsims/tests/utils/test_sim_utils.py:370-394
    with pytest.warns(UserWarning, match="not found in scattering parameter library"):
        I = ok.kinematical_intensities([[0, 0, 0]], [0.0], ["UnOb"], [[0, 0, 0]], [1], [0], "lobato")
    assert I[0] == 0.0


def test_nickel_f0_kat():
    # diffsims/tests/utils/test_sim_utils.py:330-353: Ni at g = 0 -> 43.0979; None -> 1
    I = ok.kinematical_intensities([[0, 0, 0]], [0.0], ["Ni"], [[0, 0, 0]], [1], [0], "lobato")
    np.testing.assert_almost_equal(I[0], 43.0979, decimal=4)
    I = ok.kinematical_intensities([[0, 0, 0]], [0.0], ["Ni"], [[0, 0, 0]], [1], [0], None)
    np.testing.assert_almost_equal(I[0], 1.0)


def test_enumeration_kats():
    # doctest diffsims/crystallography/reciprocal_lattice_vector.py:1107-1127
    al = ok.Crystal((4.04,) * 3 + (90, 90, 90), ["Al"], [[0, 0, 1]])
    h = ok.enumerate_hkl(al.rbase, 0.7)
    assert len(h) == 798 and list(h[0]) == [5, 2, 2] and list(h[-1]) == [-5, -2, -2]
    assert len(ok.enumerate_hkl(al.rbase, 1.0)) == 256
    # diffsims/tests/crystallography/test_reciprocal_lattice_vector.py:76-87
    fe = ok.Crystal((2.8665,) * 3 + (90, 90, 90), ["Fe"] * 2, [[0, 0, 0], [.5, .5, .5]])
    for d, n in [(2, 18), (1, 92), (0.5, 750)]:
        assert len(ok.enumerate_hkl(fe.rbase, d)) == n
        assert len(ok.enumerate_hkl(fe.rbase, d, n_zero=1)) == n + 1
    assert list(ok.enumerate_hkl(fe.rbase, 2)[0]) == [1, 1, 0]
    # diffsims/tests/crystallography/test_reciprocal_lattice_vector.py:244-250 (SiC, d = 3)
    sic = ok.Crystal((3.073, 3.073, 10.053, 90, 90, 120), ["Si"], [[0, 0, 0]])
    np.testing.assert_array_equal(ok.enumerate_hkl(sic.rbase, 3),
                                  [[0, 0, 3], [0, 0, 2], [0, 0, 1], [0, 0, -1], [0, 0, -2], [0, 0, -3]])


@pytest.mark.parametrize("kw, count", [
    (dict(), 70),
    (dict(precession_angle=0.5), 250),
    (dict(precession_angle=0.5, approximate_precession=False), 250),
])
def test_spot_counts_kat(kw, count):
    # diffsims/tests/generators/test_simulation_generator.py:137-161
    p = ok.SimParams(accelerating_voltage=300, reciprocal_radius=5.0, **kw)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        pat = ok.simulate(si_crystal(), ok.euler_to_quaternion([0, 0, 0]), p)[0]
    assert pat.hkl.shape[0] == count


def test_direct_beam_brightest_and_absent():
    # diffsims/tests/generators/test_simulation_generator.py:188-208
    p = ok.SimParams(accelerating_voltage=300, reciprocal_radius=0.5)
    pat = ok.simulate(si_crystal(), ok.euler_to_quaternion([0, 0, 0]), p)[0]
    i0 = [tuple(h) for h in pat.hkl].index((0, 0, 0))
    assert np.all(pat.intensity[i0] >= pat.intensity)
    p = ok.SimParams(accelerating_voltage=300, reciprocal_radius=0.5, with_direct_beam=False)
    pat = ok.simulate(si_crystal(), ok.euler_to_quaternion([0, 0, 0]), p)[0]
    assert (0, 0, 0) not in [tuple(h) for h in pat.hkl]


def test_scaling_with_lattice():
    # diffsims/tests/generators/test_simulation_generator.py:170-186
    p = ok.SimParams(accelerating_voltage=300, reciprocal_radius=5.0)
    q = ok.euler_to_quaternion([0, 0, 0])
    a = ok.simulate(si_crystal(5), q, p)[0]
    b = ok.simulate(si_crystal(10), q, p)[0]
    ia = [tuple(h) for h in a.hkl].index((2, 2, 0))
    ib = [tuple(h) for h in b.hkl].index((2, 2, 0))
    np.testing.assert_allclose(a.xyz[ia], 2 * b.xyz[ib])


def graphite_golden_image(tie_tol=1e-9):
    """The oracle's image for the reference's golden case.

    Sixteen spots of this case sit exactly on pixel boundaries in exact
    arithmetic (beam-frame x or y = 0).  The reference's own float noise on
    those coordinates is zero, so they truncate to the integer; the oracle
    resolves coordinates within ``tie_tol`` of an integer the same way.
    """
    from scipy import ndimage as ndi
    gr = ok.Crystal((2.464, 2.464, 6.711, 90, 90, 120), ["C"] * 4,
                    [[0, 0, .25], [0, 0, .75], [1 / 3, 2 / 3, .25], [2 / 3, 1 / 3, .75]])
    p = ok.SimParams(accelerating_voltage=200, reciprocal_radius=1.6768, max_excitation_error=0.1,
                     with_direct_beam=False, shape_factor_model="lorentzian")
    pat = ok.simulate(gr, ok.euler_to_quaternion([0, 90, 90], degrees=True), p)[0]
    t = ok.transformed_pixel_coordinates(pat.xyz, (128, 128), 0.0262)
    near = np.abs(t[:, :2] - np.round(t[:, :2])) < tie_tol
    t[:, :2][near] = np.round(t[:, :2])[near]
    inf = (t[:, 0] >= 0) & (t[:, 0] < 128) & (t[:, 1] >= 0) & (t[:, 1] < 128)
    co = t[inf].astype(int)
    img = np.zeros((128, 128))
    img[co[:, 1], co[:, 0]] = pat.intensity[inf]
    img = ndi.gaussian_filter(img, 1.4)
    return img / img.max(), int(near.any(axis=1).sum())


def test_graphite_golden_pattern(golden_dir):
    # diffsims/tests/generators/test_simulation_generator.py:283-343 (atol 1e-8)
    old = np.load(os.path.join(golden_dir, "graphite_pattern_128.npy"))
    img, n_ties = graphite_golden_image()
    assert n_ties == 16
    np.testing.assert_allclose(img, old, atol=1e-8)
