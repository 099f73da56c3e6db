"""Pin the legacy-path oracle (``DiffractionGenerator.calculate_ed_data``)
against the reference's own outputs and tests, and check the host logic of
``diffsims_gb300.diffraction_generator`` -- CPU only.

Fixtures: tests/golden/reference_legacy.npz, from the reference's
diffsims/generators/diffraction_generator.py run by tests/golden/make_golden.py.
Structural checks restate diffsims/tests/generators/test_diffraction_generator.py:131-215.
"""
import os
import warnings

import numpy as np
import pytest

from oracle import legacy as ol
from tests.golden.make_golden import legacy_cases, legacy_structures


@pytest.fixture(scope="module")
def ref(golden_dir):
    return dict(np.load(os.path.join(golden_dir, "reference_legacy.npz")))


def oracle_case(i, quad=True):
    name, gk, ck = legacy_cases()[i]
    lat, els, xyz, occ = legacy_structures()[name]
    dwd = ck.get("debye_waller_factors", {})
    kw = dict(reciprocal_radius=ck["reciprocal_radius"], rotation=ck.get("rotation", (0, 0, 0)),
              max_excitation_error=ck.get("max_excitation_error", 1e-2),
              shape_factor_width=ck.get("shape_factor_width"),
              shape_factor_model=gk.get("shape_factor_model", "lorentzian"),
              precession_angle=gk.get("precession_angle", 0),
              approximate_precession=gk.get("approximate_precession", True),
              scattering_params=gk.get("scattering_params", "lobato"), quad=quad)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        return ol.calculate_ed_data(ol.DiffpyLattice(*lat), els, xyz, occ, [dwd.get(e, 0) for e in els],
                                    gk["accelerating_voltage"], **kw)


@pytest.mark.parametrize("i", range(len(legacy_cases())))
def test_oracle_matches_reference_fixtures(ref, i):
    c, idx, inten, _ = oracle_case(i)
    np.testing.assert_array_equal(idx, ref[f"case{i}_indices"])
    np.testing.assert_allclose(c, ref[f"case{i}_coordinates"], rtol=0, atol=1e-13)
    np.testing.assert_allclose(inten, ref[f"case{i}_intensities"], rtol=1e-12,
                               atol=1e-14 * np.max(ref[f"case{i}_intensities"]))


def si(a=5.431):
    xyz = []
    for c in [[0, 0, 0], [0.5, 0, 0.5], [0, 0.5, 0.5], [0.5, 0.5, 0]]:
        xyz += [c, [c[0] + .25, c[1] + .25, c[2] + .25]]
    return ol.DiffpyLattice(a, a, a, 90, 90, 90), ["Si"] * 8, xyz, [1.0] * 8, [0.0] * 8


def test_oracle_reference_structural_checks():
    # test_appropriate_scaling: doubling the cell halves the spacing
    a = ol.calculate_ed_data(*si(5), 300, 5.0)
    b = ol.calculate_ed_data(*si(10), 300, 5.0)
    ia = [tuple(x) for x in a[1]]
    ib = [tuple(x) for x in b[1]]
    assert (2, 2, 0) in ia and (2, 2, 0) in ib
    np.testing.assert_allclose(a[0][ia.index((2, 2, 0))], 2 * b[0][ib.index((2, 2, 0))])
    # test_appropriate_intensities: the direct beam is the strongest spot
    c, idx, inten, _ = ol.calculate_ed_data(*si(), 300, 5.0)
    assert np.all(inten[[tuple(x) for x in idx].index((0, 0, 0))] >= inten)
    # test_shape_factor_custom: a wider cutoff changes the pattern
    t1 = ol.calculate_ed_data(*si(), 300, 2.0, max_excitation_error=0.02)
    t2 = ol.calculate_ed_data(*si(), 300, 2.0, max_excitation_error=0.4)
    assert np.sum(t1[2]) != np.sum(t2[2])


def test_diffpy_frame_and_euler_convention():
    from diffsims_gb300.crystal import Lattice, Rotation, diffpy_base
    from diffsims_gb300.diffraction_generator import euler_rzxz_quaternions, structure_base
    for p in [(5.431,) * 3 + (90, 90, 90), (2.464, 2.464, 6.711, 90, 90, 120), (6.3, 7.1, 8.2, 84, 97, 103),
              (9.1, 11.3, 12.7, 81.0, 97.0, 104.0)]:
        np.testing.assert_allclose(diffpy_base(*p), ol.diffpy_stdbase(*p), rtol=0, atol=1e-14 * max(p[:3]))
        np.testing.assert_array_equal(structure_base(Lattice(*p)), diffpy_base(*p))
        lat = ol.DiffpyLattice(*p)
        np.testing.assert_array_equal(structure_base(lat), lat.base)
    rng = np.random.default_rng(2)
    e = rng.uniform(-180, 180, (50, 3))
    R = Rotation(euler_rzxz_quaternions(e)).to_matrix()
    for k in range(50):
        np.testing.assert_allclose(R[k], ol.euler2mat_rzxz(*np.deg2rad(e[k])), atol=1e-14)


def test_sphere_box_rule_matches_oracle():
    """The table's box half-widths are the reference's floor(r / |a*|)."""
    for p, r in [((5.431,) * 3 + (90, 90, 90), 5.0), ((6.3, 7.1, 8.2, 84, 97, 103), 1.5),
                 ((2.464, 2.464, 6.711, 90, 90, 120), 3.0)]:
        lat = ol.DiffpyLattice(*p)
        rl = lat.reciprocal()
        want = [np.floor(r / x) for x in (rl.a, rl.b, rl.c)]
        recip = np.linalg.inv(lat.base).T
        got = np.floor(r / np.linalg.norm(recip, axis=1))
        np.testing.assert_array_equal(got, want)


def test_diffraction_simulation_container():
    from diffsims_gb300.diffraction_simulation import DiffractionSimulation
    c = np.array([[0.0, 0.0, 0.0], [0.1, 0.2, 0.0], [-0.3, 0.1, 0.01]])
    sim = DiffractionSimulation(c, indices=np.array([[0, 0, 0], [1, 1, 0], [2, 0, 0]]),
                                intensities=np.array([3.0, 1.0, 2.0]))
    assert len(sim) == 2 and sim.size == 2                  # direct beam masked out by default
    sim.with_direct_beam = True
    assert len(sim) == 3
    with pytest.raises(Exception):
        sim.calibrated_coordinates
    sim.calibration = 0.01
    np.testing.assert_allclose(sim.calibrated_coordinates, c[:, :2] / 0.01)
    with pytest.raises(ValueError):
        sim.calibration = 0
    with pytest.raises(ValueError):
        sim.calibration = (1, 2, 3)
    s1 = sim[1:]
    assert len(s1) == 2 and s1.calibration is not None
    assert len(sim[0]) == 1
    with pytest.raises(ValueError):
        DiffractionSimulation(c, indices=np.zeros((2, 3)))
    sim.rotate_shift_coordinates(90, center=(1, 0))
    np.testing.assert_allclose(sim.coordinates[1, :2], [1 - 0.2, 0.1], atol=1e-15)
    assert len(sim + sim) == 6


def test_structure_and_diffraction_library_containers(tmp_path):
    # diffsims/tests/library/test_structure_library.py, test_diffraction_library.py (host logic)
    from diffsims_gb300.library import DiffractionLibrary, StructureLibrary, load_DiffractionLibrary
    lib = StructureLibrary(["a", "b"], [None, None], [[(0, 0, 0)], [(0, 0, 0), (0, 10, 0), (5, 5, 5)]])
    assert lib.get_library_size() == 4 and set(lib.struct_lib) == {"a", "b"}
    with pytest.raises(ValueError):
        StructureLibrary(["a"], [None, None], [[(0, 0, 0)]])
    with pytest.raises(ValueError):
        StructureLibrary(["a", "b"], [None, None], [[(0, 0, 0)]])
    dl = DiffractionLibrary()
    dl["a"] = {"simulations": ["s0", "s1"], "orientations": [(0, 0, 0), (0, 10, 0)],
               "pixel_coords": [np.zeros((1, 2)), np.ones((1, 2))], "intensities": [np.array([3.0, 4.0]),
                                                                                   np.array([1.0])]}
    e = dl.get_library_entry("a", (0, 10.001, 0))
    assert e["Sim"] == "s1" and e["pattern_norm"] == 1.0
    assert dl.get_library_entry()["pattern_norm"] == 5.0
    with pytest.raises(ValueError):
        dl.get_library_entry("a", (1, 1, 1))
    with pytest.raises(ValueError):
        dl.get_library_entry(angle=(0, 0, 0))
    f = tmp_path / "lib.pickle"
    dl.pickle_library(f)
    with pytest.raises(RuntimeError):
        load_DiffractionLibrary(f)
    assert load_DiffractionLibrary(f, safety=True)["a"]["orientations"] == dl["a"]["orientations"]


def profile_structures():
    from tests.golden.make_golden import legacy_structures as ls
    return dict(ls(), ni_hex=((3.0, 3.0, 5.0, 90, 90, 120), ["Ni"], [[0, 0, 0]], [1.0]))


@pytest.mark.parametrize("j", range(6))
def test_oracle_profiles_match_reference_fixtures(ref, j):
    from tests.golden.make_golden import profile_cases
    name, r, kw = profile_cases()[j]
    lat, els, xyz, occ = profile_structures()[name]
    x, y, h = ol.calculate_profile_data(ol.DiffpyLattice(*lat), els, xyz, occ, np.zeros(len(els)), r,
                                        scattering_params=kw.get("scattering_params", "lobato"))
    assert list(h) == list(ref[f"profile{j}_hkls"])
    np.testing.assert_allclose(x, ref[f"profile{j}_magnitudes"], rtol=1e-14)
    np.testing.assert_allclose(y, ref[f"profile{j}_intensities"], rtol=1e-12, atol=1e-11)


@pytest.mark.parametrize("angle, mirrored, center", [(0, False, (0, 0)), (33.0, False, (5, -2)),
                                                     (-120.5, True, (256, 256)), (90, True, (0, 0))])
def test_diffraction_simulation_transform_matches_reference_order(angle, mirrored, center):
    """The container's in-plane turn (complex form) against the reference's
    atan2 / sqrt / cos / sin order (oracle restatement): equal to round-off."""
    from diffsims_gb300.diffraction_simulation import DiffractionSimulation
    rng = np.random.default_rng(5)
    c = rng.normal(0, 1, (50, 3))
    sim = DiffractionSimulation(c, intensities=rng.random(50), with_direct_beam=True)
    sim.calibration = 0.02
    for units, src in (("real", c), ("pixel", c[:, :2] / 0.02)):
        got = sim._get_transformed_coordinates(angle, center, mirrored, units=units)
        want = ol.transformed_coordinates(src, angle, center, mirrored)
        np.testing.assert_allclose(got[:, :2], want[:, :2], rtol=0, atol=1e-12 * max(1.0, np.abs(want).max()))
