"""Pin the per-family structure-factor oracle, and the host logic of
``diffsims_gb300.structure_factor``, against the reference -- CPU only.

Known answers are the reference's own EMsoft-checked values
(diffsims/tests/structure_factor/test_structure_factor.py:79-181,
test_atomic_scattering_factor.py:27-110, test_atomic_scattering_parameters.py:25-70);
fixtures come from running the reference's structure_factor modules
(tests/golden/make_golden.py).
"""
import math
import os

import numpy as np
import pytest

from oracle import structure_factor_families as osf
from tests.golden.make_golden import sf_phases

B_REF = 8 * math.pi ** 2 * 0.006332
NICKEL = (225, (3.5236,) * 3 + (90, 90, 90), [("Ni0+", [0, 0, 0], 1.0, B_REF)])
FERRITE = (229, (2.8665,) * 3 + (90, 90, 90), [("Fe", [0, 0, 0], 1.0, B_REF), ("Fe", [.5, .5, .5], 1.0, B_REF)])
SIC4H = (186, (3.073, 3.073, 10.053, 90, 90, 120),
         [("Si", [0, 0, 0], 1.0, B_REF), ("Si", [0.33, 0.667, 0.25], 1.0, B_REF),
          ("C", [0, 0, 0.188], 1.0, B_REF), ("C", [0.333, 0.667, 0.438], 1.0, B_REF)])
PHASES = {"nickel": NICKEL, "ferrite": FERRITE, "sic4h": SIC4H}


@pytest.fixture(scope="module")
def ref(golden_dir):
    return dict(np.load(os.path.join(golden_dir, "reference_structure_factor.npz")))


# test_structure_factor.py:79-96
@pytest.mark.parametrize("name, hkl, s, want", [
    ("nickel", [1, 1, 1], 0.245778, 79.665427), ("ferrite", [1, 1, 0], 0.2466795, 35.783295),
    ("ferrite", [1, 1, 1], 0.2466795, 0), ("sic4h", [0, 0, 4], 0.198945, 19.027004)])
def test_kinematical_kat(name, hkl, s, want):
    sg, _, atoms = PHASES[name]
    assert np.allclose(osf.kinematical_structure_factor(atoms, osf.space_group_operations(sg), hkl, s), want)


# test_structure_factor.py:99-121 and :124-144
@pytest.mark.parametrize("name, hkl, s, kv, want", [
    ("nickel", [1, 1, 1], 0.245778, 15e3, 8.606363), ("ferrite", [1, 1, 0], 0.2466795, 20e3, 8.096651),
    ("ferrite", [1, 1, 1], 0.2466795, 20e3, 0), ("sic4h", [0, 0, 4], 0.198945, 200e3, 2.744304),
    ("ferrite", [2, 0, 0], 0.348857, 20e3, 5.581301)])
def test_doyleturner_kat(name, hkl, s, kv, want):
    sg, lat, atoms = PHASES[name]
    v, params = osf.doyleturner_structure_factor(atoms, osf.space_group_operations(sg), hkl, s,
                                                 osf.cell_volume(*lat), kv)
    assert np.allclose(v, want)
    if name == "ferrite" and kv == 20e3 and hkl != [1, 1, 1]:
        want_p = {(1, 1, 0): [1.03, 12.17, 1.22e-16, 12.17 + 2.45e-15j],
                  (2, 0, 0): [1.03, 8.39, 1.22e-16, 8.39 + 1.02e-15j]}[tuple(hkl)]
        assert np.allclose(list(params.values()), want_p, atol=1e-2)


# test_structure_factor.py:147-164
@pytest.mark.parametrize("name, kv, want", [
    ("nickel", 20e3, 0.008582), ("nickel", 200e3, 0.002507), ("ferrite", 10e3, 0.012186), ("sic4h", 100e3, 0.003701)])
def test_refraction_corrected_wavelength_kat(name, kv, want):
    sg, lat, atoms = PHASES[name]
    got = osf.refraction_corrected_wavelength(atoms, osf.space_group_operations(sg), osf.cell_volume(*lat), kv)
    assert np.allclose(got, want, atol=1e-6)


# test_atomic_scattering_factor.py:27-54
@pytest.mark.parametrize("el, occ, u, s, want", [
    ("fe", 1, 0.5, 0.17442875, 6.306987), ("fe", 1, 0.5, 0.90635835, 5.911219e-14),
    ("ni", 1, 0.5, 0.14190033, 10.964046), ("ni", 0.5, 0.5, 0.14190033, 5.482023)])
def test_atomic_kinematical_kat(el, occ, u, s, want):
    b = 8 * math.pi ** 2 * u
    assert np.allclose(osf.atomic_f_kinematical(el, s, b, occ), want)
    assert np.allclose(osf.atomic_f_kinematical(osf.element_id(el), s, b, occ), want)


# test_atomic_scattering_factor.py:57-110
@pytest.mark.parametrize("el, lat, u, s, want", [
    ("fe", (2.8665,) * 3 + (90, 90, 90), 0.5, 0.17442875, 2.422658),
    ("fe", (2.8665,) * 3 + (90, 90, 90), 0.5, 0.90635835, 9.172283e-15),
    ("fe", (2.8665,) * 3 + (90, 90, 90), 0, 0.90635835, 1.114444),
    ("ni", (3.5236,) * 3 + (90, 90, 90), 0.5, 0.14190033, 2.186904),
    ("si", (3.073, 3.073, 10.053, 90, 90, 120), 0, 0.19894559, 1.512963)])
def test_atomic_doyleturner_kat(el, lat, u, s, want):
    got = osf.atomic_f_doyleturner(el, s, osf.cell_volume(*lat), 8 * math.pi ** 2 * u)
    assert np.allclose(got, want)


# test_atomic_scattering_parameters.py:25-45
@pytest.mark.parametrize("el, unit, want", [
    (10, "m", [0.303, 0.720, 0.475, 0.153, 17.640, 5.860, 1.762, 0.266]),
    ("Fe", None, [2.544, 2.343, 1.759, 0.506, 64.424, 14.880, 2.854, 0.350]),
    ("Fe", "NM", [0.02544, 0.02343, 0.01759, 0.00506, 0.64424, 0.14880, 0.02854, 0.00350]),
    ("bk", "Å", [6.502, 5.478, 2.510, 0.000, 28.375, 4.975, 0.561, 0.0])])
def test_parameters_kat(el, unit, want):
    a, b = osf.doyleturner_parameters(el, unit)
    assert np.allclose(a, want[:4]) and np.allclose(b, want[4:])


def test_element_ids_round_trip():
    # test_atomic_scattering_parameters.py:48-70
    for z in range(1, 99):
        sym = osf.element_symbol_from_id(z)
        assert osf.element_id(sym.upper()) == z and osf.element_id(sym.lower()) == z


@pytest.mark.parametrize("name", list(sf_phases()))
def test_oracle_matches_reference_fixtures(ref, name):
    sg, lat, atoms = sf_phases()[name]
    ops = osf.space_group_operations(sg)
    hkl, s = ref[f"{name}_hkl"], ref[f"{name}_s"]
    np.testing.assert_array_equal(osf.asymmetric_mask([a[1] for a in atoms]), ref[f"{name}_asym"])
    kin = np.array([osf.kinematical_structure_factor(atoms, ops, h, si) for h, si in zip(hkl, s)])
    scale = np.max(np.abs(ref[f"{name}_kin"]))
    np.testing.assert_allclose(kin, ref[f"{name}_kin"], rtol=0, atol=1e-12 * scale)
    vol = osf.cell_volume(*lat)
    for kv in (20e3, 200e3):
        dt = np.array([osf.doyleturner_structure_factor(atoms, ops, h, si, vol, kv)[0] for h, si in zip(hkl, s)])
        want = ref[f"{name}_dt{int(kv)}"]
        np.testing.assert_allclose(dt, want, rtol=0, atol=1e-12 * np.max(np.abs(want)))
    wl = [osf.refraction_corrected_wavelength(atoms, ops, vol, v) for v in ref[f"{name}_voltages"]]
    np.testing.assert_allclose(wl, ref[f"{name}_wavelength"], rtol=1e-14)


def test_oracle_atomic_factors_match_reference_fixtures(ref):
    for i, el in enumerate(ref["atom_elements"]):
        kin = [osf.atomic_f_kinematical(str(el), s, 0.45, 0.7) for s in ref["atom_s"]]
        dt = [osf.atomic_f_doyleturner(str(el), s, 61.3, 0.45, 0.7) for s in ref["atom_s"]]
        np.testing.assert_allclose(kin, ref["atom_kin"][i], rtol=1e-14, atol=1e-14)
        np.testing.assert_allclose(dt, ref["atom_dt"][i], rtol=1e-14, atol=1e-14)
        np.testing.assert_array_equal(np.concatenate(osf.doyleturner_parameters(str(el))), ref["atom_params"][i])


# ------------------------------------------------- host logic of the package
def test_host_orbits_and_mask_match_oracle():
    from diffsims_gb300 import structure_factor as gsf
    for sg in (1, 2, 186, 221, 225, 229):
        ops = osf.space_group_operations(sg)
        for xyz in ([0, 0, 0], [0.11, 0.23, 0.37], [0.5, 0.5, 0.5], [1 / 3, 2 / 3, 0.25], [0.999999999, 0, 0.5]):
            a = gsf.expand_position(ops, xyz)
            b = osf.orbit(ops, xyz)
            assert a.shape == b.shape
            np.testing.assert_allclose(a, b, atol=1e-12)
    assert gsf.expand_position(None, [0.2, 0.3, 0.4]).shape == (1, 3)
    assert len(gsf.expand_position(osf.space_group_operations(225), [0, 0, 0])) == 4
    assert len(gsf.expand_position(osf.space_group_operations(221), [0.11, 0.23, 0.37])) == 48
    # test_structure_factor.py:62-76
    assert list(gsf.find_asymmetric_positions([[0, 0, 0], [0, 0.5, 0.5]], None)) == [True, False]
    assert list(gsf.find_asymmetric_positions([[0.0349, 0.3106, 0.2607]] * 2, None)) == [True, True]


def test_host_space_group_forms():
    from diffsims_gb300 import structure_factor as gsf

    class Op:
        def __init__(self, R, t):
            self.R, self.t = R, t

    class SG:
        def __init__(self, ops):
            self.ops = ops

        def iter_symops(self):
            return iter([Op(R, t) for R, t in self.ops])

    ops = osf.space_group_operations(229)
    a = gsf.expand_position(SG(ops), [0, 0, 0])
    assert a.shape == (2, 3)
    with pytest.raises(NotImplementedError):
        gsf.expand_position(229, [0, 0, 0])


def test_host_element_table():
    from diffsims_gb300 import structure_factor as gsf
    for z in range(1, 99):
        sym = gsf._get_string_from_element_id(z)
        assert gsf.get_element_id_from_string(sym) == z == osf.element_id(sym)
        np.testing.assert_array_equal(np.concatenate(gsf.get_atomic_scattering_parameters(z)),
                                      np.concatenate(osf.doyleturner_parameters(z)))
    np.testing.assert_array_equal(gsf.get_atomic_scattering_parameters("Fe", "nm")[0],
                                  osf.doyleturner_parameters("Fe", "nm")[0])
    with pytest.raises(KeyError):
        gsf.get_element_id_from_string("Xx")


# --------------------------------- ReciprocalLatticeVector.calculate_structure_factor
def _al_phase(sg=225):
    from diffsims_gb300.crystal import Atom, Lattice, Phase, Structure
    atoms = [Atom("Al", x) for x in ([0, 0, 0], [0, .5, .5], [.5, 0, .5], [.5, .5, 0])]
    return Phase("al", Structure(atoms, Lattice(4.04, 4.04, 4.04)), space_group=osf.space_group_operations(sg))


def _ni_phase():
    from diffsims_gb300.crystal import Atom, Lattice, Phase, Structure
    atoms = [Atom("Ni", x, Uisoequiv=0.006332) for x in ([0, 0, 0], [0, .5, .5], [.5, 0, .5], [.5, .5, 0])]
    return Phase("nickel", Structure(atoms, Lattice(3.5236, 3.5236, 3.5236)),
                 space_group=osf.space_group_operations(225))


def _oracle_sf(monkeypatch):
    from diffsims_gb300 import structure_factor as gsf
    from oracle import kinematic as ok

    def fp64(structure, hkl, g2, sp):
        els = [a.element for a in structure]
        xyz = [a.xyz for a in structure]
        occ = [a.occupancy for a in structure]
        return ok.structure_factor(hkl, np.sqrt(g2), els, xyz, occ, np.zeros(len(els)), sp)

    monkeypatch.setattr(gsf, "_structure_factors_fp64", fp64)
    return gsf


def test_calculate_structure_factor_doctest(monkeypatch):
    # diffsims/crystallography/reciprocal_lattice_vector.py:665-690 (Al, a = 4.04)
    gsf = _oracle_sf(monkeypatch)
    F = gsf.calculate_structure_factor(_al_phase(), [[1, 1, 1], [2, 0, 0]])
    np.testing.assert_allclose(F.real, [8.46881663, 7.04777513], rtol=1e-8)
    assert np.all(np.abs(F.imag) < 1e-12)
    F = gsf.calculate_structure_factor(_al_phase(), [[1, 1, 1], [2, 0, 0]], "lobato")
    np.testing.assert_allclose(F.real, [8.44934816, 7.0387957], rtol=1e-8)


def test_calculate_structure_factor_table_kat(monkeypatch):
    # diffsims/tests/crystallography/test_reciprocal_lattice_vector.py:330-338 (print_table)
    gsf = _oracle_sf(monkeypatch)
    F = np.abs(gsf.calculate_structure_factor(_ni_phase(), [[1, 1, 1], [2, 0, 0]]))
    assert [f"{v:.1f}" for v in F] == ["11.8", "10.4"]
    assert [f"{v:.1f}" for v in F ** 2] == ["140.0", "108.2"]
    assert f"{(F ** 2 / (F ** 2).max() * 100)[1]:.1f}" == "77.3"


def test_calculate_structure_factor_sets(monkeypatch):
    """Every vector gets the value of its set's first vector (get_hkl_sets):
    in a non-centrosymmetric, non-symmorphic group (P6_3mc) equivalent
    reflections can differ in phase, and the reference copies the first."""
    from diffsims_gb300.crystal import Atom, Lattice, Phase, Structure
    gsf = _oracle_sf(monkeypatch)
    atoms = [Atom("Si", [0, 0, 0]), Atom("Si", [1 / 3, 2 / 3, 0.5]), Atom("C", [0, 0, 0.188]),
             Atom("C", [1 / 3, 2 / 3, 0.688])]
    phase = Phase("sic", Structure(atoms, Lattice(3.073, 3.073, 10.053, 90, 90, 120)),
                  space_group=osf.space_group_operations(186))
    hkl = np.array([[1, 0, 1], [0, 1, 1], [-1, 0, 1], [1, 0, -1], [0, 0, 4], [1, 1, 0], [-1, -1, 0], [1, 0, 1]])
    F = gsf.calculate_structure_factor(phase, hkl.reshape(2, 4, 3))
    assert F.shape == (2, 4)
    F = F.reshape(-1)
    rot = np.unique(np.array([np.rint(R).astype(int) for R, _ in osf.space_group_operations(186)]), axis=0)
    orbit = [{tuple(r) for r in (h @ rot).tolist()} for h in hkl]
    for i in range(len(hkl)):
        first = next(j for j in range(len(hkl)) if tuple(hkl[i]) in orbit[j])
        assert F[i] == F[first]
    assert F[0] == F[2]  # (-1, 0, 1) is in the set of (1, 0, 1) and copies its value
