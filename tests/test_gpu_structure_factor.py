"""GPU parity of the per-family structure factors (ds_family_structure_factors)
against the reference's known answers, the reference's own outputs
(tests/golden/reference_structure_factor.npz) and the FP64 oracle.

Tolerances: the GPU form is FP64 with the phase reduced modulo 1 before
sincospi; against the reference (which takes cos(2 pi h.x) unreduced) and
the oracle the bar is 1e-11 of the largest magnitude in each set, and the
reference's own np.allclose for its known answers.
"""
import math
import os

import numpy as np
import pytest

from oracle import structure_factor_families as osf
from tests.golden.make_golden import sf_phases

pytestmark = pytest.mark.gpu

B_REF = 8 * math.pi ** 2 * 0.006332


class _Atom:
    def __init__(self, element, xyz, occ, biso):
        self.element, self.xyz, self.occupancy, self.Bisoequiv = element, np.asarray(xyz, float), occ, biso


def phase_of(sg, lat, atoms):
    from diffsims_gb300.crystal import Lattice, Phase, Structure
    return Phase(structure=Structure([_Atom(*a) for a in atoms], Lattice(*lat)),
                 space_group=osf.space_group_operations(sg))


def kat_phase(name):
    from diffsims_gb300.crystal import Atom, Lattice, Phase, Structure
    u = 0.006332
    if name == "nickel":
        sg, lat, atoms = 225, (3.5236,) * 3 + (90, 90, 90), [Atom("Ni0+", [0, 0, 0], Uisoequiv=u)]
    elif name == "ferrite":
        sg, lat, atoms = 229, (2.8665,) * 3 + (90, 90, 90), [Atom("Fe", [0, 0, 0], Uisoequiv=u),
                                                              Atom("Fe", [.5, .5, .5], Uisoequiv=u)]
    else:
        sg, lat = 186, (3.073, 3.073, 10.053, 90, 90, 120)
        atoms = [Atom("Si", [0, 0, 0], Uisoequiv=u), Atom("Si", [0.33, 0.667, 0.25], Uisoequiv=u),
                 Atom("C", [0, 0, 0.188], Uisoequiv=u), Atom("C", [0.333, 0.667, 0.438], Uisoequiv=u)]
    return Phase(structure=Structure(atoms, Lattice(*lat)), space_group=osf.space_group_operations(sg))


@pytest.fixture(scope="module")
def ref(golden_dir):
    return dict(np.load(os.path.join(golden_dir, "reference_structure_factor.npz")))


# diffsims/tests/structure_factor/test_structure_factor.py:79-96
@pytest.mark.parametrize("name, hkl, s, want", [
    ("nickel", [1, 1, 1], 0.245778, 79.665427), ("ferrite", [1, 1, 0], 0.2466795, 35.783295),
    ("ferrite", [1, 1, 1], 0.2466795, 0), ("sic4h", [0, 0, 4], 0.198945, 19.027004)])
def test_kinematical_kat(name, hkl, s, want):
    from diffsims_gb300.structure_factor import get_kinematical_structure_factor
    got = get_kinematical_structure_factor(kat_phase(name), hkl, s)
    assert np.ndim(got) == 0
    assert np.allclose(got, want)


# test_structure_factor.py:99-144
@pytest.mark.parametrize("name, hkl, s, kv, want", [
    ("nickel", [1, 1, 1], 0.245778, 15e3, 8.606363), ("ferrite", [1, 1, 0], 0.2466795, 20e3, 8.096651),
    ("ferrite", [1, 1, 1], 0.2466795, 20e3, 0), ("sic4h", [0, 0, 4], 0.198945, 200e3, 2.744304)])
def test_doyleturner_kat(name, hkl, s, kv, want):
    from diffsims_gb300.structure_factor import get_doyleturner_structure_factor
    assert np.allclose(get_doyleturner_structure_factor(kat_phase(name), hkl, s, kv), want)


@pytest.mark.parametrize("hkl, s, want, want_p", [
    ([1, 1, 0], 0.2466795, 8.096628, [1.03, 12.17, 1.22e-16, 12.17 + 2.45e-15j]),
    ([2, 0, 0], 0.348857, 5.581301, [1.03, 8.39, 1.22e-16, 8.39 + 1.02e-15j])])
def test_doyleturner_parameters_kat(hkl, s, want, want_p):
    from diffsims_gb300.structure_factor import get_doyleturner_structure_factor
    sf, params = get_doyleturner_structure_factor(kat_phase("ferrite"), hkl, s, 20e3, return_parameters=True)
    assert np.allclose(sf, want)
    assert list(params) == ["gamma_relcor", "v_mod", "v_phase", "v_g"]
    assert np.allclose(list(params.values()), want_p, atol=1e-2)


# test_structure_factor.py:147-164
@pytest.mark.parametrize("name, kv, want", [
    ("nickel", 20e3, 0.008582), ("nickel", 200e3, 0.002507), ("ferrite", 10e3, 0.012186), ("sic4h", 100e3, 0.003701)])
def test_refraction_corrected_wavelength_kat(name, kv, want):
    from diffsims_gb300.structure_factor import get_refraction_corrected_wavelength
    assert np.allclose(get_refraction_corrected_wavelength(kat_phase(name), kv), want, atol=1e-6)


# test_atomic_scattering_factor.py:27-110
def test_atomic_factor_kats():
    from diffsims_gb300.crystal import Atom
    from diffsims_gb300.structure_factor import (get_doyleturner_atomic_scattering_factor,
                                                 get_kinematical_atomic_scattering_factor)
    for el, occ, u, s, want in [("fe", 1, 0.5, 0.17442875, 6.306987), ("fe", 1, 0.5, 0.90635835, 5.911219e-14),
                                ("ni", 1, 0.5, 0.14190033, 10.964046), ("ni", 0.5, 0.5, 0.14190033, 5.482023)]:
        atom = Atom(el, [0, 0, 0], occ, Uisoequiv=u)
        assert np.allclose(get_kinematical_atomic_scattering_factor(atom, s), want)
        atom.element = osf.element_id(el)
        assert np.allclose(get_kinematical_atomic_scattering_factor(atom, s), want)
    fe_v, ni_v = 2.8665 ** 3, 3.5236 ** 3
    sic_v = osf.cell_volume(3.073, 3.073, 10.053, 90, 90, 120)
    for el, v, u, s, want in [("fe", fe_v, 0.5, 0.17442875, 2.422658), ("fe", fe_v, 0.5, 0.90635835, 9.172283e-15),
                              ("fe", fe_v, 0, 0.90635835, 1.114444), ("ni", ni_v, 0.5, 0.14190033, 2.186904),
                              ("si", sic_v, 0, 0.19894559, 1.512963)]:
        atom = Atom(el, [0, 0, 0], 1.0, Uisoequiv=u)
        assert np.allclose(get_doyleturner_atomic_scattering_factor(atom, s, v), want)


@pytest.mark.parametrize("name", list(sf_phases()))
def test_batched_matches_reference_fixtures(ref, name):
    from diffsims_gb300.structure_factor import (find_asymmetric_positions, get_doyleturner_structure_factor,
                                                 get_kinematical_structure_factor, get_refraction_corrected_wavelength)
    sg, lat, atoms = sf_phases()[name]
    phase = phase_of(sg, lat, atoms)
    hkl, s = ref[f"{name}_hkl"], ref[f"{name}_s"]
    np.testing.assert_array_equal(find_asymmetric_positions([a[1] for a in atoms], phase.space_group),
                                  ref[f"{name}_asym"])
    kin = get_kinematical_structure_factor(phase, hkl, s)
    assert kin.shape == (hkl.shape[0],)
    want = ref[f"{name}_kin"]
    np.testing.assert_allclose(kin, want, rtol=0, atol=1e-11 * np.max(np.abs(want)))
    for kv in (20e3, 200e3):
        dt, params = get_doyleturner_structure_factor(phase, hkl, s, kv, return_parameters=True)
        want = ref[f"{name}_dt{int(kv)}"]
        np.testing.assert_allclose(dt, want, rtol=0, atol=1e-11 * np.max(np.abs(want)))
        np.testing.assert_allclose(params["v_mod"], ref[f"{name}_dt{int(kv)}_vmod"], rtol=1e-11,
                                   atol=1e-11 * np.max(ref[f"{name}_dt{int(kv)}_vmod"]))
        vg, vg_want = params["v_g"], ref[f"{name}_dt{int(kv)}_vg"]
        np.testing.assert_allclose(vg, vg_want, rtol=0, atol=1e-11 * np.max(np.abs(vg_want)))
    wl = [get_refraction_corrected_wavelength(phase, v) for v in ref[f"{name}_voltages"]]
    np.testing.assert_allclose(wl, ref[f"{name}_wavelength"], rtol=1e-13)
    # one family at a time gives the batched values
    for i in (0, 7, hkl.shape[0] - 1):
        assert get_kinematical_structure_factor(phase, hkl[i], s[i]) == pytest.approx(kin[i], rel=1e-14, abs=1e-12)


def test_atomic_factors_match_reference_fixtures(ref):
    from diffsims_gb300.structure_factor import (get_doyleturner_atomic_scattering_factor,
                                                 get_kinematical_atomic_scattering_factor)
    for i, el in enumerate(ref["atom_elements"]):
        atom = _Atom(str(el), [0, 0, 0], 0.7, 0.45)
        kin = get_kinematical_atomic_scattering_factor(atom, ref["atom_s"])
        dt = get_doyleturner_atomic_scattering_factor(atom, ref["atom_s"], 61.3)
        np.testing.assert_allclose(kin, ref["atom_kin"][i], rtol=1e-13, atol=1e-13)
        np.testing.assert_allclose(dt, ref["atom_dt"][i], rtol=1e-13, atol=1e-13)


def test_large_batch_matches_oracle():
    """8192 families of a 48-position orbit (a mixed site at a general position
    of Pm-3m): every family within 1e-11 of the largest |F| of the oracle."""
    from diffsims_gb300.structure_factor import get_doyleturner_structure_factor, get_kinematical_structure_factor
    sg, lat, atoms = sf_phases()["mixed_pm3m"]
    phase = phase_of(sg, lat, atoms)
    rng = np.random.default_rng(5)
    hkl = rng.integers(-40, 41, (8192, 3)).astype(np.float64)
    s = rng.uniform(0.0, 3.0, hkl.shape[0])
    ops = osf.space_group_operations(sg)
    idx = rng.choice(hkl.shape[0], 400, replace=False)
    kin = get_kinematical_structure_factor(phase, hkl, s)
    want = np.array([osf.kinematical_structure_factor(atoms, ops, hkl[i], s[i]) for i in idx])
    np.testing.assert_allclose(kin[idx], want, rtol=0, atol=1e-11 * np.max(np.abs(want)))
    vol = osf.cell_volume(*lat)
    dt = get_doyleturner_structure_factor(phase, hkl, s, 300e3)
    want = np.array([osf.doyleturner_structure_factor(atoms, ops, hkl[i], s[i], vol, 300e3)[0] for i in idx])
    np.testing.assert_allclose(dt[idx], want, rtol=0, atol=1e-11 * np.max(np.abs(want)))


def test_entry_rejects_bad_arguments():
    import torch
    from diffsims_gb300 import _native as N
    from diffsims_gb300.sim_utils import PackedAtoms
    from diffsims_gb300.structure_factor import get_kinematical_structure_factor
    lib = N.load_library()
    dev = torch.device("cuda", torch.cuda.current_device())
    atoms = PackedAtoms(["Fe"], np.zeros((1, 3)), [1.0], [0.0], "lobato", dev)
    hkl = torch.zeros((4, 3), dtype=torch.float64, device=dev)
    s = torch.zeros(4, dtype=torch.float64, device=dev)
    F = torch.zeros((4, 2), dtype=torch.float64, device=dev)
    status = torch.zeros(1, dtype=torch.int32, device=dev)
    rc = lib.ds_family_structure_factors(atoms.cstruct(), N.ptr(hkl), N.ptr(s), 4, N.ptr(F), N.ptr(status),
                                         N.stream_handle())
    assert rc == N.DS_ERR_INVALID_ARGUMENT  # a lobato table is not a per-family kind
    rc = lib.ds_family_structure_factors(atoms.cstruct(), N.ptr(hkl), N.ptr(s), 0, N.ptr(F), N.ptr(status),
                                         N.stream_handle())
    assert rc == N.DS_ERR_INVALID_ARGUMENT  # the kind is checked before the empty-call shortcut
    phase = kat_phase("nickel")
    phase.structure[0].element = "Xx"
    with pytest.raises(KeyError):
        get_kinematical_structure_factor(phase, [1, 1, 1], 0.2)
    phase = kat_phase("nickel")
    phase.space_group = 225
    with pytest.raises(NotImplementedError):
        get_kinematical_structure_factor(phase, [1, 1, 1], 0.2)
    assert get_kinematical_structure_factor(kat_phase("nickel"), np.zeros((0, 3)), np.zeros(0)).shape == (0,)


def test_calculate_structure_factor_on_gpu():
    """ReciprocalLatticeVector.calculate_structure_factor on the GPU: the
    reference's doctest (Al, xtables and lobato) and table (Ni) values, and
    the FP64 oracle for every set of a P6_3mc phase (1e-12 of the largest)."""
    from diffsims_gb300.crystal import Atom, Lattice, Phase, Structure
    from diffsims_gb300.structure_factor import calculate_structure_factor
    from oracle import kinematic as ok
    from tests.test_oracle_structure_factor import _al_phase, _ni_phase
    F = calculate_structure_factor(_al_phase(), [[1, 1, 1], [2, 0, 0]])
    np.testing.assert_allclose(F.real, [8.46881663, 7.04777513], rtol=1e-8)
    F = calculate_structure_factor(_al_phase(), [[1, 1, 1], [2, 0, 0]], "lobato")
    np.testing.assert_allclose(F.real, [8.44934816, 7.0387957], rtol=1e-8)
    F = np.abs(calculate_structure_factor(_ni_phase(), [[1, 1, 1], [2, 0, 0]]))
    assert [f"{v:.1f}" for v in F] == ["11.8", "10.4"]
    atoms = [Atom("Si", [0, 0, 0]), Atom("Si", [1 / 3, 2 / 3, 0.5]), Atom("C", [0, 0, 0.188]),
             Atom("C", [1 / 3, 2 / 3, 0.688])]
    lat = (3.073, 3.073, 10.053, 90, 90, 120)
    phase = Phase("sic", Structure(atoms, Lattice(*lat)), space_group=osf.space_group_operations(186))
    rb = ok.reciprocal_base(ok.lattice_base(*lat))
    hkl = ok.enumerate_hkl(rb, 0.8)
    F = calculate_structure_factor(phase, hkl, "lobato")
    rot = np.unique(np.array([np.rint(R).astype(int) for R, _ in osf.space_group_operations(186)]), axis=0)
    key = [frozenset(tuple(r) for r in (h @ rot).tolist()) for h in hkl]
    first = {}
    for i, k in enumerate(key):
        first.setdefault(k, i)
    src = np.array([first[k] for k in key])
    g = np.sqrt(ok.g_squared(ok.g_cartesian(hkl[src], rb)))
    want = ok.structure_factor(hkl[src], g, [a.element for a in atoms], [a.xyz for a in atoms], [1.0] * 4,
                               np.zeros(4), "lobato")
    np.testing.assert_allclose(F, want, rtol=0, atol=1e-12 * np.max(np.abs(want)))
