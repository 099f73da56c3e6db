"""GPU parity of the legacy ``DiffractionGenerator.calculate_ed_data`` path
(sphere enumeration + the orientation kernel) against the reference's own
outputs (tests/golden/reference_legacy.npz) and the FP64 oracle.

Bars, as for the current path: identical spot sets except selection flips
within 1e-9 1/Angstrom of the cutoff (counted) and spots that are FP64
round-off on the reference side; intensities within 1e-5 relative;
positions within 1e-5 |g|.
"""
import os
import warnings

import numpy as np
import pytest

from oracle import kinematic as ok
from oracle import legacy as ol
from tests.golden.make_golden import _LegacySite, _LegacyStructure, legacy_cases, legacy_structures

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ref(golden_dir):
    return dict(np.load(os.path.join(golden_dir, "reference_legacy.npz")))


def structure_of(name, diffpy_lattice=True):
    from diffsims_gb300.crystal import Lattice
    lat, els, xyz, occ = legacy_structures()[name]
    lattice = ol.DiffpyLattice(*lat) if diffpy_lattice else Lattice(*lat)
    return _LegacyStructure([_LegacySite(e, x, o) for e, x, o in zip(els, xyz, occ)], lattice)


def run_case(i, form="mixed", diffpy_lattice=True):
    from diffsims_gb300.diffraction_generator import DiffractionGenerator
    name, gk, ck = legacy_cases()[i]
    gen = DiffractionGenerator(**gk)
    return gen.calculate_ed_data(structure_of(name, diffpy_lattice), form=form, **ck)


def excitation_error_of(i, hkl):
    """FP64 excitation error of one reflection in case i, and whether the
    boundary test is the precession band."""
    name, gk, ck = legacy_cases()[i]
    lat = ol.DiffpyLattice(*legacy_structures()[name][0])
    g = ol.euler2mat_rzxz(*np.deg2rad(ck.get("rotation", (0, 0, 0)))) @ (np.asarray(hkl, float) @ lat.recbase.T)
    k0 = 1 / ok.electron_wavelength(gk["accelerating_voltage"])
    r = np.hypot(g[0], g[1])
    s = -np.sqrt(k0 ** 2 - r ** 2) + k0 - g[2]
    eps = ck.get("max_excitation_error", 1e-2)
    phi = np.deg2rad(gk.get("precession_angle", 0))
    if phi == 0:
        return abs(abs(s) - eps)
    pz, pt = k0 * np.cos(phi), k0 * np.sin(phi)
    up = pz - np.sqrt(k0 ** 2 - (r + pt) ** 2)
    do = pz - np.sqrt(k0 ** 2 - (r - pt) ** 2)
    return min(abs(up - (g[2] - eps)), abs((g[2] + eps) - do))


def compare(i, sim, coords, idx, inten, rtol=1e-5, atol_rel=0.0):
    got = {tuple(h): k for k, h in enumerate(sim._hkl)}
    want = {tuple(h): k for k, h in enumerate(idx)}
    flips = 0
    scale = np.max(inten) if inten.size else 1.0
    for h in set(got) ^ set(want):
        if h in want and inten[want[h]] <= 1e-24 * scale:
            continue
        d = excitation_error_of(i, h)
        assert d < 1e-9, f"case {i}: hkl {h} differs (on gpu: {h in got}), boundary distance {d:.3e}"
        flips += 1
    common = sorted(set(got) & set(want), key=lambda h: want[h])
    # the reference's order is kept
    order = [got[h] for h in common]
    assert order == sorted(order)
    a = np.array([got[h] for h in common], dtype=int)
    b = np.array([want[h] for h in common], dtype=int)
    Ig, Ir = sim._I[a], inten[b]
    np.testing.assert_allclose(Ig, Ir, rtol=rtol, atol=max(1e-24 * scale, atol_rel * scale))
    gn = np.maximum(np.linalg.norm(coords[b], axis=1), 1e-3)
    assert np.all(np.abs(sim._xyz[a] - coords[b]).max(axis=1) <= 1e-5 * gn)
    return flips


@pytest.mark.parametrize("i", range(len(legacy_cases())))
def test_matches_reference_fixtures(ref, i):
    sim = run_case(i)
    assert sim.with_direct_beam
    # the precession average is checked against the reference's adaptive
    # quadrature within that quadrature's own absolute error
    atol_rel = 1e-8 if legacy_cases()[i][1].get("approximate_precession", True) is False else 0.0
    flips = compare(i, sim, ref[f"case{i}_coordinates"], ref[f"case{i}_indices"], ref[f"case{i}_intensities"],
                    atol_rel=atol_rel)
    assert flips <= 2


@pytest.mark.parametrize("i", [0, 3, 5, 9, 11])
def test_fp64_form_and_parameter_lattice(i):
    """The FP64 form against the oracle; a lattice given by parameters
    (diffpy's standard frame built here) gives the same spots."""
    from tests.test_oracle_legacy import oracle_case
    c, idx, inten, _ = oracle_case(i, quad=False)
    compare(i, run_case(i, form="fp64"), c, idx, inten, rtol=1e-6)  # FP64 arithmetic, float32 output
    compare(i, run_case(i, diffpy_lattice=False), c, idx, inten)


def test_many_rotations_in_one_launch():
    """A batch of Euler triples gives, bit for bit, the single-call results."""
    from diffsims_gb300.diffraction_generator import DiffractionGenerator
    gen = DiffractionGenerator(200, shape_factor_model="sinc")
    st = structure_of("p1")
    rng = np.random.default_rng(8)
    eul = rng.uniform(-180, 180, (64, 3))
    many = gen.calculate_ed_data(st, 1.5, rotation=eul)
    assert len(many) == 64
    for k in (0, 17, 63):
        one = gen.calculate_ed_data(st, 1.5, rotation=eul[k])
        np.testing.assert_array_equal(one._hkl, many[k]._hkl)
        np.testing.assert_array_equal(one._I, many[k]._I)
        np.testing.assert_array_equal(one._xyz, many[k]._xyz)


def test_sphere_enumeration_matches_oracle():
    """ds_enumerate_sphere: the reference's hkl list, in its order, for
    several cells and radii (down to a sphere holding only 000)."""
    import torch
    from diffsims_gb300.engine import PhaseTable
    from diffsims_gb300.sim_utils import PackedAtoms
    dev = torch.device("cuda", 0)
    atoms = PackedAtoms(["Si"], np.zeros((1, 3)), [1.0], [0.0], "lobato", dev)
    for p, r in [((5.431,) * 3 + (90, 90, 90), 5.0), ((6.3, 7.1, 8.2, 84, 97, 103), 1.5),
                 ((2.464, 2.464, 6.711, 90, 90, 120), 3.0), ((4.0, 4.0, 4.0, 90, 90, 90), 0.2),
                 ((12.1, 3.3, 7.7, 95, 88, 101), 2.2)]:
        lat = ol.DiffpyLattice(*p)
        want, _, gsp = ol.points_in_sphere(lat.reciprocal(), r)
        t = PhaseTable.sphere(np.linalg.inv(lat.base).T, atoms, r, device=dev)
        np.testing.assert_array_equal(t.hkl.cpu().numpy(), want.astype(np.int32))
        np.testing.assert_allclose(np.sqrt(t.g2.cpu().numpy()), gsp, rtol=1e-14)


def test_reference_structural_checks():
    # diffsims/tests/generators/test_diffraction_generator.py:131-215
    from diffsims_gb300.diffraction_generator import DiffractionGenerator

    def si(a):
        xyz = []
        for c in [[0, 0, 0], [0.5, 0, 0.5], [0, 0.5, 0.5], [0.5, 0.5, 0]]:
            xyz += [c, [c[0] + .25, c[1] + .25, c[2] + .25]]
        return _LegacyStructure([_LegacySite("Si", x, 1.0) for x in xyz], ol.DiffpyLattice(a, a, a, 90, 90, 90))

    gen = DiffractionGenerator(300)
    assert gen.scattering_params == "lobato" and gen.precession_angle == 0
    assert gen.approximate_precession is True and gen.minimum_intensity == 1e-20
    d = gen.calculate_ed_data(si(5.431), reciprocal_radius=5.0)
    assert len(d.indices) == len(d.coordinates) == len(d.intensities)
    small, big = gen.calculate_ed_data(si(5), 5.0), gen.calculate_ed_data(si(10), 5.0)
    ia, ib = [tuple(x) for x in small.indices], [tuple(x) for x in big.indices]
    assert (2, 2, 0) in ia and (2, 2, 0) in ib
    np.testing.assert_allclose(small.coordinates[ia.index((2, 2, 0))], 2 * big.coordinates[ib.index((2, 2, 0))],
                               rtol=1e-6)
    i0 = [tuple(x) for x in d.indices].index((0, 0, 0))
    assert np.all(d.intensities[i0] >= d.intensities)
    t1 = gen.calculate_ed_data(si(5.431), 2, max_excitation_error=0.02)
    t2 = gen.calculate_ed_data(si(5.431), 2, max_excitation_error=0.4)
    assert np.sum(t1.intensities) != np.sum(t2.intensities)
    for kw in (dict(precession_angle=0.5, approximate_precession=True),
               dict(precession_angle=0.5, approximate_precession=False)):
        p = DiffractionGenerator(300, **kw).calculate_ed_data(si(5.431), reciprocal_radius=5.0)
        assert len(p.indices) == len(p.coordinates) == len(p.intensities) > 0
    with pytest.raises(NotImplementedError):
        DiffractionGenerator(300, shape_factor_model="dracula")
    with pytest.raises(NotImplementedError):
        DiffractionGenerator(300, scattering_params="_empty")
    nobeam = gen.calculate_ed_data(si(5.431), 2.0, with_direct_beam=False)
    assert (0, 0, 0) not in [tuple(x) for x in nobeam.indices]


def test_library_generator_matches_single_calls():
    """get_diffraction_library (library_generator.py:51-155): every entry
    equals its own calculate_ed_data call; pixel coordinates are
    rint(calibrated xy + half_shape)."""
    from diffsims_gb300.diffraction_generator import DiffractionGenerator
    from diffsims_gb300.library import DiffractionLibraryGenerator, StructureLibrary
    gen = DiffractionGenerator(300)
    eul_si = [(0, 0, 0), (10, 20, 30), (45, 54.7356, 0)]
    eul_p1 = [(12, 34, 56)]
    sl = StructureLibrary(["si", "p1"], [structure_of("si"), structure_of("p1")], [eul_si, eul_p1])
    lib = DiffractionLibraryGenerator(gen).get_diffraction_library(sl, 0.02, 1.5, (72, 72), with_direct_beam=False)
    assert lib.reciprocal_radius == 1.5 and lib.with_direct_beam is False
    for name, eul in (("si", eul_si), ("p1", eul_p1)):
        entry = lib[name]
        assert list(entry["orientations"]) == eul
        for k, e in enumerate(eul):
            one = gen.calculate_ed_data(structure_of(name), 1.5, rotation=e, with_direct_beam=False)
            sim = entry["simulations"][k]
            np.testing.assert_array_equal(sim.indices, one.indices)
            np.testing.assert_array_equal(entry["intensities"][k], one.intensities)
            np.testing.assert_array_equal(entry["pixel_coords"][k],
                                          np.rint(one.coordinates[:, :2] / 0.02 + 72).astype(int))
    e = lib.get_library_entry("si", (10, 20, 30))
    assert e["Sim"] is lib["si"]["simulations"][1]


@pytest.mark.parametrize("j", range(6))
def test_profiles_match_reference_fixtures(ref, j):
    """calculate_profile_data (diffraction_generator.py:333-416): the
    reference's labels in its order, magnitudes and intensities (1e-9 on the
    0-100 scale: FP64 on both sides)."""
    from diffsims_gb300.diffraction_generator import DiffractionGenerator
    from tests.golden.make_golden import profile_cases
    from tests.test_oracle_legacy import profile_structures
    name, r, kw = profile_cases()[j]
    lat, els, xyz, occ = profile_structures()[name]
    st = _LegacyStructure([_LegacySite(e, x, o) for e, x, o in zip(els, xyz, occ)], ol.DiffpyLattice(*lat))
    prof = DiffractionGenerator(300, **kw).calculate_profile_data(st, reciprocal_radius=r)
    assert list(prof.hkls) == list(ref[f"profile{j}_hkls"])
    np.testing.assert_allclose(prof.magnitudes, ref[f"profile{j}_magnitudes"], rtol=1e-13)
    np.testing.assert_allclose(prof.intensities, ref[f"profile{j}_intensities"], rtol=1e-9, atol=1e-9)


@pytest.mark.parametrize("kw", [dict(), dict(in_plane_angle=30.0), dict(mirrored=True, sigma=2.0),
                                dict(shape=(200, 200), direct_beam_position=(80, 120), sigma=3.0)])
def test_legacy_drawing_methods_match_reference_recipe(kw):
    """DiffractionSimulation.get_diffraction_pattern (GPU rasteriser) and
    get_as_mask against the reference's recipes restated in the oracle
    (diffsims/sims/diffraction_simulation.py:235-354).  Patterns with a spot
    within 1e-4 px of a pixel edge (float32 positions may truncate the other
    way) are left out and counted."""
    compared = 0
    for case in (1, 3, 4, 9):
        sim = run_case(case)
        sim.calibration = 0.01
        shape = kw.get("shape", (512, 512))
        args = {k: v for k, v in kw.items() if k != "shape"}
        dbp = args.get("direct_beam_position") or (shape[1] // 2, shape[0] // 2)
        pos = ol.transformed_coordinates(sim.calibrated_coordinates, args.get("in_plane_angle", 0), dbp,
                                         args.get("mirrored", False))
        fr = pos[:, :2] - np.floor(pos[:, :2])
        if np.any(((fr < 1e-4) | (fr > 1 - 1e-4)) & (np.abs(sim.calibrated_coordinates) > 0)):
            continue
        got = sim.get_diffraction_pattern(shape, **args)
        want = ol.legacy_diffraction_pattern(sim.calibrated_coordinates, sim.intensities, shape, **args)
        np.testing.assert_allclose(got, want, rtol=0, atol=2e-6 * max(np.abs(want).max(), 1e-300))
        margs = {k: v for k, v in args.items() if k != "sigma"}
        for negative, rf in ((True, None), (False, np.sqrt)):
            m = sim.get_as_mask(shape, radius=4.5, negative=negative, radius_function=rf, **margs)
            mw = ol.legacy_mask(sim.calibrated_coordinates, sim.intensities, shape, radius=4.5, negative=negative,
                                radius_function=rf, **margs)
            assert np.array_equal(m, mw)
        compared += 1
    assert compared >= 1
