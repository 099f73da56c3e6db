"""1-D profiles (``SimulationGenerator.calculate_diffraction1d``): the oracle
and the package's symmetry-family logic against the reference's known
answers, and the package's host path against the oracle -- CPU only (the
GPU enumeration / structure-factor helper is replaced by the oracle here;
tests/test_gpu_diffraction1d.py runs the real one).

Known answers: diffsims/tests/crystallography/test_reciprocal_lattice_vector.py:155-186
(ferrite families at d >= 1 Angstrom after unique(use_symmetry=True)), the
multiplicity doctest at diffsims/crystallography/reciprocal_lattice_vector.py:303-311,
diffsims/tests/simulations/test_simulations1d.py:66-73 (repr, theta) and
diffsims/tests/generators/test_simulation_generator.py:225-246 (hkil).
"""
import numpy as np
import pytest

from oracle import kinematic as ok
from oracle import structure_factor_families as osf

FERRITE_G = [0.34885749, 0.69771498, 0.493359, 0.78006907, 0.98671799, 0.604238, 0.85452285]
FERRITE_D = [2.8665, 1.43325, 2.02692159, 1.28193777, 1.01346079, 1.65497455, 1.17024372]
FERRITE_S = [0.17442875, 0.34885749, 0.2466795, 0.39003453, 0.493359, 0.30211945, 0.42726142]


def rotations(sg):
    return np.unique(np.array([np.rint(R).astype(int) for R, _ in osf.space_group_operations(sg)]), axis=0)


def crystals():
    return {
        "al": (225, ok.Crystal((4.05,) * 3 + (90, 90, 90), ["Al"] * 4,
                               [[0, 0, 0], [0, .5, .5], [.5, 0, .5], [.5, .5, 0]], B=[0.5] * 4)),
        "ferrite": (229, ok.Crystal((2.8665,) * 3 + (90, 90, 90), ["Fe"] * 2, [[0, 0, 0], [.5, .5, .5]])),
        "sic": (186, ok.Crystal((3.073, 3.073, 10.053, 90, 90, 120), ["Si", "Si", "C", "C"],
                                [[0, 0, 0], [1 / 3, 2 / 3, 0.5], [0, 0, 0.188], [1 / 3, 2 / 3, 0.688]])),
        "p1": (1, ok.Crystal((5.1, 6.2, 7.3, 84.0, 97.0, 103.0), ["C", "O", "Fe"],
                             [[0.1, 0.2, 0.3], [0.6, 0.1, 0.8], [0.4, 0.7, 0.2]])),
        "pm1": (2, ok.Crystal((5.1, 6.2, 7.3, 84.0, 97.0, 103.0), ["Si", "O"], [[0.1, 0.2, 0.3], [0.6, 0.1, 0.8]])),
    }


def ferrite_families(fn):
    rb = crystals()["ferrite"][1].rbase
    hkl = ok.enumerate_hkl(rb, 1.0)
    reps, mult = fn(hkl, rb, rotations(229))
    return hkl[reps], np.sqrt(ok.g_squared(ok.g_cartesian(hkl[reps], rb))), mult


@pytest.mark.parametrize("which", ["oracle", "package"])
def test_ferrite_families_kat(which):
    from diffsims_gb300.generator import symmetry_families
    fn = ok.unique_with_symmetry if which == "oracle" else symmetry_families
    hkl, g, mult = ferrite_families(fn)
    assert np.allclose(g, FERRITE_G)
    assert np.allclose(1 / g, FERRITE_D)
    assert np.allclose(g / 2, FERRITE_S)
    assert hkl.tolist() == [[1, 0, 0], [2, 0, 0], [1, 1, 0], [2, 1, 0], [2, 2, 0], [1, 1, 1], [2, 1, 1]]
    assert mult.tolist() == [6, 6, 12, 24, 12, 8, 24]


def test_multiplicity_doctest():
    from diffsims_gb300.generator import symmetry_families
    rb = crystals()["al"][1].rbase
    reps, mult = symmetry_families(np.array([[1, 1, 1], [2, 0, 0]]), rb, rotations(225))
    assert sorted(mult.tolist()) == [6, 8]
    assert dict(zip(reps.tolist(), mult.tolist())) == {0: 8, 1: 6}


@pytest.mark.parametrize("name", list(crystals()))
def test_package_symmetry_families_match_oracle(name):
    from diffsims_gb300.generator import symmetry_families
    sg, cr = crystals()[name]
    hkl = ok.enumerate_hkl(cr.rbase, 0.7)
    a = symmetry_families(hkl, cr.rbase, rotations(sg))
    b = ok.unique_with_symmetry(hkl, cr.rbase, rotations(sg))
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1], b[1])
    assert a[1].sum() == hkl.shape[0]  # the families partition the set


def _phase_of(name):
    from diffsims_gb300.crystal import Atom, Lattice, Phase, Structure
    sg, cr = crystals()[name]
    atoms = [Atom(e, x) for e, x in zip(cr.elements, cr.xyz)]
    return Phase(name, Structure(atoms, Lattice(*cr.lattice)), space_group=osf.space_group_operations(sg)), cr


@pytest.mark.parametrize("name", list(crystals()))
def test_package_host_path_matches_oracle(monkeypatch, name):
    import diffsims_gb300 as ds
    from diffsims_gb300 import generator
    phase, cr = _phase_of(name)

    def rows(phase_, dmin, sp, dw):
        # the oracle in place of the GPU enumeration and structure factors
        assert dmin == 0.7
        hkl = ok.enumerate_hkl(cr.rbase, dmin)
        g = np.sqrt(ok.g_squared(ok.g_cartesian(hkl, cr.rbase)))
        B = [dw.get(e, 0) for e in cr.elements] if dw else np.zeros(len(cr.elements))
        F2 = ok.kinematical_intensities(hkl, g, cr.elements, cr.xyz, cr.occupancy, B, sp)
        return hkl.astype(np.int64), g, F2

    monkeypatch.setattr(generator, "_min_dspacing_rows", rows)
    dw = {e: b for e, b in zip(cr.elements, cr.B)}
    sim = ds.SimulationGenerator(300).calculate_diffraction1d(phase, 0.5, debye_waller_factors=dw)
    g, inten, idx = ok.diffraction1d(cr, rotations(crystals()[name][0]))
    np.testing.assert_array_equal(sim.hkl, idx)
    np.testing.assert_allclose(sim.reciprocal_spacing, g, rtol=1e-15)
    np.testing.assert_allclose(sim.intensities, inten, rtol=1e-12, atol=1e-12)
    assert sim.reciprocal_radius == 0.5 and sim.wavelength == ds.SimulationGenerator(300).wavelength
    assert len(sim.hkl[0]) == (4 if name == "sic" else 3)
    assert np.max(sim.intensities) == 100


def test_simulation1d_container():
    # diffsims/tests/simulations/test_simulations1d.py:66-73
    from diffsims_gb300.crystal import Phase
    from diffsims_gb300.simulation1d import Simulation1D
    sim = Simulation1D(Phase("Al"), np.array([1, 2, 3]), np.array([1, 2, 3]),
                       np.array([[1, 0, 0], [1, 1, 0], [1, 1, 1]]), 4.0, 0.025)
    assert repr(sim) == "Simulation1D(name: Al, wavelength: 0.025)"
    np.testing.assert_almost_equal(sim.theta, np.array([0.02499479, 0.0499584, 0.07485985]))
