"""Generate the golden fixtures in this folder from the reference itself.

Runs only where a diffsims checkout is available (its path is the one
required argument); the fixtures it writes are committed so the tests never
need the reference.  What it does:

* copies the reference's golden detector image
  ``diffsims/tests/generators/old_simulation.npy`` (graphite P6/mmm, 200 kV,
  Euler (0, 90, 90) deg, 128x128, sigma 1.4, calibration 0.0262; checked at
  diffsims/tests/generators/test_simulation_generator.py:283-343);
* imports the reference's own ``diffsims/utils/sim_utils.py`` and
  ``diffsims/utils/shape_factor_models.py`` (unchanged; orix, diffpy and numba
  are absent, so the package ``__init__`` files are bypassed and ``diffpy`` is
  a stub module -- sim_utils uses it only in docstrings) and records their
  outputs on seeded inputs: wavelengths, every shape-factor model, the
  Lorentzian precession form, the ``quad`` precession integral and
  ``get_kinematical_intensities`` on several structures;
* imports the reference's own ``diffsims/structure_factor/`` modules
  (``atomic_scattering_parameters``, ``atomic_scattering_factor``,
  ``structure_factor``; diffpy's ``expandPosition`` / ``SymmetryConstraints``
  are stubbed by the oracle's restatement of them, over space-group
  operations the oracle generates) and records the family structure factors,
  Doyle-Turner parameters, atomic scattering factors and refraction-corrected
  wavelengths of several phases (``reference_structure_factor.npz``);
* imports the reference's own ``diffsims/generators/diffraction_generator.py``
  (numba, matplotlib and PIL stubbed -- used only by code this path does not
  run; transforms3d's ``euler2mat`` and diffpy's ``Lattice`` are the
  oracle's restatements) and records ``DiffractionGenerator.calculate_ed_data``
  outputs for several structures, rotations, shape models and precession
  settings (``reference_legacy.npz``).

Usage::

    python tests/golden/make_golden.py [/path/to/diffsims-checkout]
"""
import pathlib
import sys
import types

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parents[1]))

from oracle import kinematic as ok  # noqa: E402  (oracle provides hkl sets and lattices)


def load_reference(ref_root):
    for name in ["diffpy", "diffpy.structure", "diffpy.structure.symmetryutilities"]:
        sys.modules.setdefault(name, types.ModuleType(name))
    sys.modules["diffpy"].structure = sys.modules["diffpy.structure"]
    sym = sys.modules["diffpy.structure.symmetryutilities"]
    sys.modules["diffpy.structure"].symmetryutilities = sym
    sym.expandPosition = None
    sym.SymmetryConstraints = None
    for pkg, sub in [("diffsims", "diffsims"), ("diffsims.utils", "diffsims/utils"),
                     ("diffsims.structure_factor", "diffsims/structure_factor")]:
        if pkg not in sys.modules:
            m = types.ModuleType(pkg)
            m.__path__ = [str(pathlib.Path(ref_root) / sub)]
            sys.modules[pkg] = m
    import diffsims.utils.sim_utils as su
    import diffsims.utils.shape_factor_models as sfm
    return su, sfm


class _Site:
    def __init__(self, element, xyz, occ):
        self.element, self.xyz, self.occupancy = element, np.asarray(xyz, float), float(occ)


class _Lattice:
    """stdbase/recbase such that inv(stdbase @ recbase) is the identity,
    the x || a, z || c* case of diffsims/utils/sim_utils.py:290-291."""
    def __init__(self, base):
        self.stdbase = base
        self.recbase = np.linalg.inv(base)


class _Structure(list):
    def __init__(self, sites, base):
        super().__init__(sites)
        self.lattice = _Lattice(base)


def structures():
    """Named test structures: (lattice params, elements, xyz, occupancy, per-element B)."""
    out = {}
    out["al_fcc"] = ((4.05, 4.05, 4.05, 90, 90, 90), ["Al"] * 4,
                     [[0, 0, 0], [0, .5, .5], [.5, 0, .5], [.5, .5, 0]], [1.0] * 4, {"Al": 0.5})
    xyz = []
    for c in [[0, 0, 0], [0.5, 0, 0.5], [0, 0.5, 0.5], [0.5, 0.5, 0]]:
        xyz += [c, [c[0] + .25, c[1] + .25, c[2] + .25]]
    out["si_fd3m"] = ((5.431,) * 3 + (90, 90, 90), ["Si"] * 8, xyz, [1.0] * 8, {})
    rng = np.random.default_rng(7)
    n = 60
    els = list(rng.choice(["C", "N", "O", "Si", "Fe"], n))
    out["p1_60"] = ((9.1, 11.3, 12.7, 81.0, 97.0, 104.0), els, rng.random((n, 3)).tolist(),
                    rng.uniform(0.5, 1.0, n).tolist(), {"C": 0.4, "N": 0.6, "O": 0.8, "Si": 1.1, "Fe": 1.4})
    out["graphite"] = ((2.464, 2.464, 6.711, 90, 90, 120), ["C"] * 4,
                       [[0, 0, .25], [0, 0, .75], [1 / 3, 2 / 3, .25], [2 / 3, 1 / 3, .75]], [1.0] * 4, {})
    out["unknown"] = ((3.5236,) * 3 + (90, 90, 90), ["UnOb", "Ni2+"], [[0, 0, 0], [.5, .5, 0]],
                      [1.0, 1.0], {"Ni": 0.3})
    return out


def main(ref_root):
    su, sfm = load_reference(ref_root)
    old = np.load(pathlib.Path(ref_root) / "diffsims/tests/generators/old_simulation.npy")
    np.save(HERE / "graphite_pattern_128.npy", old)

    g = {}
    g["wavelength_kv"] = np.array([100.0, 200.0, 300.0, 80.0, 120.0])
    g["wavelength"] = np.array([su.get_electron_wavelength(v) for v in g["wavelength_kv"]])

    rng = np.random.default_rng(11)
    for w in (0.01, 0.015, 0.02):
        s = np.concatenate([[0.0, w, -w, w / 5, -2 * w / 5, 1e-12, -1e-12],
                            np.linspace(-1.3 * w, 1.3 * w, 101), rng.uniform(-w, w, 64)])
        key = f"w{w}"
        g[f"shape_s_{key}"] = s
        g[f"shape_linear_{key}"] = sfm.linear(s.copy(), w)
        g[f"shape_sinc_{key}"] = sfm.sinc(s.copy(), w)
        g[f"shape_sinc3_{key}"] = sfm.sinc(s.copy(), w, minima_number=3)
        g[f"shape_sin2c_{key}"] = sfm.sin2c(s.copy(), w)
        with np.errstate(invalid="ignore", divide="ignore"):
            g[f"shape_atanc_{key}"] = sfm.atanc(s.copy(), w)
        g[f"shape_lorentzian_{key}"] = sfm.lorentzian(s.copy(), w)
        r = rng.uniform(0.0, 2.0, s.shape)
        g[f"shape_r_{key}"] = r
        for deg in (0.5, 1.0):
            g[f"shape_lprec{deg}_{key}"] = sfm.lorentzian_precession(s.copy(), w, r, np.deg2rad(deg))

    # adaptive-quadrature precession integral, a few spots per model
    s = np.array([-0.012, -0.004, 0.0, 0.003, 0.0095, 0.02])
    r = np.array([0.3, 1.1, 0.7, 1.9, 0.05, 1.4])
    g["quad_s"], g["quad_r"] = s, r
    for name in ("linear", "sinc", "sin2c", "atanc", "lorentzian", "binary"):
        fn = getattr(sfm, name)
        with np.errstate(invalid="ignore", divide="ignore"):
            g[f"quad_{name}"] = sfm._shape_factor_precession(s, r, np.deg2rad(0.5), fn, 0.01)

    # kinematical intensities through the reference's get_kinematical_intensities
    for name, (lat, els, xyz, occ, dw) in structures().items():
        base = ok.lattice_base(*lat)
        rb = ok.reciprocal_base(base)
        hkl = ok.enumerate_hkl(rb, 1.0 / 1.5, n_zero=1)
        if hkl.shape[0] > 600:
            hkl = np.vstack([hkl[rng.choice(hkl.shape[0] - 1, 599, replace=False)], hkl[-1:]])
        gsp = np.sqrt(ok.g_squared(ok.g_cartesian(hkl, rb)))
        struct = _Structure([_Site(e, x, o) for e, x, o in zip(els, xyz, occ)], base)
        pref = rng.uniform(0.1, 1.0, hkl.shape[0])
        for sp in ("lobato", "xtables", None):
            import warnings
            with warnings.catch_warnings():
                warnings.simplefilter("ignore")
                val = su.get_kinematical_intensities(struct, hkl, gsp, debye_waller_factors=dw,
                                                     scattering_params=sp, prefactor=pref)
            g[f"kin_{name}_{sp}"] = val
        g[f"kin_{name}_hkl"] = hkl
        g[f"kin_{name}_gspacing"] = gsp
        g[f"kin_{name}_prefactor"] = pref
    np.savez_compressed(HERE / "reference_numerics.npz", **g)
    print("wrote", HERE / "reference_numerics.npz", len(g), "arrays")


class _SfAtom:
    def __init__(self, element, xyz, occ, biso):
        self.element, self.xyz, self.occupancy, self.Bisoequiv = element, np.asarray(xyz, float), occ, biso


class _SfLattice:
    def __init__(self, params):
        from oracle import structure_factor_families as osf
        self.volume = osf.cell_volume(*params)


class _SfStructure(list):
    def __init__(self, atoms, params):
        super().__init__(atoms)
        self.lattice = _SfLattice(params)
        self.xyz = np.array([a.xyz for a in atoms])


class _SfSpaceGroup:
    def __init__(self, number):
        from oracle import structure_factor_families as osf
        self.number = number
        self.ops = osf.space_group_operations(number)


class _SfPhase:
    def __init__(self, sg, atoms, params):
        self.space_group = _SfSpaceGroup(sg)
        self.structure = _SfStructure(atoms, params)


def sf_phases():
    """Named phases: (space group, lattice params, atoms (element, xyz, occupancy, Bisoequiv))."""
    b = 8 * np.pi ** 2 * 0.006332
    rng = np.random.default_rng(23)
    out = {
        "nickel": (225, (3.5236,) * 3 + (90, 90, 90), [("Ni0+", [0, 0, 0], 1.0, b)]),
        "ferrite": (229, (2.8665,) * 3 + (90, 90, 90), [("Fe", [0, 0, 0], 1.0, b), ("Fe", [.5, .5, .5], 1.0, b)]),
        "sic4h": (186, (3.073, 3.073, 10.053, 90, 90, 120),
                  [("Si", [0, 0, 0], 1.0, b), ("Si", [0.33, 0.667, 0.25], 1.0, b),
                   ("C", [0, 0, 0.188], 1.0, b), ("C", [0.333, 0.667, 0.438], 1.0, b)]),
        # a mixed site at a general position of Pm-3m (orbit of 48), then other atoms
        "mixed_pm3m": (221, (4.1,) * 3 + (90, 90, 90),
                       [("Fe", [0.11, 0.23, 0.37], 0.6, 0.4), ("Ni", [0.11, 0.23, 0.37], 0.4, 0.7),
                        ("O", [0.5, 0.5, 0.5], 1.0, 0.9)]),
        "p1_random": (1, (7.3, 8.1, 9.6, 84.0, 96.0, 101.0),
                      [(str(e), x, float(o), float(bb)) for e, x, o, bb in
                       zip(rng.choice(["C", "N", "O", "Si", "Fe", "Cu"], 30), rng.random((30, 3)),
                           rng.uniform(0.5, 1.0, 30), rng.uniform(0.2, 1.5, 30))]),
        "pm1_centric": (2, (5.2, 6.3, 7.4, 88.0, 92.0, 95.0),
                        [("Ti", [0.21, 0.34, 0.45], 1.0, 0.5), ("O", [0.1, 0.6, 0.2], 1.0, 0.8)]),
    }
    return out


def load_reference_structure_factor(ref_root):
    from oracle import structure_factor_families as osf
    load_reference(ref_root)
    sym = sys.modules["diffpy.structure.symmetryutilities"]

    def expand_position(spacegroup, xyz, sgoffset=(0, 0, 0), eps=None):
        # (positions, operations per position, multiplicity); the reference reads [0]
        return list(osf.orbit(spacegroup.ops, xyz)), None, None

    class SymmetryConstraints:
        def __init__(self, spacegroup, positions):
            core = []
            for p in positions:
                p = np.asarray(p, float)
                if not any(any(np.all(np.abs((q - p) - np.rint(q - p)) < 1e-5) for q in osf.orbit(spacegroup.ops, c))
                           for c in core):
                    core.append(p)
            self.corepos = core

    sym.expandPosition = expand_position
    sym.SymmetryConstraints = SymmetryConstraints
    import diffsims.structure_factor.atomic_scattering_parameters as asp
    import diffsims.structure_factor.atomic_scattering_factor as asf
    import diffsims.structure_factor.structure_factor as ssf
    return asp, asf, ssf


def main_structure_factor(ref_root):
    asp, asf, ssf = load_reference_structure_factor(ref_root)
    rng = np.random.default_rng(29)
    g = {}
    for name, (sg, params, atoms) in sf_phases().items():
        phase = _SfPhase(sg, [_SfAtom(*a) for a in atoms], params)
        hkl = rng.integers(-7, 8, (48, 3)).astype(np.float64)
        hkl = np.vstack([hkl, [[0, 0, 0], [1, 1, 1], [0.5, -1.25, 2.0]]])
        s = rng.uniform(0.0, 1.6, hkl.shape[0])
        s[-3] = 0.0
        g[f"{name}_hkl"], g[f"{name}_s"] = hkl, s
        g[f"{name}_asym"] = np.asarray(ssf.find_asymmetric_positions(phase.structure.xyz, phase.space_group))
        g[f"{name}_kin"] = np.array([ssf.get_kinematical_structure_factor(phase, h, si) for h, si in zip(hkl, s)])
        for kv in (20e3, 200e3):
            vals = [ssf.get_doyleturner_structure_factor(phase, h, si, kv, return_parameters=True)
                    for h, si in zip(hkl, s)]
            g[f"{name}_dt{int(kv)}"] = np.array([v[0] for v in vals])
            g[f"{name}_dt{int(kv)}_vg"] = np.array([v[1]["v_g"] for v in vals])
            g[f"{name}_dt{int(kv)}_vmod"] = np.array([v[1]["v_mod"] for v in vals])
        g[f"{name}_voltages"] = np.array([10e3, 20e3, 100e3, 200e3, 300e3])
        g[f"{name}_wavelength"] = np.array([ssf.get_refraction_corrected_wavelength(phase, v)
                                            for v in g[f"{name}_voltages"]])
    # atomic scattering factors and parameters
    els = ["H", "C", "O", "Si", "Fe", "Ni", "Cu", "Au", "U", "Bk"]
    s = np.linspace(0.0, 1.8, 13)
    g["atom_elements"] = np.array(els)
    g["atom_s"] = s
    g["atom_kin"] = np.array([[asf.get_kinematical_atomic_scattering_factor(_SfAtom(e, [0, 0, 0], 0.7, 0.45), si)
                               for si in s] for e in els])
    g["atom_dt"] = np.array([[asf.get_doyleturner_atomic_scattering_factor(_SfAtom(e, [0, 0, 0], 0.7, 0.45), si, 61.3)
                              for si in s] for e in els])
    g["atom_params"] = np.array([np.concatenate(asp.get_atomic_scattering_parameters(e)) for e in els])
    np.savez_compressed(HERE / "reference_structure_factor.npz", **g)
    print("wrote", HERE / "reference_structure_factor.npz", len(g), "arrays")


def _stub_module(name, **attrs):
    m = sys.modules.get(name) or types.ModuleType(name)
    for k, v in attrs.items():
        setattr(m, k, v)
    sys.modules[name] = m
    return m


def load_reference_legacy(ref_root):
    from oracle import legacy as ol
    load_reference(ref_root)

    def _decorator(*args, **kwargs):
        if len(args) == 1 and callable(args[0]) and not kwargs:
            return args[0]
        return lambda f: f

    _stub_module("numba", jit=_decorator, njit=_decorator, prange=range,
                 config=types.SimpleNamespace(NUMBA_DEFAULT_NUM_THREADS=1))
    _stub_module("matplotlib")
    _stub_module("matplotlib.pyplot")
    _stub_module("PIL", ImageDraw=None, Image=None)
    _stub_module("PIL.ImageDraw")
    _stub_module("PIL.Image")

    def euler2mat(ai, aj, ak, axes="sxyz"):
        assert axes == "rzxz"
        return ol.euler2mat_rzxz(ai, aj, ak)

    _stub_module("transforms3d")
    _stub_module("transforms3d.euler", euler2mat=euler2mat)
    for pkg, sub in [("diffsims.generators", "diffsims/generators"), ("diffsims.sims", "diffsims/sims"),
                     ("diffsims.pattern", "diffsims/pattern")]:
        if pkg not in sys.modules:
            m = types.ModuleType(pkg)
            m.__path__ = [str(pathlib.Path(ref_root) / sub)]
            sys.modules[pkg] = m
    import diffsims.generators.diffraction_generator as dg
    return dg


class _LegacySite:
    def __init__(self, element, xyz, occ):
        self.element, self.xyz, self.occupancy = element, np.asarray(xyz, float), float(occ)


class _LegacyStructure(list):
    def __init__(self, sites, lattice):
        super().__init__(sites)
        self.lattice = lattice


def legacy_structures():
    """Named structures for the legacy path: (lattice params, elements, xyz, occupancy)."""
    xyz = []
    for c in [[0, 0, 0], [0.5, 0, 0.5], [0, 0.5, 0.5], [0.5, 0.5, 0]]:
        xyz += [c, [c[0] + .25, c[1] + .25, c[2] + .25]]
    rng = np.random.default_rng(31)
    return {
        "si": ((5.431,) * 3 + (90, 90, 90), ["Si"] * 8, xyz, [1.0] * 8),
        "graphite": ((2.464, 2.464, 6.711, 90, 90, 120), ["C"] * 4,
                     [[0, 0, .25], [0, 0, .75], [1 / 3, 2 / 3, .25], [2 / 3, 1 / 3, .75]], [1.0] * 4),
        "p1": ((6.3, 7.1, 8.2, 84.0, 97.0, 103.0), list(rng.choice(["C", "O", "Si", "Fe"], 12)),
               rng.random((12, 3)).tolist(), rng.uniform(0.6, 1.0, 12).tolist()),
    }


def legacy_cases():
    """(structure, kwargs of DiffractionGenerator, kwargs of calculate_ed_data)."""
    cases = []
    for name, rot in [("si", (0, 0, 0)), ("si", (10, 20, 30)), ("graphite", (0, 90, 90)),
                      ("p1", (35, 47, 112)), ("p1", (-80, 133, 5))]:
        cases.append((name, dict(accelerating_voltage=300), dict(reciprocal_radius=2.0, rotation=rot)))
    for model in ("linear", "sinc", "sin2c", "atanc"):
        cases.append(("si", dict(accelerating_voltage=200, shape_factor_model=model),
                      dict(reciprocal_radius=2.5, rotation=(5, 12, 40), max_excitation_error=0.02)))
    cases.append(("p1", dict(accelerating_voltage=200, precession_angle=0.5),
                  dict(reciprocal_radius=1.5, rotation=(12, 34, 56))))
    cases.append(("p1", dict(accelerating_voltage=200, precession_angle=0.5, approximate_precession=False,
                             shape_factor_model="linear"),
                  dict(reciprocal_radius=1.2, rotation=(12, 34, 56))))
    cases.append(("graphite", dict(accelerating_voltage=200, scattering_params="xtables"),
                  dict(reciprocal_radius=3.0, rotation=(0, 0, 0), shape_factor_width=0.05,
                       debye_waller_factors={"C": 0.6})))
    cases.append(("si", dict(accelerating_voltage=300), dict(reciprocal_radius=5.0)))
    return cases


def profile_cases():
    """(structure, reciprocal_radius, DiffractionGenerator kwargs) of the 1-D profiles."""
    return [("si", 1.0, {}), ("si", 2.5, {}), ("ni_hex", 1.0, {}), ("graphite", 2.0, {}),
            ("p1", 1.2, {}), ("p1", 1.6, {"scattering_params": "xtables"})]


def main_legacy(ref_root):
    from oracle import legacy as ol
    dg = load_reference_legacy(ref_root)
    g = {}
    structs = legacy_structures()
    for i, (name, gen_kw, call_kw) in enumerate(legacy_cases()):
        lat, els, xyz, occ = structs[name]
        structure = _LegacyStructure([_LegacySite(e, x, o) for e, x, o in zip(els, xyz, occ)],
                                     ol.DiffpyLattice(*lat))
        gen = dg.DiffractionGenerator(**gen_kw)
        sim = gen.calculate_ed_data(structure, **call_kw)
        g[f"case{i}_coordinates"] = np.asarray(sim._coordinates)
        g[f"case{i}_indices"] = np.asarray(sim._indices)
        g[f"case{i}_intensities"] = np.asarray(sim._intensities)
    g["n_cases"] = np.array(len(legacy_cases()))
    # 1-D profiles (calculate_profile_data)
    profile_structs = dict(structs, ni_hex=((3.0, 3.0, 5.0, 90, 90, 120), ["Ni"], [[0, 0, 0]], [1.0]))
    for j, (name, r, kw) in enumerate(profile_cases()):
        lat, els, xyz, occ = profile_structs[name]
        structure = _LegacyStructure([_LegacySite(e, x, o) for e, x, o in zip(els, xyz, occ)],
                                     ol.DiffpyLattice(*lat))
        prof = dg.DiffractionGenerator(300, **kw).calculate_profile_data(structure, reciprocal_radius=r)
        g[f"profile{j}_magnitudes"] = np.asarray(prof.magnitudes, dtype=np.float64)
        g[f"profile{j}_intensities"] = np.asarray(prof.intensities, dtype=np.float64)
        g[f"profile{j}_hkls"] = np.asarray(prof.hkls, dtype=str)
    np.savez_compressed(HERE / "reference_legacy.npz", **g)
    print("wrote", HERE / "reference_legacy.npz", len(g), "arrays")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py /path/to/diffsims-checkout")
    main(sys.argv[1])
    main_structure_factor(sys.argv[1])
    main_legacy(sys.argv[1])
