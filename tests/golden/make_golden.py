"""Generate the golden fixtures in this folder from the reference itself.

Runs only where a diffsims checkout is available (default
``/root/reference``); the fixtures it writes are committed so the tests never
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
  ``get_kinematical_intensities`` on several structures.

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


def main(ref_root="/root/reference"):
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


if __name__ == "__main__":
    main(*sys.argv[1:])
