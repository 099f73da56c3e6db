"""CPU tests of the host side: the C-ABI library loads and exports every
declared entry, the host-only box rule matches the oracle, the conventions
of the drop-in types, and the reference's error behaviour."""
import ctypes
import pathlib
import re

import numpy as np
import pytest

from oracle import kinematic as ok

ROOT = pathlib.Path(__file__).resolve().parents[1]


@pytest.fixture(scope="module")
def lib():
    from diffsims_gb300 import _build, _native
    _build.build()
    return _native.load_library(require_cuda=False)


def declared_functions():
    names = []
    for h in (ROOT / "include").glob("*.h"):
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names += re.findall(r"\b(ds_[a-z0-9_]+)\s*\(", text)
    return sorted(set(names))


def test_library_exports_every_declared_symbol(lib):
    names = declared_functions()
    assert "ds_simulate" in names and "ds_enumerate_hkl" in names
    for name in names:
        assert hasattr(lib, name), f"{name} declared in include/ but not exported"
    from diffsims_gb300 import _native
    assert set(_native.EXPORTED_SYMBOLS) <= set(names)
    assert lib.ds_version().decode().startswith("diffsims_gb300")


@pytest.mark.parametrize("lat, r", [
    ((4.05, 4.05, 4.05, 90, 90, 90), 1.0),
    ((4.04, 4.04, 4.04, 90, 90, 90), 1 / 0.7),
    ((2.464, 2.464, 6.711, 90, 90, 120), 1.6768),
    ((9.1, 11.3, 12.7, 81.0, 97.0, 104.0), 2.0),
    ((7.1, 9.3, 12.4, 90, 90, 90), 1.5),
    ((3.0, 20.0, 7.5, 85.0, 95.0, 100.0), 1.5),
])
def test_box_extent_matches_oracle(lib, lat, r):
    from diffsims_gb300.engine import box_extent, reciprocal_basis
    from diffsims_gb300.crystal import Lattice
    recip = reciprocal_basis(Lattice(*lat))
    np.testing.assert_allclose(recip, ok.reciprocal_base(ok.lattice_base(*lat)), rtol=0, atol=0)
    np.testing.assert_array_equal(box_extent(recip, 1 / r), ok.highest_hkl(ok.reciprocal_base(ok.lattice_base(*lat)), 1 / r))


def test_box_extent_rejects_bad_arguments(lib):
    r = (ctypes.c_double * 9)(*([0.0] * 9))
    out = (ctypes.c_int32 * 3)()
    assert lib.ds_box_extent(r, -1.0, out) == 1
    assert "min_dspacing" in lib.ds_last_error().decode()


def test_euler_and_rotation_conventions():
    import diffsims_gb300 as ds
    e = np.array([[0, 90, 90], [10, 20, 30], [123, 45, 300]], dtype=float)
    np.testing.assert_allclose(ds.Rotation.from_euler(e, degrees=True).data, ok.euler_to_quaternion(e, True),
                               atol=1e-15)
    q = ok.random_quaternions(5, seed=3)
    np.testing.assert_allclose(ds.Rotation(q).to_matrix(), ok.quaternion_to_matrix(q), atol=1e-15)
    np.testing.assert_allclose(ds.Rotation.random(7, seed=0).data, ok.random_quaternions(7, seed=0))


def test_wavelength_matches_oracle():
    import diffsims_gb300 as ds
    for kv in (100, 200, 300, 80.5):
        assert ds.get_electron_wavelength(kv) == ok.electron_wavelength(kv)
    assert ds.get_electron_wavelength("inf") == 0


def test_generator_errors_and_repr():
    # diffsims/tests/generators/test_simulation_generator.py:122-135,268-280
    import diffsims_gb300 as ds
    g = ds.SimulationGenerator(300)
    assert repr(g) == "SimulationGenerator(accelerating_voltage=300, scattering_params=lobato, approximate_precession=True)"
    assert g.scattering_params == "lobato" and g.precession_angle == 0 and g.minimum_intensity == 1e-20
    with pytest.raises(NotImplementedError):
        ds.SimulationGenerator(300, scattering_params="_empty")
    with pytest.raises(NotImplementedError):
        ds.SimulationGenerator(300, shape_factor_model="dracula")
    for sp in ("lobato", "xtables", None):
        ds.SimulationGenerator(300, scattering_params=sp)


def test_settings_mapping():
    import diffsims_gb300 as ds
    from diffsims_gb300 import _native as N
    s = ds.SimulationGenerator(200, precession_angle=-0.5).settings(0.02)
    assert s.precession_mode == N.DS_PRECESSION_LORENTZIAN and np.isclose(s.precession_angle_rad, np.deg2rad(0.5))
    s = ds.SimulationGenerator(200, precession_angle=1, approximate_precession=False).settings(0.02, 0.03)
    assert s.precession_mode == N.DS_PRECESSION_INTEGRAL and s.shape_width == 0.03
    s = ds.SimulationGenerator(300, shape_factor_model="sinc", minima_number=3).settings()
    assert s.shape_model == "sinc" and s.minima_number == 3 and np.isclose(s.k0, 1 / ok.electron_wavelength(300))


def test_packed_atoms_layout():
    from diffsims_gb300 import _native as N
    assert ctypes.sizeof(N.ds_atom) == 48
    assert ctypes.sizeof(N.ds_sim_params) == 6 * 8 + 8 * 4
    assert N.ds_phase_table.recip.offset % 8 == 0


def test_debye_waller_rules():
    from diffsims_gb300.sim_utils import debye_waller_per_atom
    np.testing.assert_array_equal(debye_waller_per_atom(["Al", "Fe2+", "O"], {"Al": 0.5, "Fe": 0.3}), [0.5, 0.3, 0])
    np.testing.assert_array_equal(debye_waller_per_atom(["Al", "O"], [0.1, 0.2]), [0.1, 0.2])
    with pytest.raises(ValueError):
        debye_waller_per_atom(["Al", "O"], [0.1])


def test_get_closest_matches_reference_rule():
    from diffsims_gb300.simulation2d import _get_closest
    a = np.array([0.0, 1.0, 2.0, 3.0])
    np.testing.assert_array_equal(_get_closest(a, np.array([-1, 0.4, 0.5, 0.6, 2.9, 7.0])), [0, 0, 1, 1, 3, 3])


def test_raster_settings_struct():
    """ds_raster_params layout and the direct-beam default of
    get_diffraction_pattern (diffsims/simulations/simulation2d.py:404-411)."""
    import ctypes
    from diffsims_gb300 import _native as N
    from diffsims_gb300.engine import RasterSettings
    assert ctypes.sizeof(N.ds_raster_params) == 88
    p = RasterSettings((128, 100)).cstruct()
    assert (p.height, p.width, p.center_x, p.center_y, p.fast, p.normalize) == (128, 100, 50.0, 64.0, 1, 1)
    p = RasterSettings((128, 100), fast=False).cstruct()
    assert (p.center_x, p.center_y) == (49.5, 63.5)
    p = RasterSettings((10, 20), direct_beam_position=(3.5, 4.25), mirrored=True, sigma=2, truncate=3).cstruct()
    assert (p.center_x, p.center_y, p.mirrored, p.sigma, p.truncate) == (3.5, 4.25, 1, 2.0, 3.0)
    with pytest.raises(ValueError):
        RasterSettings(None).cstruct()


def test_precession_tight_quadrature_agrees_with_reference_quadrature():
    """The oracle's tight rotation average and the reference's adaptive
    quadrature agree where the latter converges (smooth models)."""
    s = np.array([0.001, -0.012, 0.02, 0.0, 0.03])
    r = np.array([0.5, 1.0, 1.3, 0.0, 1.6])
    for m in ("linear", "sin2c", "atanc", "lorentzian"):
        a = ok.sf_precession_integral_tight(s, r, np.deg2rad(1.0), m, 0.015)
        b = ok.sf_precession_integral(s, r, np.deg2rad(1.0), ok.ALL_SHAPE_MODELS[m], 0.015)
        np.testing.assert_allclose(a, b, rtol=1e-7, atol=1e-9)


# ---------------------------------------------------------------- failures on the host
def test_degenerate_and_non_finite_inputs_raise():
    """Bad cells and rotations are rejected on the host before any launch."""
    from diffsims_gb300.crystal import Rotation, diffpy_base, lattice_base
    for bad in [(4.0, 4.0, 4.0, 90, 90, 180), (4.0, 4.0, float("nan"), 90, 90, 90), (1, 1, 1, 10, 170, 90)]:
        with pytest.raises(ValueError):
            lattice_base(*bad)
        with pytest.raises(ValueError):
            diffpy_base(*bad)
    for q in ([0, 0, 0, 0], [1, float("nan"), 0, 0], [float("inf"), 0, 0, 0]):
        with pytest.raises(ValueError):
            Rotation(q)


def test_unknown_element_warns_with_zero_coefficients():
    """diffsims/utils/sim_utils.py:213-219: a warning and zero scattering
    coefficients (the packing runs on the host; a CPU tensor suffices)."""
    import torch
    from diffsims_gb300.sim_utils import PackedAtoms
    with pytest.warns(UserWarning, match="Xx"):
        a = PackedAtoms(["Fe", "Xx2+"], np.zeros((2, 3)), [1.0, 1.0], [0.0, 0.0], "lobato", torch.device("cpu"))
    coeffs = a.coeffs.numpy().reshape(-1, 10)
    assert np.any(coeffs[0] != 0) and np.all(coeffs[1] == 0)
    with pytest.raises(NotImplementedError):
        PackedAtoms(["Fe"], np.zeros((1, 3)), [1.0], [0.0], "waasmaier", torch.device("cpu"))


def test_new_entries_reject_bad_arguments_before_any_launch(lib):
    """Argument errors come back as DS_ERR_INVALID_ARGUMENT with a message,
    checked before any CUDA call (so this runs without a GPU)."""
    from diffsims_gb300 import _native as N
    r = (ctypes.c_double * 9)(*([0.25, 0, 0, 0, 0.25, 0, 0, 0, 0.25]))
    hm = (ctypes.c_int32 * 3)(2, 2, 2)
    fake = ctypes.c_void_p(4096)  # never dereferenced: validation fails first
    assert lib.ds_enumerate_sphere(r, hm, -1.0, fake, fake, 125, fake, fake, 1 << 20, fake, None) == N.DS_ERR_INVALID_ARGUMENT
    assert "radius" in lib.ds_last_error().decode()
    assert lib.ds_enumerate_sphere(r, hm, 1.0, fake, fake, 124, fake, fake, 1 << 20, fake, None) == N.DS_ERR_INVALID_ARGUMENT
    assert "capacity" in lib.ds_last_error().decode()
    neg = (ctypes.c_int32 * 3)(2, -1, 2)
    assert lib.ds_enumerate_sphere(r, neg, 1.0, fake, fake, 125, fake, fake, 1 << 20, fake, None) == N.DS_ERR_INVALID_ARGUMENT
    atoms = N.ds_atoms(1, 1, 4096, 4096, N.DS_SCATTER["lobato"], 0)
    assert lib.ds_family_structure_factors(atoms, fake, fake, 4, fake, fake, None) == N.DS_ERR_INVALID_ARGUMENT
    assert "kind" in lib.ds_last_error().decode()
    atoms = N.ds_atoms(1, 40, 4096, 4096, N.DS_SCATTER_DOYLETURNER, 0)
    assert lib.ds_family_structure_factors(atoms, fake, fake, 4, fake, fake, None) == N.DS_ERR_INVALID_ARGUMENT
    atoms = N.ds_atoms(1, 1, 4096 + 8, 4096, N.DS_SCATTER_KINEMATICAL, 0)
    assert lib.ds_family_structure_factors(atoms, fake, fake, 4, fake, fake, None) == N.DS_ERR_INVALID_ARGUMENT
    assert "aligned" in lib.ds_last_error().decode()
    atoms = N.ds_atoms(1, 1, 4096, 4096, N.DS_SCATTER_KINEMATICAL, 0)
    assert lib.ds_family_structure_factors(atoms, None, fake, 4, fake, fake, None) == N.DS_ERR_INVALID_ARGUMENT
    assert lib.ds_family_structure_factors(atoms, fake, fake, -1, fake, fake, None) == N.DS_ERR_INVALID_ARGUMENT


@pytest.mark.skipif(__import__("torch").cuda.is_available(), reason="checks the behaviour without a CUDA device")
def test_compute_calls_fail_loudly_without_a_gpu():
    """No CPU fallback: every compute entry of the package raises."""
    import diffsims_gb300 as ds
    from diffsims_gb300 import _native as N
    from diffsims_gb300 import structure_factor as gsf
    al = ds.Phase("Al", ds.Structure([ds.Atom("Al", [0, 0, 0])], ds.Lattice(4.05, 4.05, 4.05)))
    calls = [
        lambda: ds.SimulationGenerator(200).calculate_diffraction2d(al, ds.Rotation.identity()),
        lambda: ds.SimulationGenerator(200).calculate_diffraction1d(al),
        lambda: ds.get_kinematical_intensities(al.structure, [[1, 1, 1]], [0.4]),
        lambda: ds.DiffractionGenerator(200).calculate_ed_data(al.structure, 1.0),
        lambda: gsf.get_kinematical_structure_factor(al, [1, 1, 1], 0.2),
        lambda: gsf.calculate_structure_factor(al, [[1, 1, 1]]),
    ]
    for call in calls:
        with pytest.raises(N.NativeError):
            call()


def test_autotuner_disk_cache(tmp_path, monkeypatch):
    """Tile choices persist per GPU name and problem class; without a path
    nothing is read or written."""
    from diffsims_gb300.engine import Autotuner
    k = (32, 20, 17, "sinc", 0, "mixed")
    mem = Autotuner()
    assert mem.lookup("GB300", k) is None
    mem.store("GB300", k, (16, 6144))  # no path: a no-op
    assert not list(tmp_path.iterdir())
    path = tmp_path / "tiles.json"
    a = Autotuner(path=str(path))
    assert a.lookup("GB300", k) is None
    a.store("GB300", k, (32, 12288, 4))
    a.store("GB300", (1, 2, 3, "linear", 2, "fp64"), (8, 3072, 0))
    a.store("Other GPU", k, (8, 3072, 1))
    b = Autotuner(path=str(path))
    assert b.lookup("GB300", k) == (32, 12288, 4)
    assert b.lookup("Other GPU", k) == (8, 3072, 1)
    assert b.lookup("GB300", (1, 2, 3, "linear", 2, "fp64")) == (8, 3072, 0)
    # an entry written before the refine parts were tuned reads as the library's choice
    import json
    data = json.loads(path.read_text())
    data["GB300"][Autotuner._key_str(k)] = [16, 6144]
    path.write_text(json.dumps(data))
    assert Autotuner(path=str(path)).lookup("GB300", k) == (16, 6144, 0)
    path.write_text("not json")
    assert Autotuner(path=str(path)).lookup("GB300", k) is None  # a damaged file is ignored


def test_wait_limit_entries_reject_bad_arguments(lib):
    """ds_probe_wait_timeout validates its arguments before any CUDA call;
    ds_set_wait_limits accepts any value (<= 0 restores the defaults)."""
    from diffsims_gb300 import _native as N
    fake = ctypes.c_void_p(4096)
    assert lib.ds_probe_wait_timeout(0, fake, 512, fake, fake, None) == N.DS_ERR_INVALID_ARGUMENT
    assert "polls" in lib.ds_last_error().decode()
    assert lib.ds_probe_wait_timeout(1 << 21, fake, 512, fake, fake, None) == N.DS_ERR_INVALID_ARGUMENT
    assert lib.ds_probe_wait_timeout(100, fake, 16, fake, fake, None) == N.DS_ERR_INVALID_ARGUMENT
    assert "scratch" in lib.ds_last_error().decode()
    assert lib.ds_probe_wait_timeout(100, None, 512, fake, fake, None) == N.DS_ERR_INVALID_ARGUMENT
    assert lib.ds_set_wait_limits(5, 7) == N.DS_OK
    assert lib.ds_set_wait_limits(0, -1) == N.DS_OK


def test_custom_shape_functions_are_accepted():
    """A shape-factor function of the caller's (diffsims/generators/simulation_generator.py:117-120)
    is kept with its keyword arguments; the kernels then run with the model
    switched off (the function is applied between two launches); the
    reference's own model functions still map to their names."""
    import diffsims_gb300 as ds

    def local_excite(excitation_error, maximum_excitation_error, t):
        return (np.sin(t) * excitation_error) / maximum_excitation_error

    g = ds.SimulationGenerator(300, shape_factor_model=local_excite, t=0.2)
    assert g.shape_factor_model is local_excite and g.shape_factor_kwargs == {"t": 0.2}
    assert g._custom_shape is local_excite and g.settings().shape_model == "binary"
    with pytest.raises(TypeError):
        ds.SimulationGenerator(300, shape_factor_model="sinc", t=0.2)
    with pytest.raises(NotImplementedError):
        ds.SimulationGenerator(300, shape_factor_model=3.0)
    from diffsims_gb300.autograd import SpotModel
    with pytest.raises(NotImplementedError):
        SpotModel(["Si"], g, device="cpu")


def test_apply_shape_factors_rejects_bad_arguments(lib):
    from diffsims_gb300 import _native as N
    fake = ctypes.c_void_p(4096)
    out = N.ds_spots(4096, 4096, 4096, 10, 4096, None)
    assert lib.ds_apply_shape_factors(fake, fake, fake, fake, fake, -1, 1e-20, out, fake, 1 << 20, fake,
                                      None) == N.DS_ERR_INVALID_ARGUMENT
    assert lib.ds_apply_shape_factors(fake, fake, fake, fake, fake, 5, float("nan"), out, fake, 1 << 20, fake,
                                      None) == N.DS_ERR_INVALID_ARGUMENT
    assert "finite" in lib.ds_last_error().decode()
    assert lib.ds_apply_shape_factors(fake, fake, fake, fake, fake, 5, 1e-20, out, fake, 8, fake,
                                      None) == N.DS_ERR_INVALID_ARGUMENT
    assert "scratch" in lib.ds_last_error().decode()
    assert lib.ds_apply_shape_factors_scratch_bytes(100) >= 100 * 8


def test_status_bits_mirror_the_header_and_decode():
    """Every DS_ERR_* of include/diffsims_gb300.h has its value in _native,
    and the device-word bits raise their own errors (DS_ERR_BOUNDS comes from
    the bounds-checked build only)."""
    from diffsims_gb300 import _native as N
    text = (ROOT / "include" / "diffsims_gb300.h").read_text()
    found = dict((k, int(v)) for k, v in re.findall(r"\b(DS_ERR_[A-Z_]+)\s*=\s*(\d+)", text))
    assert found and found["DS_ERR_BOUNDS"] == 64
    for k, v in found.items():
        assert getattr(N, k) == v, k
    assert N.check_status_value(0, "x") == 0
    assert N.check_status_value(N.DS_ERR_CAPACITY, "x", allow=N.DS_ERR_CAPACITY) == N.DS_ERR_CAPACITY
    with pytest.raises(N.NativeError, match="bounds-checked"):
        N.check_status_value(N.DS_ERR_BOUNDS, "x")
    with pytest.raises(N.NativeError, match="timed out"):
        N.check_status_value(N.DS_ERR_TIMEOUT | N.DS_ERR_BOUNDS, "x")


def test_bounds_checked_build_is_a_separate_library():
    from diffsims_gb300 import _build, _native as N
    assert _build.LIB_DEBUG.name == "libdiffsims_gb300_debug.so" and _build.LIB_DEBUG != _build.LIB
    assert N._LIB_PATH.name == ("libdiffsims_gb300_debug.so" if N.DEBUG_BOUNDS else "libdiffsims_gb300.so")


def test_refine_parts_is_validated(lib):
    """refine_parts (reflections per refine / write unit) travels in the
    params struct; values other than 0, 1, 2, 4 and 8 are rejected with a
    message before any CUDA call."""
    import ctypes as C
    from diffsims_gb300 import _native as N
    from diffsims_gb300.engine import SimSettings
    for parts in (0, 1, 2, 4, 8):
        assert SimSettings(39.87, 0.02, 0.02, "lorentzian", refine_parts=parts).cstruct().refine_parts == parts
    t = N.ds_phase_table()
    t.n_hkl = 0
    fake = C.c_void_p(16)
    out = N.ds_spots(fake, fake, fake, 0, fake, None)
    for parts in (3, 16, -1):
        p = SimSettings(39.87, 0.02, 0.02, "lorentzian", refine_parts=parts).cstruct()
        assert lib.ds_simulate(p, t, fake, 1, out, fake, 1 << 20, fake, None) == N.DS_ERR_INVALID_ARGUMENT
        assert "refine_parts" in lib.ds_last_error().decode()
        assert lib.ds_simulate_batch(p, None, 0, out, fake, 1 << 20, fake, None) == N.DS_ERR_INVALID_ARGUMENT


def test_row_index_width_is_validated(lib):
    """ds_spots.hkl_index_bytes: 0 or 4 (int32 rows) everywhere, 2 (uint16
    rows) for ds_simulate with tables of at most 65536 rows; anything else is
    rejected with a message before any CUDA call."""
    import ctypes as C
    from diffsims_gb300 import _native as N
    from diffsims_gb300.engine import SimSettings
    p = SimSettings(39.87, 0.02, 0.02, "lorentzian").cstruct()
    fake = C.c_void_p(16)
    t = N.ds_phase_table()
    for n_hkl, width in ((70000, 2), (100, 3), (100, 8), (100, -4)):
        t.n_hkl = n_hkl
        out = N.ds_spots(fake, fake, fake, 0, fake, None, width, 0)
        assert lib.ds_simulate(p, t, fake, 1, out, fake, 1 << 20, fake, None) == N.DS_ERR_INVALID_ARGUMENT
        assert "hkl_index_bytes" in lib.ds_last_error().decode()
    out = N.ds_spots(fake, fake, fake, 0, fake, None, 2, 0)
    phases = (N.ds_batch_phase * 1)()
    assert lib.ds_simulate_batch(p, phases, 1, out, fake, 1 << 20, fake, None) == N.DS_ERR_INVALID_ARGUMENT
    assert "hkl_index_bytes" in lib.ds_last_error().decode()
    assert lib.ds_apply_shape_factors(fake, fake, fake, fake, fake, 5, 1e-20, out, fake, 1 << 20, fake,
                                      None) == N.DS_ERR_INVALID_ARGUMENT
    assert "hkl_index_bytes" in lib.ds_last_error().decode()
    assert C.sizeof(N.ds_spots) == 6 * 8 + 2 * 4


def test_phase_spots_select_and_copy():
    """PhaseSpots.select gathers whole patterns of the CSR (an index, a slice
    or an array, in the given order) and deepcopy owns its arrays; checked
    on CPU tensors against a direct numpy gather."""
    import copy
    import torch
    from diffsims_gb300.engine import PhaseSpots
    rng = np.random.default_rng(2)
    counts = rng.integers(0, 5, 9)
    off = np.zeros(10, dtype=np.int64)
    off[1:] = np.cumsum(counts)
    total = int(off[-1])
    idx = rng.integers(0, 100, total).astype(np.int32)
    xyzi = rng.random((total, 4)).astype(np.float32)
    s = rng.random(total)
    sp = PhaseSpots(None, torch.as_tensor(off), torch.as_tensor(idx), torch.as_tensor(xyzi), total, torch.as_tensor(s))
    sp._hkl_rows = rng.integers(-5, 5, (100, 3)).astype(np.float64)
    for pick in (3, slice(2, 7), slice(None, None, -2), np.array([8, 0, 0, 5])):
        sel = sp.select(pick)
        want = np.atleast_1d(np.arange(9)[pick])
        assert sel.n_orient == len(want)
        rows = np.concatenate([np.arange(off[i], off[i + 1]) for i in want]) if len(want) else np.zeros(0, int)
        np.testing.assert_array_equal(sel.offsets.numpy(), np.r_[0, np.cumsum(counts[want])])
        np.testing.assert_array_equal(sel.hkl_index.numpy(), idx[rows])
        np.testing.assert_array_equal(sel.xyzi.numpy(), xyzi[rows])
        np.testing.assert_array_equal(sel.excitation_error.numpy(), s[rows])
        assert sel.total == len(rows) and sel._hkl_rows is sp._hkl_rows
    c = copy.deepcopy(sp)
    c.xyzi.zero_()
    assert np.array_equal(sp.xyzi.numpy(), xyzi) and c.total == total


def test_row_storage_helpers_and_pool_by_index_type(monkeypatch):
    """uint16 table rows (held in int16 tensors) widen to their unsigned
    values on the device and read as uint16 on the host; tables above 65536
    rows keep int32; the page-locked pool hands out a set only for the index
    type it was made with (checked on CPU tensors)."""
    import torch
    from diffsims_gb300 import engine
    rows = torch.tensor([0, 1, 32767, -32768, -1], dtype=torch.int16)
    assert engine._rows_int32(rows).dtype == torch.int32
    assert engine._rows_int32(rows).tolist() == [0, 1, 32767, 32768, 65535]
    host = engine._rows_numpy(rows)
    assert host.dtype == np.uint16 and host.tolist() == [0, 1, 32767, 32768, 65535]
    wide = torch.tensor([5, 70000], dtype=torch.int32)
    assert engine._rows_int32(wide) is wide and engine._rows_numpy(wide).dtype == np.int32

    class Table:
        n = 65536
    assert engine._row_index_dtype(Table) == torch.int16
    Table.n = 65537
    assert engine._row_index_dtype(Table) == torch.int32

    real_empty = torch.empty
    monkeypatch.setattr(engine.torch, "empty", lambda *a, pin_memory=False, **k: real_empty(*a, **k))
    pool = engine.HostSpotPool()
    a = pool.acquire(10, 100, torch.int16)
    assert a[1].dtype == torch.int16 and pool.allocated_bytes == 14 * 8 + 1024 * 18
    b = pool.acquire(10, 100, torch.int32)  # the free int16 set is not of this type
    assert b is not a and b[1].dtype == torch.int32
    assert pool.acquire(10, 50, torch.int16) is a


def test_polar_and_pointer_query_arguments(lib):
    """ds_polar_flatten and ds_polar_flatten_f32 reject negative sizes, one
    axis without the other and empty axes before any CUDA call;
    ds_host_mapped needs its output pointer and reports null as unmapped."""
    import ctypes as C
    from diffsims_gb300 import _native as N
    fake = C.c_void_p(16)
    for entry in (lib.ds_polar_flatten, lib.ds_polar_flatten_f32):
        assert entry(fake, fake, -1, 4, None, 0, None, 0, fake, fake, fake, None) == N.DS_ERR_INVALID_ARGUMENT
        assert "negative size" in lib.ds_last_error().decode()
        assert entry(fake, fake, 3, 4, fake, 5, None, 0, fake, fake, fake, None) == N.DS_ERR_INVALID_ARGUMENT
        assert "both axes" in lib.ds_last_error().decode()
        assert entry(fake, fake, 3, 4, fake, 0, fake, 7, fake, fake, fake, None) == N.DS_ERR_INVALID_ARGUMENT
        assert "empty axes" in lib.ds_last_error().decode()
        assert entry(fake, fake, 0, 4, None, 0, None, 0, fake, fake, fake, None) == N.DS_OK  # nothing to do
    assert lib.ds_host_mapped(None, None) == N.DS_ERR_INVALID_ARGUMENT
    out = C.c_int32(7)
    assert lib.ds_host_mapped(None, C.byref(out)) == N.DS_OK and out.value == 0
