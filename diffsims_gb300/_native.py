"""ctypes binding of libdiffsims_gb300.so (the C ABI in include/diffsims_gb300.h).

There is no CPU fallback: if the library is missing or no CUDA device is
present, every compute entry raises.
"""
from __future__ import annotations

import ctypes as C
import os
import pathlib
import threading

import torch

# DIFFSIMS_GB300_DEBUG_BOUNDS=1 loads the bounds-checked build
# (libdiffsims_gb300_debug.so, kernels compiled with -DDS_DEBUG_BOUNDS: every
# checked index outside its array sets DS_ERR_BOUNDS in the status word and
# the access is skipped); `python -m diffsims_gb300._build --debug` builds it.
DEBUG_BOUNDS = os.environ.get("DIFFSIMS_GB300_DEBUG_BOUNDS", "") == "1"
_LIB_PATH = pathlib.Path(__file__).resolve().parent / (
    "libdiffsims_gb300_debug.so" if DEBUG_BOUNDS else "libdiffsims_gb300.so")
_lock = threading.Lock()
_lib = None

# status codes / enums (mirror include/diffsims_gb300.h)
DS_OK = 0
DS_ERR_INVALID_ARGUMENT = 1
DS_ERR_CUDA = 2
DS_ERR_CAPACITY = 4
DS_ERR_TIMEOUT = 8
DS_ERR_UNSUPPORTED = 16
DS_ERR_NONFINITE = 32
DS_ERR_BOUNDS = 64

DS_FORM_MIXED = 0
DS_FORM_FP64 = 1

DS_SCATTER = {"lobato": 0, "xtables": 1, None: 2}
DS_SCATTER_KINEMATICAL = 3
DS_SCATTER_DOYLETURNER = 4
DS_SHAPE = {"linear": 0, "atanc": 1, "sinc": 2, "sin2c": 3, "lorentzian": 4, "binary": 5}
DS_SCREEN = {"auto": 0, "rows": 1, "lines": 2, "bricks": 3}
DS_PRECESSION_NONE = 0
DS_PRECESSION_LORENTZIAN = 1
DS_PRECESSION_INTEGRAL = 2

EXPORTED_SYMBOLS = (
    "ds_box_extent", "ds_enumerate_scratch_bytes", "ds_enumerate_hkl", "ds_enumerate_sphere",
    "ds_structure_factor_scratch_bytes", "ds_structure_factors", "ds_kinematical_intensities",
    "ds_family_structure_factors", "ds_simulate_scratch_bytes", "ds_simulate", "ds_simulate_noalloc",
    "ds_simulate_batch_scratch_bytes", "ds_simulate_batch_tile",
    "ds_simulate_batch", "ds_rasterize_scratch_bytes", "ds_rasterize",
    "ds_simulate_backward_scratch_bytes", "ds_simulate_backward", "ds_structure_factors_backward_scratch_bytes",
    "ds_axis_angle_compose", "ds_axis_angle_compose_backward", "ds_polar_flatten", "ds_structure_factors_backward",
    "ds_probe_fp32_fma", "ds_set_wait_limits", "ds_probe_wait_timeout", "ds_apply_shape_factors_scratch_bytes",
    "ds_apply_shape_factors", "ds_host_mapped", "ds_polar_flatten_f32", "ds_last_error", "ds_version",
)


class ds_atom(C.Structure):
    _fields_ = [("x", C.c_double), ("y", C.c_double), ("z", C.c_double), ("occupancy", C.c_double),
                ("B", C.c_double), ("species", C.c_int32), ("_pad", C.c_int32)]


class ds_atoms(C.Structure):
    _fields_ = [("n_atoms", C.c_int32), ("n_species", C.c_int32), ("atoms", C.c_void_p),
                ("coeffs", C.c_void_p), ("kind", C.c_int32), ("_pad", C.c_int32)]


class ds_sim_params(C.Structure):
    _fields_ = [("k0", C.c_double), ("max_excitation_error", C.c_double), ("shape_width", C.c_double),
                ("precession_angle", C.c_double), ("minimum_intensity", C.c_double),
                ("minima_number", C.c_double), ("shape_model", C.c_int32), ("precession_mode", C.c_int32),
                ("form", C.c_int32), ("orient_tile", C.c_int32), ("stage_cap", C.c_int32), ("screen", C.c_int32),
                ("refine_parts", C.c_int32), ("_reserved", C.c_int32)]


class ds_phase_table(C.Structure):
    _fields_ = [("n_hkl", C.c_int64), ("hkl", C.c_void_p), ("g2", C.c_void_p), ("F2", C.c_void_p),
                ("F2d", C.c_void_p), ("recip", C.c_double * 9), ("hmax", C.c_int32 * 3), ("_pad", C.c_int32)]


class ds_batch_phase(C.Structure):
    _fields_ = [("table", ds_phase_table), ("quats", C.c_void_p), ("n_orient", C.c_int64)]


class ds_spots(C.Structure):
    _fields_ = [("offsets", C.c_void_p), ("hkl_index", C.c_void_p), ("xyzi", C.c_void_p),
                ("capacity", C.c_int64), ("total", C.c_void_p), ("excitation_error", C.c_void_p),
                ("hkl_index_bytes", C.c_int32), ("_reserved", C.c_int32)]


class ds_raster_params(C.Structure):
    _fields_ = [("height", C.c_int32), ("width", C.c_int32), ("mirrored", C.c_int32), ("fast", C.c_int32),
                ("normalize", C.c_int32), ("_pad", C.c_int32), ("sigma", C.c_double), ("calibration", C.c_double),
                ("center_x", C.c_double), ("center_y", C.c_double), ("in_plane_angle", C.c_double),
                ("clip_threshold", C.c_double), ("truncate", C.c_double), ("pixel_snap", C.c_double)]


assert C.sizeof(ds_atom) == 48
assert C.sizeof(ds_sim_params) == 80


class NativeError(RuntimeError):
    """A C-ABI call returned an error status."""


def library_path() -> pathlib.Path:
    return _LIB_PATH


def load_library(require_cuda: bool = True):
    """Load the CUDA library once; raise if it is missing (no fallback)."""
    global _lib
    with _lock:
        if _lib is None:
            if not _LIB_PATH.exists():
                raise NativeError(f"{_LIB_PATH.name} is not built: run `python -c \"import __graft_entry__ as g; "
                                  f"g.build()\"` (the CUDA path has no CPU fallback)")
            lib = C.CDLL(str(_LIB_PATH))
            vp, i32, i64, sz, dp = C.c_void_p, C.c_int32, C.c_int64, C.c_size_t, C.c_double
            lib.ds_box_extent.argtypes = [C.POINTER(C.c_double), dp, C.POINTER(C.c_int32)]
            lib.ds_enumerate_scratch_bytes.argtypes = [C.POINTER(C.c_int32)]
            lib.ds_enumerate_scratch_bytes.restype = sz
            lib.ds_enumerate_hkl.argtypes = [C.POINTER(C.c_double), C.POINTER(C.c_int32), dp, i32, vp, vp, i64, vp,
                                             vp, sz, vp, vp]
            lib.ds_enumerate_sphere.argtypes = [C.POINTER(C.c_double), C.POINTER(C.c_int32), dp, vp, vp, i64, vp,
                                                vp, sz, vp, vp]
            lib.ds_structure_factor_scratch_bytes.argtypes = [i64, i32]
            lib.ds_structure_factor_scratch_bytes.restype = sz
            lib.ds_structure_factors.argtypes = [C.POINTER(ds_atoms), vp, vp, vp, i64, i32, vp, vp, vp, vp, sz, vp, vp]
            lib.ds_kinematical_intensities.argtypes = [C.POINTER(ds_atoms), vp, vp, vp, i64, vp, vp, sz, vp, vp]
            lib.ds_family_structure_factors.argtypes = [C.POINTER(ds_atoms), vp, vp, i64, vp, vp, vp]
            lib.ds_simulate_scratch_bytes.argtypes = [C.POINTER(ds_sim_params), C.POINTER(ds_phase_table), i64]
            lib.ds_simulate_scratch_bytes.restype = sz
            lib.ds_simulate.argtypes = [C.POINTER(ds_sim_params), C.POINTER(ds_phase_table), vp, i64,
                                        C.POINTER(ds_spots), vp, sz, vp, vp]
            lib.ds_simulate_batch_scratch_bytes.argtypes = [C.POINTER(ds_sim_params), C.POINTER(ds_batch_phase), i32]
            lib.ds_simulate_batch_scratch_bytes.restype = sz
            lib.ds_simulate_batch_tile.argtypes = [C.POINTER(ds_sim_params), C.POINTER(ds_batch_phase), i32]
            lib.ds_simulate_batch_tile.restype = i32
            lib.ds_simulate_batch.argtypes = [C.POINTER(ds_sim_params), C.POINTER(ds_batch_phase), i32,
                                              C.POINTER(ds_spots), vp, sz, vp, vp]
            lib.ds_rasterize_scratch_bytes.argtypes = [C.POINTER(ds_raster_params), i64]
            lib.ds_rasterize_scratch_bytes.restype = sz
            lib.ds_rasterize.argtypes = [C.POINTER(ds_raster_params), vp, vp, i64, i64, vp, vp, sz, vp, vp]
            lib.ds_simulate_backward_scratch_bytes.argtypes = [C.POINTER(ds_sim_params), i64, i64]
            lib.ds_simulate_backward_scratch_bytes.restype = sz
            lib.ds_simulate_backward.argtypes = [C.POINTER(ds_sim_params), C.POINTER(ds_phase_table), vp, i64, vp,
                                                 vp, i64, vp, vp, vp, vp, vp, sz, vp, vp]
            lib.ds_structure_factors_backward_scratch_bytes.argtypes = [i64, i32]
            lib.ds_structure_factors_backward_scratch_bytes.restype = sz
            lib.ds_structure_factors_backward.argtypes = [C.POINTER(ds_atoms), vp, vp, i64, C.POINTER(C.c_double), vp,
                                                          vp, vp, vp, sz, vp]
            lib.ds_axis_angle_compose.argtypes = [vp, vp, i64, vp, vp]
            lib.ds_polar_flatten.argtypes = [vp, vp, i64, i64, vp, i64, vp, i64, vp, vp, vp, vp]
            lib.ds_polar_flatten_f32.argtypes = [vp, vp, i64, i64, vp, i64, vp, i64, vp, vp, vp, vp]
            lib.ds_axis_angle_compose_backward.argtypes = [vp, vp, i64, vp, vp, vp]
            lib.ds_probe_fp32_fma.argtypes = [i64, i32, vp, vp]
            lib.ds_set_wait_limits.argtypes = [i64, i64]
            lib.ds_apply_shape_factors_scratch_bytes.argtypes = [i64]
            lib.ds_apply_shape_factors_scratch_bytes.restype = sz
            lib.ds_apply_shape_factors.argtypes = [vp, vp, vp, vp, vp, i64, dp, C.POINTER(ds_spots), vp, sz, vp, vp]
            lib.ds_probe_wait_timeout.argtypes = [i64, vp, sz, vp, vp, vp]
            lib.ds_host_mapped.argtypes = [vp, C.POINTER(C.c_int32)]
            lib.ds_last_error.restype = C.c_char_p
            lib.ds_version.restype = C.c_char_p
            for name in ("ds_box_extent", "ds_enumerate_hkl", "ds_structure_factors", "ds_kinematical_intensities",
                         "ds_family_structure_factors", "ds_enumerate_sphere",
                         "ds_simulate", "ds_simulate_batch", "ds_rasterize", "ds_simulate_backward",
                         "ds_structure_factors_backward",
                         "ds_axis_angle_compose", "ds_axis_angle_compose_backward", "ds_polar_flatten",
                         "ds_probe_fp32_fma", "ds_set_wait_limits", "ds_probe_wait_timeout",
                         "ds_apply_shape_factors", "ds_host_mapped", "ds_polar_flatten_f32"):
                getattr(lib, name).restype = C.c_int32
            _lib = lib
    if require_cuda and not torch.cuda.is_available():
        raise NativeError("diffsims_gb300 needs a CUDA device (GB300, sm_103a); none is visible")
    return _lib


def check(status: int, what: str):
    if status != DS_OK:
        msg = _lib.ds_last_error().decode() if _lib is not None else ""
        if status == DS_ERR_INVALID_ARGUMENT:
            raise ValueError(f"{what}: {msg}")
        if status == DS_ERR_UNSUPPORTED:
            raise NotImplementedError(f"{what}: {msg}")
        raise NativeError(f"{what}: status {status}: {msg}")


def check_device_status(status_tensor: torch.Tensor, what: str, allow=0) -> int:
    """Read the device status word (synchronises) and raise on unexpected bits."""
    return check_status_value(int(status_tensor.item()), what, allow)


def check_status_value(v: int, what: str, allow=0) -> int:
    """Raise on the unexpected bits of a status word already read."""
    bad = v & ~allow
    if bad & DS_ERR_TIMEOUT:
        raise NativeError(f"{what}: a bounded device wait timed out (status {v})")
    if bad & DS_ERR_NONFINITE:
        raise ValueError(f"{what}: non-finite input (status {v})")
    if bad & DS_ERR_BOUNDS:
        raise NativeError(f"{what}: an index check of the bounds-checked build failed (status {v})")
    if bad:
        raise NativeError(f"{what}: device status {v}")
    return v


def host_mapped(ptr: int) -> bool:
    """Whether host address ``ptr`` is page-locked memory that kernels address
    at the same value (``ds_host_mapped``)."""
    out = C.c_int32(0)
    check(load_library().ds_host_mapped(C.c_void_p(int(ptr)), C.byref(out)), "host_mapped")
    return bool(out.value)


def set_wait_limits(lookback_polls: int = 0, mbarrier_polls: int = 0):
    """Polls before the kernels' bounded waits give up (DS_ERR_TIMEOUT) for
    launches set up from now on: the decoupled look-back's wait for an
    earlier tile and the structure-factor kernels' wait for a staging copy.
    0 restores the defaults (2^24 and 2^22 polls)."""
    check(load_library(require_cuda=False).ds_set_wait_limits(int(lookback_polls), int(mbarrier_polls)),
          "set_wait_limits")


def ptr(t: torch.Tensor | None):
    return None if t is None else C.c_void_p(t.data_ptr())


def stream_handle(stream: torch.cuda.Stream | None = None):
    s = stream if stream is not None else torch.cuda.current_stream()
    return C.c_void_p(s.cuda_stream)
