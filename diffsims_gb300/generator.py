"""``SimulationGenerator``: drop-in for
diffsims/generators/simulation_generator.py (``calculate_diffraction2d``)
running on the CUDA library."""
from __future__ import annotations

import time
from concurrent.futures import ThreadPoolExecutor
from typing import Sequence, Union

import numpy as np
import torch

from . import _native as N
from .crystal import Phase, Rotation, lattice_params, quaternions_of, structure_of
from .engine import (HostSpotPool, PhaseBatch, PhaseTable, SimSettings, SpotBuffers, custom_shape_spots,
                     reciprocal_basis, simulate_phase, simulate_phase_streamed, simulate_phase_to_host)
from .simulation1d import Simulation1D
from .simulation2d import Simulation2D
from . import interop
from .symmetry import point_group_rotations, symmetry_families
from .sim_utils import get_electron_wavelength

_SHAPE_NAMES = ("linear", "atanc", "sinc", "sin2c", "lorentzian")


def _shape_name(model):
    """Name of a built-in shape model given by name or by function (the
    reference's functions in diffsims.utils.shape_factor_models, or any
    function with the same name and module tail)."""
    if isinstance(model, str):
        return model
    name = getattr(model, "__name__", None)
    mod = getattr(model, "__module__", "") or ""
    if name in _SHAPE_NAMES + ("binary",) and mod.endswith("shape_factor_models"):
        return name
    return None


# ------------------------------------------------------------ 1-D profiles
def _min_dspacing_rows(phase, min_dspacing, scattering_params, debye_waller_factors):
    """hkl rows of ReciprocalLatticeVector.from_min_dspacing (GPU enumeration),
    their |g| and FP64 |F|^2 (GPU structure factors)."""
    N.load_library()
    dev = torch.device("cuda", torch.cuda.current_device())
    table = PhaseTable(phase, 1.0 / min_dspacing, False, scattering_params, debye_waller_factors, form="fp64",
                       device=dev)
    if table.n == 0:
        return np.zeros((0, 3), dtype=np.int64), np.zeros(0), np.zeros(0)
    torch.cuda.current_stream().synchronize()
    return (table.hkl_host().astype(np.int64), np.sqrt(table.g2.cpu().numpy()),
            table.F2d[:table.n].cpu().numpy())


def _caller_rotations(caller_rotation, rots, single_phase):
    """The caller's rotation objects for a reference-type result (orix
    ``Rotation``); the identity as an orix ``Rotation`` when none was given."""
    if caller_rotation is None:
        from orix.quaternion import Rotation as OrixRotation
        ident = OrixRotation.identity()
        return ident if single_phase else [ident] * len(rots)
    return caller_rotation


def _is_hexagonal(lattice) -> bool:
    return bool(np.allclose(lattice_params(lattice)[3:], [90, 90, 120]))



class SimulationGenerator:
    """Kinematic diffraction simulations on the GPU.

    Constructor arguments as diffsims/generators/simulation_generator.py:74-128:
    ``accelerating_voltage`` (kV), ``scattering_params`` ('lobato', 'xtables'
    or None), ``precession_angle`` (degrees), ``shape_factor_model`` (one of
    'linear', 'atanc', 'sinc', 'sin2c', 'lorentzian', or the reference's model
    functions), ``approximate_precession``, ``minimum_intensity`` and keyword
    arguments for the shape model (``minima_number``).
    """

    def __init__(self, accelerating_voltage: float = 200, scattering_params: str = "lobato",
                 precession_angle: float = 0, shape_factor_model="lorentzian", approximate_precession: bool = True,
                 minimum_intensity: float = 1e-20, **kwargs):
        self.accelerating_voltage = accelerating_voltage
        self.precession_angle = np.abs(precession_angle)
        self.approximate_precession = approximate_precession
        if isinstance(shape_factor_model, str):
            if shape_factor_model not in _SHAPE_NAMES:
                raise NotImplementedError(
                    f"{shape_factor_model} is not a recognized shape factor model, choose from: "
                    f"{_SHAPE_NAMES} or provide your own function.")
        elif not callable(shape_factor_model):
            raise NotImplementedError(f"{shape_factor_model} is neither a shape factor model name nor a function")
        self.shape_factor_model = shape_factor_model
        self.minimum_intensity = minimum_intensity
        self.shape_factor_kwargs = kwargs
        # a function of the caller's (not one of the reference's models) runs
        # on the host between two kernel launches (engine.custom_shape_spots)
        self._custom_shape = None if _shape_name(shape_factor_model) is not None else shape_factor_model
        unknown = set(kwargs) - {"minima_number"}
        if unknown and self._custom_shape is None:
            raise TypeError(f"unexpected shape factor keyword arguments: {sorted(unknown)}")
        if scattering_params in ["lobato", "xtables", None]:
            self.scattering_params = scattering_params
        else:
            raise NotImplementedError(
                "The scattering parameters `{}` is not implemented. See documentation for available "
                "implementations.".format(scattering_params))
        self._host_pool = HostSpotPool()  # page-locked result arrays reused across calls
        # how a single phase's spots reach the host: "copies" (chunked copies
        # overlapping the later chunks) or "stores" (the kernel writes them
        # into page-locked host memory itself; measured slower on the headline
        # workload: 154 against 180 GB/s over the host link)
        self.host_transfer = "copies"
        self._qstage = None               # page-locked quaternion staging, reused across calls
        self._qstage_done = None          # event after the last uploads out of the staging
        self._stage_pool = None           # one thread filling the staging beside the table build

    def __repr__(self):
        return (f"SimulationGenerator(accelerating_voltage={self.accelerating_voltage}, "
                f"scattering_params={self.scattering_params}, "
                f"approximate_precession={self.approximate_precession})")

    @property
    def wavelength(self):
        return get_electron_wavelength(self.accelerating_voltage)

    def settings(self, max_excitation_error=1e-2, shape_factor_width=None, form="mixed",
                 orient_tile=0) -> SimSettings:
        """The kernel constants of one ``calculate_diffraction2d`` call."""
        lam = self.wavelength
        if not lam > 0:
            raise ValueError("accelerating_voltage must be finite (wavelength > 0)")
        phi = float(np.deg2rad(self.precession_angle))
        if phi == 0:
            mode = N.DS_PRECESSION_NONE
        elif self.approximate_precession:
            mode = N.DS_PRECESSION_LORENTZIAN
        else:
            mode = N.DS_PRECESSION_INTEGRAL
        width = max_excitation_error if shape_factor_width is None else shape_factor_width
        kernel_model = "binary" if self._custom_shape is not None else _shape_name(self.shape_factor_model)
        return SimSettings(k0=1.0 / lam, max_excitation_error=float(max_excitation_error), shape_width=float(width),
                           shape_model=kernel_model, precession_angle_rad=phi,
                           precession_mode=mode, minimum_intensity=float(self.minimum_intensity),
                           minima_number=float(self.shape_factor_kwargs.get("minima_number", 5)), form=form,
                           orient_tile=orient_tile)

    def _stage_quaternions(self, arrays):
        """Host half of the orientation upload: wait for the previous call's
        uploads out of the reusable page-locked staging, then copy the (n, 4)
        quaternion arrays into it.  Runs on the generator's staging thread
        beside the table build (numpy's copy releases the GIL).  Returns the
        staging views, one per array."""
        total = sum(int(a.shape[0]) for a in arrays)
        if self._qstage_done is not None:
            self._qstage_done.synchronize()
        if self._qstage is None or self._qstage.shape[0] < total:
            self._qstage = torch.empty((max(total, 4096), 4), dtype=torch.float64, pin_memory=True)
        views, off = [], 0
        for a in arrays:
            n = int(a.shape[0])
            st = self._qstage[off:off + n]
            st.numpy()[...] = a
            views.append(st)
            off += n
        return views

    def _upload_staged(self, views, dev):
        """Device half: asynchronous copies out of the page-locked staging on
        the current stream; the next call's staging waits for them (an
        event)."""
        out = []
        for st in views:
            d = torch.empty((st.shape[0], 4), dtype=torch.float64, device=dev)
            d.copy_(st, non_blocking=True)
            out.append(d)
        self._qstage_done = torch.cuda.Event()
        self._qstage_done.record(torch.cuda.current_stream(dev))
        return out

    def _stager(self):
        if self._stage_pool is None:
            self._stage_pool = ThreadPoolExecutor(max_workers=1, thread_name_prefix="diffsims-gb300-stage")
        return self._stage_pool

    def calculate_diffraction2d(self, phase: Union[Phase, Sequence[Phase]],
                                rotation: Union[Rotation, Sequence[Rotation]] = None,
                                reciprocal_radius: float = 1.0, with_direct_beam: bool = True,
                                max_excitation_error: float = 1e-2, shape_factor_width: float = None,
                                debye_waller_factors: dict = None, show_progressbar: bool = False,
                                form: str = "mixed", orient_tile: int = 0, stream_to_host: bool = True,
                                timing: bool = False, result: str = "auto"):
        """Spot patterns of one or more phases, each under its own rotations.

        Arguments as diffsims/generators/simulation_generator.py:134-146;
        ``form`` selects the arithmetic ('mixed': FP32 bulk with FP64 phase
        reduction and FP64 excitation error near the cutoff; 'fp64': the plain
        all-FP64 comparator).  ``show_progressbar`` is accepted and ignored
        (each phase is one kernel launch).  With ``stream_to_host`` (the
        default, as the results are normally read on the host) a single
        phase's spots go to page-locked host memory: with
        ``host_transfer = "copies"`` (the default) the orientations run in
        chunks whose spots are copied while later chunks compute, with
        ``"stores"`` the orientation kernel writes them there itself in one
        launch (no device copy of the spots; chunked copies where the host
        memory is not addressable by kernels); ``False`` keeps
        the spots on the device only (for device-side consumers such as
        ``get_diffraction_patterns``); the page-locked host arrays are kept
        by the generator and reused once a previous result is released.
        With ``timing`` (single phase, streamed) the result's
        ``spots(0).timings()`` gives the call's time split.  ``result``:
        'native' returns this library's ``Simulation2D``; 'reference' the
        reference package's own ``Simulation2D`` with ``DiffractingVector``
        coordinates built per pattern on first read
        (``interop.to_reference_simulation``; needs diffsims, orix and
        diffpy); 'auto' (default) the reference's types when that package is
        importable and the phases are not this library's ``Phase`` objects,
        else the native one.
        """
        t_call = time.perf_counter()
        if result not in ("auto", "native", "reference"):
            raise ValueError("result must be 'auto', 'native' or 'reference'")
        caller_rotation = rotation
        if rotation is None:
            rotation = Rotation.from_euler((0, 0, 0), degrees=True)
        single_phase = not isinstance(phase, (list, tuple))
        phases = [phase] if single_phase else list(phase)
        rotations = [rotation] if not isinstance(rotation, (list, tuple)) else list(rotation)
        if len(phases) != len(rotations):
            raise ValueError("The number of phases and rotations must be equal. "
                             f"Got {len(phases)} phases and {len(rotations)} rotations.")
        if form not in ("mixed", "fp64"):
            raise ValueError("form must be 'mixed' or 'fp64'")
        N.load_library()
        dev = torch.device("cuda", torch.cuda.current_device())
        settings = self.settings(max_excitation_error, shape_factor_width, form, orient_tile)
        rots, tables = [], []
        t_table = 0.0
        for r in rotations:
            rots.append(r if isinstance(r, Rotation) else Rotation(quaternions_of(r)))
        # the staging thread fills the page-locked staging with the
        # orientations while this thread builds the tables; the uploads then
        # queue behind the structure-factor kernels on the same stream
        staged = self._stager().submit(self._stage_quaternions, [quaternions_of(rot) for rot in rots])
        for p in phases:
            t0 = time.perf_counter()
            tables.append(PhaseTable(p, reciprocal_radius, with_direct_beam, self.scattering_params,
                                     debye_waller_factors, form=form, device=dev))
            t_table += time.perf_counter() - t0
        t1 = time.perf_counter()
        qs = self._upload_staged(staged.result(), dev)
        t_upload = time.perf_counter() - t1
        custom = self._custom_shape is not None and settings.precession_mode != N.DS_PRECESSION_LORENTZIAN
        if custom:
            # the caller's function on the host between the selection and the
            # finishing kernel (lorentzian_precession ignores the model, as in
            # the reference, and stays on the plain path)
            spots = [custom_shape_spots(t, q, settings, reciprocal_radius, self._custom_shape,
                                        self.shape_factor_kwargs) for t, q in zip(tables, qs)]
        elif len(tables) == 1 and stream_to_host:
            t_sim = time.perf_counter()
            sp = None
            if self.host_transfer == "stores":
                sp = simulate_phase_to_host(tables[0], qs[0], settings, reciprocal_radius, host_pool=self._host_pool,
                                            timing=timing)
            if sp is None:
                sp = simulate_phase_streamed(tables[0], qs[0], settings, reciprocal_radius,
                                             host_pool=self._host_pool, timing=timing)
            sp._timing.update(table_ms=t_table * 1e3, upload_ms=t_upload * 1e3,
                              before_stream_ms=(t_sim - t_call) * 1e3)
            spots = [sp]
        elif len(tables) == 1:
            spots = [simulate_phase(tables[0], qs[0], settings, reciprocal_radius, buffers=SpotBuffers(dev))]
        else:
            # all phases in one persistent launch (per group of up to 96); tile
            # 0 = the library's choice
            tile = min(int(orient_tile), 16 if form == "mixed" else 8) if orient_tile else 0
            spots = PhaseBatch(tables, qs, settings, reciprocal_radius, orient_tile=tile).run().spots()
        if single_phase:
            native = Simulation2D(phases[0], spots, rots[0], self, reciprocal_radius)
        else:
            native = Simulation2D(phases, spots, rots, self, reciprocal_radius)
        if result == "native" or (result == "auto" and (interop.cached_reference_classes() is None or
                                                        all(isinstance(p, Phase) for p in phases))):
            return native
        user_rot = _caller_rotations(caller_rotation, rots, single_phase)
        return interop.to_reference_simulation(native, phases[0] if single_phase else phases, user_rot)

    def calculate_diffraction1d(self, phase, reciprocal_radius: float = 1.0, minimum_intensity: float = 1e-3,
                                 debye_waller_factors: dict = None):
        """1-D profile of one phase (diffsims/generators/simulation_generator.py:261-317):
        the hkl set of ``from_min_dspacing`` with its default 0.7 Angstrom (as the
        reference, ``reciprocal_radius`` is only stored in the result), one
        vector per family of the phase's point group (``symmetry_families``),
        intensities multiplicity x |F|^2 on the GPU, scaled so the largest is
        100, peaks above ``minimum_intensity`` kept; hkil indices for hexagonal
        lattices.  The point group comes from ``phase.space_group`` (a diffpy
        ``SpaceGroup``, operations with ``R`` and ``t``, ``(R, t)`` pairs, or
        ``None`` for P1)."""
        hkl, gspacing, F2 = _min_dspacing_rows(phase, 0.7, self.scattering_params, debye_waller_factors)
        structure = structure_of(phase)
        reps, mult = symmetry_families(hkl, reciprocal_basis(structure.lattice),
                                       point_group_rotations(getattr(phase, "space_group", None)))
        hkl_r = hkl[reps].astype(np.float64)
        g_vectors = gspacing[reps]
        intensities = mult * F2[reps]
        if _is_hexagonal(structure.lattice):
            hkl_r = np.column_stack([hkl_r[:, 0], hkl_r[:, 1], -(hkl_r[:, 0] + hkl_r[:, 1]), hkl_r[:, 2]])
        intensities = np.asarray(intensities) / max(intensities) * 100
        mask = intensities > minimum_intensity
        return Simulation1D(phase=phase, reciprocal_spacing=g_vectors[mask], intensities=intensities[mask],
                            hkl=hkl_r[mask], reciprocal_radius=reciprocal_radius, wavelength=self.wavelength)

