"""Physics helpers of the drop-in API: wavelength, scattering tables, atom
packing, and ``get_kinematical_intensities`` on the GPU.

Mirrors diffsims/utils/sim_utils.py (names, argument meaning, warnings and
errors); the arithmetic of ``get_kinematical_intensities`` runs in the CUDA
library (``ds_kinematical_intensities``).
"""
from __future__ import annotations

import functools
import json
import math
import pathlib
import re
import warnings

import numpy as np
import torch

from . import _native as N

# physical constants from scipy.constants, as the reference
# (diffsims/utils/sim_utils.py:25)
from scipy.constants import c as _C, e as _E, h as _H, m_e as _ME

_TABLES = json.loads((pathlib.Path(__file__).resolve().parent / "data" / "scattering_params.json").read_text())


def get_electron_wavelength(accelerating_voltage):
    """Relativistic electron wavelength (Angstrom) for a voltage in kV;
    0 for ``inf``.  diffsims/utils/sim_utils.py:57-79."""
    if accelerating_voltage in (np.inf, "inf"):
        return 0
    E = accelerating_voltage * 1e3
    return _H / math.sqrt(2 * _ME * _E * E * (1 + (_E / (2 * _ME * _C * _C)) * E)) * 1e10


def get_scattering_params_dict(scattering_params):
    """Element -> five (a, b) pairs.  diffsims/utils/sim_utils.py:139-162."""
    if scattering_params == "lobato":
        return _TABLES["lobato"]
    if scattering_params == "xtables":
        return _TABLES["xtables"]
    raise NotImplementedError(
        "The scattering parameters `{}` are not implemented. See documentation for available "
        "implementations.".format(scattering_params))


@functools.lru_cache(maxsize=4096)
def get_element(atom_type_symbol: str) -> str:
    """Alphabetic head of a CIF atom type symbol
    (diffsims/structure_factor/atomic_scattering_parameters.py:145-164);
    remembered per symbol (a structure repeats a few symbols many times)."""
    return re.match("^(?P<element>[A-Za-z]*)", atom_type_symbol).group("element")


class PackedAtoms:
    """One phase's atoms on the device in the C-ABI layout (``ds_atom``
    records + per-species coefficient rows)."""

    def __init__(self, elements, xyz, occupancy, B, scattering_params, device):
        if scattering_params not in ("lobato", "xtables", None):
            raise NotImplementedError(
                "The scattering parameters `{}` are not implemented. See documentation for available "
                "implementations.".format(scattering_params))
        table = _TABLES[scattering_params] if scattering_params is not None else {}
        species, coeff_rows, index = [], [], {}
        for el in elements:
            sym = get_element(el)
            if sym not in index:
                index[sym] = len(coeff_rows)
                row = np.zeros(10)
                if scattering_params is not None:
                    if sym in table:
                        row = np.asarray(table[sym], dtype=np.float64).reshape(10)
                    else:
                        warnings.warn(f"Element {sym} from atom type symbol {el} not found in "
                                      "scattering parameter library.")
                coeff_rows.append(row)
            species.append(index[sym])
        self._fill(species, coeff_rows, xyz, occupancy, B, N.DS_SCATTER[scattering_params], device)

    @classmethod
    def from_rows(cls, species, coeff_rows, xyz, occupancy, B, kind, device):
        """Records from explicit per-species coefficient rows (10 doubles
        each) and a ``DS_SCATTER_*`` kind."""
        out = cls.__new__(cls)
        out._fill(species, coeff_rows, xyz, occupancy, B, kind, device)
        return out

    def _fill(self, species, coeff_rows, xyz, occupancy, B, kind, device):
        if len(coeff_rows) > 32:
            raise ValueError("at most 32 distinct elements per phase are supported")
        n = len(species)
        rec = np.zeros(n, dtype=[("x", "f8"), ("y", "f8"), ("z", "f8"), ("occ", "f8"), ("B", "f8"),
                                 ("species", "i4"), ("pad", "i4")])
        xyz = np.asarray(xyz, dtype=np.float64).reshape(-1, 3)
        rec["x"], rec["y"], rec["z"] = xyz[:, 0], xyz[:, 1], xyz[:, 2]
        rec["occ"] = np.asarray(occupancy, dtype=np.float64)
        rec["B"] = np.asarray(B, dtype=np.float64)
        rec["species"] = species
        raw = np.frombuffer(rec.tobytes(), dtype=np.uint8)
        self.records = torch.from_numpy(raw.copy()).to(device)
        self.coeffs = torch.from_numpy(np.asarray(coeff_rows, dtype=np.float64).reshape(-1)).to(device)
        self.n_atoms = n
        self.n_species = len(coeff_rows)
        self.kind = kind

    def cstruct(self) -> N.ds_atoms:
        return N.ds_atoms(self.n_atoms, self.n_species, self.records.data_ptr(), self.coeffs.data_ptr(),
                          self.kind, 0)

    def with_values(self, xyz, occupancy, B):
        """A copy whose per-atom values come from device tensors (float64:
        (N, 3), (N,), (N,)); species and coefficients are shared.  Builds the
        records on the device (no host round trip)."""
        n = self.n_atoms
        rec = torch.empty((n, 12), dtype=torch.int32, device=self.records.device)
        r64 = rec.view(torch.float64)
        r64[:, 0:3] = xyz.detach().to(torch.float64)
        r64[:, 3] = occupancy.detach().to(torch.float64)
        r64[:, 4] = B.detach().to(torch.float64)
        rec[:, 10:12] = self.records.view(torch.int32).view(n, 12)[:, 10:12]
        out = PackedAtoms.__new__(PackedAtoms)
        out.records = rec.view(torch.uint8).reshape(-1)
        out.coeffs, out.n_atoms, out.n_species, out.kind = self.coeffs, n, self.n_species, self.kind
        return out


def debye_waller_per_atom(elements, debye_waller_factors):
    """Per-atom B.  A dict maps element -> B (the reference's rule,
    diffsims/utils/sim_utils.py:220; missing elements get 0); a sequence gives
    one B per atom (an extension for per-atom refinement)."""
    if debye_waller_factors is None:
        return np.zeros(len(elements))
    if isinstance(debye_waller_factors, dict):
        return np.array([float(debye_waller_factors.get(get_element(e), 0)) for e in elements])
    B = np.asarray(debye_waller_factors, dtype=np.float64).reshape(-1)
    if B.shape[0] != len(elements):
        raise ValueError("per-atom Debye-Waller factors must have one value per atom")
    return B


def get_kinematical_intensities(structure, g_indices, g_hkls_array, debye_waller_factors=None,
                                scattering_params="lobato", prefactor=1):
    """prefactor * |F_hkl|^2 for the given reflections, on the GPU (FP64).

    Same arguments as diffsims/utils/sim_utils.py:307-354: ``structure`` is an
    iterable of sites (``element``, ``xyz``, ``occupancy``); ``g_indices``
    (N, 3) Miller indices (may be non-integer); ``g_hkls_array`` (N,) |g| in
    1/Angstrom; ``prefactor`` scalar or (N,).  Fractional coordinates are
    used as given (the reference's re-basing at :290-291 is the identity in the
    x || a, z || c* frame).  Returns a float64 numpy array.
    """
    from .crystal import sites_of
    lib = N.load_library()
    dev = torch.device("cuda", torch.cuda.current_device())
    els, xyz, occ = sites_of(structure)
    B = debye_waller_per_atom(els, debye_waller_factors)
    atoms = PackedAtoms(els, xyz, occ, B, scattering_params, dev)
    hkl = torch.as_tensor(np.asarray(g_indices, dtype=np.float64).reshape(-1, 3)).to(dev)
    gs = torch.as_tensor(np.asarray(g_hkls_array, dtype=np.float64).reshape(-1)).to(dev)
    n = hkl.shape[0]
    if gs.shape[0] != n:
        raise ValueError("g_indices and g_hkls_array must have the same length")
    pref_np = np.asarray(prefactor, dtype=np.float64)
    pref = None
    if pref_np.ndim > 0:
        pref = torch.as_tensor(np.broadcast_to(pref_np, (n,)).copy()).to(dev)
    out = torch.empty(n, dtype=torch.float64, device=dev)
    status = torch.zeros(1, dtype=torch.int32, device=dev)
    a = atoms.cstruct()
    N.check(lib.ds_kinematical_intensities(a, N.ptr(hkl), N.ptr(gs), N.ptr(pref), n, N.ptr(out), None, 0,
                                           N.ptr(status), N.stream_handle()), "get_kinematical_intensities")
    N.check_device_status(status, "get_kinematical_intensities")
    res = out.cpu().numpy()
    if pref is None:
        res = res * float(pref_np)
    return res
