"""Differentiable kinematical spot intensities (no counterpart in the reference).

``simulate_intensities`` is a ``torch.autograd.Function`` whose forward is the
CUDA path (hkl enumeration, structure factors, the orientation kernel) and
whose backward is the hand-written adjoint (``ds_simulate_backward``,
``ds_structure_factors_backward``): gradients of any loss on the spot
intensities with respect to fractional coordinates, Debye-Waller B,
occupancies, the reciprocal basis (so, through ``reciprocal_basis``, the six
lattice parameters) and the orientation quaternions (so, through
``axis_angle_quaternion``, axis-angle corrections).  Structure factors are
recomputed in the backward pass, never stored per orientation.  The spot
selection is piecewise constant in the parameters and is not differentiated.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass

import numpy as np
import torch

from . import _native as N
from .engine import PhaseTable, SpotBuffers, simulate_phase
from .sim_utils import PackedAtoms


# ------------------------------------------------- differentiable geometry ----
def reciprocal_basis(lattice: torch.Tensor) -> torch.Tensor:
    """Rows a*, b*, c* (1/Angstrom) of the lattice (a, b, c, alpha, beta,
    gamma; degrees) in the x || a, z || c* frame, differentiably."""
    a, b, c, al, be, ga = [lattice[i] for i in range(6)]
    d = math.pi / 180.0
    ca, cb, cg, sg = torch.cos(al * d), torch.cos(be * d), torch.cos(ga * d), torch.sin(ga * d)
    cx = c * cb
    cy = c * (ca - cb * cg) / sg
    cz = torch.sqrt(c * c - cx * cx - cy * cy)
    zero = torch.zeros_like(a)
    base = torch.stack([torch.stack([a, zero, zero]), torch.stack([b * cg, b * sg, zero]), torch.stack([cx, cy, cz])])
    return torch.linalg.inv(base).transpose(0, 1)


def axis_angle_quaternion(v: torch.Tensor) -> torch.Tensor:
    """Unit quaternions (w, x, y, z) of rotation vectors v (n, 3) (angle = |v|
    in radians about v / |v|), differentiable at v = 0."""
    th = torch.linalg.norm(v, dim=-1, keepdim=True)
    half = 0.5 * th
    small = th < 1e-6
    safe = torch.where(small, torch.ones_like(th), th)
    k = torch.where(small, 0.5 - th * th / 48.0, torch.sin(half) / safe)  # sin(th/2)/th
    return torch.cat([torch.cos(half), k * v], dim=-1)


def quaternion_multiply(p: torch.Tensor, q: torch.Tensor) -> torch.Tensor:
    """Hamilton product p q of (..., 4) quaternions (w, x, y, z)."""
    pw, px, py, pz = p.unbind(-1)
    qw, qx, qy, qz = q.unbind(-1)
    return torch.stack([pw * qw - px * qx - py * qy - pz * qz, pw * qx + px * qw + py * qz - pz * qy,
                        pw * qy - px * qz + py * qw + pz * qx, pw * qz + px * qy - py * qx + pz * qw], dim=-1)


def quaternion_matrix(q: torch.Tensor) -> torch.Tensor:
    """Active rotation matrices (n, 3, 3) of quaternions (normalised first),
    the kernels' convention."""
    q = q / torch.linalg.norm(q, dim=-1, keepdim=True)
    w, x, y, z = q.unbind(-1)
    return torch.stack([
        torch.stack([1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)], -1),
        torch.stack([2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)], -1),
        torch.stack([2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)], -1)], -2)


# ------------------------------------------------------------ the problem ----
class SpotModel:
    """The fixed part of a differentiable simulation: element species and
    scattering coefficients, the generator's settings, reciprocal radius,
    direct beam and arithmetic form."""

    def __init__(self, elements, generator, reciprocal_radius=1.0, max_excitation_error=1e-2,
                 shape_factor_width=None, with_direct_beam=True, form="mixed", device=None):
        dev = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
        n = len(elements)
        self.device = dev
        self.elements = list(elements)
        self._atoms = PackedAtoms(self.elements, np.zeros((n, 3)), np.ones(n), np.zeros(n),
                                  generator.scattering_params, dev)
        self.settings = generator.settings(max_excitation_error, shape_factor_width, form)
        self.reciprocal_radius = float(reciprocal_radius)
        self.with_direct_beam = bool(with_direct_beam)
        self.form = form

    def table(self, recip: np.ndarray, xyz, occ, B) -> PhaseTable:
        atoms = self._atoms.with_values(xyz, occ, B)
        return PhaseTable.from_parts(recip, atoms, self.reciprocal_radius, self.with_direct_beam, self.form,
                                     self.device)


@dataclass
class SpotIntensities:
    """Spots of a differentiable simulation: ``intensity`` (total,) float64
    (carries the graph), ``offsets`` (n_orient + 1,) int64 and ``hkl``
    (total, 3) int32, both constant."""
    intensity: torch.Tensor
    offsets: torch.Tensor
    hkl: torch.Tensor


class _KinematicalIntensities(torch.autograd.Function):
    @staticmethod
    def forward(ctx, xyz, B, occ, recip, quats, model: SpotModel):
        recip_np = recip.detach().cpu().numpy().astype(np.float64)
        table = model.table(recip_np, xyz, occ, B)
        q = quats.detach().to(torch.float64).contiguous()
        spots = simulate_phase(table, q, model.settings, model.reciprocal_radius, SpotBuffers(model.device))
        idx = spots.hkl_index.contiguous()
        inten = spots.xyzi[:, 3].to(torch.float64)
        hkl = table.hkl[idx.long()] if spots.total else torch.zeros((0, 3), dtype=torch.int32, device=q.device)
        ctx.save_for_backward(q)
        ctx.table, ctx.offsets, ctx.idx, ctx.model = table, spots.offsets, idx, model
        ctx.mark_non_differentiable(spots.offsets, hkl)
        return inten, spots.offsets, hkl

    @staticmethod
    def backward(ctx, g_inten, g_off=None, g_hkl=None):
        lib = N.load_library()
        (q,) = ctx.saved_tensors
        table, model = ctx.table, ctx.model
        dev = q.device
        n_o = q.shape[0]
        n_a = table.atoms.n_atoms
        g_inten = (torch.zeros(ctx.idx.shape[0], dtype=torch.float64, device=dev) if g_inten is None
                   else g_inten.to(torch.float64).contiguous())
        gF2 = torch.zeros(max(table.n, 1), dtype=torch.float64, device=dev)
        gR = torch.zeros((n_o, 9), dtype=torch.float64, device=dev)
        grecip = torch.zeros(9, dtype=torch.float64, device=dev)
        gatoms = torch.zeros((n_a, 5), dtype=torch.float64, device=dev)
        st = N.stream_handle()
        N.check(lib.ds_simulate_backward(model.settings.cstruct(), table.cstruct(), N.ptr(q), n_o, N.ptr(ctx.offsets),
                                         N.ptr(ctx.idx), N.ptr(g_inten), N.ptr(gF2), N.ptr(gR), N.ptr(grecip), st),
                "simulate_backward")
        nbytes = lib.ds_structure_factors_backward_scratch_bytes(table.n)
        scratch = torch.empty(max(nbytes, 16), dtype=torch.uint8, device=dev)
        rb = (C.c_double * 9)(*table.recip.reshape(-1).tolist())
        N.check(lib.ds_structure_factors_backward(table.atoms.cstruct(), N.ptr(table.hkl) if table.n else None,
                                                  N.ptr(table.g2) if table.n else None, table.n, rb, N.ptr(gF2),
                                                  N.ptr(gatoms), N.ptr(grecip), N.ptr(scratch), nbytes, st),
                "structure_factors_backward")
        with torch.enable_grad():
            qq = q.detach().requires_grad_(True)
            (gq,) = torch.autograd.grad(quaternion_matrix(qq), qq, gR.view(n_o, 3, 3))
        return gatoms[:, 0:3], gatoms[:, 4], gatoms[:, 3], grecip.view(3, 3), gq, None


def simulate_intensities(model: SpotModel, xyz: torch.Tensor, B: torch.Tensor, occupancy: torch.Tensor,
                         recip: torch.Tensor, quats: torch.Tensor) -> SpotIntensities:
    """Spot intensities of every orientation, differentiable with respect to
    xyz (N, 3) fractional coordinates, B (N,), occupancy (N,), recip (3, 3)
    (rows a*, b*, c*) and quats (n, 4); all float64 on the device."""
    inten, off, hkl = _KinematicalIntensities.apply(xyz, B, occupancy, recip, quats, model)
    return SpotIntensities(inten, off, hkl)


def _spot_keys(sp: SpotIntensities, K: int) -> torch.Tensor:
    counts = sp.offsets[1:] - sp.offsets[:-1]
    o = torch.repeat_interleave(torch.arange(counts.shape[0], device=counts.device), counts)
    h = sp.hkl.to(torch.int64) + K // 2
    return ((o * K + h[:, 0]) * K + h[:, 1]) * K + h[:, 2]


def spot_loss(sim: SpotIntensities, target: SpotIntensities) -> torch.Tensor:
    """Sum of squared intensity differences over the union of the two spot
    sets, matched by (orientation, hkl); a spot missing from one side counts
    with intensity 0."""
    hmax = 1
    for sp in (sim, target):
        if sp.hkl.numel():
            hmax = max(hmax, int(sp.hkl.abs().max().item()))
    K = 2 * hmax + 3
    ks, kt = _spot_keys(sim, K), _spot_keys(target, K)
    t_int = target.intensity.detach()
    if kt.numel() == 0:
        return (sim.intensity ** 2).sum()
    kt_sorted, perm = torch.sort(kt)
    pos = torch.searchsorted(kt_sorted, ks).clamp(max=kt.numel() - 1)
    match = kt_sorted[pos] == ks
    matched_t = torch.where(match, t_int[perm[pos]], torch.zeros_like(sim.intensity))
    used = torch.zeros(kt.numel(), dtype=torch.bool, device=kt.device)
    used[perm[pos[match]]] = True
    return ((sim.intensity - matched_t) ** 2).sum() + (t_int[~used] ** 2).sum()
