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
def _direct_base(p):
    """Rows a, b, c of the lattice (a, b, c, alpha, beta, gamma; degrees) in
    the x || a, z || c* frame, and d(base)/d(param) (6 x 3 x 3)."""
    a, b, c, al, be, ga = p
    d = np.pi / 180.0
    ca, cb, cg = np.cos(al * d), np.cos(be * d), np.cos(ga * d)
    sa, sb, sg = np.sin(al * d), np.sin(be * d), np.sin(ga * d)
    cx = c * cb
    cy = c * (ca - cb * cg) / sg
    cz = np.sqrt(c * c - cx * cx - cy * cy)
    L = np.array([[a, 0, 0], [b * cg, b * sg, 0], [cx, cy, cz]])
    dL = np.zeros((6, 3, 3))
    dL[0, 0, 0] = 1.0
    dL[1, 1, 0], dL[1, 1, 1] = cg, sg
    # c row: (c cb, c (ca - cb cg) / sg, sqrt(c^2 - cx^2 - cy^2))
    def c_row(dcx, dcy):
        return dcx, dcy, -(cx * dcx + cy * dcy) / cz
    dL[2, 2] = [cb, (ca - cb * cg) / sg, cz / c]                                   # d/dc
    dL[3, 2] = c_row(0.0, c * (-sa * d) / sg)                                        # d/dalpha
    dL[4, 2] = c_row(c * (-sb * d), c * (sb * d * cg) / sg)                          # d/dbeta
    dcy_dg = c * ((cb * sg * d) * sg - (ca - cb * cg) * cg * d) / (sg * sg)
    dL[5, 1, 0], dL[5, 1, 1] = -b * sg * d, b * cg * d                               # d/dgamma, b row
    dL[5, 2] = c_row(0.0, dcy_dg)
    return L, dL


class _ReciprocalBasis(torch.autograd.Function):
    @staticmethod
    def forward(ctx, lattice):
        p = lattice.detach().cpu().numpy().astype(np.float64)
        L, dL = _direct_base(p)
        rec = np.linalg.inv(L).T
        ctx.rec, ctx.dL, ctx.dev = rec, dL, lattice.device
        return torch.as_tensor(rec, dtype=torch.float64).to(lattice.device)

    @staticmethod
    def backward(ctx, g):
        G = g.detach().cpu().numpy().astype(np.float64)
        # recip = L^-T: d recip = -recip dL^T recip
        grads = [float(-(G * (ctx.rec @ ctx.dL[k].T @ ctx.rec)).sum()) for k in range(6)]
        return torch.as_tensor(grads, dtype=torch.float64).to(ctx.dev)


def reciprocal_basis(lattice: torch.Tensor) -> torch.Tensor:
    """Rows a*, b*, c* (1/Angstrom) of the lattice (a, b, c, alpha, beta,
    gamma; degrees) in the x || a, z || c* frame, differentiable.  Evaluated
    on the host (3 x 3); keep the lattice parameters on the CPU in a loop to
    avoid a device round trip."""
    return _ReciprocalBasis.apply(lattice)


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


class _AxisAngleCompose(torch.autograd.Function):
    @staticmethod
    def forward(ctx, q0, v):
        lib = N.load_library()
        q0c, vc = q0.detach().to(torch.float64).contiguous(), v.detach().to(torch.float64).contiguous()
        out = torch.empty_like(q0c)
        N.check(lib.ds_axis_angle_compose(N.ptr(q0c), N.ptr(vc), q0c.shape[0], N.ptr(out), N.stream_handle()),
                "axis_angle_compose")
        ctx.save_for_backward(q0c, vc)
        return out

    @staticmethod
    def backward(ctx, gq):
        lib = N.load_library()
        q0c, vc = ctx.saved_tensors
        gv = torch.empty_like(vc)
        N.check(lib.ds_axis_angle_compose_backward(N.ptr(q0c), N.ptr(vc), q0c.shape[0],
                                                   N.ptr(gq.to(torch.float64).contiguous()), N.ptr(gv),
                                                   N.stream_handle()), "axis_angle_compose_backward")
        return None, gv


def compose_axis_angle(q0: torch.Tensor, v: torch.Tensor) -> torch.Tensor:
    """q0 (x) exp(v) on the device, one fused kernel each way: orientation
    quaternions q0 (n, 4) corrected by rotation vectors v (n, 3, radians),
    differentiable in v."""
    return _AxisAngleCompose.apply(q0, v)


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
        if getattr(generator, "_custom_shape", None) is not None:
            raise NotImplementedError("gradients are available for the built-in shape-factor models only "
                                      "(a function of the caller's has no adjoint kernel)")
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
        ctx.recip_device = recip.device
        model.last_hmax = int(np.max(table.hmax))  # bound on |h|, |k|, |l| of every spot
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
        gq = torch.empty((n_o, 4), dtype=torch.float64, device=dev)
        grecip = torch.zeros(9, dtype=torch.float64, device=dev)
        gatoms = torch.zeros((n_a, 5), dtype=torch.float64, device=dev)
        st = N.stream_handle()
        p = model.settings.cstruct()
        n_sp = int(ctx.idx.shape[0])
        bbytes = lib.ds_simulate_backward_scratch_bytes(p, n_sp, n_o)
        bscr = torch.empty(max(bbytes, 16), dtype=torch.uint8, device=dev)
        status = torch.zeros(1, dtype=torch.int32, device=dev)
        N.check(lib.ds_simulate_backward(p, table.cstruct(), N.ptr(q), n_o, N.ptr(ctx.offsets), N.ptr(ctx.idx), n_sp,
                                         N.ptr(g_inten), N.ptr(gF2), N.ptr(gq), N.ptr(grecip), N.ptr(bscr), bbytes,
                                         N.ptr(status), st), "simulate_backward")
        nbytes = lib.ds_structure_factors_backward_scratch_bytes(table.n, table.atoms.n_species)
        scratch = torch.empty(max(nbytes, 16), dtype=torch.uint8, device=dev)
        rb = (C.c_double * 9)(*table.recip.reshape(-1).tolist())
        N.check(lib.ds_structure_factors_backward(table.atoms.cstruct(), N.ptr(table.hkl) if table.n else None,
                                                  N.ptr(table.g2) if table.n else None, table.n, rb, N.ptr(gF2),
                                                  N.ptr(gatoms), N.ptr(grecip), N.ptr(scratch), nbytes, st),
                "structure_factors_backward")
        N.check_device_status(status, "simulate_backward")
        return gatoms[:, 0:3], gatoms[:, 4], gatoms[:, 3], grecip.view(3, 3).to(ctx.recip_device), gq, None


def simulate_intensities(model: SpotModel, xyz: torch.Tensor, B: torch.Tensor, occupancy: torch.Tensor,
                         recip: torch.Tensor, quats: torch.Tensor) -> SpotIntensities:
    """Spot intensities of every orientation, differentiable with respect to
    xyz (N, 3) fractional coordinates, B (N,), occupancy (N,), recip (3, 3)
    (rows a*, b*, c*) and quats (n, 4); float64.  recip is read on the host by
    the forward (hkl enumeration): keeping it, and the lattice parameters it
    comes from, on the CPU saves a device round trip; the rest live on the
    device."""
    inten, off, hkl = _KinematicalIntensities.apply(xyz, B, occupancy, recip, quats, model)
    out = SpotIntensities(inten, off, hkl)
    out._hmax = model.last_hmax
    return out


def _spot_keys(sp: SpotIntensities, K: int) -> torch.Tensor:
    counts = sp.offsets[1:] - sp.offsets[:-1]
    o = torch.repeat_interleave(torch.arange(counts.shape[0], device=counts.device), counts,
                                output_size=int(sp.hkl.shape[0]))
    h = sp.hkl.to(torch.int64) + K // 2
    return ((o * K + h[:, 0]) * K + h[:, 1]) * K + h[:, 2]


def spot_loss(sim: SpotIntensities, target: SpotIntensities) -> torch.Tensor:
    """Sum of squared intensity differences over the union of the two spot
    sets, matched by (orientation, hkl); a spot missing from one side counts
    with intensity 0.  (Keys are unique per side, so every target spot is
    matched at most once: the unmatched targets contribute
    sum T^2 - sum over matched T^2.)"""
    hmax = 1
    for sp in (sim, target):
        if sp.hkl.numel():
            hm = getattr(sp, "_hmax", None)
            if hm is None:
                hm = int(sp.hkl.abs().max().item())
                sp._hmax = hm
            hmax = max(hmax, hm)
    K = 2 * hmax + 3
    t_int = target.intensity.detach()
    if t_int.numel() == 0:
        return (sim.intensity ** 2).sum()
    cache = getattr(target, "_sorted_keys", None)
    if cache is None or cache[0] != K:
        kt_sorted, perm = torch.sort(_spot_keys(target, K))
        cache = (K, kt_sorted, perm, (t_int ** 2).sum())
        target._sorted_keys = cache  # the target is constant: sort its keys once
    _, kt_sorted, perm, t_sq = cache
    ks = _spot_keys(sim, K)
    pos = torch.searchsorted(kt_sorted, ks).clamp(max=kt_sorted.numel() - 1)
    match = kt_sorted[pos] == ks
    matched_t = torch.where(match, t_int[perm[pos]], torch.zeros_like(sim.intensity))
    return ((sim.intensity - matched_t) ** 2).sum() + (t_sq - (matched_t ** 2).sum())
