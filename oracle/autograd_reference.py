"""FP64 torch transcription of the reference's spot-intensity formulas, for
gradient checks.

TEST INFRASTRUCTURE ONLY (the checker): imported by tests/ and by the CPU or
comparison legs of ``bench.py``; never by the ``diffsims_gb300`` package.

For a FIXED set of spots (orientation index and hkl of every spot) it computes
I = shf(s, r) |F_hkl|^2 with torch autograd enabled, following
diffsims/utils/sim_utils.py:227-304 (scattering factors, Debye-Waller, the
structure factor), diffsims/generators/simulation_generator.py:355-411
(excitation error, shape-factor dispatch) and
diffsims/utils/shape_factor_models.py (the models, lorentzian_precession and
the rotation average of :222-268, here by 16-point Gauss-Legendre quadrature
on pieces cut at the model's kinks, with the cuts held fixed -- the models are
continuous there, so the cut positions carry no derivative).
"""
from __future__ import annotations

import math

import numpy as np
import torch

from . import kinematic as ok


def quaternion_matrix(q):
    q = q / torch.linalg.norm(q, dim=-1, keepdim=True)
    w, x, y, z = q.unbind(-1)
    return torch.stack([
        torch.stack([1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)], -1),
        torch.stack([2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)], -1),
        torch.stack([2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)], -1)], -2)


def reciprocal_basis_torch(lattice):
    """Rows a*, b*, c* of the lattice (a, b, c, alpha, beta, gamma; degrees),
    x || a, z || c* frame, as plain torch operations (autograd)."""
    a, b, c, al, be, ga = [lattice[i] for i in range(6)]
    d = math.pi / 180.0
    ca, cb, cg, sg = torch.cos(al * d), torch.cos(be * d), torch.cos(ga * d), torch.sin(ga * d)
    cx = c * cb
    cy = c * (ca - cb * cg) / sg
    cz = torch.sqrt(c * c - cx * cx - cy * cy)
    zero = torch.zeros_like(a)
    base = torch.stack([torch.stack([a, zero, zero]), torch.stack([b * cg, b * sg, zero]), torch.stack([cx, cy, cz])])
    return torch.inverse(base.cpu()).to(base.device).transpose(0, 1)


def compose_axis_angle_torch(q0, v):
    """q0 (x) exp(v) (Hamilton product with the unit quaternion of rotation
    vector v) as plain torch operations (autograd)."""
    th = torch.linalg.vector_norm(v, dim=-1, keepdim=True)
    half = 0.5 * th
    small = th < 1e-6
    safe = torch.where(small, torch.ones_like(th), th)
    k = torch.where(small, 0.5 - th * th / 48.0, torch.sin(half) / safe)
    e = torch.cat([torch.cos(half), k * v], dim=-1)
    pw, px, py, pz = q0.unbind(-1)
    qw, qx, qy, qz = e.unbind(-1)
    return torch.stack([pw * qw - px * qx - py * qy - pz * qz, pw * qx + px * qw + py * qz - pz * qy,
                        pw * qy - px * qz + py * qw + pz * qx, pw * qz + px * qy - py * qx + pz * qw], dim=-1)


def _model(name, s, w, n):
    pi = math.pi
    if name == "linear":
        return torch.clamp(1 - torch.abs(s) / w, min=0.0)
    if name in ("sinc", "sin2c"):
        fac = pi * n / w
        x = fac * s
        safe = torch.where(x == 0, torch.ones_like(x), x)
        v = torch.where(x == 0, torch.zeros_like(x), torch.abs(torch.sin(safe) / safe))
        return v * v if name == "sin2c" else v
    if name == "atanc":
        fac = pi * n / abs(w)
        y = fac * s
        safe = torch.where(y == 0, torch.ones_like(y), y)
        return torch.where(y == 0, torch.ones_like(y), torch.atan(safe) / safe)
    if name == "lorentzian":
        sigma = pi / w
        return sigma / (pi * (sigma ** 2 * s ** 2 + 1)) * w
    return torch.ones_like(s)


_GL16 = np.polynomial.legendre.leggauss(16)


def _rotation_average(name, s0, a, w, n):
    """(1/pi) int_0^pi f(s0 + a cos t) dt per spot (tensors of equal shape).
    Every spot's cut list is padded to the longest with empty pieces."""
    h = ok.precession_breakpoint_step(name, w, n)
    x, wt = (torch.as_tensor(v, dtype=torch.float64, device=s0.device) for v in _GL16)
    s0d, ad = s0.detach().cpu().numpy(), a.detach().cpu().numpy()
    n_sp = s0d.shape[0]
    # cut angles of every spot at once: acos((k h - s0) / a) for the grid
    # points k h inside [s0 - a, s0 + a], padded with pi (empty pieces)
    if h > 0 and n_sp:
        pos = ad > 0
        safe_a = np.where(pos, ad, 1.0)
        k_lo = np.where(pos, np.ceil((s0d - ad) / h), 0.0)
        k_hi = np.where(pos, np.floor((s0d + ad) / h), -1.0)
        cnt = np.maximum(k_hi - k_lo + 1, 0).astype(np.int64)
        width = int(cnt.max(initial=0))
        ks = k_lo[:, None] + np.arange(width)[None, :]
        ang = np.arccos(np.clip((ks * h - s0d[:, None]) / safe_a[:, None], -1, 1))
        ang = np.where(np.arange(width)[None, :] < cnt[:, None], ang, math.pi)
    else:
        ang = np.zeros((n_sp, 0))
    cuts = np.concatenate([np.zeros((n_sp, 1)), ang, np.full((n_sp, 1), math.pi)], axis=1)
    cuts.sort(axis=1)
    ct = torch.as_tensor(cuts, dtype=torch.float64, device=s0.device)
    mid, half = 0.5 * (ct[:, 1:] + ct[:, :-1]), 0.5 * (ct[:, 1:] - ct[:, :-1])   # (spots, pieces)
    t = mid[:, :, None] + half[:, :, None] * x                                     # (spots, pieces, 16)
    f = _model(name, s0[:, None, None] + a[:, None, None] * torch.cos(t), w, n)
    avg = (half[:, :, None] * wt * f).sum((1, 2)) / math.pi
    return torch.where(a > 0, avg, _model(name, s0, w, n))


def spot_intensities(xyz, B, occ, recip, quats, elements, scattering_params, spot_orient, spot_hkl, p: ok.SimParams):
    """I per spot (FP64, differentiable in xyz, B, occ, recip, quats)."""
    dev = xyz.device
    k0 = 1 / ok.electron_wavelength(p.accelerating_voltage)
    w = p.max_excitation_error if p.shape_factor_width is None else p.shape_factor_width
    n = p.shape_kwargs.get("minima_number", 5)
    hkl = spot_hkl.to(torch.float64)
    recip = recip.to(dev)
    g = hkl @ recip                                   # g = B*^T h
    R = quaternion_matrix(quats)[spot_orient]          # (m, 3, 3)
    u = torch.einsum("mkc,mk->mc", R, g)              # R^T g
    r2 = u[:, 0] ** 2 + u[:, 1] ** 2
    r = torch.where(r2 > 0, torch.sqrt(torch.where(r2 > 0, r2, torch.ones_like(r2))), torch.zeros_like(r2))
    s = (-torch.sqrt(k0 ** 2 - r ** 2) + k0) - u[:, 2]
    phi = math.radians(abs(p.precession_angle))
    model = p.shape_factor_model
    if phi == 0:
        shf = _model(model, s, w, n)
    elif p.approximate_precession:
        sigma = math.pi / w
        uu = sigma ** 2 * (r ** 2 * phi ** 2 - s ** 2) + 1
        z = torch.sqrt(uu ** 2 + 4 * sigma ** 2 * s ** 2)
        shf = (sigma / math.pi) * torch.sqrt(2 * (uu + z) / z ** 2)
    else:
        shf = _rotation_average(model, s, r * phi, w, n)
    # structure factor
    g2 = (g * g).sum(-1)
    cf = torch.as_tensor(ok.scattering_coefficients(list(elements), scattering_params), dtype=torch.float64,
                         device=dev)  # (N, 5, 2)
    gb = g2[:, None, None] * cf[None, :, :, 1]
    if scattering_params == "lobato":
        f = (cf[None, :, :, 0] * (2 + gb) / (1 + gb) ** 2).sum(-1)
    elif scattering_params == "xtables":
        f = (cf[None, :, :, 0] * torch.exp(-0.25 * gb)).sum(-1)
    else:
        f = torch.ones((g2.shape[0], len(elements)), dtype=torch.float64, device=dev)
    amp = occ[None, :] * f * torch.exp(-0.25 * B[None, :] * g2[:, None])
    ph = 2 * math.pi * (hkl @ xyz.T)
    re = (amp * torch.cos(ph)).sum(-1)
    im = (amp * torch.sin(ph)).sum(-1)
    return shf * (re * re + im * im)


class MatchedLoss:
    """L(I) = sum of squared intensity differences over the union of two
    spot sets matched by (orientation, hkl), a spot missing on one side
    counting with intensity 0 (the loss of the differentiation workload).
    The match is made once on the host with a dictionary (equal keys -- the
    two direct-beam rows -- pair up in order), so FP64 finite differences can
    re-evaluate the loss of a fixed spot set cheaply."""

    def __init__(self, offsets, hkl, target_I, target_offsets, target_hkl):
        def keys(off, h):
            off = np.asarray(off.detach().cpu() if torch.is_tensor(off) else off, dtype=np.int64)
            h = np.asarray(h.detach().cpu() if torch.is_tensor(h) else h, dtype=np.int64)
            o = np.repeat(np.arange(off.shape[0] - 1), np.diff(off))
            return list(zip(o.tolist(), map(tuple, h.tolist())))
        ks, kt = keys(offsets, hkl), keys(target_offsets, target_hkl)
        pos_t = {}
        for i, k in enumerate(kt):
            pos_t.setdefault(k, []).append(i)
        match_s, match_t = [], []
        for i, k in enumerate(ks):
            js = pos_t.get(k)
            if js:
                match_s.append(i)
                match_t.append(js.pop(0))
        T = target_I.detach().to(torch.float64)
        dev = T.device
        ms = torch.as_tensor(match_s, dtype=torch.int64, device=dev)
        mt = torch.as_tensor(match_t, dtype=torch.int64, device=dev)
        # per simulated spot: its matched target intensity, or 0
        self.target_per_spot = torch.zeros(len(ks), dtype=torch.float64, device=dev)
        self.target_per_spot[ms] = T[mt]
        unmatched_t = torch.ones(T.shape[0], dtype=torch.bool, device=dev)
        unmatched_t[mt] = False
        self.constant = (T[unmatched_t] ** 2).sum()

    def __call__(self, I, start=0):
        """The loss of the simulated spots ``start:start + len(I)``; the
        unmatched targets' constant is added to the chunk that starts at 0,
        so the chunks' losses (and gradients) add up to the whole."""
        d = I - self.target_per_spot[start:start + I.shape[0]].to(I.device)
        out = (d * d).sum()
        return out + self.constant.to(I.device) if start == 0 else out


def gradient_errors(got, want, floor=1e-4, floors=(1e-6, 1e-4, 1e-2)):
    """Per parameter group (dict name -> array):

    * ``max_rel``: the largest |got - want| / max(|want|, floor x max|want|)
      -- every component relative to itself, components below ``floor`` of
      the group's largest measured against that floor;
    * ``max_rel_at_floor``: the same for each of ``floors``;
    * ``norm_rel``: ||got - want|| / ||want|| over the group;
    * ``below_floor``: components below ``floor`` of the group's largest."""
    out = {}
    for name in want:
        a = np.asarray(got[name], dtype=np.float64).reshape(-1)
        b = np.asarray(want[name], dtype=np.float64).reshape(-1)
        scale = float(np.abs(b).max()) if b.size else 0.0

        def rel(fl):
            den = np.maximum(np.abs(b), fl * scale) if scale > 0 else np.ones_like(b)
            return float((np.abs(a - b) / den).max()) if b.size else 0.0
        nb = float(np.linalg.norm(b))
        out[name] = {"max_rel": rel(floor), "max_rel_at_floor": {f"{fl:g}": rel(fl) for fl in floors},
                     "norm_rel": float(np.linalg.norm(a - b)) / nb if nb > 0 else 0.0,
                     "components": int(b.size), "below_floor": int((np.abs(b) < floor * scale).sum())}
    return out
