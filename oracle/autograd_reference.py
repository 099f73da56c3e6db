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
    cut_lists = []
    for i in range(s0.shape[0]):
        cuts = [0.0, math.pi]
        if h > 0 and ad[i] > 0:
            ks = np.arange(np.ceil((s0d[i] - ad[i]) / h), np.floor((s0d[i] + ad[i]) / h) + 1)
            cuts += np.arccos(np.clip((ks * h - s0d[i]) / ad[i], -1, 1)).tolist()
        cut_lists.append(np.unique(cuts))
    m = max((len(c) for c in cut_lists), default=2)
    cuts = np.array([np.concatenate([c, np.full(m - len(c), math.pi)]) for c in cut_lists]).reshape(-1, m)
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
