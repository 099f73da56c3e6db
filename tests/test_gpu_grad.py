"""Gradients of a loss on spot intensities through the hand-written adjoint
kernels, against (a) autograd through the FP64 torch transcription of the
reference formulas on the same spots and (b) FP64 central finite differences
(h = 1e-6) of that transcription.  Bar: 1e-5 of the largest gradient of each
parameter group (coordinates, B, occupancies, lattice, orientations).
"""
import warnings

import numpy as np
import pytest

from oracle import autograd_reference as ar
from oracle import kinematic as ok
from tests import parity_util as pu

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import __graft_entry__
    __graft_entry__.build()
    torch.cuda.set_device(0)


def cone_quaternions(n, deg, seed):
    """Rotations within ``deg`` of the identity (axis uniform, cos(angle)
    uniform): beams within a cone about [001]."""
    rng = np.random.default_rng(seed)
    ax = rng.standard_normal((n, 3))
    ax /= np.linalg.norm(ax, axis=1, keepdims=True)
    th = np.arccos(rng.uniform(np.cos(np.radians(deg)), 1.0, n))
    return np.c_[np.cos(th / 2), np.sin(th / 2)[:, None] * ax]


def make_case(n_atoms=12, n_orient=24, seed=0):
    rng = np.random.default_rng(seed)
    els = list(rng.choice(["O", "Si", "Fe"], n_atoms))
    base = dict(lattice=np.array([7.1, 9.3, 12.4, 90.0, 90.0, 90.0]), xyz=rng.random((n_atoms, 3)),
                B=rng.uniform(0.3, 1.5, n_atoms), occ=np.ones(n_atoms), q=cone_quaternions(n_orient, 5.0, seed + 1))
    # target: the perturbations of the differentiation workload
    ax = rng.standard_normal((n_orient, 3))
    ax /= np.linalg.norm(ax, axis=1, keepdims=True)
    dq = np.c_[np.cos(np.radians(0.1)) * np.ones(n_orient), np.sin(np.radians(0.1)) * ax]
    w1, v1 = base["q"][:, :1], base["q"][:, 1:]
    w2, v2 = dq[:, :1], dq[:, 1:]
    qt = np.c_[w1 * w2 - (v1 * v2).sum(1, keepdims=True), w1 * v2 + w2 * v1 + np.cross(v1, v2)]
    tgt = dict(lattice=base["lattice"] * np.array([1.002, 1.002, 1.002, 1, 1, 1]),
               xyz=base["xyz"] + rng.normal(0, 0.01, (n_atoms, 3)), B=base["B"] * (1 + rng.normal(0, 0.1, n_atoms)),
               occ=base["occ"] * rng.uniform(0.9, 1.0, n_atoms), q=qt)
    return els, base, tgt


CASES = [
    dict(shape_factor_model="sinc", precession_angle=1.0, approximate_precession=False),
    dict(shape_factor_model="sinc", precession_angle=1.0),
    dict(shape_factor_model="linear"),
    dict(shape_factor_model="lorentzian"),
    dict(shape_factor_model="atanc", precession_angle=0.5, approximate_precession=False),
]


@pytest.mark.parametrize("kw", CASES, ids=lambda k: "-".join(f"{v}" for v in k.values()))
def test_gradient_matches_reference_and_finite_differences(kw):
    import torch
    from diffsims_gb300.autograd import (SpotIntensities, SpotModel, compose_axis_angle, reciprocal_basis,
                                         simulate_intensities, spot_loss)
    dev = torch.device("cuda", 0)
    els, base, tgt = make_case()
    p = ok.SimParams(accelerating_voltage=300, reciprocal_radius=1.0, max_excitation_error=0.015, **kw)
    model = SpotModel(els, pu.generator_for(p), p.reciprocal_radius, p.max_excitation_error)
    T = lambda a: torch.as_tensor(np.asarray(a, dtype=np.float64), device=dev)
    with torch.no_grad():
        target = simulate_intensities(model, T(tgt["xyz"]), T(tgt["B"]), T(tgt["occ"]),
                                      reciprocal_basis(T(tgt["lattice"])), T(tgt["q"]))

    def params():
        # a non-zero starting rotation vector exercises the general axis-angle Jacobian
        rv0 = np.random.default_rng(11).normal(0, 1e-3, (len(base["q"]), 3))
        return [T(base["xyz"]).requires_grad_(), T(base["B"]).requires_grad_(), T(base["occ"]).requires_grad_(),
                torch.as_tensor(base["lattice"], dtype=torch.float64).requires_grad_(), T(rv0).requires_grad_()]

    q0 = T(base["q"])
    xyz, B, occ, lat, rv = params()
    sim = simulate_intensities(model, xyz, B, occ, reciprocal_basis(lat), compose_axis_angle(q0, rv))
    L = spot_loss(sim, target)
    L.backward()
    g_gpu = [t.grad.detach().cpu().numpy() for t in (xyz, B, occ, lat, rv)]
    assert sim.intensity.shape[0] > 200

    counts = (sim.offsets[1:] - sim.offsets[:-1])
    orient = torch.repeat_interleave(torch.arange(counts.shape[0], device=dev), counts)
    hkl = sim.hkl

    def ref_loss(xyz, B, occ, lat, rv):
        I = ar.spot_intensities(xyz, B, occ, ar.reciprocal_basis_torch(lat), ar.compose_axis_angle_torch(q0, rv),
                                els, "lobato", orient, hkl, p)
        return spot_loss(SpotIntensities(I, sim.offsets, hkl), target)

    xyz2, B2, occ2, lat2, rv2 = params()
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        Lr = ref_loss(xyz2, B2, occ2, lat2, rv2)
        Lr.backward()
    g_ref = [t.grad.detach().cpu().numpy() for t in (xyz2, B2, occ2, lat2, rv2)]
    assert abs(float(L) - float(Lr)) <= 1e-5 * float(Lr)
    names = ["xyz", "B", "occupancy", "lattice", "axis-angle"]
    for name, a, b in zip(names, g_gpu, g_ref):
        scale = np.abs(b).max()
        assert scale > 0, name
        err = np.abs(a - b).max() / scale
        assert err <= 1e-5, (name, err)

    # FP64 central differences of the transcription, a few components per group
    h = 1e-6
    rng = np.random.default_rng(7)
    with torch.no_grad():
        vals = [t.detach().clone() for t in params()]
        for gi, name in enumerate(names):
            flat = vals[gi].view(-1)
            picks = rng.choice(flat.numel(), size=min(3, flat.numel()), replace=False)
            if name == "lattice":
                picks = np.arange(6)
            for k in picks:
                old = flat[k].item()
                flat[k] = old + h
                lp = float(ref_loss(*vals))
                flat[k] = old - h
                lm = float(ref_loss(*vals))
                flat[k] = old
                fd = (lp - lm) / (2 * h)
                got = g_gpu[gi].reshape(-1)[k]
                assert abs(got - fd) <= 1e-5 * np.abs(g_ref[gi]).max() + 1e-5 * abs(fd), (name, k, got, fd)


def test_gradient_flows_only_where_asked():
    """A loss on a subset of spots: zero upstream gradient elsewhere gives the
    same result as dropping those spots."""
    import torch
    from diffsims_gb300.autograd import SpotModel, reciprocal_basis, simulate_intensities
    dev = torch.device("cuda", 0)
    els, base, _ = make_case(8, 10, seed=3)
    p = ok.SimParams(accelerating_voltage=300, reciprocal_radius=1.0, max_excitation_error=0.015,
                     shape_factor_model="lorentzian")
    model = SpotModel(els, pu.generator_for(p), p.reciprocal_radius, p.max_excitation_error)
    T = lambda a: torch.as_tensor(np.asarray(a, dtype=np.float64), device=dev)
    xyz = T(base["xyz"]).requires_grad_()
    sim = simulate_intensities(model, xyz, T(base["B"]), T(base["occ"]), reciprocal_basis(T(base["lattice"])),
                               T(base["q"]))
    (sim.intensity[:5].sum() * 0.0).backward()
    assert torch.count_nonzero(xyz.grad) == 0
