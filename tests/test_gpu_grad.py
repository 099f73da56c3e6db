"""Gradients of a loss on spot intensities through the hand-written adjoint
kernels, against (a) autograd through the FP64 torch transcription of the
reference formulas on the same spots and (b) FP64 central finite differences
(h = 1e-6) of that transcription with the spot set held fixed.

Bars, per parameter group (fractional coordinates, B, occupancies, lattice
parameters, orientation axis-angle corrections):

* the FP64 reference gradient (autograd of the transcription) against its
  own central differences: every sampled component within 1e-5 of itself
  (floored at 1e-4 of the group's largest; 5e-5 with the precession rotation
  average, whose quadrature cuts autograd holds fixed while finite
  differences move them);
* the GPU gradient -- the adjoint alone (same upstream dL/dI) and the whole
  loss gradient -- within 1e-5 of FP64 over the group (norm-wise), against
  autograd on every component and against central differences on the
  sampled ones;
* component by component, for components above 1e-2 of their group's
  largest: within 1e-4 (adjoint) and 1e-3 (loss gradient).  Smaller
  components carry the FP32 rounding of the forward intensities (which enter
  the residual I - T) and of the adjoint's per-spot products, relative to
  much larger terms that cancel in their sums; every test prints the full
  error distribution.
"""
import warnings

import numpy as np
import pytest

import bench
from oracle import autograd_reference as ar
from oracle import kinematic as ok
from tests import parity_util as pu

pytestmark = pytest.mark.gpu

FLOOR = 1e-4
NAMES = ["xyz", "B", "occupancy", "lattice", "axis-angle"]


@pytest.fixture(scope="module", autouse=True)
def cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import __graft_entry__
    __graft_entry__.build()
    torch.cuda.set_device(0)


def make_case(n_atoms=12, n_orient=24, seed=0):
    rng = np.random.default_rng(seed)
    els = list(rng.choice(["O", "Si", "Fe"], n_atoms))
    base = dict(lattice=np.array([7.1, 9.3, 12.4, 90.0, 90.0, 90.0]), xyz=rng.random((n_atoms, 3)),
                B=rng.uniform(0.3, 1.5, n_atoms), occ=np.ones(n_atoms),
                q=bench.cone_quaternions(n_orient, 5.0, seed + 1))
    # target: the perturbations of the differentiation workload
    ax = rng.standard_normal((n_orient, 3))
    ax *= np.radians(0.2) / np.linalg.norm(ax, axis=1, keepdims=True)
    tgt = dict(lattice=base["lattice"] * np.array([1.002, 1.002, 1.002, 1, 1, 1]),
               xyz=base["xyz"] + rng.normal(0, 0.01, (n_atoms, 3)), B=base["B"] * (1 + rng.normal(0, 0.1, n_atoms)),
               occ=base["occ"] * rng.uniform(0.9, 1.0, n_atoms), rotvec=ax)
    return els, base, tgt


def workload_case(n_orient):
    """The differentiation workload of ``bench.py`` (64 atoms, 300 kV,
    r = 1.5, sinc, 1 deg precession) on its first ``n_orient`` orientations."""
    G = bench.grad_problem(n_orient)
    base = dict(lattice=G["lattice"], xyz=G["xyz"], B=G["B"], occ=G["occ"], q=G["q0"])
    tgt = dict(lattice=G["target_lattice"], xyz=G["target_xyz"], B=G["target_B"], occ=G["target_occ"],
               rotvec=G["target_rotvec"])
    return G["elements"], base, tgt


def run_and_check(els, base, tgt, p, n_fd=10, min_spots=200, rv0_scale=1e-3):
    """The GPU gradients against the FP64 transcription on the same spots:

    * the adjoint alone: the GPU's and the transcription's vector-Jacobian
      products with the same upstream dL/dI = 2 (I - T);
    * the loss gradient: the whole chain (the GPU forward's FP32 intensities
      in the residual) against autograd of the FP64 loss, and against FP64
      central differences of that loss on ``n_fd`` components per group
      (all six lattice parameters), which also pin the transcription's
      autograd.
    Returns the error summary; asserts after collecting it."""
    import torch
    from diffsims_gb300.autograd import SpotModel, compose_axis_angle, reciprocal_basis, simulate_intensities, spot_loss
    dev = torch.device("cuda", 0)
    model = SpotModel(els, pu.generator_for(p), p.reciprocal_radius, p.max_excitation_error)
    T = lambda a: torch.as_tensor(np.asarray(a, dtype=np.float64), device=dev)
    q0 = T(base["q"])
    with torch.no_grad():
        target = simulate_intensities(model, T(tgt["xyz"]), T(tgt["B"]), T(tgt["occ"]),
                                      reciprocal_basis(torch.as_tensor(tgt["lattice"])),
                                      compose_axis_angle(q0, T(tgt["rotvec"])))
    # a non-zero starting rotation vector exercises the general axis-angle Jacobian
    rv0 = np.random.default_rng(11).normal(0, rv0_scale, (len(base["q"]), 3))

    def params():
        return [T(base["xyz"]).requires_grad_(), T(base["B"]).requires_grad_(), T(base["occ"]).requires_grad_(),
                torch.as_tensor(base["lattice"], dtype=torch.float64).requires_grad_(), T(rv0).requires_grad_()]

    ps = params()
    sim = simulate_intensities(model, ps[0], ps[1], ps[2], reciprocal_basis(ps[3]), compose_axis_angle(q0, ps[4]))
    assert sim.intensity.shape[0] > min_spots
    loss_ref = ar.MatchedLoss(sim.offsets, sim.hkl, target.intensity, target.offsets, target.hkl)
    gI = 2.0 * (sim.intensity.detach() - loss_ref.target_per_spot)
    g_adj = {n: g.detach().cpu().numpy() for n, g in
             zip(NAMES, torch.autograd.grad(sim.intensity, ps, gI, retain_graph=True))}
    L = spot_loss(sim, target)
    g_gpu = {n: g.detach().cpu().numpy() for n, g in zip(NAMES, torch.autograd.grad(L, ps))}

    counts = sim.offsets[1:] - sim.offsets[:-1]
    orient = torch.repeat_interleave(torch.arange(counts.shape[0], device=dev), counts)
    hkl = sim.hkl

    def ref_I(xyz_, B_, occ_, lat_, rv_):
        with warnings.catch_warnings():
            warnings.simplefilter("ignore")
            return ar.spot_intensities(xyz_, B_, occ_, ar.reciprocal_basis_torch(lat_),
                                       ar.compose_axis_angle_torch(q0, rv_), els, "lobato", orient, hkl, p)

    ps2 = params()
    I2 = ref_I(*ps2)
    v_ref = {n: g.detach().cpu().numpy() for n, g in zip(NAMES, torch.autograd.grad(I2, ps2, gI, retain_graph=True))}
    Lr = loss_ref(I2)
    g_ref = {n: g.detach().cpu().numpy() for n, g in zip(NAMES, torch.autograd.grad(Lr, ps2))}
    adj = ar.gradient_errors(g_adj, v_ref, FLOOR)
    full = ar.gradient_errors(g_gpu, g_ref, FLOOR)

    # FP64 central differences of the transcription's loss (spot set fixed),
    # h = 1e-6.  L(I+) - L(I-) is summed per spot as (I+ - I-)(I+ + I- - 2T):
    # the same difference without subtracting two large totals.
    h = 1e-6
    T_spot = loss_ref.target_per_spot
    rng = np.random.default_rng(7)
    fd_ref, fd_gpu = {}, {}
    with torch.no_grad():
        vals = [t.detach().clone() for t in params()]
        for gi, name in enumerate(NAMES):
            flat = vals[gi].view(-1)
            picks = np.arange(6) if name == "lattice" else rng.choice(flat.numel(), min(n_fd, flat.numel()), False)
            scale = np.abs(g_ref[name]).max()
            fds = []
            for k in picks:
                old = flat[k].item()
                flat[k] = old + h
                Ip = ref_I(*vals)
                flat[k] = old - h
                Im = ref_I(*vals)
                flat[k] = old
                fds.append(float(((Ip - Im) * (Ip + Im - 2.0 * T_spot)).sum()) / (2 * h))
            fds = np.array(fds)
            den = np.maximum(np.abs(fds), FLOOR * scale)
            fd_ref[name] = float(np.max(np.abs(g_ref[name].reshape(-1)[picks] - fds) / den))
            a = g_gpu[name].reshape(-1)[picks]
            fd_gpu[name] = {"max_rel": float(np.max(np.abs(a - fds) / den)),
                            "norm_rel": float(np.linalg.norm(a - fds) / max(np.linalg.norm(fds), 1e-300)),
                            "components": int(len(picks))}
    res = {"adjoint": adj, "loss_gradient": full, "fd_vs_transcription": fd_ref, "fd_vs_gpu": fd_gpu,
           "spots": int(sim.intensity.shape[0]),
           "loss_rel": abs(float(L.detach()) - float(Lr.detach())) / float(Lr.detach())}
    print(res)
    assert res["loss_rel"] <= 1e-5
    for name in NAMES:
        # the FP64 reference gradient itself, every sampled component (5e-5
        # with the rotation average: autograd holds its quadrature cuts fixed,
        # finite differences move them with the parameters)
        fd_tol = 5e-5 if p.precession_angle and not p.approximate_precession else 1e-5
        assert fd_ref[name] <= fd_tol, (name, "transcription autograd vs its central differences", res)
        # the GPU gradient: within 1e-5 of FP64 over each parameter group
        assert adj[name]["norm_rel"] <= 1e-5, (name, "adjoint", res)
        assert full[name]["norm_rel"] <= 1e-5, (name, "loss gradient", res)
        assert fd_gpu[name]["norm_rel"] <= 1e-5, (name, "GPU gradient vs central differences", res)
        # and component by component, for components above 1e-2 of their
        # group's largest: 1e-4 for the adjoint alone, 1e-3 for the loss
        # gradient (the FP32 forward intensities enter the residual I - T)
        assert adj[name]["max_rel_at_floor"]["0.01"] <= 1e-4, (name, "adjoint per component", res)
        assert full[name]["max_rel_at_floor"]["0.01"] <= 1e-3, (name, "loss gradient per component", res)
    return res


CASES = [
    dict(shape_factor_model="sinc", precession_angle=1.0, approximate_precession=False),
    dict(shape_factor_model="sinc", precession_angle=1.0),
    dict(shape_factor_model="linear"),
    dict(shape_factor_model="lorentzian"),
    dict(shape_factor_model="atanc", precession_angle=0.5, approximate_precession=False),
]


@pytest.mark.parametrize("kw", CASES, ids=lambda k: "-".join(f"{v}" for v in k.values()))
def test_gradient_matches_reference_and_finite_differences(kw):
    els, base, tgt = make_case()
    p = ok.SimParams(accelerating_voltage=300, reciprocal_radius=1.0, max_excitation_error=0.015, **kw)
    run_and_check(els, base, tgt, p)


@pytest.mark.parametrize("approximate", [False, True])
def test_gradient_differentiation_workload(approximate):
    """The differentiation workload's own crystal and settings (64 atoms,
    300 kV, r = 1.5, s_max = 0.015, sinc with 1 deg precession: the rotation
    average, and the reference's default lorentzian_precession) on its first
    256 cone orientations, 20 finite-difference components per group."""
    W = bench.GRAD_WORKLOAD
    els, base, tgt = workload_case(256)
    p = ok.SimParams(accelerating_voltage=W["accelerating_voltage"], reciprocal_radius=W["reciprocal_radius"],
                     max_excitation_error=W["max_excitation_error"], shape_factor_model=W["shape_factor_model"],
                     precession_angle=W["precession_angle"], approximate_precession=approximate)
    res = run_and_check(els, base, tgt, p, n_fd=20, min_spots=20000, rv0_scale=0.0)
    print(approximate, res)


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
