"""Benchmark of the kinematical spot-pattern path on one GB300.

Workload (the large single-phase case): synthetic triclinic P1 cell, a, b, c
uniform in [8, 15] Angstrom, alpha, beta, gamma uniform in [70, 110] deg, 200
atoms with fractional coordinates uniform in [0, 1)^3, Z uniform in
{6, 7, 8, 14, 26}, occupancy 1, B uniform in [0.3, 1.5] Angstrom^2;
200 kV, reciprocal_radius 2.0 1/Angstrom, max_excitation_error 0.02,
lorentzian shape factor, Lobato scattering factors; 100,000 orientations
uniform on SO(3).  Seeded synthetic data (no dataset is involved).

A step = one pass of the hot path over the batch: hkl enumeration, the
structure-factor table, and the per-orientation kernel (rotation, excitation
error, selection, shape factor, intensity, mask, ordered CSR output).

Arms:
  default           the CUDA path (mixed form).  value = patterns/s with the
                    inputs resident in HBM; e2e = the same through the public
                    API with host quaternions in and all spots copied back.
                    Extra legs in the same line: "grad" (gradient step of the
                    differentiation workload against its forward pass),
                    "batched_phases" (32 uneven phases in one launch, graph
                    replay, tile by the autotuner),
                    "template_library" (three phases simulated and rasterised
                    to 256x256 detectors in 8192-orientation chunks),
                    "family_structure_factors" (Doyle-Turner structure
                    factors of 2^20 lattice-plane families in one launch,
                    against the oracle's per-family loop on one core),
                    "legacy_ed_data" (the legacy DiffractionGenerator:
                    100,000 Euler triples of one structure in one launch,
                    against the oracle's per-orientation call on one core),
                    "polar_templates" (polar_flatten_simulations of the
                    headline's 100,000 patterns, unbinned and binned, HBM
                    roofline, against the oracle's numpy restatement),
                    "profiles_1d" (calculate_diffraction1d of the headline's
                    200-atom cell, public call, against the oracle).
  --impl reference  the reference's CPU path restated in numpy (the FP64
                    oracle) on all host cores, a bounded sample per step.

Several GPUs (torchrun): every rank runs the same per-GPU workload (weak
scaling; orientations are independent, there is no exchange), the timed
region is bracketed by barriers, the slowest rank's time counts and rank 0
reports; the extra legs run on rank 0 only.
"""
from __future__ import annotations

import argparse
import json
import math
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = dict(workload="triclinic P1, 200 atoms, 200 kV, r=2.0, s_max=0.02, lorentzian, lobato, 100k orientations",
                cell_seed=1, orientation_seed=0, n_orientations=100_000, n_atoms=200, reciprocal_radius=2.0,
                max_excitation_error=0.02, accelerating_voltage=200, shape_factor_model="lorentzian")
METRIC = "orientation patterns/s"
# measured: (dram__bytes_read.sum + dram__bytes_write.sum) / spots written, one
# simulate_kernel launch on 8192 orientations of the workload below
DRAM_BYTES_PER_SPOT = 21.8
UNIT = "patterns/s"


GRAD_WORKLOAD = dict(workload="orthorhombic 7.1/9.3/12.4, 64 atoms, 4096 orientations in a 5 deg cone about [001], "
                              "300 kV, r=1.5, sinc with 1 deg precession (rotation average), loss = sum of squared "
                              "spot-intensity differences to perturbed-parameter targets",
                     seed=4, n_atoms=64, n_orientations=4096, cone_deg=5.0, accelerating_voltage=300,
                     reciprocal_radius=1.5, max_excitation_error=0.015, shape_factor_model="sinc",
                     precession_angle=1.0, approximate_precession=False)
BATCH_WORKLOAD = dict(workload="32 phases, cell edges 3-20 A, angles 80-100 deg, 1-500 atoms, 1k-50k orientations each, "
                               "200 kV, r=1.5, sinc, s_max=0.015; one persistent launch in a CUDA graph, tile by the "
                               "autotuner",
                      n_phases=32, seed=3, accelerating_voltage=200, reciprocal_radius=1.5, max_excitation_error=0.015,
                      shape_factor_model="sinc")
LIBRARY_WORKLOAD = dict(workload="template library: Al FCC, Fe BCC, P1 60 atoms; 200k orientations per phase, 200 kV, "
                                 "r=1.2, linear with 0.5 deg precession (rotation average), 256x256 float32 detector, "
                                 "sigma 1 px, 8192-orientation chunks",
                        n_orientations=200_000, chunk=8192, accelerating_voltage=200, reciprocal_radius=1.2,
                        max_excitation_error=0.01, shape_factor_model="linear", precession_angle=0.5,
                        approximate_precession=False, shape=(256, 256), sigma=1.0, calibration=1.2 / 128, seed=5)


def make_crystal(seed=1, n_atoms=200):
    rng = np.random.default_rng(seed)
    lat = tuple(rng.uniform(8, 15, 3)) + tuple(rng.uniform(70, 110, 3))
    els = list(rng.choice(["C", "N", "O", "Si", "Fe"], n_atoms))
    xyz = rng.random((n_atoms, 3))
    B = rng.uniform(0.3, 1.5, n_atoms)
    return lat, els, xyz, B


def uniform_quaternions(n, seed=0):
    rng = np.random.default_rng(seed)
    q = rng.standard_normal((n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    q[q[:, 0] < 0] *= -1
    return q


BATCH_ELEMENTS = ["C", "N", "O", "Al", "Si", "Ti", "Fe", "Cu"]


def batch_phase_specs(seed=BATCH_WORKLOAD["seed"], n_phases=BATCH_WORKLOAD["n_phases"]):
    """The uneven phases of the batched workload, in draw order: per phase
    (lattice (a, b, c, alpha, beta, gamma), elements, fractional xyz, B,
    orientation count, orientation seed)."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n_phases):
        lat = tuple(rng.uniform(3, 20, 3)) + tuple(rng.uniform(80, 100, 3))
        n_a = int(rng.integers(1, 501))
        els = list(rng.choice(BATCH_ELEMENTS, n_a))
        xyz = rng.random((n_a, 3))
        B = rng.uniform(0.3, 1.5, n_a)
        out.append((lat, els, xyz, B, int(rng.integers(1000, 50001)), 1000 + k))
    return out


def library_phase_specs(seed=LIBRARY_WORKLOAD["seed"]):
    """The template library's three phases: per phase (name, lattice,
    elements, fractional xyz, B); Al FCC, Fe BCC, and a 60-atom P1 cell."""
    rng = np.random.default_rng(seed)
    lat = tuple(rng.uniform(6, 10, 3)) + tuple(rng.uniform(70, 110, 3))
    p1_els = list(rng.choice(["C", "N", "O", "Si", "Fe"], 60))
    p1_xyz = rng.random((60, 3))
    p1_B = rng.uniform(0.3, 1.5, 60)
    return [("Al", (4.05, 4.05, 4.05, 90, 90, 90), ["Al"] * 4,
             np.array([[0, 0, 0], [0, .5, .5], [.5, 0, .5], [.5, .5, 0]], dtype=np.float64), np.full(4, 0.5)),
            ("Fe", (2.87, 2.87, 2.87, 90, 90, 90), ["Fe"] * 2, np.array([[0, 0, 0], [.5, .5, .5]], dtype=np.float64),
             np.full(2, 0.35)),
            ("P1", lat, p1_els, p1_xyz, p1_B)]


def phase_of(name, lat, els, xyz):
    import diffsims_gb300 as ds
    return ds.Phase(name, ds.Structure([ds.Atom(e, x) for e, x in zip(els, xyz)], ds.Lattice(*lat)))


# --------------------------------------------------------------------- CPU
def _cpu_worker(args):
    """Reference CPU path (oracle restatement) on a slice of orientations."""
    os.environ.setdefault("OMP_NUM_THREADS", "1")
    from oracle import kinematic as ok
    lat, els, xyz, B, q, kv, r, eps, shape = args
    cr = ok.Crystal(lat, els, xyz, B=B)
    p = ok.SimParams(accelerating_voltage=kv, reciprocal_radius=r, max_excitation_error=eps, shape_factor_model=shape)
    table = ok.phase_table(cr, p)
    n = 0
    for R in ok.quaternion_to_matrix(q):
        n += ok.simulate_orientation(cr, p, table, R).hkl.shape[0]
    return n


def cpu_reference_rate(n_sample, cores, seed=0):
    """patterns/s of the FP64 numpy restatement of the reference's path on
    ``cores`` worker processes (spawned), OMP_NUM_THREADS=1 each."""
    lat, els, xyz, B = make_crystal(WORKLOAD["cell_seed"], WORKLOAD["n_atoms"])
    q = uniform_quaternions(n_sample, seed)
    chunks = np.array_split(q, cores)
    args = [(lat, els, xyz, B, c, WORKLOAD["accelerating_voltage"], WORKLOAD["reciprocal_radius"],
             WORKLOAD["max_excitation_error"], WORKLOAD["shape_factor_model"]) for c in chunks if len(c)]
    ctx = mp.get_context("spawn")
    with ctx.Pool(len(args)) as pool:
        pool.map(_cpu_worker, [(a[0], a[1], a[2], a[3], a[4][:1]) + a[5:] for a in args])  # warm the workers
        t0 = time.perf_counter()
        spots = sum(pool.map(_cpu_worker, args))
        dt = time.perf_counter() - t0
    return n_sample / dt, dt, spots


def _cpu_phase_worker(args):
    """The oracle's per-orientation path (the reference's algorithm) over a
    slice of one phase's orientations; optionally each pattern rasterised by
    the reference's recipe.  Returns the spot count."""
    os.environ.setdefault("OMP_NUM_THREADS", "1")
    import warnings
    from oracle import kinematic as ok
    lat, els, xyz, B, q, params, raster = args
    cr = ok.Crystal(lat, els, xyz, B=B)
    p = ok.SimParams(**params)
    table = ok.phase_table(cr, p)
    n = 0
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        for R in ok.quaternion_to_matrix(q):
            pat = ok.simulate_orientation(cr, p, table, R)
            n += pat.hkl.shape[0]
            if raster is not None:
                ok.diffraction_pattern(pat.xyz, pat.intensity, raster["shape"], sigma=raster["sigma"],
                                       calibration=raster["calibration"])
    return n


def cpu_phases_rate(jobs, cores):
    """patterns/s of the oracle over ``jobs`` (each: lat, els, xyz, B,
    quaternions, SimParams keywords, raster settings or None), every job's
    orientations split over ``cores`` spawned workers."""
    tasks = []
    for lat, els, xyz, B, q, params, raster in jobs:
        for part in np.array_split(q, max(1, min(cores, len(q)))):
            if len(part):
                tasks.append((lat, els, xyz, B, part, params, raster))
    n_pat = sum(len(t[4]) for t in tasks)
    ctx = mp.get_context("spawn")
    with ctx.Pool(cores) as pool:
        pool.map(_cpu_phase_worker, [t[:4] + (t[4][:1],) + t[5:] for t in tasks[:cores]])  # warm the workers
        t0 = time.perf_counter()
        spots = sum(pool.map(_cpu_phase_worker, tasks, chunksize=1))
        dt = time.perf_counter() - t0
    return n_pat / dt, dt, n_pat, spots


# --------------------------------------------------------------- clocks
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, out_path=None):
        self.out_path = out_path
        self.proc = None

    def __enter__(self):
        try:
            self.f = open(self.out_path, "w") if self.out_path else subprocess.DEVNULL
            self.tmp = self.out_path or os.path.join("/tmp", f"clocks_{os.getpid()}.csv")
            if not self.out_path:
                self.f = open(self.tmp, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-lms", "200", "-i", os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0]],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            time.sleep(0.25)
            self.proc.terminate()
            self.proc.wait(timeout=5)
            self.f.close()

    def summary(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.tmp) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    smax = float(parts[2])
                except ValueError:
                    continue
                for nm, v in zip(names, parts[5:9]):
                    if v.lower() == "active":
                        reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax, "samples": len(sm),
                "reasons": sorted(reasons)}


# ------------------------------------------------------------------ GPU
def fp32_peak_tflops(torch, lib, N):
    """Measured FP32 FMA throughput of this GPU (the screening kernel's
    roofline denominator); best of 5."""
    blocks = 152 * 8
    iters = 4096
    out = torch.empty(blocks * 256, dtype=torch.float32, device="cuda")
    st = torch.cuda.current_stream()
    best = 0.0
    for _ in range(6):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        N.check(lib.ds_probe_fp32_fma(iters, blocks, N.ptr(out), N.stream_handle()), "probe")
        e1.record(st)
        e1.synchronize()
        ms = e0.elapsed_time(e1)
        best = max(best, blocks * 256 * iters * 256 / (ms * 1e-3) / 1e12)
    return best


def fp32_nominal_tflops(torch):
    """Nominal FP32 FMA peak of this GPU: SMs x 128 FP32 lanes x 2 FLOP x the
    maximum SM clock (2.07 GHz on GB300: 152 x 128 x 2 x 2.07e9 = 80.5
    TFLOP/s), stated beside the measured figure."""
    n_sm = torch.cuda.get_device_properties(0).multi_processor_count
    mhz = 2070.0
    try:
        import subprocess
        out = subprocess.run(["nvidia-smi", "--query-gpu=clocks.max.sm", "--format=csv,noheader,nounits", "-i", "0"],
                             capture_output=True, text=True, timeout=20).stdout.strip().splitlines()
        if out:
            mhz = float(out[0])
    except (OSError, ValueError, subprocess.SubprocessError):
        pass
    return {"tflops": n_sm * 128 * 2 * mhz * 1e6 / 1e12, "basis": f"{n_sm} SMs x 128 FP32 lanes x 2 FLOP x {mhz:.0f} MHz"}


def _hbm_peak():
    """(GB/s, source) of the HBM copy bandwidth: MEASURED_PEAKS.json when
    present, else the fallback figure."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            v = json.load(f).get("hbm_gbs")
        if v:
            return float(v), "MEASURED_PEAKS.json"
    except (OSError, ValueError):
        pass
    return 6800.0, "fallback"


def rank_shard(n_per_rank, seed, rank):
    """This rank's orientations: an independent uniform set drawn from
    ``seed + 1000 * rank`` (weak scaling -- each rank simulates its own
    shard; rank 0's shard is the single-GPU workload)."""
    return uniform_quaternions(n_per_rank, seed + 1000 * rank)


def max_over_ranks(value, dist, device):
    """The largest value over all ranks (one all-reduce of one number; the
    slowest rank's step time sets the whole job's)."""
    import torch
    if dist is None:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def run_gpu(args):
    import torch
    import diffsims_gb300 as ds
    from diffsims_gb300 import _native as N
    from diffsims_gb300.engine import PhaseTable, SpotBuffers, simulate_phase

    lib = N.load_library()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)
    lat, els, xyz, B = make_crystal(WORKLOAD["cell_seed"], WORKLOAD["n_atoms"])
    phase = ds.Phase("P1", ds.Structure([ds.Atom(e, x) for e, x in zip(els, xyz)], ds.Lattice(*lat)))
    n_o = args.orientations
    q_host = rank_shard(n_o, WORKLOAD["orientation_seed"], rank)
    gen = ds.SimulationGenerator(WORKLOAD["accelerating_voltage"], "lobato",
                                 shape_factor_model=WORKLOAD["shape_factor_model"])
    gen.host_transfer = args.host_transfer
    r = WORKLOAD["reciprocal_radius"]
    settings = gen.settings(WORKLOAD["max_excitation_error"], form="mixed")
    settings.screen = args.screen
    q_dev = torch.from_numpy(q_host).to(dev)
    table = PhaseTable(phase, r, True, "lobato", list(B), form="mixed", device=dev, build=True)
    buffers = SpotBuffers(dev)
    st = torch.cuda.current_stream()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)  # 256 MB > L2

    def step():
        table.build()
        return simulate_phase(table, q_dev, settings, r, buffers)

    for _ in range(args.warmup):
        spots = step()
    torch.cuda.synchronize()
    step_ms, kern_ms = [], []
    with ClockSampler(os.path.join(args.out_dir, "clocks.csv") if args.out_dir and rank == 0 else None) as clk:
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        t_all = time.perf_counter()
        for _ in range(args.steps):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(st)
            spots = step()
            e1.record(st)
            e1.synchronize()
            step_ms.append(e0.elapsed_time(e1))
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        wall = time.perf_counter() - t_all
        # the dominant kernel alone (simulate), timed on its launch stream
        for _ in range(args.steps):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(st)
            simulate_phase(table, q_dev, settings, r, buffers, sync=False)
            e1.record(st)
            e1.synchronize()
            kern_ms.append(e0.elapsed_time(e1))
    clocks = clk.summary()
    ms = statistics.mean(step_ms)
    if dist:
        ms = max_over_ranks(ms, dist, dev)  # the slowest rank's step time
        if rank != 0:
            dist.destroy_process_group()
            return
    if args.device_only:
        print(json.dumps({"device_only": True, "ms_per_step": ms, "kernel_ms": statistics.mean(kern_ms),
                          "patterns_per_s": n_o / (ms * 1e-3), "n_hkl": table.n, "spots": spots.total}))
        return
    value = world * n_o / (ms * 1e-3)
    total_spots = spots.total
    n_h = table.n

    # ---- end to end through the public API with host buffers
    rot_host = ds.Rotation(q_host)
    e2e_ms, e2e_split = [], []
    h2d = q_host.nbytes
    d2h = 0
    for it in range(args.warmup + args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        sim = gen.calculate_diffraction2d(phase, rot_host, reciprocal_radius=r,
                                          max_excitation_error=WORKLOAD["max_excitation_error"],
                                          debye_waller_factors=list(B), timing=True)
        sp = sim.spots(0)
        sp.host(pinned=True)
        dt = time.perf_counter() - t0
        if it >= args.warmup:
            e2e_ms.append(dt * 1e3)
            e2e_split.append(sp.timings())
        d2h = sp.nbytes()
        transfer = "stores" if type(sp).__name__ == "HostSpots" else "copies"
        del sim, sp
    e2e_value = n_o / (statistics.mean(e2e_ms) * 1e-3)
    breakdown = {k: statistics.mean(t[k] for t in e2e_split) for k in e2e_split[0] if k != "chunks"}
    breakdown["chunks"] = e2e_split[0].get("chunks")
    breakdown["d2h_bytes"] = int(d2h)
    breakdown["copy_span_gbs"] = d2h / (breakdown["copy_span_ms"] * 1e-3) / 1e9 if breakdown.get(
        "copy_span_ms") else None
    breakdown["pinned_pool_bytes"] = gen._host_pool.allocated_bytes
    breakdown["calls_ms"] = [round(x, 3) for x in e2e_ms]  # every timed call (the link is shared with the host's other load)
    breakdown["median_call_ms"] = statistics.median(e2e_ms)  # beside the mean that value and ms_per_step report
    breakdown["host_transfer"] = transfer
    breakdown["note"] = ("host ms per call: table (enumeration + structure factors, one count read), quaternion "
                         "upload, launch set-up, waits for the kernel (chunk_wait_ms), pinned-pool allocation (0 once "
                         "warm), the wrap in host(); device ms from CUDA events: the kernel's span and the transfer's "
                         "span, the same span when the kernel stores the spots into page-locked host memory itself "
                         "(host_transfer 'stores', one launch); copy_span_gbs = the spots' bytes over the transfer "
                         "span (the device-to-host rate the call achieved)")

    # ---- roofline of the dominant kernel (FP32 issue-bound screen)
    peak32 = fp32_peak_tflops(torch, lib, N)
    kms = statistics.mean(kern_ms)
    flops = 10.0 * n_o * n_h  # algorithmic FP32 FLOP per (orientation, row) pair
    achieved = flops / (kms * 1e-3) / 1e12
    bytes_alg = total_spots * 20 + (n_o + 1) * 8 + n_o * 32 + n_h * 32
    hbm_peak, hbm_src = _hbm_peak()
    # DRAM bytes of one launch: the per-spot figure of the ncu capture in
    # profiles/simulate_kernel_p1_8192.md (8192 orientations of this workload)
    # scaled by the spots of this launch
    traffic = DRAM_BYTES_PER_SPOT * total_spots

    # ---- the all-FP64 GPU form on the same 100k orientations (tables built
    # outside the timed launches; the table builds timed on their own)
    t64 = PhaseTable(phase, r, True, "lobato", list(B), form="fp64", device=dev)
    s64 = gen.settings(WORKLOAD["max_excitation_error"], form="fp64")
    b64 = SpotBuffers(dev)
    simulate_phase(t64, q_dev, s64, r, b64)  # sizes the outputs

    def ev_time(fn, reps):
        out = []
        for _ in range(reps):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(st)
            fn()
            e1.record(st)
            e1.synchronize()
            out.append(e0.elapsed_time(e1))
        return statistics.mean(out)

    reps64 = max(1, min(args.steps, 3))
    fp64_kernel_ms = ev_time(lambda: simulate_phase(t64, q_dev, s64, r, b64, sync=False), reps64)
    fp64_table_ms = ev_time(t64.build, reps64)
    mixed_table_ms = ev_time(table.build, reps64)
    fp64_rate = n_o / (fp64_kernel_ms * 1e-3)
    # error of the mixed form against the FP64 form on a subset (per pair, with excitation errors)
    n_cmp = min(args.fp64_orientations, n_o)
    q_cmp = q_dev[:n_cmp].contiguous()
    b64s = SpotBuffers(dev, with_excitation_error=True)
    ref64 = simulate_phase(t64, q_cmp, s64, r, b64s)
    mixed = simulate_phase(table, q_cmp, settings, r, SpotBuffers(dev, with_excitation_error=True))
    err = compare_forms(mixed, ref64, table, q_host[:n_cmp], settings)
    # both forms against the FP64 oracle on the first orientations (the checker; untimed)
    err_oracle = None
    if not args.no_oracle_check:
        err_oracle = oracle_errors(lat, els, xyz, B, q_host[:args.oracle_orientations],
                                   {"mixed": host_csr_first(table, q_dev, settings, r, args.oracle_orientations),
                                    "fp64": host_csr_first(t64, q_dev, s64, r, args.oracle_orientations)})

    grad = None if args.skip_grad else run_grad(args, torch, dev)
    batched = None if args.skip_batch else run_batch(args, torch, dev)
    library = None if args.skip_library else run_library(args, torch, dev, hbm_peak)
    families = None if args.skip_families else run_families(args, torch, dev)
    legacy = None if args.skip_legacy else run_legacy(args, torch, dev)
    polar = None if args.skip_polar else run_polar(args, torch, dev, hbm_peak, spots)
    profiles = None if args.skip_profiles else run_profiles(args, torch, dev)

    cpu = None
    if not args.no_cpu_baseline:
        cores = os.cpu_count() or 1
        rate, dt, _ = cpu_reference_rate(args.cpu_sample, cores)
        cpu = {"value": rate, "unit": UNIT, "cores": cores, "kind": "port",
               "sample": f"{args.cpu_sample} orientations of the same workload, FP64 numpy restatement of the "
                         f"reference path, {cores} spawned processes, {dt:.1f} s"}

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
        "data": "synthetic (seeded P1 cell and uniform SO(3) orientations)",
        "config": dict(WORKLOAD, n_orientations=n_o, n_hkl=n_h, spots_per_step=total_spots,
                       l2="256 MB buffer written between timed steps", form="mixed"),
        "spots_per_s": total_spots / (ms * 1e-3),
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                "ms_per_step": statistics.mean(e2e_ms), "ranks": 1, "breakdown": breakdown},
        "roofline": {"bound": "fp32", "achieved": achieved, "peak": peak32, "unit": "TFLOP/s",
                     "frac": achieved / peak32, "traffic": traffic, "kernel": "simulate_kernel",
                     "kernel_ms": kms, "peak_source": "measured by bench.py FMA probe (ds_probe_fp32_fma)",
                     "peak_nominal": fp32_nominal_tflops(torch),
                     "hbm": {"achieved_gbs": bytes_alg / (kms * 1e-3) / 1e9, "peak_gbs": hbm_peak,
                             "frac": bytes_alg / (kms * 1e-3) / 1e9 / hbm_peak,
                             "peak_source": hbm_src}},
        "fp64_form": {"value": fp64_rate, "unit": UNIT, "orientations": n_o, "kernel_ms": fp64_kernel_ms,
                      "table_ms": fp64_table_ms, "mixed_kernel_ms": kms, "mixed_table_ms": mixed_table_ms,
                      "mixed_over_fp64": fp64_kernel_ms / kms,
                      "mixed_over_fp64_with_tables": (fp64_kernel_ms + fp64_table_ms) / (kms + mixed_table_ms),
                      "note": "both forms on the same orientations with their tables resident; table builds "
                              "(enumeration + structure factors) timed separately"},
        "error_vs_fp64_form": err,
        "error_vs_oracle": err_oracle,
        "grad": grad,
        "batched_phases": batched,
        "template_library": library,
        "family_structure_factors": families,
        "legacy_ed_data": legacy,
        "polar_templates": polar,
        "profiles_1d": profiles,
        "cpu_baseline": cpu,
        "clocks": clocks,
        "gpu_launches": 5 * args.steps,
        "wall_s_timed_region": wall,
    }
    print(json.dumps(line))
    if dist:
        dist.destroy_process_group()


def cone_quaternions(n, deg, seed):
    """Rotations within ``deg`` of the identity (axis uniform, cos(angle)
    uniform): beam directions in a cone about [001]."""
    rng = np.random.default_rng(seed)
    ax = rng.standard_normal((n, 3))
    ax /= np.linalg.norm(ax, axis=1, keepdims=True)
    th = np.arccos(rng.uniform(np.cos(np.radians(deg)), 1.0, n))
    return np.c_[np.cos(th / 2), np.sin(th / 2)[:, None] * ax]


def grad_problem(n_orient=None):
    """The differentiation workload's parameters and target perturbations, in
    draw order: orthorhombic 7.1/9.3/12.4 cell, 64 atoms (O, Si, Fe), B in
    [0.3, 1.5], cone orientations q0 (5 deg about [001]); the target has
    fractional coordinates + N(0, 0.01), B x (1 + N(0, 0.1)), occupancy x
    U(0.9, 1), lattice lengths + 0.2 % and orientations turned by 0.2 deg
    about random axes (``target_rotvec``).  ``n_orient`` keeps the first
    orientations of the full set."""
    W = GRAD_WORKLOAD
    rng = np.random.default_rng(W["seed"])
    n_a, n_o = W["n_atoms"], W["n_orientations"]
    els = list(rng.choice(["O", "Si", "Fe"], n_a))
    lat = np.array([7.1, 9.3, 12.4, 90.0, 90.0, 90.0])
    xyz, B, occ = rng.random((n_a, 3)), rng.uniform(0.3, 1.5, n_a), np.ones(n_a)
    q0 = cone_quaternions(n_o, W["cone_deg"], W["seed"] + 1)
    ax = rng.standard_normal((n_o, 3))
    ax *= np.radians(0.2) / np.linalg.norm(ax, axis=1, keepdims=True)
    out = dict(elements=els, lattice=lat, xyz=xyz, B=B, occ=occ, q0=q0, target_rotvec=ax,
               target_xyz=xyz + rng.normal(0, 0.01, xyz.shape), target_B=B * (1 + rng.normal(0, 0.1, n_a)),
               target_occ=occ * rng.uniform(0.9, 1.0, n_a), target_lattice=lat * [1.002, 1.002, 1.002, 1, 1, 1])
    if n_orient is not None:
        out["q0"], out["target_rotvec"] = q0[:n_orient], ax[:n_orient]
    return out


def run_grad(args, torch, dev):
    """Gradient step of the differentiation workload: forward (tables,
    spots, loss) and forward + adjoint, timed with the device synchronised on
    both sides (the forward reads the row and spot counts on the host); for
    the rotation average (the workload's sinc with 1 deg precession) and for
    the reference's default ``approximate_precession=True``
    (lorentzian_precession).  The rotation-average gradients are checked
    against autograd through the FP64 transcription of the reference
    formulas on the same spots (every component), and that transcription
    is timed on the host cores on a bounded sample."""
    import diffsims_gb300 as ds
    from diffsims_gb300.autograd import (SpotModel, compose_axis_angle, reciprocal_basis, simulate_intensities,
                                         spot_loss)
    W = GRAD_WORKLOAD
    G = grad_problem()
    els, lat, xyz, B, occ, q0 = G["elements"], G["lattice"], G["xyz"], G["B"], G["occ"], G["q0"]
    n_o = q0.shape[0]
    T = lambda a: torch.as_tensor(np.asarray(a, dtype=np.float64), device=dev)
    q0t = T(q0)

    def leg(approximate):
        gen = ds.SimulationGenerator(W["accelerating_voltage"], "lobato", W["precession_angle"],
                                     W["shape_factor_model"], approximate)
        model = SpotModel(els, gen, W["reciprocal_radius"], W["max_excitation_error"])
        with torch.no_grad():
            tq = compose_axis_angle(q0t, T(G["target_rotvec"]))
            target = simulate_intensities(model, T(G["target_xyz"]), T(G["target_B"]), T(G["target_occ"]),
                                          reciprocal_basis(torch.as_tensor(G["target_lattice"])), tq)
        # parameters resident where they live in a refinement loop: per-atom and
        # per-orientation values on the device, the six lattice parameters on the
        # host (the forward reads the reciprocal basis on the host)
        ps = [T(xyz), T(B), T(occ), torch.as_tensor(lat, dtype=torch.float64),
              torch.zeros((n_o, 3), dtype=torch.float64, device=dev)]

        def forward(grad):
            for t in ps:
                t.requires_grad_(grad)
                t.grad = None
            sim = simulate_intensities(model, ps[0], ps[1], ps[2], reciprocal_basis(ps[3]),
                                       compose_axis_angle(q0t, ps[4]))
            L = spot_loss(sim, target)
            if grad:
                L.backward()
            return L, sim

        def timed(grad):
            out = []
            for it in range(args.warmup + args.steps):
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                L, sim = forward(grad)
                torch.cuda.synchronize()
                if it >= args.warmup:
                    out.append((time.perf_counter() - t0) * 1e3)
            return statistics.mean(out), L, sim

        fwd_ms, L, _ = timed(False)
        grad_ms, Lg, sim = timed(True)
        return dict(gen=gen, model=model, target=target, ps=ps, fwd_ms=fwd_ms, grad_ms=grad_ms, loss=float(L),
                    sim=sim, loss_grad=float(Lg.detach()))

    main = leg(W["approximate_precession"])
    approx = leg(True)
    names = ("xyz", "B", "occupancy", "lattice", "axis_angle")
    g_gpu = {n: t.grad.detach().cpu().numpy() for n, t in zip(names, main["ps"])}
    gnorm = {n: float(np.linalg.norm(v)) for n, v in g_gpu.items()}
    check = None if args.no_oracle_check else grad_check(torch, dev, main, els, q0t, names)
    cpu = None if args.no_cpu_baseline else grad_cpu_baseline(torch, main, els, q0, n_o)
    return {"ms_per_step": main["grad_ms"], "forward_ms": main["fwd_ms"],
            "grad_over_forward": main["grad_ms"] / main["fwd_ms"], "unit": "ms", "loss": main["loss"],
            "spots": int(main["sim"].intensity.shape[0]), "gradient_norms": gnorm,
            "approximate_precession_true": {"ms_per_step": approx["grad_ms"], "forward_ms": approx["fwd_ms"],
                                            "grad_over_forward": approx["grad_ms"] / approx["fwd_ms"],
                                            "spots": int(approx["sim"].intensity.shape[0])},
            "error_vs_fp64_autograd": check, "cpu_baseline": cpu,
            "config": {k: v for k, v in W.items()}, "dtype": "f32 forward with f64 phase; f64 adjoint"}


def _reference_grads(torch, sim, target, ps, els, q0t, p, upstream=None, chunk=131072):
    """Autograd through the FP64 transcription of the reference formulas on
    the spots of ``sim`` (orientation and hkl fixed), in chunks of spots:
    the gradient of the loss (in the returned leaves' ``.grad``), its value,
    and, with ``upstream`` (dL/dI per spot), the vector-Jacobian product
    upstream . dI/dparams (a list per parameter group)."""
    from oracle import autograd_reference as ar
    loss = ar.MatchedLoss(sim.offsets, sim.hkl, target.intensity, target.offsets, target.hkl)
    dev = q0t.device
    counts = sim.offsets[1:] - sim.offsets[:-1]
    orient = torch.repeat_interleave(torch.arange(counts.shape[0], device=counts.device), counts).to(dev)
    hkl = sim.hkl.to(dev)
    leaves = [t.detach().clone().requires_grad_() for t in ps]
    recip = ar.reciprocal_basis_torch(leaves[3])
    quats = ar.compose_axis_angle_torch(q0t[:counts.shape[0]], leaves[4])
    n = int(hkl.shape[0])
    total = 0.0
    vjp = [torch.zeros_like(t) for t in leaves] if upstream is not None else None
    for a in range(0, max(n, 1), chunk):
        b = min(n, a + chunk)
        I = ar.spot_intensities(leaves[0], leaves[1], leaves[2], recip, quats, els, "lobato", orient[a:b], hkl[a:b], p)
        if upstream is not None:
            for acc, g in zip(vjp, torch.autograd.grad(I, leaves, upstream[a:b].to(I.device), retain_graph=True)):
                acc += g
        La = loss(I, a)
        La.backward(retain_graph=True)
        total += float(La.detach())
    return leaves, total, vjp


def _grad_params(W, approximate):
    from oracle import kinematic as ok
    return ok.SimParams(accelerating_voltage=W["accelerating_voltage"], reciprocal_radius=W["reciprocal_radius"],
                        max_excitation_error=W["max_excitation_error"], shape_factor_model=W["shape_factor_model"],
                        precession_angle=W["precession_angle"], approximate_precession=approximate)


def grad_check(torch, dev, main, els, q0t, names):
    """Errors of the workload's GPU gradients against the FP64 transcription
    of the reference formulas on the same spots (the checker; untimed):

    * ``adjoint``: the hand-written adjoint alone -- the GPU's and the
      transcription's vector-Jacobian products with the same upstream
      dL/dI = 2 (I - T) (the GPU forward's intensities);
    * ``loss_gradient``: the whole chain -- the GPU gradient of the loss
      (FP32 forward intensities in the residual I - T) against autograd of
      the FP64 loss.
    Per group: every component relative to itself with floors, and the
    group's norm-wise relative error."""
    import warnings
    from diffsims_gb300.autograd import compose_axis_angle, reciprocal_basis, simulate_intensities, spot_loss
    from oracle import autograd_reference as ar
    W = GRAD_WORKLOAD
    t0 = time.perf_counter()
    model, target = main["model"], main["target"]
    ps = [t.detach().clone().requires_grad_() for t in main["ps"]]
    sim = simulate_intensities(model, ps[0], ps[1], ps[2], reciprocal_basis(ps[3]), compose_axis_angle(q0t, ps[4]))
    loss = ar.MatchedLoss(sim.offsets, sim.hkl, target.intensity, target.offsets, target.hkl)
    gI = 2.0 * (sim.intensity.detach() - loss.target_per_spot)
    g_adj = torch.autograd.grad(sim.intensity, ps, gI, retain_graph=True)
    L = spot_loss(sim, target)
    g_full = torch.autograd.grad(L, ps)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        leaves, L_ref, vjp = _reference_grads(torch, sim, target, ps, els, q0t,
                                              _grad_params(W, W["approximate_precession"]), upstream=gI)
    npy = lambda ts: {n: t.detach().cpu().numpy() for n, t in zip(names, ts)}
    adj = ar.gradient_errors(npy(g_adj), npy(vjp))
    full = ar.gradient_errors(npy(g_full), npy([t.grad for t in leaves]))
    return {"adjoint": adj, "loss_gradient": full,
            "adjoint_max_norm_rel": max(v["norm_rel"] for v in adj.values()),
            "loss_gradient_max_norm_rel": max(v["norm_rel"] for v in full.values()),
            "loss_rel_error": abs(float(L.detach()) - L_ref) / abs(L_ref), "spots": int(sim.intensity.shape[0]),
            "reference": "autograd through the FP64 torch transcription (oracle/autograd_reference.py), same spots",
            "seconds": time.perf_counter() - t0}


def grad_cpu_baseline(torch, main, els, q0, n_o, n_sample=64):
    """The FP64 transcription's forward + backward on the host cores (torch
    threads) for the spots of the first ``n_sample`` orientations, scaled to
    the workload's orientations: ms per gradient step."""
    import warnings
    W = GRAD_WORKLOAD
    sim = main["sim"]
    off = sim.offsets.cpu()
    m = int(off[n_sample])

    class Sub:
        pass
    sub, tgt = Sub(), Sub()
    sub.offsets, sub.hkl = off[:n_sample + 1].clone(), sim.hkl[:m].cpu()
    toff = main["target"].offsets.cpu()
    tm = int(toff[n_sample])
    tgt.offsets, tgt.hkl, tgt.intensity = toff[:n_sample + 1].clone(), main["target"].hkl[:tm].cpu(), \
        main["target"].intensity[:tm].detach().cpu()
    ps = [t.detach().cpu() if i != 4 else t.detach()[:n_sample].cpu() for i, t in enumerate(main["ps"])]
    q0c = torch.as_tensor(q0[:n_sample], dtype=torch.float64)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        _reference_grads(torch, sub, tgt, ps, els, q0c, _grad_params(W, W["approximate_precession"]))  # warm
        t0 = time.perf_counter()
        _reference_grads(torch, sub, tgt, ps, els, q0c, _grad_params(W, W["approximate_precession"]))
        dt = time.perf_counter() - t0
    return {"value": dt * 1e3 * n_o / n_sample, "unit": "ms", "cores": torch.get_num_threads(), "kind": "port",
            "sample": f"forward + backward of the FP64 torch transcription of the reference formulas on the "
                      f"{m} spots of the first {n_sample} orientations ({dt:.2f} s), scaled by {n_o}/{n_sample}"}


def run_batch(args, torch, dev):
    """Batched uneven phases: every phase's orientations in one persistent
    launch (CUDA graph replay), against the same phases launched one by one."""
    import diffsims_gb300 as ds
    from diffsims_gb300 import _native as N
    from diffsims_gb300.engine import AUTOTUNER, Autotuner, PhaseBatch, PhaseTable, SpotBuffers, simulate_phase
    W = BATCH_WORKLOAD
    gen = ds.SimulationGenerator(W["accelerating_voltage"], "lobato", shape_factor_model=W["shape_factor_model"])
    settings = gen.settings(W["max_excitation_error"])
    r = W["reciprocal_radius"]
    tables, qs = [], []
    t_tab = time.perf_counter()
    for k, (lat, els, xyz, B, n_q, q_seed) in enumerate(batch_phase_specs()):
        tables.append(PhaseTable(phase_of(f"p{k}", lat, els, xyz), r, True, "lobato", list(B), device=dev))
        qs.append(torch.from_numpy(uniform_quaternions(n_q, q_seed)).to(dev))
    torch.cuda.synchronize()
    table_s = time.perf_counter() - t_tab
    n_pat = sum(int(q.shape[0]) for q in qs)
    batch = PhaseBatch(tables, qs, settings, r)  # tile from the autotuner
    key = Autotuner.key(batch)
    batch.run()
    batch.capture()
    st = torch.cuda.current_stream()

    def timed(fn):
        for _ in range(args.warmup):
            fn()
        torch.cuda.synchronize()
        ms = []
        for _ in range(args.steps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(st)
            fn()
            e1.record(st)
            e1.synchronize()
            ms.append(e0.elapsed_time(e1))
        return statistics.mean(ms)

    graph_ms = timed(batch.replay)
    if int(batch.status.abs().sum()) != 0:
        raise RuntimeError("batched launch reported a device status")
    spots = batch.spots()
    n_spots = sum(s.total for s in spots)
    bufs = [SpotBuffers(dev) for _ in tables]
    for t, q, b in zip(tables, qs, bufs):
        simulate_phase(t, q, settings, r, b)  # size the buffers
    seq_ms = timed(lambda: [simulate_phase(t, q, settings, r, b, sync=False) for t, q, b in zip(tables, qs, bufs)])
    # roofline: FP32 screen over every (orientation, row) pair, and the bytes written
    peak32 = fp32_peak_tflops(torch, N.load_library(), N)
    pairs = sum(int(q.shape[0]) * t.n for t, q in zip(tables, qs))
    flops = 10.0 * pairs / (graph_ms * 1e-3) / 1e12
    bytes_alg = n_spots * 20 + (n_pat + 1) * 8 + n_pat * 32 + sum(t.n for t in tables) * 28
    hbm_peak = _hbm_peak()[0]
    roof = {"bound": "fp32", "achieved": flops, "peak": peak32, "unit": "TFLOP/s", "frac": flops / peak32,
            "pairs": pairs, "kernel": "simulate_batch_kernel", "kernel_ms": graph_ms,
            "peak_source": "measured by bench.py FMA probe (ds_probe_fp32_fma)", "peak_nominal": fp32_nominal_tflops(torch),
            "hbm": {"achieved_gbs": bytes_alg / (graph_ms * 1e-3) / 1e9, "peak_gbs": hbm_peak,
                    "frac": bytes_alg / (graph_ms * 1e-3) / 1e9 / hbm_peak}}
    cpu = None
    if not args.no_cpu_baseline:
        params = dict(accelerating_voltage=W["accelerating_voltage"], reciprocal_radius=r,
                      max_excitation_error=W["max_excitation_error"], shape_factor_model=W["shape_factor_model"])
        jobs = [(lat, els, xyz, Bv, uniform_quaternions(n_q, q_seed)[:max(1, n_q // 256)], params, None)
                for lat, els, xyz, Bv, n_q, q_seed in batch_phase_specs()]
        cores = os.cpu_count() or 1
        rate, dt, n_s, _ = cpu_phases_rate(jobs, cores)
        cpu = {"value": rate, "unit": "patterns/s", "cores": cores, "kind": "port",
               "sample": f"the first 1/256 of every phase's orientations ({n_s} patterns, {dt:.1f} s), FP64 numpy "
                         f"restatement of the reference path, {cores} spawned processes"}
    return {"metric": "orientation patterns/s (32 uneven phases, one launch)", "value": n_pat / (graph_ms * 1e-3),
            "unit": "patterns/s", "ms_per_step": graph_ms, "patterns_per_step": n_pat, "spots_per_step": int(n_spots),
            "per_phase_launches_ms": seq_ms, "speedup_over_per_phase_launches": seq_ms / graph_ms,
            "orient_tile": batch.orient_tile, "stage_cap": batch.stage_cap, "refine_parts": batch.refine_parts,
            "autotuner_ms": AUTOTUNER.timings.get(key),
            "n_hkl_range": [min(t.n for t in tables), max(t.n for t in tables)],
            "orientations_range": [min(int(q.shape[0]) for q in qs), max(int(q.shape[0]) for q in qs)],
            "table_build_s": table_s, "launches_per_step": len(tables) + 2, "roofline": roof, "cpu_baseline": cpu,
            "config": {k: v for k, v in W.items()}}


def pm3m_operations():
    """The 48 operations (R, 0) of Pm-3m: the closure of a 4-fold about z, a
    3-fold about [111] and the inversion (the per-family leg's input)."""
    gens = [np.array([[0, -1, 0], [1, 0, 0], [0, 0, 1]]), np.array([[0, 0, 1], [1, 0, 0], [0, 1, 0]]), -np.eye(3, dtype=int)]
    group = {tuple(np.eye(3, dtype=int).ravel())}
    frontier = [np.eye(3, dtype=int)]
    while frontier:
        new = []
        for R in frontier:
            for G in gens:
                P = G @ R
                if tuple(P.ravel()) not in group:
                    group.add(tuple(P.ravel()))
                    new.append(P)
        frontier = new
    return [(np.array(k, dtype=np.float64).reshape(3, 3), np.zeros(3)) for k in sorted(group)]


def run_families(args, torch, dev):
    """Per-family structure factors (diffsims/structure_factor/structure_factor.py:103-185):
    2^20 Doyle-Turner families at 200 kV of a mixed site at a general
    position of Pm-3m (two 48-position orbits), one ds_family_structure_factors
    launch; and the public call from host arrays (copies in, values out)."""
    from diffsims_gb300 import _native as N
    from diffsims_gb300 import structure_factor as gsf
    from diffsims_gb300.crystal import Atom, Lattice, Phase, Structure
    lib = N.load_library()
    ops = pm3m_operations()
    atoms = [Atom("Fe", [0.11, 0.23, 0.37], 0.6, 0.005), Atom("Ni", [0.11, 0.23, 0.37], 0.4, 0.009),
             Atom("O", [0.5, 0.5, 0.5], 1.0, 0.011)]
    phase = Phase(structure=Structure(atoms, Lattice(4.1, 4.1, 4.1)), space_group=ops)
    rng = np.random.default_rng(3)
    n = 1 << 20
    hkl = rng.integers(-25, 26, (n, 3)).astype(np.float64)
    s = np.sqrt(np.sum(hkl * hkl, axis=1)) / (2 * 4.1)
    sites = gsf._asymmetric_sites(phase.structure, phase.space_group)
    n_pos = sum(len(p) for _, p, _, _ in sites)
    volume = phase.structure.lattice.volume
    # device-resident launch
    from diffsims_gb300.sim_utils import PackedAtoms
    species, rows, xyz, occ, B = [], [], [], [], []
    for k, (z, positions, o, biso) in enumerate(sites):
        rows.append(gsf._coeff_row(z, N.DS_SCATTER_DOYLETURNER, volume))
        for p in positions:
            species.append(k); xyz.append(p); occ.append(o); B.append(4.0 * biso)
    packed = PackedAtoms.from_rows(species, rows, np.asarray(xyz), occ, B, N.DS_SCATTER_DOYLETURNER, dev)
    hkl_d = torch.from_numpy(hkl).to(dev)
    s_d = torch.from_numpy(s).to(dev)
    F = torch.empty((n, 2), dtype=torch.float64, device=dev)
    status = torch.zeros(1, dtype=torch.int32, device=dev)
    st = torch.cuda.current_stream()

    def launch():
        N.check(lib.ds_family_structure_factors(packed.cstruct(), N.ptr(hkl_d), N.ptr(s_d), n, N.ptr(F),
                                                N.ptr(status), N.stream_handle()), "families")

    def timed(fn):
        for _ in range(args.warmup):
            fn()
        torch.cuda.synchronize()
        ms = []
        for _ in range(args.steps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(st)
            fn()
            e1.record(st)
            e1.synchronize()
            ms.append(e0.elapsed_time(e1))
        return statistics.mean(ms)

    k_ms = timed(launch)
    N.check_device_status(status, "families")
    t_e2e = []
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        gsf.get_doyleturner_structure_factor(phase, hkl, s, 200e3)
        if i >= args.warmup:
            t_e2e.append(time.perf_counter() - t0)
    # the oracle's per-family loop (the reference's algorithm) on one core, a bounded sample
    from oracle import structure_factor_families as osf
    atoms_o = [(a.element, a.xyz, a.occupancy, a.Bisoequiv) for a in atoms]
    n_cpu = 2000
    t0 = time.perf_counter()
    for i in range(n_cpu):
        osf.doyleturner_structure_factor(atoms_o, ops, hkl[i], s[i], volume, 200e3)
    cpu_rate = n_cpu / (time.perf_counter() - t0)
    return {"metric": "lattice-plane families/s (Doyle-Turner structure factor, 200 kV)",
            "value": n / (k_ms * 1e-3), "unit": "families/s", "kernel_ms": k_ms, "families": n,
            "orbit_positions": n_pos, "terms_per_s": n * n_pos / (k_ms * 1e-3),
            "e2e": {"value": n / statistics.mean(t_e2e), "unit": "families/s",
                    "h2d_bytes_per_step": n * 32, "d2h_bytes_per_step": n * 8},
            "cpu_baseline": {"value": cpu_rate, "unit": "families/s", "cores": 1, "kind": "port",
                             "sample": f"{n_cpu} families, FP64 numpy restatement of the reference's per-family loop"},
            "dtype": "f64"}


def run_polar(args, torch, dev, hbm_peak, spots):
    """Polar templates (Simulation2D.polar_flatten_simulations,
    diffsims/simulations/simulation2d.py:313-355) of the headline leg's
    100,000 patterns on the device: padded (r, theta, I) float64 arrays,
    unbinned and binned to 256 radial x 360 azimuthal axes.  Bytes = the spot
    records read (16 B) + the three arrays written (24 B per slot).  CPU
    baseline: the oracle's numpy restatement on one core over a sample."""
    from diffsims_gb300.engine import polar_flatten
    from oracle import kinematic as ok
    st = torch.cuda.current_stream()
    n = spots.n_orient
    m = int((spots.offsets[1:] - spots.offsets[:-1]).max().item())
    rax = np.linspace(0.0, 2.0, 256)
    aax = np.linspace(-np.pi, np.pi, 360)
    out = {}
    binned = dict(radial_axes=rax, azimuthal_axes=aax)
    for name, kw in (("unbinned", {}), ("binned", binned), ("unbinned_fp32", dict(precision="fp32")),
                     ("binned_fp32", dict(binned, precision="fp32"))):
        for _ in range(args.warmup):
            res = polar_flatten([spots], **kw)
        del res
        torch.cuda.synchronize()
        ms = []
        for _ in range(args.steps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(st)
            res = polar_flatten([spots], **kw)
            e1.record(st)
            e1.synchronize()
            ms.append(e0.elapsed_time(e1))
            del res
        t = statistics.median(ms)
        nbytes = spots.total * 16 + 3 * n * m * 8
        out[name] = {"ms": t, "patterns_per_s": n / (t * 1e-3), "achieved_gbs": nbytes / (t * 1e-3) / 1e9,
                     "frac": nbytes / (t * 1e-3) / 1e9 / hbm_peak, "bytes": int(nbytes)}
    # the FP32 mode against the FP64 one on every slot: r and theta relative
    # error (unbinned), index mismatches (binned)
    err = {}
    a, b = polar_flatten([spots]), polar_flatten([spots], precision="fp32")
    for k, name in ((0, "r"), (1, "theta")):
        d = (a[k] - b[k]).abs() / a[k].abs().clamp_min(1e-30)
        err[f"max_rel_{name}"] = float(torch.where(a[k] != 0, d, torch.zeros_like(d)).max().item())
    del a, b
    a, b = polar_flatten([spots], **binned), polar_flatten([spots], **binned, precision="fp32")
    err["binned_slots_differing"] = int(((a[0] != b[0]) | (a[1] != b[1]) | (a[2] != b[2])).sum().item())
    err["binned_patterns_differing"] = int(((a[0] != b[0]) | (a[1] != b[1]) | (a[2] != b[2])).any(1).sum().item())
    del a, b
    off, _, xyzi = spots.host()
    n_cpu = 2000
    pats = [(xyzi[off[k]:off[k + 1], :3].astype(np.float64), xyzi[off[k]:off[k + 1], 3].astype(np.float64))
            for k in range(n_cpu)]
    t0 = time.perf_counter()
    ok.polar_flatten(pats)
    cpu_rate = n_cpu / (time.perf_counter() - t0)
    return {"metric": "polar templates/s (padded r, theta, I)", "value": out["unbinned"]["patterns_per_s"],
            "unit": "patterns/s", "patterns": n, "max_spots": m, "spots": int(spots.total), **out,
            "roofline": {"bound": "hbm", "achieved": out["unbinned"]["achieved_gbs"], "peak": hbm_peak,
                         "unit": "GB/s", "frac": out["unbinned"]["frac"]},
            "fp32_vs_fp64": err,
            "cpu_baseline": {"value": cpu_rate, "unit": "patterns/s", "cores": 1, "kind": "port",
                             "sample": f"{n_cpu} patterns of the same spots, the oracle's numpy polar_flatten"},
            "note": "the launch plus its three float64 output allocations (the kernel writes the padding); "
                    "value and roofline: the FP64 (reference-exact) unbinned mode; *_fp32: r and theta in FP32 "
                    "(ds_polar_flatten_f32)"}


def run_profiles(args, torch, dev):
    """1-D profiles (SimulationGenerator.calculate_diffraction1d,
    diffsims/generators/simulation_generator.py:261-317) of the headline's
    200-atom P1 cell: the from_min_dspacing set at 0.7 Angstrom, enumeration
    and FP64 structure factors on the GPU, families on the host; the public
    call timed against the oracle's restatement (numpy, one core)."""
    import diffsims_gb300 as ds
    from oracle import kinematic as ok
    lat, els, xyz, B = make_crystal(WORKLOAD["cell_seed"], WORKLOAD["n_atoms"])
    phase = phase_of("P1", lat, els, xyz)
    gen = ds.SimulationGenerator(WORKLOAD["accelerating_voltage"])
    for _ in range(max(1, args.warmup)):
        prof = gen.calculate_diffraction1d(phase, 1.0)
    torch.cuda.synchronize()
    ts = []
    for _ in range(max(3, args.steps)):
        t0 = time.perf_counter()
        prof = gen.calculate_diffraction1d(phase, 1.0)
        ts.append(time.perf_counter() - t0)
    t = statistics.median(ts)
    cr = ok.Crystal(lat, els, xyz)
    t0 = time.perf_counter()
    ok.diffraction1d(cr, np.eye(3, dtype=int)[None])
    cpu_s = time.perf_counter() - t0
    return {"metric": "1-D profiles/s (calculate_diffraction1d, 200-atom P1, d_min 0.7 A)", "value": 1.0 / t,
            "unit": "profiles/s", "ms_per_call": t * 1e3, "peaks": int(len(prof.intensities)),
            "cpu_baseline": {"value": 1.0 / cpu_s, "unit": "profiles/s", "cores": 1, "kind": "port",
                             "sample": "one profile, the oracle's numpy restatement (FP64 structure factors, "
                                       "families)"},
            "note": "public call: host families and result objects included"}


def run_legacy(args, torch, dev):
    """Legacy DiffractionGenerator.calculate_ed_data
    (diffsims/generators/diffraction_generator.py:192-331): a 12-atom P1 cell
    (a, b, c = 6.3, 7.1, 8.2 A), 200 kV, r = 2.0, lorentzian, 100,000 Euler
    triples in one call (the loop of DiffractionLibraryGenerator.get_diffraction_library,
    diffsims/generators/library_generator.py:51-155, for one phase)."""
    from diffsims_gb300.crystal import Atom, Lattice, Structure
    from diffsims_gb300.diffraction_generator import DiffractionGenerator, euler_rzxz_quaternions, structure_base
    from diffsims_gb300.engine import PhaseTable, SpotBuffers, simulate_phase
    from diffsims_gb300.sim_utils import PackedAtoms
    from oracle import legacy as ol
    rng = np.random.default_rng(31)
    els = list(rng.choice(["C", "O", "Si", "Fe"], 12))
    xyz = rng.random((12, 3))
    occ = rng.uniform(0.6, 1.0, 12)
    lat = (6.3, 7.1, 8.2, 84.0, 97.0, 103.0)
    structure = Structure([Atom(e, x, o) for e, x, o in zip(els, xyz, occ)], Lattice(*lat))
    n, r = 100_000, 2.0
    eul = np.random.default_rng(7).uniform(-180, 180, (n, 3))
    gen = DiffractionGenerator(200)
    # device-resident: the sphere table and the orientation launch
    recip = np.ascontiguousarray(np.linalg.inv(structure_base(structure.lattice)).T)
    atoms = PackedAtoms(els, xyz, occ, np.zeros(12), "lobato", dev)
    q = euler_rzxz_quaternions(eul)
    q[:, 1:] *= -1
    quats = torch.from_numpy(q).to(dev)
    settings = gen._gen.settings(1e-2)
    bufs = SpotBuffers(dev)
    st = torch.cuda.current_stream()

    def step():
        t = PhaseTable.sphere(recip, atoms, r, device=dev)
        return simulate_phase(t, quats, settings, r, bufs)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    ms = []
    for _ in range(args.steps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        spots = step()
        e1.record(st)
        e1.synchronize()
        ms.append(e0.elapsed_time(e1))
    dev_ms = statistics.mean(ms)
    # the public call, host Euler angles in, DiffractionSimulation objects out
    t0 = time.perf_counter()
    sims = gen.calculate_ed_data(structure, r, rotation=eul)
    e2e_s = time.perf_counter() - t0
    # the oracle's per-orientation call (the reference's algorithm), one core
    n_cpu = 500
    dl = ol.DiffpyLattice(*lat)
    t0 = time.perf_counter()
    for k in range(n_cpu):
        ol.calculate_ed_data(dl, els, xyz, occ, np.zeros(12), 200, r, rotation=eul[k])
    cpu_rate = n_cpu / (time.perf_counter() - t0)
    return {"metric": "orientation patterns/s (legacy calculate_ed_data, Euler rzxz)", "value": n / (dev_ms * 1e-3),
            "unit": "patterns/s", "ms_per_step": dev_ms, "patterns_per_step": n, "spots_per_step": int(spots.total),
            "n_hkl": int(spots.table.n),
            "e2e": {"value": n / e2e_s, "unit": "patterns/s", "s": e2e_s, "simulations": len(sims),
                    "note": "public call with host Euler angles; includes building 100k DiffractionSimulation objects"},
            "cpu_baseline": {"value": cpu_rate, "unit": "patterns/s", "cores": 1, "kind": "port",
                             "sample": f"{n_cpu} orientations, FP64 numpy restatement of calculate_ed_data"},
            "config": {"workload": "legacy calculate_ed_data: P1 12 atoms (6.3, 7.1, 8.2 A; 84, 97, 103 deg), "
                                   "200 kV, r=2.0, s_max=0.01, lorentzian, 100k Euler triples", "seed": 31}}


def run_library(args, torch, dev, hbm_peak):
    """Template-library throughput: three phases simulated and rasterised in
    8192-orientation chunks through one reused detector buffer; with the
    rotation average (the workload's linear with 0.5 deg precession) and with
    the reference's default ``approximate_precession=True``."""
    import diffsims_gb300 as ds
    from diffsims_gb300 import _native as N
    from diffsims_gb300.engine import PhaseTable, RasterBuffers, RasterSettings, SpotBuffers, rasterize, simulate_phase
    W = LIBRARY_WORKLOAD
    specs = library_phase_specs()
    phases = [phase_of(nm, lat, els, xyz) for nm, lat, els, xyz, _ in specs]
    dws = [list(B) for *_, B in specs]
    r = W["reciprocal_radius"]
    n_o, chunk = W["n_orientations"], W["chunk"]
    H, Wd = W["shape"]
    qs = [torch.from_numpy(uniform_quaternions(n_o, 100 + i)).to(dev) for i in range(3)]
    tables = [PhaseTable(ph, r, True, "lobato", dw, device=dev) for ph, dw in zip(phases, dws)]
    bufs = [SpotBuffers(dev) for _ in range(3)]
    rs = RasterSettings((H, Wd), sigma=W["sigma"], calibration=W["calibration"])
    rb = RasterBuffers(dev)
    img = torch.empty((chunk, H, Wd), dtype=torch.float32, device=dev)
    st = torch.cuda.current_stream()
    n_pat = 3 * n_o
    bytes_img = n_pat * H * Wd * 4

    def measure(approximate):
        gen = ds.SimulationGenerator(W["accelerating_voltage"], "lobato", W["precession_angle"],
                                     W["shape_factor_model"], approximate)
        settings = gen.settings(W["max_excitation_error"])

        def step(time_raster):
            spots = [simulate_phase(t, q, settings, r, b) for t, q, b in zip(tables, qs, bufs)]
            maxes = [int((s.offsets[1:] - s.offsets[:-1]).max().item()) for s in spots]
            ras_ms = 0.0
            for s, m in zip(spots, maxes):
                for a in range(0, n_o, chunk):
                    b = min(a + chunk, n_o)
                    if time_raster:
                        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                        e0.record(st)
                    rasterize(s, rs, a, b, out=img[:b - a], max_spots=m, buffers=rb, sync=False)
                    if time_raster:
                        e1.record(st)
                        e1.synchronize()
                        ras_ms += e0.elapsed_time(e1)
            return spots, ras_ms

        for _ in range(args.warmup):
            step(False)
        torch.cuda.synchronize()
        ms = []
        for _ in range(args.steps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            spots, _ = step(False)
            torch.cuda.synchronize()
            ms.append((time.perf_counter() - t0) * 1e3)
        _, ras_ms = step(True)
        N.check_device_status(rb.status, "rasterize")
        ras_gbs = bytes_img / (ras_ms * 1e-3) / 1e9
        return {"value": n_pat / (statistics.mean(ms) * 1e-3), "ms_per_step": statistics.mean(ms),
                "spots_per_step": int(sum(s.total for s in spots)),
                "raster": {"ms": ras_ms, "achieved_gbs": ras_gbs, "peak_gbs": hbm_peak, "frac": ras_gbs / hbm_peak,
                           "bytes_written": bytes_img, "launches": 3 * ((n_o + chunk - 1) // chunk),
                           "note": "CUDA events around each chunk's launch; bytes = images written"}}

    main = measure(W["approximate_precession"])
    approx = measure(True)
    cpu = None
    if not args.no_cpu_baseline:
        params = dict(accelerating_voltage=W["accelerating_voltage"], reciprocal_radius=r,
                      max_excitation_error=W["max_excitation_error"], shape_factor_model=W["shape_factor_model"],
                      precession_angle=W["precession_angle"], approximate_precession=W["approximate_precession"])
        raster = {"shape": W["shape"], "sigma": W["sigma"], "calibration": W["calibration"]}
        n_cpu = args.library_cpu_sample
        jobs = [(lat, els, xyz, Bv, uniform_quaternions(n_o, 100 + i)[:n_cpu], params, raster)
                for i, (_, lat, els, xyz, Bv) in enumerate(specs)]
        cores = os.cpu_count() or 1
        rate, dt, n_s, _ = cpu_phases_rate(jobs, cores)
        cpu = {"value": rate, "unit": "patterns/s", "cores": cores, "kind": "port",
               "sample": f"the first {n_cpu} orientations of each phase ({n_s} patterns, {dt:.1f} s): FP64 numpy "
                         f"restatement of the reference path (scipy quad rotation average) and its rasteriser "
                         f"(scipy gaussian_filter), {cores} spawned processes"}
    return {"metric": "orientation patterns/s (simulated and rasterised)", "value": main["value"],
            "unit": "patterns/s", "ms_per_step": main["ms_per_step"], "patterns_per_step": n_pat,
            "spots_per_step": main["spots_per_step"], "n_hkl": [t.n for t in tables], "raster": main["raster"],
            "approximate_precession_true": approx, "cpu_baseline": cpu,
            "config": {k: (list(v) if isinstance(v, tuple) else v) for k, v in W.items()}}


def run_case(args):
    """Small fixed cases for profiler captures (one kernel of interest each;
    a few GB on the device at most).  Prints what ran."""
    import torch
    import diffsims_gb300 as ds
    from diffsims_gb300 import _native as N
    from diffsims_gb300.engine import (PhaseBatch, PhaseTable, RasterSettings, SpotBuffers, rasterize,
                                       simulate_phase)
    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    out = {"case": args.case}
    if args.case == "raster":
        # the template library's 60-atom P1 phase, 2048 patterns, two rasterisations
        W = LIBRARY_WORKLOAD
        nm, lat, els, xyz, B = library_phase_specs()[2]
        gen = ds.SimulationGenerator(W["accelerating_voltage"], "lobato", W["precession_angle"],
                                     W["shape_factor_model"], W["approximate_precession"])
        tab = PhaseTable(phase_of(nm, lat, els, xyz), W["reciprocal_radius"], True, "lobato", list(B), device=dev)
        q = torch.from_numpy(uniform_quaternions(2048, 1)).to(dev)
        sp = simulate_phase(tab, q, gen.settings(W["max_excitation_error"]), W["reciprocal_radius"], SpotBuffers(dev))
        img = torch.empty((2048,) + tuple(W["shape"]), dtype=torch.float32, device=dev)
        rs = RasterSettings(W["shape"], sigma=W["sigma"], calibration=W["calibration"])
        for _ in range(2):
            rasterize(sp, rs, 0, 2048, out=img)
        out.update(patterns=2048, spots=sp.total)
    elif args.case == "adjoint":
        # the differentiation workload at 1024 orientations: forward, then the adjoint kernels
        from diffsims_gb300.autograd import SpotModel, reciprocal_basis
        W = GRAD_WORKLOAD
        rng = np.random.default_rng(W["seed"])
        els = list(rng.choice(["O", "Si", "Fe"], W["n_atoms"]))
        lat = torch.tensor([7.1, 9.3, 12.4, 90.0, 90.0, 90.0], dtype=torch.float64)
        xyz = torch.as_tensor(rng.random((W["n_atoms"], 3))).to(dev)
        B = torch.as_tensor(rng.uniform(0.3, 1.5, W["n_atoms"])).to(dev)
        gen = ds.SimulationGenerator(W["accelerating_voltage"], "lobato", W["precession_angle"],
                                     W["shape_factor_model"], W["approximate_precession"])
        model = SpotModel(els, gen, W["reciprocal_radius"], W["max_excitation_error"])
        table = model.table(reciprocal_basis(lat).numpy(), xyz, torch.ones_like(B), B)
        q = torch.as_tensor(cone_quaternions(1024, W["cone_deg"], W["seed"] + 1)).to(dev)
        sp = simulate_phase(table, q, model.settings, W["reciprocal_radius"], SpotBuffers(dev))
        lib = N.load_library()
        p = model.settings.cstruct()
        n = sp.total
        gI = torch.ones(n, dtype=torch.float64, device=dev)
        gF2 = torch.zeros(table.n, dtype=torch.float64, device=dev)
        gq = torch.zeros((1024, 4), dtype=torch.float64, device=dev)
        grec = torch.zeros(9, dtype=torch.float64, device=dev)
        nb = lib.ds_simulate_backward_scratch_bytes(p, n, 1024)
        scr = torch.empty(max(nb, 16), dtype=torch.uint8, device=dev)
        st = torch.zeros(1, dtype=torch.int32, device=dev)
        idx = sp.hkl_index.contiguous()
        for _ in range(2):
            N.check(lib.ds_simulate_backward(p, table.cstruct(), N.ptr(q), 1024, N.ptr(sp.offsets), N.ptr(idx), n,
                                             N.ptr(gI), N.ptr(gF2), N.ptr(gq), N.ptr(grec), N.ptr(scr), nb, N.ptr(st),
                                             N.stream_handle()), "simulate_backward")
        N.check_device_status(st, "simulate_backward")
        out.update(orientations=1024, spots=n)
    elif args.case == "batch":
        # the 32 uneven phases with 1/16 of their orientations, one batched launch (tile 16)
        W = BATCH_WORKLOAD
        gen = ds.SimulationGenerator(W["accelerating_voltage"], "lobato", shape_factor_model=W["shape_factor_model"])
        tables, qs = [], []
        for k, (lat, els, xyz, B, n_q, q_seed) in enumerate(batch_phase_specs()):
            tables.append(PhaseTable(phase_of(f"p{k}", lat, els, xyz), W["reciprocal_radius"], True, "lobato",
                                     list(B), device=dev))
            qs.append(torch.from_numpy(uniform_quaternions(n_q // 16, q_seed)).to(dev))
        batch = PhaseBatch(tables, qs, gen.settings(W["max_excitation_error"]), W["reciprocal_radius"], orient_tile=16)
        batch.run()
        batch.run()
        out.update(patterns=sum(int(x.shape[0]) for x in qs), spots=int(batch.totals.sum()))
    elif args.case == "families":
        # the per-family leg's 2^20 Doyle-Turner families (96 orbit positions), two launches
        from diffsims_gb300 import structure_factor as gsf
        from diffsims_gb300.sim_utils import PackedAtoms
        atoms = [ds.Atom("Fe", [0.11, 0.23, 0.37], 0.6, 0.005), ds.Atom("Ni", [0.11, 0.23, 0.37], 0.4, 0.009)]
        sites = gsf._asymmetric_sites(atoms, pm3m_operations())
        species, rows, xyz, occ, B = [], [], [], [], []
        for k, (z, positions, o, biso) in enumerate(sites):
            rows.append(gsf._coeff_row(z, N.DS_SCATTER_DOYLETURNER, 4.1 ** 3))
            for p_ in positions:
                species.append(k); xyz.append(p_); occ.append(o); B.append(4.0 * biso)
        packed = PackedAtoms.from_rows(species, rows, np.asarray(xyz), occ, B, N.DS_SCATTER_DOYLETURNER, dev)
        rng = np.random.default_rng(3)
        n = 1 << 20
        hkl = torch.from_numpy(rng.integers(-25, 26, (n, 3)).astype(np.float64)).to(dev)
        s_ = torch.linalg.norm(hkl, dim=1) / (2 * 4.1)
        F = torch.empty((n, 2), dtype=torch.float64, device=dev)
        st = torch.zeros(1, dtype=torch.int32, device=dev)
        lib = N.load_library()
        for _ in range(2):
            N.check(lib.ds_family_structure_factors(packed.cstruct(), N.ptr(hkl), N.ptr(s_), n, N.ptr(F), N.ptr(st),
                                                    N.stream_handle()), "families")
        N.check_device_status(st, "families")
        out.update(families=n, orbit_positions=len(species))
    elif args.case == "polar":
        # polar templates of 8192 headline orientations, unbinned then binned
        from diffsims_gb300.engine import polar_flatten
        lat, els, xyz, B = make_crystal(WORKLOAD["cell_seed"], WORKLOAD["n_atoms"])
        gen = ds.SimulationGenerator(WORKLOAD["accelerating_voltage"], "lobato",
                                     shape_factor_model=WORKLOAD["shape_factor_model"])
        tab = PhaseTable(phase_of("P1", lat, els, xyz), WORKLOAD["reciprocal_radius"], True, "lobato", list(B),
                         device=dev)
        q = torch.from_numpy(uniform_quaternions(8192, WORKLOAD["orientation_seed"])).to(dev)
        sp = simulate_phase(tab, q, gen.settings(WORKLOAD["max_excitation_error"]), WORKLOAD["reciprocal_radius"],
                            SpotBuffers(dev))
        polar_flatten([sp])
        polar_flatten([sp], np.linspace(0.0, 2.0, 256), np.linspace(-np.pi, np.pi, 360))
        polar_flatten([sp], precision="fp32")
        polar_flatten([sp], np.linspace(0.0, 2.0, 256), np.linspace(-np.pi, np.pi, 360), precision="fp32")
        out.update(patterns=8192, spots=sp.total)
    elif args.case == "legacy":
        # the legacy leg's 12-atom P1 sphere table at r = 2.0 and 8192 Euler triples
        from diffsims_gb300.diffraction_generator import DiffractionGenerator, euler_rzxz_quaternions, structure_base
        from diffsims_gb300.sim_utils import PackedAtoms
        rng = np.random.default_rng(31)
        els = list(rng.choice(["C", "O", "Si", "Fe"], 12))
        xyz, occ = rng.random((12, 3)), rng.uniform(0.6, 1.0, 12)
        recip = np.ascontiguousarray(np.linalg.inv(structure_base(ds.Lattice(6.3, 7.1, 8.2, 84.0, 97.0, 103.0))).T)
        atoms = PackedAtoms(els, xyz, occ, np.zeros(12), "lobato", dev)
        q = euler_rzxz_quaternions(np.random.default_rng(7).uniform(-180, 180, (8192, 3)))
        q[:, 1:] *= -1
        quats = torch.from_numpy(q).to(dev)
        settings = DiffractionGenerator(200)._gen.settings(1e-2)
        for _ in range(2):
            tab = PhaseTable.sphere(recip, atoms, 2.0, device=dev)
            sp = simulate_phase(tab, quats, settings, 2.0, SpotBuffers(dev))
        out.update(patterns=8192, spots=sp.total, n_hkl=tab.n)
    torch.cuda.synchronize()
    print(json.dumps(out))


def host_csr_first(table, q_dev, settings, r, n):
    """Host CSR (offsets, rows, xyzi, s) of the first ``n`` orientations, run
    on their own with excitation errors."""
    from diffsims_gb300.engine import SpotBuffers, simulate_phase
    sp = simulate_phase(table, q_dev[:n].contiguous(), settings, r, SpotBuffers(table.device, with_excitation_error=True))
    return (sp.offsets.cpu().numpy(), sp.hkl_index.cpu().numpy(), sp.xyzi.cpu().numpy(),
            sp.excitation_error.cpu().numpy())


def oracle_errors(lat, els, xyz, B, q, runs):
    """Errors of GPU results (``runs``: name -> host CSR of the orientations
    ``q``) against the FP64 oracle, computed in spawned worker processes:
    max relative intensity error, max |s| error, max position error (per
    |g|), cutoff flips within 1e-9 1/Angstrom, FP64 round-off spots of
    systematic absences, and differences neither explains."""
    from oracle import compare as oc
    from oracle import kinematic as ok
    crystal = ok.Crystal(lat, els, xyz, B=B)
    p = ok.SimParams(accelerating_voltage=WORKLOAD["accelerating_voltage"], reciprocal_radius=WORKLOAD["reciprocal_radius"],
                     max_excitation_error=WORKLOAD["max_excitation_error"],
                     shape_factor_model=WORKLOAD["shape_factor_model"])
    t0 = time.perf_counter()
    ref = oc.simulate_parallel(crystal, q, p)
    out = {"orientations": int(len(q)), "oracle_s": time.perf_counter() - t0}
    for name, (off, idx, xyzi, s) in runs.items():
        st = oc.spot_errors(off, idx, xyzi, s, crystal, q, p, ref)
        out[name] = {"max_rel_intensity": st["max_rel_I"], "max_abs_excitation_error": st["max_abs_s"],
                     "max_rel_position": st["max_abs_pos"], "flips_within_1e-9": st["boundary_flips"],
                     "max_flip_distance": st["max_flip_distance"], "noise_spots": st["noise_spots"],
                     "unexplained": len(st["unexplained"]), "spots": st["spots"], "ordered": st["ordered"]}
    return out


def compare_forms(mixed, ref, table, q_host, settings):
    """Errors of the mixed form against the all-FP64 GPU form: max relative
    intensity error, max |s| difference, selection flips (and how far from
    the cutoff they sit, from an FP64 host evaluation of those pairs)."""
    om, im, xm, sm = (mixed.offsets.cpu().numpy(), mixed.hkl_index.cpu().numpy(), mixed.xyzi.cpu().numpy(),
                      mixed.excitation_error.cpu().numpy())
    of, jf, xf, sf = (ref.offsets.cpu().numpy(), ref.hkl_index.cpu().numpy(), ref.xyzi.cpu().numpy(),
                      ref.excitation_error.cpu().numpy())
    hkl = table.hkl_host().astype(np.float64)
    from diffsims_gb300.crystal import Rotation
    Rs = Rotation(q_host).to_matrix()
    k0, eps = settings.k0, settings.max_excitation_error
    max_rel, max_ds, flips, max_fd = 0.0, 0.0, 0, 0.0
    for i in range(len(q_host)):
        a, b = im[om[i]:om[i + 1]], jf[of[i]:of[i + 1]]
        common, ia, ib = np.intersect1d(a, b, return_indices=True)
        I1, I2 = xm[om[i]:om[i + 1]][ia, 3].astype(np.float64), xf[of[i]:of[i + 1]][ib, 3].astype(np.float64)
        nz = I2 != 0
        if nz.any():
            max_rel = max(max_rel, float(np.max(np.abs(I1[nz] - I2[nz]) / np.abs(I2[nz]))))
        if common.size:
            max_ds = max(max_ds, float(np.max(np.abs(sm[om[i]:om[i + 1]][ia] - sf[of[i]:of[i + 1]][ib]))))
        for j in np.setxor1d(a, b):
            g = hkl[j] @ table.recip
            rot = g @ Rs[i]
            rr = math.hypot(rot[0], rot[1])
            s = (-math.sqrt(k0 * k0 - rr * rr) + k0) - rot[2]
            flips += 1
            max_fd = max(max_fd, abs(abs(s) - eps))
    return {"max_rel_intensity": max_rel, "max_abs_excitation_error": max_ds, "flips": flips,
            "max_flip_distance_from_cutoff": max_fd, "orientations": int(len(q_host))}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    n = args.cpu_sample
    rates = []
    for it in range(args.warmup + args.steps):
        rate, dt, _ = cpu_reference_rate(n, cores, seed=it)
        if it >= args.warmup:
            rates.append(rate)
    value = statistics.mean(rates)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": n / value * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded P1 cell and uniform SO(3) orientations)",
        "config": dict(WORKLOAD, sample_orientations_per_step=n), "impl": "reference",
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"{n} orientations per step of the same workload; FP64 numpy restatement of "
                                   f"diffsims' calculate_diffraction2d loop, {cores} spawned processes"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--orientations", type=int, default=WORKLOAD["n_orientations"])
    ap.add_argument("--fp64-orientations", type=int, default=4096)
    ap.add_argument("--cpu-sample", type=int, default=16384)
    ap.add_argument("--library-cpu-sample", type=int, default=512,
                    help="orientations per phase of the template library's CPU baseline")
    ap.add_argument("--oracle-orientations", type=int, default=2048,
                    help="orientations of the headline workload checked against the FP64 oracle")
    ap.add_argument("--no-oracle-check", action="store_true", help="leave out the error report against the oracle")
    ap.add_argument("--skip-grad", action="store_true", help="leave out the gradient-step leg")
    ap.add_argument("--skip-library", action="store_true", help="leave out the template-library leg")
    ap.add_argument("--skip-batch", action="store_true", help="leave out the batched-phases leg")
    ap.add_argument("--skip-families", action="store_true", help="leave out the per-family structure-factor leg")
    ap.add_argument("--skip-legacy", action="store_true", help="leave out the legacy calculate_ed_data leg")
    ap.add_argument("--host-transfer", default="copies", choices=["stores", "copies"],
                    help="how the e2e leg's spots reach the host: chunked copies (default) or the kernel's own "
                         "stores into page-locked memory")
    ap.add_argument("--skip-polar", action="store_true", help="leave out the polar-template leg")
    ap.add_argument("--skip-profiles", action="store_true", help="leave out the 1-D profile leg")
    ap.add_argument("--case", default=None, choices=["raster", "adjoint", "batch", "families", "legacy", "polar"],
                    help="run one small profiling case instead of the benchmark")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--out-dir", default=None)
    ap.add_argument("--screen", default="auto", choices=["auto", "rows", "lines", "bricks"],
                    help="candidate screen of the orientation kernel (results are identical)")
    ap.add_argument("--device-only", action="store_true",
                    help="time only the device-resident step (for profiling); no e2e, FP64 form or CPU legs")
    args = ap.parse_args()
    if args.case:
        run_case(args)
        return
    if args.impl == "reference":
        run_reference(args)
        return
    run_gpu(args)


if __name__ == "__main__":
    main()
