"""Batched multi-phase launch (ds_simulate_batch): one persistent launch over
many phases gives, phase by phase, exactly the spots of the single-phase
launches (bit for bit), inside and outside a CUDA graph, for every tile size
the autotuner may pick."""
import numpy as np
import pytest

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


def random_cell(seed, n_atoms, edges=(3, 20), angles=(80, 100),
                zs=("C", "N", "O", "Al", "Si", "Ti", "Fe", "Cu")):
    rng = np.random.default_rng(seed)
    lat = tuple(rng.uniform(*edges, 3)) + tuple(rng.uniform(*angles, 3))
    return ok.Crystal(lat, list(rng.choice(zs, n_atoms)), rng.random((n_atoms, 3)), B=rng.uniform(0.3, 1.5, n_atoms))


def _phase_set(torch, dev, p, specs):
    from diffsims_gb300.engine import PhaseTable
    tables, qs = [], []
    for seed, n_atoms, n_orient, edges in specs:
        cr = random_cell(seed, n_atoms, edges=edges)
        tables.append(PhaseTable(pu.to_phase(cr), p.reciprocal_radius, True, "lobato", list(cr.B), form="mixed",
                                 device=dev))
        qs.append(torch.as_tensor(ok.random_quaternions(n_orient, seed=seed + 100)).to(dev))
    return tables, qs


SPECS = [(1, 3, 50, (3, 5)), (2, 40, 300, (8, 12)), (3, 7, 0, (5, 7)), (4, 120, 777, (10, 16)),
         (5, 1, 33, (3, 4)), (6, 60, 129, (6, 9))]


def _same(a, b):
    assert a.total == b.total
    assert np.array_equal(a.offsets.cpu().numpy(), b.offsets.cpu().numpy())
    assert np.array_equal(a.hkl_index.cpu().numpy(), b.hkl_index.cpu().numpy())
    assert np.array_equal(a.xyzi.cpu().numpy(), b.xyzi.cpu().numpy())


@pytest.mark.parametrize("kw", [dict(shape_factor_model="sinc"),
                                dict(shape_factor_model="linear", precession_angle=0.5, approximate_precession=False),
                                dict(shape_factor_model="lorentzian", precession_angle=0.5)])
@pytest.mark.parametrize("tile", [1, 4, 16])
def test_batch_matches_single_phase_launches(kw, tile):
    import torch
    from diffsims_gb300.engine import PhaseBatch, SpotBuffers, simulate_phase
    dev = torch.device("cuda", 0)
    p = ok.SimParams(accelerating_voltage=200, reciprocal_radius=1.2, max_excitation_error=0.015, **kw)
    settings = pu.generator_for(p).settings(p.max_excitation_error)
    tables, qs = _phase_set(torch, dev, p, SPECS)
    batch = PhaseBatch(tables, qs, settings, p.reciprocal_radius, orient_tile=tile).run()
    for t, q, got in zip(tables, qs, batch.spots()):
        want = simulate_phase(t, q, settings, p.reciprocal_radius, SpotBuffers(dev))
        _same(got, want)


def test_batch_fp64_form_and_oracle():
    import torch
    from diffsims_gb300.engine import PhaseBatch, PhaseTable
    dev = torch.device("cuda", 0)
    p = ok.SimParams(accelerating_voltage=200, reciprocal_radius=1.0, max_excitation_error=0.015,
                     shape_factor_model="sinc")
    crystals = [random_cell(11, 8, edges=(4, 6)), random_cell(12, 30, edges=(7, 10))]
    qs = [ok.random_quaternions(40, seed=3), ok.random_quaternions(17, seed=4)]
    for form in ("mixed", "fp64"):
        tables = [PhaseTable(pu.to_phase(c), 1.0, True, "lobato", list(c.B), form=form, device=dev) for c in crystals]
        settings = pu.generator_for(p).settings(p.max_excitation_error, form=form)
        spots = PhaseBatch(tables, [torch.as_tensor(q).to(dev) for q in qs], settings, 1.0, orient_tile=0).run().spots()
        for c, q, sp in zip(crystals, qs, spots):
            pu.compare(sp, c, q, p, rtol=1e-5 if form == "mixed" else 1e-6)


def test_graph_replay_follows_inputs():
    """A captured batch re-run on new orientations written in place equals a
    fresh launch."""
    import torch
    from diffsims_gb300.engine import PhaseBatch
    dev = torch.device("cuda", 0)
    p = ok.SimParams(accelerating_voltage=200, reciprocal_radius=1.2, max_excitation_error=0.015,
                     shape_factor_model="sinc")
    settings = pu.generator_for(p).settings(p.max_excitation_error)
    tables, qs = _phase_set(torch, dev, p, SPECS)
    batch = PhaseBatch(tables, qs, settings, p.reciprocal_radius, orient_tile=8).capture()
    for seed in (21, 22):
        for q in batch.quats:
            if q.shape[0]:
                q.copy_(torch.as_tensor(ok.random_quaternions(q.shape[0], seed=seed + q.shape[0])).to(dev))
        batch.replay()
        torch.cuda.synchronize()
        assert int(batch.status.abs().sum()) == 0
        got = batch.spots()
        fresh = PhaseBatch(tables, [q.clone() for q in batch.quats], settings, p.reciprocal_radius,
                           orient_tile=8).run().spots()
        for a, b in zip(got, fresh):
            _same(a, b)


def test_autotuner_picks_and_caches():
    import torch
    from diffsims_gb300.engine import Autotuner, PhaseBatch
    dev = torch.device("cuda", 0)
    p = ok.SimParams(accelerating_voltage=200, reciprocal_radius=1.2, max_excitation_error=0.015,
                     shape_factor_model="sinc")
    settings = pu.generator_for(p).settings(p.max_excitation_error)
    tables, qs = _phase_set(torch, dev, p, SPECS)
    tuner = Autotuner(repeats=2)
    batch = PhaseBatch(tables, qs, settings, p.reciprocal_radius, autotuner=tuner)
    key = Autotuner.key(batch)
    assert batch.orient_tile in Autotuner.TILES
    assert batch.stage_cap in [batch.orient_tile * s for s in Autotuner.STAGE_PER_ORIENT]
    assert batch.refine_parts in (0,) + Autotuner.PARTS
    assert tuner.cache[key] == (batch.orient_tile, batch.stage_cap, batch.refine_parts) and tuner.timings[key]
    assert any("_parts" in name for name in tuner.timings[key])  # the reflections-per-unit sweep ran
    batch.run()
    again = PhaseBatch(tables, qs, settings, p.reciprocal_radius, autotuner=tuner)
    assert (again.orient_tile, again.stage_cap, again.refine_parts) == \
        (batch.orient_tile, batch.stage_cap, batch.refine_parts)


@pytest.mark.parametrize("parts", [1, 4, 8])
def test_refine_parts_give_identical_spots(parts):
    """The reflections per refine / write unit change the work split, not
    the result: single-phase and batched launches equal the default split."""
    import dataclasses
    import torch
    from diffsims_gb300.engine import PhaseBatch, SpotBuffers, simulate_phase
    dev = torch.device("cuda", 0)
    p = ok.SimParams(accelerating_voltage=200, reciprocal_radius=1.2, max_excitation_error=0.015,
                     shape_factor_model="sinc")
    settings = pu.generator_for(p).settings(p.max_excitation_error)
    other = dataclasses.replace(settings, refine_parts=parts)
    tables, qs = _phase_set(torch, dev, p, SPECS)
    for t, q in zip(tables, qs):
        a = simulate_phase(t, q, settings, p.reciprocal_radius, SpotBuffers(dev))
        b = simulate_phase(t, q, other, p.reciprocal_radius, SpotBuffers(dev))
        _same(a, b)
    ba = PhaseBatch(tables, qs, settings, p.reciprocal_radius, orient_tile=8).run()
    bb = PhaseBatch(tables, qs, other, p.reciprocal_radius, orient_tile=8).run()
    assert bb.refine_parts == parts
    for a, b in zip(ba.spots(), bb.spots()):
        _same(a, b)


def test_more_phases_than_one_launch_holds():
    """100 phases: two launches, same spots as single-phase launches."""
    import torch
    from diffsims_gb300.engine import PhaseBatch, SpotBuffers, simulate_phase
    dev = torch.device("cuda", 0)
    p = ok.SimParams(accelerating_voltage=200, reciprocal_radius=0.8, max_excitation_error=0.02,
                     shape_factor_model="lorentzian")
    settings = pu.generator_for(p).settings(p.max_excitation_error)
    specs = [(200 + i, 1 + i % 5, 3 + i % 7, (3, 6)) for i in range(100)]
    tables, qs = _phase_set(torch, dev, p, specs)
    batch = PhaseBatch(tables, qs, settings, p.reciprocal_radius, orient_tile=4).run()
    assert len(batch.groups) == 2
    for t, q, got in zip(tables, qs, batch.spots()):
        _same(got, simulate_phase(t, q, settings, p.reciprocal_radius, SpotBuffers(dev)))


def test_calculate_diffraction2d_phases_in_one_launch():
    import diffsims_gb300 as ds
    crystals = [random_cell(31, 5, edges=(4, 6)), random_cell(32, 12, edges=(6, 9))]
    rots = [ds.Rotation(ok.random_quaternions(20, seed=5)), ds.Rotation(ok.random_quaternions(9, seed=6))]
    gen = ds.SimulationGenerator(200, shape_factor_model="sinc")
    multi = gen.calculate_diffraction2d([pu.to_phase(c) for c in crystals], rots, reciprocal_radius=1.0)
    for k, (c, r) in enumerate(zip(crystals, rots)):
        one = gen.calculate_diffraction2d(pu.to_phase(c), r, reciprocal_radius=1.0)
        for a, b in zip(multi.coordinates[k], one.coordinates):
            assert np.array_equal(a.data, b.data) and np.array_equal(a.intensity, b.intensity)
            assert np.array_equal(a.hkl, b.hkl)


@pytest.mark.parametrize("tile", [4, 16, 32])
def test_batch_brick_screen_matches_row_screen(tile):
    """The batched launch with every phase on the brick screen (its own
    bricks per phase) against the row screen, bit for bit, including a phase
    whose candidate table is empty."""
    import torch
    from diffsims_gb300.engine import PhaseBatch, PhaseTable
    dev = torch.device("cuda", 0)
    p = ok.SimParams(accelerating_voltage=200, reciprocal_radius=1.2, max_excitation_error=0.015,
                     shape_factor_model="sinc")
    tables, qs = _phase_set(torch, dev, p, SPECS)
    empty = random_cell(7, 3, edges=(3, 4))
    tables.append(PhaseTable(pu.to_phase(empty), 0.05, False, "lobato", list(empty.B), device=dev))
    qs.append(torch.as_tensor(ok.random_quaternions(25, seed=8)).to(dev))
    assert tables[-1].n == 0
    out = {}
    for screen in ("rows", "bricks"):
        settings = pu.generator_for(p).settings(p.max_excitation_error)
        settings.screen = screen
        out[screen] = PhaseBatch(tables, qs, settings, p.reciprocal_radius, orient_tile=tile).run().spots()
    for a, b in zip(out["rows"], out["bricks"]):
        _same(a, b)
