"""Chunked simulation with the spots streamed to host memory
(``simulate_phase_streamed``, the default single-phase path of
``calculate_diffraction2d``): the host CSR and the assembled device CSR equal
a single ``simulate_phase`` launch bit for bit, for any chunking, with chunks
that overflow their region, and with no orientations at all."""
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


def _case(torch, n_orient, seed=1, model="sinc"):
    from diffsims_gb300.engine import PhaseTable
    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(seed)
    cr = ok.Crystal(tuple(rng.uniform(5, 9, 3)) + (90.0, 95.0, 90.0), list(rng.choice(["O", "Si", "Fe"], 20)),
                    rng.random((20, 3)), B=rng.uniform(0.3, 1.2, 20))
    p = ok.SimParams(accelerating_voltage=200, reciprocal_radius=1.5, max_excitation_error=0.02,
                     shape_factor_model=model)
    settings = pu.generator_for(p).settings(p.max_excitation_error)
    table = PhaseTable(pu.to_phase(cr), p.reciprocal_radius, True, "lobato", list(cr.B), device=dev)
    q = torch.as_tensor(ok.random_quaternions(n_orient, seed=seed + 7)).to(dev)
    return table, q, settings, p.reciprocal_radius


def _check(torch, got, want):
    off, idx, xyzi = got.host()
    w_off, w_idx, w_xyzi = want.host()
    assert got.total == want.total
    assert np.array_equal(off, w_off)
    assert np.array_equal(idx, w_idx)
    assert np.array_equal(xyzi, w_xyzi)
    assert torch.equal(got.offsets, want.offsets)
    assert torch.equal(got.hkl_index, want.hkl_index)
    assert torch.equal(got.xyzi, want.xyzi)


@pytest.mark.parametrize("n_orient,chunk,first", [(5000, 1024, 300), (777, 16384, 4096), (3000, 1000, 1000),
                                                   (1, 16, 16)])
def test_streamed_equals_one_launch(n_orient, chunk, first):
    import torch
    from diffsims_gb300.engine import SpotBuffers, simulate_phase, simulate_phase_streamed
    table, q, settings, r = _case(torch, n_orient)
    want = simulate_phase(table, q, settings, r, SpotBuffers(q.device))
    got = simulate_phase_streamed(table, q, settings, r, chunk=chunk, first_chunk=first)
    _check(torch, got, want)


def test_streamed_chunk_overflow_and_host_growth(monkeypatch):
    """An estimate far too small: every chunk overflows its region and is
    re-run, and the page-locked host arrays grow."""
    import torch
    from diffsims_gb300 import engine
    table, q, settings, r = _case(torch, 2500, seed=4, model="lorentzian")
    want = engine.simulate_phase(table, q, settings, r, engine.SpotBuffers(q.device))
    monkeypatch.setattr(engine, "estimate_spots", lambda *a: 1)
    got = engine.simulate_phase_streamed(table, q, settings, r, chunk=700, first_chunk=200)
    _check(torch, got, want)


def test_streamed_no_orientations():
    import torch
    from diffsims_gb300.engine import simulate_phase_streamed
    table, q, settings, r = _case(torch, 0)
    got = simulate_phase_streamed(table, q, settings, r)
    off, idx, xyzi = got.host()
    assert got.total == 0 and off.tolist() == [0] and idx.shape == (0,) and xyzi.shape == (0, 4)


def test_calculate_diffraction2d_streamed_and_device_only_agree():
    import diffsims_gb300 as ds
    rng = np.random.default_rng(9)
    cr = ok.Crystal((5.1, 6.2, 7.3, 90.0, 90.0, 90.0), ["Si"] * 4, rng.random((4, 3)), B=[0.5] * 4)
    rot = ds.Rotation(ok.random_quaternions(6000, seed=2))
    gen = ds.SimulationGenerator(200, shape_factor_model="linear")
    a = gen.calculate_diffraction2d(pu.to_phase(cr), rot, reciprocal_radius=1.2)
    b = gen.calculate_diffraction2d(pu.to_phase(cr), rot, reciprocal_radius=1.2, stream_to_host=False)
    for x, y in zip(a.coordinates[::97], b.coordinates[::97]):
        assert np.array_equal(x.data, y.data) and np.array_equal(x.intensity, y.intensity)
        assert np.array_equal(x.hkl, y.hkl)


def test_host_mapped_query():
    import torch
    from diffsims_gb300 import _native as N
    pinned = torch.empty(1024, dtype=torch.int32, pin_memory=True)
    assert N.host_mapped(pinned.data_ptr())
    assert N.host_mapped(pinned[100:].data_ptr())  # inside a page-locked block
    assert not N.host_mapped(torch.empty(1024, dtype=torch.int32, device="cuda").data_ptr())
    assert not N.host_mapped(np.zeros(1024, np.int32).ctypes.data)
    assert not N.host_mapped(0)


@pytest.mark.parametrize("n_orient", [5000, 777, 1])
def test_kernel_stores_to_host_equal_one_launch(n_orient):
    """The orientation kernel writing its spots straight into page-locked host
    memory gives the device launch's CSR bit for bit, on the host and after
    the upload of the device CSR."""
    import torch
    from diffsims_gb300.engine import SpotBuffers, simulate_phase, simulate_phase_to_host
    table, q, settings, r = _case(torch, n_orient, model="lorentzian")
    want = simulate_phase(table, q, settings, r, SpotBuffers(q.device))
    got = simulate_phase_to_host(table, q, settings, r, timing=True)
    assert got is not None
    _check(torch, got, want)
    t = got.timings()
    assert t["chunks"] == 1 and t["kernel_span_ms"] > 0 and t["copy_span_ms"] == t["kernel_span_ms"]
    assert got.host()[1].dtype == np.uint16  # a small table: 2-byte rows
    assert got.nbytes() == (n_orient + 1) * 8 + got.total * 18


def test_kernel_stores_to_host_overflow_and_pool_reuse(monkeypatch):
    """An estimate far too small: the launch overflows the host arrays and is
    re-run with the exact size; the pool then remembers the density, and a
    later call reuses the released set without overflowing."""
    import gc
    import torch
    from diffsims_gb300 import engine
    table, q, settings, r = _case(torch, 2500, seed=4, model="sinc")
    want = engine.simulate_phase(table, q, settings, r, engine.SpotBuffers(q.device))
    pool = engine.HostSpotPool()
    monkeypatch.setattr(engine, "estimate_spots", lambda *a: 1)
    got = engine.simulate_phase_to_host(table, q, settings, r, host_pool=pool)
    _check(torch, got, want)
    assert len(pool.density) == 1 and abs(list(pool.density.values())[0] * 2500 - want.total) < 1e-6
    n_bytes = pool.allocated_bytes
    first_set = got._set
    del got
    gc.collect()
    again = engine.simulate_phase_to_host(table, q, settings, r, host_pool=pool)
    _check(torch, again, want)
    assert again._set is first_set and pool.allocated_bytes == n_bytes
    # a live result's arrays are never handed out again
    third = engine.simulate_phase_to_host(table, q, settings, r, host_pool=pool)
    assert third._set is not again._set
    _check(torch, third, want)
    _check(torch, again, want)


def test_kernel_stores_to_host_no_orientations():
    import torch
    from diffsims_gb300.engine import simulate_phase_to_host
    table, q, settings, r = _case(torch, 0)
    assert simulate_phase_to_host(table, q, settings, r) is None


def test_calculate_diffraction2d_host_transfers_agree():
    import diffsims_gb300 as ds
    from diffsims_gb300.engine import HostSpots, StreamedSpots
    rng = np.random.default_rng(11)
    cr = ok.Crystal((5.4, 6.0, 7.7, 90.0, 90.0, 90.0), ["Si", "O", "O"], rng.random((3, 3)), B=[0.5] * 3)
    rot = ds.Rotation(ok.random_quaternions(3000, seed=5))
    gen = ds.SimulationGenerator(200, shape_factor_model="linear")
    b = gen.calculate_diffraction2d(pu.to_phase(cr), rot, reciprocal_radius=1.2, result="native")
    assert isinstance(b.spots(0), StreamedSpots)
    gen.host_transfer = "stores"
    a = gen.calculate_diffraction2d(pu.to_phase(cr), rot, reciprocal_radius=1.2, result="native")
    assert isinstance(a.spots(0), HostSpots)
    for x, y in zip(a.coordinates[::53], b.coordinates[::53]):
        assert np.array_equal(x.data, y.data) and np.array_equal(x.intensity, y.intensity)
        assert np.array_equal(x.hkl, y.hkl)
    # a device-side consumer of a host result: the device CSR is uploaded
    img = a.get_diffraction_patterns((64, 64), sigma=1, calibration=0.02, stop=8)
    img_b = b.get_diffraction_patterns((64, 64), sigma=1, calibration=0.02, stop=8)
    assert bool((img == img_b).all())


def _large_case(torch, n_orient, cell, radius, seed=3):
    from diffsims_gb300.engine import PhaseTable
    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(seed)
    cr = ok.Crystal((cell, cell * 1.07, cell * 0.93, 90.0, 90.0, 90.0), list(rng.choice(["O", "Si"], 6)),
                    rng.random((6, 3)), B=rng.uniform(0.3, 1.0, 6))
    p = ok.SimParams(accelerating_voltage=200, reciprocal_radius=radius, max_excitation_error=0.01,
                     shape_factor_model="lorentzian")
    settings = pu.generator_for(p).settings(p.max_excitation_error)
    table = PhaseTable(pu.to_phase(cr), radius, True, "lobato", list(cr.B), device=dev)
    q = torch.as_tensor(ok.random_quaternions(n_orient, seed=seed + 1)).to(dev)
    return table, q, settings, radius


@pytest.mark.parametrize("cell,radius,row_dtype", [(12.0, 2.0, np.uint16), (19.0, 1.6, np.int32)])
def test_row_width_by_table_size(cell, radius, row_dtype):
    """Rows go to the host as uint16 for tables of at most 65536 rows (here
    ~60k, so rows above 32767 exercise the unsigned widening) and as int32
    above that; both transfers equal the device launch."""
    import torch
    from diffsims_gb300.engine import SpotBuffers, simulate_phase, simulate_phase_streamed, simulate_phase_to_host
    table, q, settings, r = _large_case(torch, 600, cell, radius)
    assert (table.n <= 65536) == (row_dtype == np.uint16)
    want = simulate_phase(table, q, settings, r, SpotBuffers(q.device))
    assert want.total > 0 and (row_dtype == np.int32 or int(want.hkl_index.max()) > 32767)
    for got in (simulate_phase_streamed(table, q, settings, r, chunk=256, first_chunk=64),
                simulate_phase_to_host(table, q, settings, r)):
        _check(torch, got, want)
        assert got.host()[1].dtype == row_dtype and got.hkl_index.dtype == torch.int32
        assert got.nbytes() == 601 * 8 + got.total * (16 + np.dtype(row_dtype).itemsize)


def test_streamed_reports_a_later_chunks_status():
    """A non-finite orientation in the last chunk: the kernel flags it in that
    chunk's status word, which travels behind the spot copies; reading the
    result (host or device) raises."""
    import torch
    from diffsims_gb300.engine import simulate_phase_streamed
    table, q, settings, r = _case(torch, 3000)
    q = q.clone()
    q[2900] = float("nan")
    got = simulate_phase_streamed(table, q, settings, r, chunk=1000, first_chunk=500)
    with pytest.raises(ValueError, match="non-finite"):
        got.host()
    got = simulate_phase_streamed(table, q, settings, r, chunk=1000, first_chunk=500)
    with pytest.raises(ValueError, match="non-finite"):
        got.hkl_index


def test_streamed_without_mapped_counts(monkeypatch):
    """Where page-locked memory is not addressable by kernels, each chunk's
    count and status word come back by copies instead (the same results, the
    overflow re-run included)."""
    import torch
    from diffsims_gb300 import _native as N
    from diffsims_gb300 import engine
    table, q, settings, r = _case(torch, 2500, seed=6, model="lorentzian")
    want = engine.simulate_phase(table, q, settings, r, engine.SpotBuffers(q.device))
    monkeypatch.setattr(N, "host_mapped", lambda ptr: False)
    _check(torch, engine.simulate_phase_streamed(table, q, settings, r, chunk=700, first_chunk=200), want)
    monkeypatch.setattr(engine, "estimate_spots", lambda *a: 1)
    _check(torch, engine.simulate_phase_streamed(table, q, settings, r, chunk=700, first_chunk=200), want)
    # and the kernel-stores route declines, leaving the copies to the caller
    assert engine.simulate_phase_to_host(table, q, settings, r) is None
