"""ds_simulate_noalloc: the orientation kernel with its scratch in the
library's static device array, for callers that cannot allocate device
memory (a loop that must not enter the CUDA allocator, a host whose memory
manager owns all device memory).  Checked through the C ABI against the
regular ds_simulate (caller-owned scratch) on the same inputs, twice in a row
(the static array keeps the previous call's contents).
"""
import ctypes

import numpy as np
import pytest

from oracle import kinematic as ok
from tests import parity_util as pu

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import __graft_entry__
    __graft_entry__.build()
    from diffsims_gb300 import _native as N
    lib = N.load_library()
    lib.ds_simulate_noalloc.argtypes = [ctypes.POINTER(N.ds_sim_params), ctypes.POINTER(N.ds_phase_table),
                                        ctypes.c_void_p, ctypes.c_int64, ctypes.POINTER(N.ds_spots),
                                        ctypes.c_void_p, ctypes.c_void_p]
    lib.ds_simulate_noalloc.restype = ctypes.c_int32
    torch.cuda.set_device(0)
    return lib


def _run_noalloc(lib, table, settings, q, capacity):
    import torch
    from diffsims_gb300 import _native as N
    dev = q.device
    n = q.shape[0]
    offsets = torch.empty(n + 1, dtype=torch.int64, device=dev)
    idx = torch.empty(capacity, dtype=torch.int32, device=dev)
    xyzi = torch.empty((capacity, 4), dtype=torch.float32, device=dev)
    total = torch.zeros(1, dtype=torch.int64, device=dev)
    status = torch.zeros(1, dtype=torch.int32, device=dev)
    out = N.ds_spots(offsets.data_ptr(), idx.data_ptr(), xyzi.data_ptr(), capacity, total.data_ptr(), None)
    rc = lib.ds_simulate_noalloc(settings.cstruct(), table.cstruct(), q.data_ptr(), n, out, status.data_ptr(),
                                 N.stream_handle())
    assert rc == 0, lib.ds_last_error().decode()
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    t = int(total.item())
    return offsets.cpu().numpy(), idx[:t].cpu().numpy(), xyzi[:t].cpu().numpy()


@pytest.mark.parametrize("shape, n_orient", [("lorentzian", 3000), ("linear", 257)])
def test_noalloc_matches_ds_simulate_twice(lib, shape, n_orient):
    import torch
    from diffsims_gb300.engine import PhaseTable, SpotBuffers, simulate_phase
    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(4)
    crystal = ok.Crystal(tuple(rng.uniform(8, 12, 3)) + (88.0, 95.0, 101.0), list(rng.choice(["C", "O", "Si"], 40)),
                         rng.random((40, 3)), B=rng.uniform(0.3, 1.5, 40))
    p = ok.SimParams(accelerating_voltage=200, shape_factor_model=shape, reciprocal_radius=1.6,
                     max_excitation_error=0.02)
    table = PhaseTable(pu.to_phase(crystal), 1.6, True, "lobato", list(crystal.B), device=dev)
    settings = pu.generator_for(p).settings(0.02)
    for call in range(2):
        q = torch.as_tensor(ok.random_quaternions(n_orient, seed=10 + call)).to(dev)
        ref = simulate_phase(table, q, settings, 1.6, SpotBuffers(dev))
        off, idx, xyzi = _run_noalloc(lib, table, settings, q, ref.total + 64)
        np.testing.assert_array_equal(off, ref.offsets.cpu().numpy())
        np.testing.assert_array_equal(idx, ref.hkl_index.cpu().numpy())
        rx = ref.xyzi.cpu().numpy()
        np.testing.assert_allclose(xyzi[:, 3], rx[:, 3], rtol=1e-6)      # intensities
        np.testing.assert_allclose(xyzi[:, :3], rx[:, :3], atol=1e-6)    # beam-frame positions


def test_noalloc_rejects_oversized_problem(lib):
    import torch
    from diffsims_gb300.engine import PhaseTable
    from diffsims_gb300 import _native as N
    dev = torch.device("cuda", 0)
    crystal = ok.Crystal((5.0, 5.0, 5.0, 90, 90, 90), ["Si"], [[0, 0, 0]])
    p = ok.SimParams(accelerating_voltage=200, reciprocal_radius=1.0)
    table = PhaseTable(pu.to_phase(crystal), 1.0, True, device=dev)
    settings = pu.generator_for(p).settings(0.01)
    n = 400_000_000  # 12.5M tiles of 32: their look-back states alone exceed the static scratch
    out = N.ds_spots(None, None, None, 0, None, None)
    status = torch.zeros(1, dtype=torch.int32, device=dev)
    rc = lib.ds_simulate_noalloc(settings.cstruct(), table.cstruct(), None, n, out, status.data_ptr(),
                                 N.stream_handle())
    assert rc == N.DS_ERR_INVALID_ARGUMENT
    assert "static scratch" in lib.ds_last_error().decode()


def test_noalloc_reports_the_plans_own_error(lib):
    """A candidate table too large for one orientation tile: the entry point
    returns the launch plan's own status and message (not a generic one).
    The table's arrays are null, so nothing could launch even if planning
    passed (ds_simulate rejects missing arrays before any launch)."""
    import torch
    from diffsims_gb300 import _native as N
    dev = torch.device("cuda", 0)
    p = ok.SimParams(accelerating_voltage=200, reciprocal_radius=1.0)
    settings = pu.generator_for(p).settings(0.01)
    t = N.ds_phase_table()
    t.n_hkl = 1 << 30
    out = N.ds_spots(None, None, None, 0, None, None)
    status = torch.zeros(1, dtype=torch.int32, device=dev)
    rc = lib.ds_simulate_noalloc(settings.cstruct(), t, None, 1000, out, status.data_ptr(), N.stream_handle())
    assert rc == N.DS_ERR_INVALID_ARGUMENT
    assert "too large for one orientation tile" in lib.ds_last_error().decode()
