"""Bounded device waits on the GPU: a wait that nothing satisfies gives up,
sets DS_ERR_TIMEOUT and returns; the Python layer raises; the context stays
usable.  No test here faults, traps or hangs the GPU: every wait has a small
limit, and the probe issues no copy that could still be in flight.
"""
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


def _small_case():
    crystal = ok.Crystal((7.3, 8.1, 6.6, 88.0, 95.0, 101.0), ["Si", "O", "O", "Fe"],
                         [[0.1, 0.2, 0.3], [0.4, 0.1, 0.7], [0.8, 0.6, 0.2], [0.3, 0.9, 0.5]], B=[0.5] * 4)
    p = ok.SimParams(accelerating_voltage=200, shape_factor_model="lorentzian", reciprocal_radius=1.2,
                     max_excitation_error=0.02)
    return crystal, p


def test_waits_on_flags_nothing_sets_give_up():
    import torch
    from diffsims_gb300 import _native as N
    lib = N.load_library()
    dev = torch.device("cuda", 0)
    scratch = torch.empty(512, dtype=torch.uint8, device=dev)
    out = torch.full((2,), 7, dtype=torch.int64, device=dev)
    status = torch.zeros(1, dtype=torch.int32, device=dev)
    N.check(lib.ds_probe_wait_timeout(1000, N.ptr(scratch), 512, N.ptr(out), N.ptr(status), N.stream_handle()),
            "probe_wait_timeout")
    torch.cuda.synchronize()
    assert int(status.item()) & N.DS_ERR_TIMEOUT
    assert out.cpu().tolist() == [-1, 0]
    with pytest.raises(N.NativeError, match="timed out"):
        N.check_device_status(status, "probe_wait_timeout")
    # the context is still usable: a simulation afterwards matches the oracle
    crystal, p = _small_case()
    q = ok.random_quaternions(64, seed=1)
    spots, _ = pu.gpu_run(crystal, q, p, "mixed")
    pu.compare(spots, crystal, q, p)


def test_kernels_honour_a_short_wait_limit():
    """With one poll per wait the look-back and staging waits of a
    multi-tile launch may give up: the call then raises (DS_ERR_TIMEOUT),
    and never returns spots that differ from the default-limit run.  The
    defaults restored, the same call gives the reference result again."""
    import torch
    from diffsims_gb300 import _native as N
    crystal, p = _small_case()
    q = ok.random_quaternions(20000, seed=2)
    ref, _ = pu.gpu_run(crystal, q, p, "mixed", with_s=False)
    ref_off, ref_idx = ref.offsets.cpu().numpy(), ref.hkl_index.cpu().numpy()
    outcomes = []
    try:
        N.set_wait_limits(1, 1)
        for _ in range(3):
            try:
                sp, _ = pu.gpu_run(crystal, q, p, "mixed", with_s=False)
            except N.NativeError as e:
                assert "timed out" in str(e)
                outcomes.append("timeout")
                continue
            assert np.array_equal(sp.offsets.cpu().numpy(), ref_off)
            assert np.array_equal(sp.hkl_index.cpu().numpy(), ref_idx)
            outcomes.append("complete")
    finally:
        N.set_wait_limits(0, 0)
    torch.cuda.synchronize()
    again, _ = pu.gpu_run(crystal, q, p, "mixed", with_s=False)
    assert np.array_equal(again.offsets.cpu().numpy(), ref_off)
    assert np.array_equal(again.hkl_index.cpu().numpy(), ref_idx)
    print(outcomes)
