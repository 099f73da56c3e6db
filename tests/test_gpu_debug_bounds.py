"""The parity suites under the bounds-checked build (-DDS_DEBUG_BOUNDS).

That build checks the computed indices of the kernels' staging, table,
bitmap, slice-list and row-buffer accesses; an index outside its array sets
DS_ERR_BOUNDS in the status word (the access is skipped) and the Python layer
raises.  The parity, batch, rasteriser and custom-shape suites run again in a
child process with DIFFSIMS_GB300_DEBUG_BOUNDS=1: every status word must stay
clean and every result must still match the oracle.
"""
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SUITES = ["tests/test_gpu_parity.py", "tests/test_gpu_batch.py", "tests/test_gpu_raster.py",
          "tests/test_gpu_custom_shape.py"]
CHECK_LOADED = ("from diffsims_gb300 import _native as N; N.load_library(); "
                "assert N.DEBUG_BOUNDS and N._LIB_PATH.name == 'libdiffsims_gb300_debug.so'; print('checked build')")


def test_parity_suites_under_bounds_checked_build():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from diffsims_gb300 import _native as N
    if N.DEBUG_BOUNDS:
        pytest.skip("this process already runs the checked build")
    import __graft_entry__
    __graft_entry__.build()
    from diffsims_gb300 import _build
    _build.build(debug=True)
    env = dict(os.environ, DIFFSIMS_GB300_DEBUG_BOUNDS="1")
    r = subprocess.run([sys.executable, "-c", CHECK_LOADED], cwd=ROOT, env=env, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0 and "checked build" in r.stdout, r.stdout + r.stderr
    cmd = [sys.executable, "-m", "pytest", "-x", "-q", "-p", "no:cacheprovider", "-m", "gpu", *SUITES]
    r = subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=2400)
    tail = (r.stdout + r.stderr)[-4000:]
    print(tail[-600:])
    assert r.returncode == 0 and " passed" in tail, tail
