"""The plain C caller (tests/c_caller/main_w03_gpu.c) run on the GPU: the
reference driver's call sequence, unchanged but for device allocations,
meets the accuracy gates through the library's own checks."""
import subprocess

import pytest

import lila_cases as C

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("args", [[], ["4000", "1000", "128", "256"], ["1413", "692", "7", "9"]])
def test_c_caller_runs(gpu_lib, tmp_path, args):
    exe = C.build_c_caller(tmp_path / "main_w03_gpu")
    if exe is None:
        pytest.skip("gcc or the CUDA runtime headers are not available")
    r = subprocess.run([exe] + args, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, (r.returncode, r.stdout, r.stderr)
    assert "rc 0 status 0" in r.stdout, r.stdout
