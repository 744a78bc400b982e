"""Bounds-checked debug build (-DFDTD_CHECK): parity cases of the fused Yee
step, the batched plan and the 4th-order stage pairs run in a child process
against libfdtd_gb300_check.so, whose kernels check every wrapped global index
against its array's extent and record the first one outside it instead of
accessing it; the run must stay bit-exact and record nothing."""
import json
import os
import subprocess
import sys

import pytest

from tests.conftest import cuda_available

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not cuda_available(), reason="needs a CUDA GPU")]

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_checked_build_records_no_out_of_range_index():
    from fdtd_accelerate_gb300 import buildlib
    lib = buildlib.build(check=True)
    assert os.path.basename(lib) == "libfdtd_gb300_check.so"
    env = dict(os.environ, FDTD_GB300_CHECKED="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "tests", "checked_cases.py")], env=env,
                       capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-4000:]
    out = json.loads(r.stdout.strip().splitlines()[-1])
    assert out["lib"] == "libfdtd_gb300_check.so"
    assert out["cases"] == 7
    bad = out["first_bad"]
    assert bad == 0, "index outside its array: source line %d, index %d" % ((bad >> 40) & 0x7FFFFF, bad & 0xFFFFFFFFFF)
