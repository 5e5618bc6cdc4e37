"""Bounds-checked debug build on the GPU.

compute-sanitizer is not available for these runs, so the library carries
its own checks: liblbx_cuda_checked.so tests every global element index of
every kernel against the array it addresses and counts (and skips) the
misses.  tests/checked_driver.py drives every device path -- single level in
all precisions on tiny and prime extents (with a readout fused into the
next step), the three AMR couplings with two and three levels (FP64, paired
FP64, FP32) and a regrid onto the periodic corner, the batched ensemble with
its autotuner, and the server with 1-3 level requests -- and reports the
counters, which must stay at zero.
"""
import json
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


def test_checked_build_has_no_out_of_range_access():
    from lambrex_gb300 import build as B
    B.build("checked")
    env = dict(os.environ, LBX_LIBRARY="checked")
    p = subprocess.run([sys.executable, os.path.join(HERE, "checked_driver.py")], env=env,
                       capture_output=True, text=True, timeout=900)
    assert p.returncode == 0, p.stderr[-3000:]
    line = json.loads([ln for ln in p.stdout.splitlines() if ln.startswith("{")][-1])
    assert line["variant"] == "checked"
    assert line["cases"] == 21
    assert line["count"] == 0, "out-of-range accesses: %d, first index %d" % (line["count"], line["first"])
