"""The paired-FP32 collision (csrc/df32.cuh, scalar form) built for the host
and checked cell by cell against the oracle's reference-order FP64 collision
(src/AmrSim.cpp:25-107), without a GPU.

On the host the approximate reciprocal is an exact division (the device uses
the hardware's approximation, which the residual refinement absorbs), so this
pins the pair arithmetic's accuracy, not the device's bits; the GPU tests pin
those.  Measured: at most 2.5e-14 relative per collision (median 6e-15),
against 1.1e-15 for the FP64 form of the same restructured collision."""
import os
import shutil
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CUDA_INCLUDE = "/usr/local/cuda/include"


def build_harness(tmp_path):
    gxx = shutil.which("g++")
    if not gxx or not os.path.exists(os.path.join(CUDA_INCLUDE, "cuda_runtime.h")):
        pytest.skip("g++ or the CUDA headers are not available")
    exe = str(tmp_path / "paired_host_check")
    cmd = [gxx, "-std=c++17", "-O2", "-ffp-contract=off", "-I" + CUDA_INCLUDE,
           "-I" + os.path.join(ROOT, "lambrex_gb300", "csrc"),
           os.path.join(HERE, "paired_host_check.cpp"), "-o", exe]
    subprocess.run(cmd, check=True, capture_output=True)
    return exe


@pytest.mark.parametrize("om_s,om_b", [(1.25, 0.9), (1.9, 1.6)])
def test_paired_collision_matches_reference_order(oracle, tmp_path, om_s, om_b):
    exe = build_harness(tmp_path)
    out = str(tmp_path / "cells.bin")
    n = 4000
    subprocess.run([exe, str(n), repr(om_s), repr(om_b), out], check=True)
    cells = np.fromfile(out, dtype=np.float64).reshape(n, 2, 15)
    worst = 0.0
    for f_in, f_out in cells:
        ref = oracle.collide_cell(f_in, om_s, om_b)
        worst = max(worst, float(np.max(np.abs(f_out - ref) / np.abs(ref))))
    assert worst <= 5e-14
