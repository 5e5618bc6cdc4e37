"""The per-cell step code of the periodic kernels (csrc/cells.cuh) built for
the host and run cell by cell over whole periodic boxes, checked against the
oracle's reference-order step (src/AmrSim.cpp:25-135), without a GPU.

This pins the kernels' index arithmetic -- the periodic wrap of the push
form, the forward and inverse gathers of the pull form, extents of 1 -- and
each precision's collision over several steps.  The host build contracts no
FMAs, so it is not the device's bits; the GPU tests compare the kernels
themselves.  Measured after 9 steps on 6x5x7, 1x3x2, 4x1x5 and 8^3: FP64
1.1e-15, paired 2.8e-14, FP32 shifted 1.8e-8 relative in every f_i; the push
and pull forms give the same bits."""
import os
import shutil
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CUDA_INCLUDE = "/usr/local/cuda/include"
STEPS, TAU_S, TAU_B = 9, 0.8, 1.1
# per-precision bound on max |f - f_ref| / |f_ref| after STEPS steps
BOUND = {"f64": 1e-14, "paired": 2e-13, "f32": 2e-7}
DIMS = [(6, 5, 7), (1, 3, 2), (4, 1, 5), (8, 8, 8)]


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    gxx = shutil.which("g++")
    if not gxx or not os.path.exists(os.path.join(CUDA_INCLUDE, "cuda_runtime.h")):
        pytest.skip("g++ or the CUDA headers are not available")
    exe = str(tmp_path_factory.mktemp("step_host") / "step_host_check")
    cmd = [gxx, "-std=c++17", "-O2", "-ffp-contract=off", "-I" + CUDA_INCLUDE,
           "-I" + os.path.join(ROOT, "lambrex_gb300", "csrc"), "-I" + os.path.join(ROOT, "include"),
           os.path.join(HERE, "step_host_check.cpp"), "-o", exe]
    subprocess.run(cmd, check=True, capture_output=True)
    return exe


def perturbed_equilibrium(oracle, dims, seed):
    """Equilibrium of a random rho, u field plus a small non-equilibrium part."""
    nx, ny, nz = dims
    rng = np.random.default_rng(seed)
    rho_c = 1.0 + 0.02 * rng.standard_normal(nx * ny * nz)
    u_c = 0.01 * rng.standard_normal(3 * nx * ny * nz)
    rho, u = oracle.c_to_fab(nx, ny, nz, rho_c, u_c)
    f = oracle.equilibrium(rho, u)
    return np.ascontiguousarray(f + 1e-4 * np.abs(f) * rng.standard_normal(f.shape))


def run(harness, tmp_path, form, prec, dims, f0):
    src, dst = str(tmp_path / "in.bin"), str(tmp_path / ("%s_%s.bin" % (form, prec)))
    f0.tofile(src)
    subprocess.run([harness, form, prec, *map(str, dims), str(STEPS), repr(TAU_S), repr(TAU_B),
                    src, dst], check=True)
    return np.fromfile(dst).reshape(f0.shape)


@pytest.mark.parametrize("dims", DIMS)
@pytest.mark.parametrize("prec", ["f64", "paired", "f32"])
def test_periodic_step_forms_match_oracle(oracle, harness, tmp_path, dims, prec):
    f0 = perturbed_equilibrium(oracle, dims, seed=sum(dims))
    ref = oracle.step(f0.copy(), TAU_S, TAU_B, STEPS, nthreads=1, style=1)
    push = run(harness, tmp_path, "push", prec, dims, f0)
    pull = run(harness, tmp_path, "pull", prec, dims, f0)
    assert np.array_equal(push, pull)
    err = float(np.max(np.abs(push - ref) / np.abs(ref)))
    assert err <= BOUND[prec], (dims, prec, err)
