"""The per-cell step code of the kernels (csrc/cells.cuh) built for the host
and run cell by cell over whole boxes, checked against the oracle without a
GPU: periodic single levels against the reference-order step
(src/AmrSim.cpp:25-135), and the conservative two- and three-level scheme
(explode, periodic and patch steps, coalesce, restrict, in the order the
library's driver launches them) against the oracle's restatement of it, and
the reference-faithful Rohde cycle over two and three levels (csrc/faithful.cuh,
in the faithful driver's order) against the oracle's restatement of
src/AmrSim.cpp:430-631.

This pins the kernels' index arithmetic -- the periodic wrap of the push
form, the forward and inverse gathers of the pull form, extents of 1 -- and
each precision's collision over several steps.  The host build contracts no
FMAs, so it is not the device's bits; the GPU tests compare the kernels
themselves.  Measured after 9 steps on 6x5x7, 1x3x2, 4x1x5 and 8^3: FP64
1.1e-15, paired 2.8e-14, FP32 shifted 1.8e-8 relative in every f_i; the push
and pull forms give the same bits, with 64-bit or 32-bit element indices;
rho and u read from the store by the hydro kernel's cell body (gathering
through the pull form): FP64 rho 5.6e-16, u 4.2e-14 of max|u|; paired
5.8e-15, 7.5e-13; FP32 shifted 8.4e-10, 3.8e-7.  Conservative levels on a 16^3 coarse box
(two levels, 6 coarse steps; three levels, 3): FP64 1.9e-15, paired 4.0e-14,
FP32 shifted 9.5e-8 on every level.  Faithful cycle, same cases (error
relative to each level's largest population, since the cycle leaves zero
entries): FP64 1.0e-15, paired 1.8e-14."""
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
HYDRO_BOUND = {"f64": 1e-14, "paired": 2e-13, "f32": 1e-7}
# velocity error against the velocity scale max|u|: u = j / rho is a small
# difference of O(rho) terms, so the population error is amplified by about
# rho / |j| (measured 4.2e-14, 7.5e-13 and 3.8e-7 of max|u|)
U_BOUND = {"f64": 1e-13, "paired": 2e-12, "f32": 1e-6}
DIMS = [(6, 5, 7), (1, 3, 2), (4, 1, 5), (8, 8, 8)]


def build_host(tmp_path_factory, name):
    gxx = shutil.which("g++")
    if not gxx or not os.path.exists(os.path.join(CUDA_INCLUDE, "cuda_runtime.h")):
        pytest.skip("g++ or the CUDA headers are not available")
    exe = str(tmp_path_factory.mktemp(name) / name)
    cmd = [gxx, "-std=c++17", "-O2", "-ffp-contract=off", "-I" + CUDA_INCLUDE,
           "-I" + os.path.join(ROOT, "lambrex_gb300", "csrc"), "-I" + os.path.join(ROOT, "include"),
           os.path.join(HERE, name + ".cpp"), "-o", exe]
    subprocess.run(cmd, check=True, capture_output=True)
    return exe


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    return build_host(tmp_path_factory, "step_host_check")


@pytest.fixture(scope="module")
def amr_harness(tmp_path_factory):
    return build_host(tmp_path_factory, "amr_host_check")


@pytest.fixture(scope="module")
def faithful_harness(tmp_path_factory):
    return build_host(tmp_path_factory, "faithful_host_check")


def perturbed_equilibrium(oracle, dims, seed):
    """Equilibrium of a random rho, u field plus a small non-equilibrium part."""
    nx, ny, nz = dims
    rng = np.random.default_rng(seed)
    rho_c = 1.0 + 0.02 * rng.standard_normal(nx * ny * nz)
    u_c = 0.01 * rng.standard_normal(3 * nx * ny * nz)
    rho, u = oracle.c_to_fab(nx, ny, nz, rho_c, u_c)
    f = oracle.equilibrium(rho, u)
    return np.ascontiguousarray(f + 1e-4 * np.abs(f) * rng.standard_normal(f.shape))


def run(harness, tmp_path, form, prec, dims, f0, hydro=False):
    """f after STEPS steps (and, with hydro, the cell hydro body's rho, u)."""
    src, dst = str(tmp_path / "in.bin"), str(tmp_path / ("%s_%s.bin" % (form, prec)))
    f0.tofile(src)
    subprocess.run([harness, form, prec, *map(str, dims), str(STEPS), repr(TAU_S), repr(TAU_B),
                    src, dst], check=True)
    out = np.fromfile(dst)
    n = f0[0].size
    f = out[:f0.size].reshape(f0.shape)
    if not hydro:
        return f
    rho = out[f0.size:f0.size + n].reshape(f0.shape[1:])
    u = out[f0.size + n:].reshape((3,) + f0.shape[1:])
    return f, rho, u


@pytest.mark.parametrize("dims", DIMS)
@pytest.mark.parametrize("prec", ["f64", "paired", "f32"])
def test_periodic_step_forms_match_oracle(oracle, harness, tmp_path, dims, prec):
    f0 = perturbed_equilibrium(oracle, dims, seed=sum(dims))
    ref = oracle.step(f0.copy(), TAU_S, TAU_B, STEPS, nthreads=1, style=1)
    push = run(harness, tmp_path, "push", prec, dims, f0)
    pull = run(harness, tmp_path, "pull", prec, dims, f0)
    assert np.array_equal(push, pull)
    for form in ("push32", "pull32"):  # the batch engine's 32-bit element indices
        assert np.array_equal(run(harness, tmp_path, form, prec, dims, f0), push)
    # hydro read from the store, gathering through the pull form (rho relative,
    # u against the velocity scale)
    rho_ref, u_ref = oracle.hydro(ref)
    for form in ("push", "pull"):
        _, rho, u = run(harness, tmp_path, form, prec, dims, f0, hydro=True)
        assert np.max(np.abs(rho - rho_ref) / rho_ref) <= HYDRO_BOUND[prec], (form, prec)
        assert np.max(np.abs(u - u_ref)) <= U_BOUND[prec] * np.max(np.abs(u_ref)), (form, prec)
    err = float(np.max(np.abs(push - ref) / np.abs(ref)))
    assert err <= BOUND[prec], (dims, prec, err)


AMR_CASES = {  # tag boxes, each in the cells of the level it refines; coarse steps
    "two levels": ([((4, 5, 6), (11, 10, 12))], 6),
    "three levels": ([((4, 4, 4), (11, 11, 11)), ((12, 12, 12), (19, 19, 19))], 3),
}
AMR_BOUND = {"f64": 1e-14, "paired": 4e-13, "f32": 1e-6}


def run_levels(oracle, exe, tmp_path, mode, case, prec):
    """Oracle levels and the harness's levels after the case's coarse steps."""
    from golden_util import smooth_random
    tags, steps = AMR_CASES[case]
    nx, ny, nz, tau = 16, 16, 16, 0.8
    o = oracle.AmrOracle(nx, ny, nz, len(tags), tau, tau, mode)
    rho_c, u_c = smooth_random(nx, ny, nz, seed=2)
    o.init(rho_c, u_c)
    f0 = np.ascontiguousarray(o.f(0))
    for L, (lo, hi) in enumerate(tags):
        o.refine(L, lo, hi)
    o.iterate(steps)
    src, dst = str(tmp_path / "in.bin"), str(tmp_path / "out.bin")
    f0.tofile(src)
    args = [exe, prec, str(nx), str(ny), str(nz), repr(tau), str(steps), str(len(tags))]
    for lo, hi in tags:
        args += [str(v) for v in lo + hi]
    subprocess.run(args + [src, dst], check=True)
    out, off, pairs = np.fromfile(dst), 0, []
    for L in range(len(tags) + 1):
        ref = o.f(L)
        pairs.append((out[off:off + ref.size].reshape(ref.shape), ref))
        off += ref.size
    assert off == out.size
    return pairs


@pytest.mark.parametrize("case", sorted(AMR_CASES))
@pytest.mark.parametrize("prec", ["f64", "paired", "f32"])
def test_conservative_levels_match_oracle(oracle, amr_harness, tmp_path, case, prec):
    for L, (got, ref) in enumerate(run_levels(oracle, amr_harness, tmp_path, 1, case, prec)):
        err = float(np.max(np.abs(got - ref) / np.abs(ref)))
        assert err <= AMR_BOUND[prec], (case, prec, L, err)


@pytest.mark.parametrize("case", sorted(AMR_CASES))
@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_conservative_levels_32bit_indices_same_bits(oracle, amr_harness, tmp_path, case, prec):
    """The batch engine runs the conservative scheme for served requests with
    32-bit element indices: the same per-cell code gives the same bits."""
    wide = run_levels(oracle, amr_harness, tmp_path, 1, case, prec)
    narrow = run_levels(oracle, amr_harness, tmp_path, 1, case, prec + "-i32")
    for (a, _), (b, _) in zip(wide, narrow):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("case", sorted(AMR_CASES))
@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_served_pull_form_same_bits_as_push_form(oracle, amr_harness, tmp_path, case, prec):
    """The server runs the conservative scheme in the pull form (explosion
    from post-collision stores, coalescence into the entries the coarse ring
    cells gather, conversion at admission and readout): the same bits as the
    push form with the same 32-bit element indices, hence the oracle's
    values to the push form's bounds."""
    push = run_levels(oracle, amr_harness, tmp_path, 1, case, prec + "-i32")
    pull = run_levels(oracle, amr_harness, tmp_path, 1, case, prec + "+p")
    for L, ((a, ref), (b, _)) in enumerate(zip(push, pull)):
        assert np.array_equal(a, b), (case, prec, L, float(np.max(np.abs(a - b))))
        assert float(np.max(np.abs(b - ref) / np.abs(ref))) <= AMR_BOUND[prec]


@pytest.mark.parametrize("case", sorted(AMR_CASES))
@pytest.mark.parametrize("prec", ["f64", "paired", "f32"])
def test_rescaled_levels_match_oracle(oracle, amr_harness, tmp_path, case, prec):
    """The rescaled coupling (covered cells active, time-interpolated and
    rescaled explosion before every fine sub-step, rescaled restriction)
    run by the kernels' per-cell functions in the rescaled driver's order."""
    for L, (got, ref) in enumerate(run_levels(oracle, amr_harness, tmp_path, 2, case, prec + "+r")):
        err = float(np.max(np.abs(got - ref) / np.abs(ref)))
        assert err <= AMR_BOUND[prec], (case, prec, L, err)


FAITHFUL_BOUND = {"f64": 1e-14, "paired": 2e-13}


@pytest.mark.parametrize("case", sorted(AMR_CASES))
@pytest.mark.parametrize("prec", ["f64", "paired"])
def test_faithful_cycle_matches_oracle(oracle, faithful_harness, tmp_path, case, prec):
    for L, (got, ref) in enumerate(run_levels(oracle, faithful_harness, tmp_path, 0, case, prec)):
        err = float(np.max(np.abs(got - ref)) / np.max(np.abs(ref)))
        assert err <= FAITHFUL_BOUND[prec], (case, prec, L, err)


@pytest.fixture(scope="module")
def batch_harness(tmp_path_factory):
    return build_host(tmp_path_factory, "batch_host_check")


BATCH_BOXES = [((6, 5, 7), 0.8), ((1, 3, 2), 1.1), ((9, 4, 3), 0.6), ((8, 8, 8), 1.3)]


@pytest.mark.parametrize("tile_cells", [97, 512])
@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_batch_walk_equals_single_boxes(oracle, harness, batch_harness, tmp_path, tile_cells, prec):
    """The persistent kernel's walk over uneven boxes (tiles that straddle
    rows, planes and boxes; fast-division decode) steps every cell exactly
    once: each box comes out bit for bit as the single-box pull form."""
    steps = 7
    f0s = [perturbed_equilibrium(oracle, dims, seed=k) for k, (dims, _) in enumerate(BATCH_BOXES)]
    src, dst = str(tmp_path / "batch_in.bin"), str(tmp_path / "batch_out.bin")
    np.concatenate([f.ravel() for f in f0s]).tofile(src)
    args = [batch_harness, prec, str(steps), str(tile_cells), str(len(BATCH_BOXES))]
    for dims, tau in BATCH_BOXES:
        args += [str(d) for d in dims] + [repr(tau)]
    subprocess.run(args + [src, dst], check=True)
    out, off = np.fromfile(dst), 0
    for f0, (dims, tau) in zip(f0s, BATCH_BOXES):
        got = out[off:off + f0.size].reshape(f0.shape)
        off += f0.size
        single = str(tmp_path / "single.bin")
        f0.tofile(str(tmp_path / "single_in.bin"))
        subprocess.run([harness, "pull32", prec, *map(str, dims), str(steps), repr(tau), repr(tau),
                        str(tmp_path / "single_in.bin"), single], check=True)
        assert np.array_equal(got, np.fromfile(single)[:f0.size].reshape(f0.shape)), dims
    assert off == out.size
