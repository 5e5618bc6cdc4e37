"""The reduction entry point that allocates nothing, for callers that cannot
let a library allocate device memory (an application that gives all of HBM
to its own pool, a latency-bound loop that must not take allocator locks).

Its result must equal the allocating lbx_reduce_mass_momentum_f64 on the same
device array, on two calls in a row (the shared scratch keeps the previous
call's partial sums, which must not leak into the next result).  This file is
collected last; it passes alone in a fresh process and after the other tests.
"""
import ctypes

import numpy as np
import pytest

from golden_util import smooth_random

pytestmark = pytest.mark.gpu

RTOL = 1e-13  # compensated FP64 sums of the same data by the same kernels


def _device_f(lbx, dims, seed, steps):
    nx, ny, nz = dims
    rho_c, u_c = smooth_random(nx, ny, nz, seed=seed, amp_u=0.03)
    sim = lbx.AmrSim(nx, ny, nz, 0, [1, 1, 1], 0.8, 0.8)
    sim.SetInitialDensity(rho_c)
    sim.SetInitialVelocity(u_c)
    sim.InitFromScratch(0.0)
    sim.Iterate(steps)
    sim.synchronize()
    ptr = ctypes.c_void_p()
    ext = (ctypes.c_int * 3)()
    g, p = ctypes.c_int(), ctypes.c_int()
    rc = lbx.lib().lbx_get_device_f(sim.handle, 0, ctypes.byref(ptr), ext, ctypes.byref(g), ctypes.byref(p))
    assert rc == 0 and g.value == 0 and p.value == 0
    return sim, ptr, nx * ny * nz


def test_no_alloc_reduction_matches_allocating_entry(gpu_lib, oracle):
    torch = pytest.importorskip("torch")
    L = gpu_lib.lib()
    sig = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_void_p]
    L.lbx_reduce_mass_momentum_f64.argtypes = sig
    L.lbx_reduce_mass_momentum_f64_noalloc.argtypes = sig
    stream = torch.cuda.current_stream().cuda_stream
    # two different arrays so that a stale partial from call 1 would show in call 2
    cases = [((33, 17, 9), 4, 3), ((20, 30, 11), 7, 5)]
    for dims, seed, steps in cases:
        sim, f, n = _device_f(gpu_lib, dims, seed, steps)
        ref_out = torch.zeros(4, dtype=torch.float64, device="cuda")
        new_out = torch.full((4,), float("nan"), dtype=torch.float64, device="cuda")
        assert L.lbx_reduce_mass_momentum_f64(f, n, ref_out.data_ptr(), stream) == 0
        assert L.lbx_reduce_mass_momentum_f64_noalloc(f, n, new_out.data_ptr(), stream) == 0
        torch.cuda.synchronize()
        ref = ref_out.cpu().numpy()
        new = new_out.cpu().numpy()
        assert abs(new[0] - ref[0]) <= RTOL * abs(ref[0])
        assert np.allclose(new[1:], ref[1:], rtol=RTOL, atol=RTOL * abs(ref[0]))
        # and both agree with the CPU oracle on the same state
        want = oracle.mass_momentum(sim.copy_f(0))
        assert abs(new[0] - want[0]) <= 1e-13 * want[0]
        sim.close()


def test_no_alloc_rejects_oversize_input(gpu_lib):
    L = gpu_lib.lib()
    L.lbx_reduce_mass_momentum_f64_noalloc.argtypes = [ctypes.c_void_p, ctypes.c_size_t,
                                                        ctypes.c_void_p, ctypes.c_void_p]
    dummy = ctypes.c_void_p(16)  # never dereferenced: the size check comes first
    assert L.lbx_reduce_mass_momentum_f64_noalloc(dummy, 1 << 31, dummy, None) == 1
    assert L.lbx_reduce_mass_momentum_f64_noalloc(dummy, 0, dummy, None) == 1
