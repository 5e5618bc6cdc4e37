"""GPU tests of the batched ensemble (one persistent launch per step for many
uneven boxes, graph-replayed steps, autotuned launch shape).  Each box must
give the same result alone (single AmrSim) and in the mix."""
import numpy as np
import pytest

from golden_util import plane_pulse, smooth_random

pytestmark = pytest.mark.gpu

DIMS = [(16, 24, 8), (8, 8, 8), (24, 16, 32), (12, 20, 16), (16, 16, 16), (40, 8, 24)]
TAUS = [0.6, 0.9, 1.2, 0.75, 1.5, 0.65]


def inputs(b):
    nx, ny, nz = DIMS[b]
    return smooth_random(nx, ny, nz, seed=100 + b, amp_rho=0.02, amp_u=0.01)


def alone(lbx, b, steps, precision):
    nx, ny, nz = DIMS[b]
    rho_c, u_c = inputs(b)
    s = lbx.AmrSim(nx, ny, nz, 0, [1, 1, 1], TAUS[b], TAUS[b], precision=precision)
    s.SetInitialDensity(rho_c)
    s.SetInitialVelocity(u_c)
    s.InitFromScratch(0.0)
    s.Iterate(steps)
    return s.copy_f(0)


def make(lbx, precision):
    e = lbx.Ensemble(DIMS, TAUS, precision=precision)
    for b in range(len(DIMS)):
        e.init_box(b, *inputs(b))
    return e


@pytest.mark.parametrize("precision,rtol", [("f64", 1e-13), ("f32s", 1e-6)])
def test_ensemble_matches_single_runs(gpu_lib, precision, rtol):
    from lambrex_gb300.lbx import Ensemble  # noqa: F401
    e = make(gpu_lib, precision)
    e.set_config(1024, 128, 2)
    e.iterate(7)    # odd: exercises the direct launch after graph replays
    e.iterate(10)   # starts from the odd parity
    for b in range(len(DIMS)):
        got = e.copy_f(b)
        ref = alone(gpu_lib, b, 17, precision)
        assert np.max(np.abs(got - ref) / np.abs(ref)) <= rtol, b


def test_ensemble_f64_matches_oracle(gpu_lib, oracle):
    e = make(gpu_lib, "f64")
    e.iterate(9)
    for b in (0, 2, 5):
        nx, ny, nz = DIMS[b]
        rho, u = oracle.c_to_fab(nx, ny, nz, *inputs(b))
        f = oracle.equilibrium(rho, u)
        oracle.step(f, TAUS[b], TAUS[b], 9, nthreads=4)
        assert np.max(np.abs(e.copy_f(b) - f) / f) <= 1e-12


def test_autotune_keeps_state(gpu_lib):
    a = make(gpu_lib, "f32s")
    b = make(gpu_lib, "f32s")
    a.iterate(3)
    b.iterate(3)
    chosen = a.autotune(trial_steps=4)
    assert chosen[1] in (128, 256, 512) and chosen[2] in (1, 2)
    a.iterate(6)
    b.iterate(6)
    for k in range(len(DIMS)):
        np.testing.assert_allclose(a.copy_f(k), b.copy_f(k), rtol=1e-6)


def test_ensemble_launch_count_and_hydro(gpu_lib):
    e = gpu_lib.Ensemble([(16, 16, 16), (32, 8, 8)], [0.8, 0.8], precision="f32s")
    for b, d in enumerate([(16, 16, 16), (32, 8, 8)]):
        e.init_box(b, plane_pulse(*d, axis=0, index=4, amplitude=0.05), np.zeros(3 * np.prod(d)))
    ms = e.iterate_timed(10)
    assert ms > 0
    assert e.launches() == 10  # one persistent launch per step for all boxes
    rho, u = e.hydro(0)
    assert abs(rho.mean() - (1 + 0.05 / 16)) < 1e-6
