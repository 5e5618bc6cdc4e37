"""CalcHydroVars fused into the next time step.

On a single periodic level the store holds the post-collision populations
of the last step (the pull form), and the next step gathers exactly the
state CalcHydroVars reads.  Once a program has stepped on after reading
fields, CalcHydroVars therefore runs that next step with rho and u of the
gathered state as its epilogue (one pass instead of a hydro pass plus a
step), and the following Iterate takes the step already made.  These tests
check that the fields and the states are the same bits as without the
fusion, that times and steps advance as before, and that a state change in
between (an import, a timed run) drops the step made ahead.
"""
import numpy as np
import pytest

from golden_util import smooth_random

pytestmark = pytest.mark.gpu
DIMS = (20, 12, 9)


def make(lbx, precision, seed=11):
    nx, ny, nz = DIMS
    rho_c, u_c = smooth_random(nx, ny, nz, seed=seed)
    s = lbx.AmrSim(nx, ny, nz, 0, [1, 1, 1], 0.75, 1.05, precision=precision)
    s.SetInitialDensity(rho_c)
    s.SetInitialVelocity(u_c)
    s.InitFromScratch(0.0)
    return s


@pytest.mark.parametrize("precision", ["f64", "f64p", "f32s"])
def test_fused_readout_loop_matches_separate_passes(gpu_lib, precision):
    """Iterate(7) + CalcHydroVars four times: from the second readout on
    CalcHydroVars runs the next step with the fields as epilogue.  Fields,
    populations, times and steps equal those of a fresh run brought to the
    same step and read once (hydro pass alone), bit for bit; lbx_iterate
    issues one launch fewer after each fused readout."""
    a = make(gpu_lib, precision)
    steps = 0
    for k in range(4):
        a.Iterate(7)
        steps += 7
        a.CalcHydroVars(0)
        ra, ua = a.density_field(0), a.velocity_field(0)
        b = make(gpu_lib, precision)
        b.Iterate(steps)
        b.CalcHydroVars(0)   # never stepped after a readout: the hydro pass alone
        assert np.array_equal(ra, b.density_field(0)), k
        assert np.array_equal(ua, b.velocity_field(0)), k
        assert np.array_equal(a.copy_f(0), b.copy_f(0)), k
        assert a.GetTimeStep(0) == b.GetTimeStep(0) == steps
        assert a.GetTime(0) == b.GetTime(0)
        b.close()
    # readouts 2..4 were fused; the steps made by readouts 2 and 3 were taken
    # by the next Iterate (+ 1: the launch entering the pull form)
    assert a.launch_count() == 1 + 28 - 2
    a.Iterate(5)   # consumes the fourth readout's step
    c = make(gpu_lib, precision)
    c.Iterate(33)
    assert np.array_equal(a.copy_f(0), c.copy_f(0))
    a.close()
    c.close()


def test_step_made_ahead_is_dropped_by_an_import_and_by_timed_runs(gpu_lib):
    a = make(gpu_lib, "f64")
    b = make(gpu_lib, "f64")
    for s in (a, b):
        s.Iterate(3)
        s.CalcHydroVars(0)
        s.Iterate(3)
        s.CalcHydroVars(0)   # fused: a step made ahead
    # import: the state is replaced, the step made ahead must not be used
    f = b.copy_f(0)
    a.set_f(0, f)
    a.Iterate(2)
    b.Iterate(2)
    assert np.array_equal(a.copy_f(0), b.copy_f(0))
    # a timed run recomputes the step it reports
    a.CalcHydroVars(0)
    b.CalcHydroVars(0)
    l0 = a.launch_count()
    a.iterate_timed(4)
    assert a.launch_count() - l0 == 4
    b.Iterate(4)
    assert np.array_equal(a.copy_f(0), b.copy_f(0))
    assert a.GetTimeStep(0) == b.GetTimeStep(0) == 12
    a.close()
    b.close()


def test_getters_after_fused_readout(gpu_lib, oracle):
    """The point getters read the fused fields (host copy refreshed)."""
    a = make(gpu_lib, "f64")
    a.Iterate(4)
    a.CalcHydroVars(0)
    a.Iterate(4)
    a.CalcHydroVars(0)
    nx, ny, nz = DIMS
    rho_c, u_c = smooth_random(nx, ny, nz, seed=11)
    f = oracle.equilibrium(*oracle.c_to_fab(nx, ny, nz, rho_c, u_c))
    oracle.step(f, 0.75, 1.05, 8, nthreads=2)
    r_ref, u_ref = oracle.hydro(f)
    assert a.GetDensity(3, 5, 7, 0) == pytest.approx(r_ref[7, 5, 3], rel=1e-13)
    assert a.GetVelocity(3, 5, 7, 1, 0) == pytest.approx(u_ref[1, 7, 5, 3], rel=1e-9, abs=1e-15)
    a.close()
