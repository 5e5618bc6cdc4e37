"""Edge cases of the device path, compared with the oracle.

* Tiny and prime extents (including an extent of 1, where both neighbours
  along that axis are the cell itself) after 1, 2 and N steps, in every
  precision; the extents exercise the periodic wrap on every face.
* The regrid lifecycle of the static-refinement API (src/AmrSim.cpp:995-1017
  of the reference): refine, step, unset, step, refine a different box, step
  -- every level against the oracle doing the same.
"""
import numpy as np
import pytest

from golden_util import smooth_random

pytestmark = pytest.mark.gpu

F64_RTOL = 1e-12
F32_RTOL = 1e-5
DIMS = [(4, 4, 4), (5, 7, 3), (1, 3, 2), (11, 13, 7), (2, 1, 5)]


def max_rel(a, b):
    return float(np.max(np.abs(a - b) / np.abs(b)))


@pytest.mark.parametrize("dims", DIMS)
@pytest.mark.parametrize("precision", ["f64", "f64p", "f32s"])
def test_small_and_prime_extents(gpu_lib, oracle, dims, precision):
    nx, ny, nz = dims
    rho_c, u_c = smooth_random(nx, ny, nz, seed=7 * nx + 3 * ny + nz)
    tau_s, tau_b = 0.7, 1.1
    sim = gpu_lib.AmrSim(nx, ny, nz, 0, [1, 1, 1], tau_s, tau_b, precision=precision)
    sim.SetInitialDensity(rho_c)
    sim.SetInitialVelocity(u_c)
    sim.InitFromScratch(0.0)
    rho, u = oracle.c_to_fab(nx, ny, nz, rho_c, u_c)
    f = oracle.equilibrium(rho, u)
    done = 0
    for n in (1, 2, 9):
        sim.Iterate(n - done)
        oracle.step(f, tau_s, tau_b, n - done, nthreads=1)
        done = n
        if precision == "f32s":
            sim.CalcHydroVars(0)
            r_ref, u_ref = oracle.hydro(f)
            assert np.max(np.abs(sim.density_field(0) - r_ref) / r_ref) <= F32_RTOL
            assert np.max(np.abs(sim.velocity_field(0) - u_ref)) <= F32_RTOL * np.max(np.abs(u_ref))
        else:
            assert max_rel(sim.copy_f(0), f) <= F64_RTOL, (dims, n)
    assert sim.GetTimeStep(0) == 9


def _compare_levels(sim, o, mode, finest):
    for lev in range(finest + 1):
        a, b = sim.copy_f(lev), o.f(lev)
        if mode == "faithful":
            # The reference's cycle zeroes cells under its coarse mask; a cell
            # of zero density then gives 0/0 in the collision, in the
            # reference as here.  Non-finite entries must coincide, finite
            # ones agree to round-off of the field's scale.
            fin = np.isfinite(b)
            assert np.array_equal(np.isfinite(a), fin), lev
            if fin.any():
                assert np.max(np.abs(a[fin] - b[fin])) <= F64_RTOL * np.max(np.abs(b[fin])), lev
        else:
            assert max_rel(a, b) <= F64_RTOL, lev


@pytest.mark.parametrize("mode", ["faithful", "conservative"])
def test_regrid_lifecycle(gpu_lib, oracle, mode):
    dims = (16, 12, 10)
    nx, ny, nz = dims
    rho_c, u_c = smooth_random(nx, ny, nz, seed=404)
    tau = 0.8
    sim = gpu_lib.AmrSim(nx, ny, nz, 1, [1, 1, 1], tau, tau, precision="f64", amr_mode=mode)
    sim.SetInitialDensity(rho_c)
    sim.SetInitialVelocity(u_c)
    sim.InitFromScratch(0.0)
    o = oracle.AmrOracle(nx, ny, nz, 1, tau, tau, 0 if mode == "faithful" else 1)
    o.init(rho_c, u_c)

    sim.SetStaticRefinement(0, (4, 3, 2), (9, 8, 6))
    o.refine(0, (4, 3, 2), (9, 8, 6))
    sim.Iterate(3)
    o.iterate(3)
    assert sim.finestLevel() == 1
    _compare_levels(sim, o, mode, 1)

    sim.UnsetStaticRefinement(0)
    o.unrefine(0)
    assert sim.finestLevel() == 0
    _compare_levels(sim, o, mode, 0)
    sim.Iterate(2)
    o.iterate(2)
    _compare_levels(sim, o, mode, 0)

    sim.SetStaticRefinement(0, (6, 2, 3), (12, 7, 8))
    o.refine(0, (6, 2, 3), (12, 7, 8))
    assert sim.GetExtent(1) == ([12, 4, 6], [25, 15, 17])
    _compare_levels(sim, o, mode, 1)
    sim.Iterate(3)
    o.iterate(3)
    _compare_levels(sim, o, mode, 1)
    if mode == "conservative":
        assert sim.total_mass() == pytest.approx(o.mass(), rel=1e-13)


GRAPH_CASES = [("f32s", "conservative", 0), ("f64", "conservative", 0), ("f64p", "conservative", 0),
               ("f64", "conservative", 1), ("f32s", "conservative", 2), ("f64", "faithful", 1),
               ("f64p", "faithful", 1)]


@pytest.mark.parametrize("precision,mode,levels", GRAPH_CASES)
def test_graph_replay_equals_direct_steps(gpu_lib, precision, mode, levels):
    """Iterate(n) with n >= 4 replays captured CUDA graphs of whole macro
    steps; one-step calls launch directly.  Both give the same state bit for
    bit, the same times, step counters and kernel counts."""
    dims = (16, 16, 12)
    rho_c, u_c = smooth_random(*dims, seed=2024)

    def make():
        s = gpu_lib.AmrSim(*dims, max(levels, 0), [1, 1, 1], 0.8, 0.8, precision=precision,
                           amr_mode=mode)
        s.SetInitialDensity(rho_c)
        s.SetInitialVelocity(u_c)
        s.InitFromScratch(0.0)
        if levels >= 1:
            s.SetStaticRefinement(0, (4, 4, 3), (11, 11, 8))
        if levels >= 2:
            s.SetStaticRefinement(1, (10, 10, 8), (17, 17, 13))
        return s

    a, b = make(), make()
    for _ in range(13):
        a.Iterate(1)
    b.Iterate(13)
    b.Iterate(2)   # below the graph threshold after a replayed run
    for _ in range(2):
        a.Iterate(1)
    for lev in range(levels + 1):
        fa, fb = a.copy_f(lev), b.copy_f(lev)
        assert np.array_equal(fa, fb, equal_nan=True), lev
        assert a.GetTime(lev) == b.GetTime(lev) and a.GetTimeStep(lev) == b.GetTimeStep(lev)
    assert a.GetTimeStep(0) == 15
    assert a.launch_count() == b.launch_count()
    if mode == "conservative":
        assert a.total_mass() == b.total_mass()


@pytest.mark.parametrize("mode", ["faithful", "conservative"])
def test_refinement_at_periodic_corner(gpu_lib, oracle, mode):
    """A patch on the domain's low corner: its ghost shell and parent ring
    wrap through the periodic faces of level 0."""
    dims = (12, 10, 8)
    nx, ny, nz = dims
    rho_c, u_c = smooth_random(nx, ny, nz, seed=99)
    tau = 0.9
    sim = gpu_lib.AmrSim(nx, ny, nz, 1, [1, 1, 1], tau, tau, precision="f64", amr_mode=mode)
    sim.SetInitialDensity(rho_c)
    sim.SetInitialVelocity(u_c)
    sim.InitFromScratch(0.0)
    o = oracle.AmrOracle(nx, ny, nz, 1, tau, tau, 0 if mode == "faithful" else 1)
    o.init(rho_c, u_c)
    sim.SetStaticRefinement(0, (0, 0, 0), (5, 4, 3))
    o.refine(0, (0, 0, 0), (5, 4, 3))
    for n in (1, 4):
        sim.Iterate(n)
        o.iterate(n)
        _compare_levels(sim, o, mode, 1)
    if mode == "conservative":
        assert sim.total_mass() == pytest.approx(o.mass(), rel=1e-13)
