"""GPU tests of the static two-level path through the C ABI.

Faithful mode (the reference's Rohde cycle, src/AmrSim.cpp:430-631), the
conservative volumetric mode and the rescaled mode (non-equilibrium
rescaling, ghost data interpolated in time) are each compared with their CPU
restatement: every f_i of every level within 1e-12 relative.  The
conservative mode also conserves the composite mass to round-off.
"""
import numpy as np
import pytest

from golden_util import plane_pulse, pulse_problem, smooth_random

pytestmark = pytest.mark.gpu
RTOL = 1e-12
MODES = {"faithful": 0, "conservative": 1, "rescaled": 2}  # oracle mode codes


def pair(lbx, O, dims, tau, mode, lo, hi, rho_c, u_c, max_level=1, precision="f64"):
    nx, ny, nz = dims
    sim = lbx.AmrSim(nx, ny, nz, max_level, [1, 1, 1], tau, tau, precision=precision,
                     amr_mode=mode)
    sim.SetInitialDensity(rho_c)
    sim.SetInitialVelocity(u_c)
    sim.InitFromScratch(0.0)
    o = O.AmrOracle(nx, ny, nz, max_level, tau, tau, MODES[mode])
    o.init(rho_c, u_c)
    if lo is not None:
        sim.SetStaticRefinement(0, lo, hi)
        o.refine(0, lo, hi)
    return sim, o


def rel(a, b):
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-300)))


@pytest.mark.parametrize("precision", ["f64", "f64p"])
@pytest.mark.parametrize("mode", ["faithful", "conservative", "rescaled"])
def test_two_level_parity(gpu_lib, oracle, mode, precision):
    """f64p: the FP64 store with every collision (base level, patch,
    explosion, faithful masked collide) in paired FP32 arithmetic."""
    dims = (16, 12, 10)
    rho_c, u_c = smooth_random(*dims, seed=31)
    sim, o = pair(gpu_lib, oracle, dims, 0.8, mode, (4, 3, 2), (11, 8, 7), rho_c, u_c,
                  precision=precision)
    assert sim.finestLevel() == 1
    assert sim.GetExtent(1) == ([8, 6, 4], [23, 17, 15])
    for n in (1, 5):
        sim.Iterate(n)
        o.iterate(n)
        f0, g0 = sim.copy_f(0), o.f(0)
        f1, g1 = sim.copy_f(1), o.f(1)
        if mode == "faithful":
            # the faithful scheme zeroes populations: compare absolutely on
            # zero entries, relatively elsewhere
            assert np.max(np.abs(f0 - g0)) <= RTOL * np.max(np.abs(g0))
            assert np.max(np.abs(f1 - g1)) <= RTOL * np.max(np.abs(g1))
        else:
            assert rel(f0, g0) <= RTOL
            assert rel(f1, g1) <= RTOL
    assert sim.GetTimeStep(0) == 6 and sim.GetTimeStep(1) == 12
    assert sim.GetTime(1) == pytest.approx(6.0)


def test_conservative_mass_conserved(gpu_lib, oracle):
    dims = (24, 24, 24)
    rho_c = plane_pulse(*dims, axis=0, index=12, amplitude=0.05)
    u_c = np.zeros(3 * 24 ** 3)
    sim, o = pair(gpu_lib, oracle, dims, 0.8, "conservative", (6, 6, 6), (17, 17, 17), rho_c, u_c)
    m0 = sim.total_mass()
    assert m0 == pytest.approx(o.mass(), rel=1e-14)
    sim.Iterate(20)
    m1 = sim.total_mass()
    assert abs(m1 - m0) <= 1e-12 * m0


def test_level_timing_and_tau(gpu_lib, oracle):
    """catch2AMRTests.cpp:306-354 and :385-422 (static refinement extents)."""
    NX, NY, NZ, TAU = 48, 24, 12, 0.01
    sim = gpu_lib.AmrSim(NX, NY, NZ, 1, [1, 1, 1], TAU, TAU)
    sim.SetInitialDensity(0.8)
    sim.SetInitialVelocity(0.1)
    sim.InitFromScratch(0.0)
    assert sim.maxLevel() == 1 and sim.refRatio(0) == [2, 2, 2]
    lo, hi = [NX // 4, NY // 4, NZ // 4], [3 * NX // 4, 3 * NY // 4, 3 * NZ // 4]
    sim.SetStaticRefinement(0, lo, hi)
    assert sim.GetDt(1) == 0.5
    ts, tb = sim.GetTau(1)
    assert ts == pytest.approx(2 * (TAU - 0.5) + 0.5)
    flo, fhi = sim.GetExtent(1)
    assert all(flo[d] <= 2 * lo[d] for d in range(3)) and all(fhi[d] >= 2 * hi[d] for d in range(3))
    # MakeNewLevelFromCoarse: fine density and velocity equal the coarse values
    assert np.allclose(sim.density_field(1), 0.8, rtol=1e-14)
    assert np.allclose(sim.velocity_field(1), 0.1, rtol=1e-13)
    sim.UnsetStaticRefinement(0)
    assert sim.finestLevel() == 0
    assert sim.GetDensity(2 * lo[0], 2 * lo[1], 2 * lo[2], 1) == -1.0


def test_ml_pulse_faithful_parity(gpu_lib, oracle):
    """ml_pulse set-up (catch2RegressionTests.cpp:95-196): whole-domain patch."""
    nx, ny, nz, tau, rho_c, u_c = pulse_problem()
    sim, o = pair(gpu_lib, oracle, (nx, ny, nz), tau, "faithful", (0, 0, 0),
                  (nx - 1, ny - 1, nz - 1), rho_c, u_c)
    sim.Iterate(10)
    o.iterate(10)
    for L in (0, 1):
        a, b = sim.copy_f(L), o.f(L)
        assert np.max(np.abs(a - b)) <= RTOL * np.max(np.abs(b))
        sim.CalcHydroVars(L)


@pytest.mark.parametrize("precision", ["f64", "f64p"])
@pytest.mark.parametrize("mode", ["conservative", "rescaled"])
def test_three_levels_parity(gpu_lib, oracle, mode, precision):
    dims = (16, 16, 16)
    rho_c, u_c = smooth_random(*dims, seed=5)
    sim, o = pair(gpu_lib, oracle, dims, 0.9, mode, (4, 4, 4), (11, 11, 11), rho_c,
                  u_c, max_level=2, precision=precision)
    sim.SetStaticRefinement(1, (12, 12, 12), (19, 19, 19))
    o.refine(1, (12, 12, 12), (19, 19, 19))
    m0 = sim.total_mass()
    sim.Iterate(3)
    o.iterate(3)
    for L in (0, 1, 2):
        assert rel(sim.copy_f(L), o.f(L)) <= RTOL
    assert sim.total_mass() == pytest.approx(o.mass(), rel=1e-13)
    if mode == "conservative":
        assert abs(sim.total_mass() - m0) <= 1e-12 * m0


@pytest.mark.parametrize("precision", ["f64", "f64p"])
def test_three_levels_faithful_parity(gpu_lib, oracle, precision):
    """The faithful cycle's recursion over three levels (src/AmrSim.cpp:454):
    every level against the oracle after 3 coarse steps, on the geometry of
    the host check of the same cycle (the cycle is unstable on long runs)."""
    dims = (16, 16, 16)
    rho_c, u_c = smooth_random(*dims, seed=2)
    sim, o = pair(gpu_lib, oracle, dims, 0.8, "faithful", (4, 4, 4), (11, 11, 11), rho_c,
                  u_c, max_level=2, precision=precision)
    sim.SetStaticRefinement(1, (12, 12, 12), (19, 19, 19))
    o.refine(1, (12, 12, 12), (19, 19, 19))
    assert sim.finestLevel() == 2
    sim.Iterate(3)
    o.iterate(3)
    for L in (0, 1, 2):
        a, b = sim.copy_f(L), o.f(L)
        assert np.max(np.abs(a - b)) <= RTOL * np.max(np.abs(b)), L
    assert sim.GetTimeStep(2) == 12


@pytest.mark.parametrize("mode", ["conservative", "rescaled"])
def test_f32_two_level(gpu_lib, oracle, mode):
    """FP32 shifted store on the two-level couplings: rho within 1e-5
    relative and mass within 1e-6 of the FP64 oracle."""
    dims = (24, 20, 16)
    rho_c = plane_pulse(*dims, axis=0, index=12, amplitude=0.05)
    u_c = np.zeros(3 * np.prod(dims))
    sim, o = pair(gpu_lib, oracle, dims, 0.8, mode, (6, 5, 4), (17, 14, 11), rho_c,
                  u_c, precision="f32s")
    sim.Iterate(20)
    o.iterate(20)
    for L in (0, 1):
        sim.CalcHydroVars(L)
        r_ref, _ = o.hydro(L)
        assert np.max(np.abs(sim.density_field(L) - r_ref) / r_ref) <= 1e-5
    assert sim.total_mass() == pytest.approx(o.mass(), rel=1e-6)
