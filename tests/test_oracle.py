"""CPU tests of the oracle: pinned against the reference's known answers,
then checked for the invariants the reference relies on."""
import hashlib
import json
import os

import numpy as np
import pytest

from conftest import reference_file
from golden_util import (catch2_approx, config1_problem, parse_mode_tables, parse_pulse_header,
                         pulse_problem, smooth_random)

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURE = json.load(open(os.path.join(HERE, "golden", "pulse_oracle.json")))


def _digest(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<f8").tobytes()).hexdigest()


def test_mode_tables_are_inverse(oracle):
    M, Mi = oracle.mode_tables()
    assert np.allclose(Mi @ M, np.eye(15), atol=1e-15)
    # rows of M: 1, c, c_a c_b - delta/3 ... first row is all ones
    assert np.array_equal(M[0], np.ones(15))


def test_mode_tables_match_reference(oracle):
    M_ref, Mi_ref = parse_mode_tables(reference_file("src/AmrSim.cpp"))
    M, Mi = oracle.mode_tables()
    assert np.array_equal(M, M_ref)       # bit-identical doubles
    assert np.array_equal(Mi, Mi_ref)


def test_pulse_regression_catch2(oracle):
    """catch2RegressionTests.cpp:6-93 with the reference's own Approx rule."""
    golden = parse_pulse_header(reference_file("tests/pulseRegression.h"))
    nx, ny, nz, tau, rho_c, u_c = pulse_problem()
    rho, u = oracle.c_to_fab(nx, ny, nz, rho_c, u_c)
    f = oracle.equilibrium(rho, u)
    done = 0
    for tag, t in (("t0", 0), ("t100", 100), ("t200", 200)):
        oracle.step(f, tau, tau, t - done, nthreads=2)
        done = t
        r, v = oracle.hydro(f) if t else (rho, u)
        assert catch2_approx(r.reshape(-1), golden["RHO_" + tag]).all()
        assert catch2_approx(np.moveaxis(v, 0, -1).reshape(-1), golden["VEL_" + tag]).all()


def test_pulse_fixture_digests(oracle):
    """The committed digests pin the oracle where the reference is absent."""
    nx, ny, nz, tau, rho_c, u_c = pulse_problem()
    rho, u = oracle.c_to_fab(nx, ny, nz, rho_c, u_c)
    f = oracle.equilibrium(rho, u)
    done = 0
    for tag, cp in sorted(FIXTURE["checkpoints"].items(), key=lambda kv: kv[1]["step"]):
        oracle.step(f, tau, tau, cp["step"] - done, nthreads=2)
        done = cp["step"]
        assert _digest(f) == cp["sha256_f"], tag
        assert cp["catch2_checks_passed"] == 20000


def test_config1_fixture_digest(oracle):
    nx, ny, nz, tau, steps, rho_c, u_c = config1_problem()
    rho, u = oracle.c_to_fab(nx, ny, nz, rho_c, u_c)
    f = oracle.equilibrium(rho, u)
    oracle.step(f, tau, tau, steps, nthreads=4)
    assert _digest(f) == FIXTURE["config1"]["sha256_f"]


@pytest.mark.parametrize("dims", [(5, 7, 3), (4, 4, 4), (11, 2, 3)])
def test_reference_style_equals_fast_style(oracle, dims):
    nx, ny, nz = dims
    rho_c, u_c = smooth_random(nx, ny, nz, seed=3)
    rho, u = oracle.c_to_fab(nx, ny, nz, rho_c, u_c)
    f0 = oracle.equilibrium(rho, u)
    a, b = f0.copy(), f0.copy()
    oracle.step(a, 0.7, 0.9, 5, style=0)
    oracle.step(b, 0.7, 0.9, 5, nthreads=3, style=1)
    assert np.array_equal(a, b)


def test_c_order_initialisation(oracle):
    """catch2InitTests.cpp:50-109: C-order element-wise initial values."""
    nx, ny, nz = 16, 9, 8
    n = nx * ny * nz
    rho, u = oracle.c_to_fab(nx, ny, nz, np.arange(n, dtype=float), np.arange(3 * n, dtype=float))
    val = 0.0
    for i in range(nx):
        for j in range(ny):
            for k in range(nz):
                assert rho[k, j, i] == val
                val += 1
    assert u[2, 3, 4, 5] == ((5 * ny + 4) * nz + 3) * 3 + 2


def test_short_initial_vector_is_an_error(oracle):
    with pytest.raises(IndexError):
        oracle.c_to_fab(4, 4, 4, np.ones(10), np.zeros(192))


def test_equilibrium_moments(oracle):
    nx, ny, nz = 6, 5, 4
    rho_c, u_c = smooth_random(nx, ny, nz, seed=5, amp_u=0.05)
    rho, u = oracle.c_to_fab(nx, ny, nz, rho_c, u_c)
    f = oracle.equilibrium(rho, u)
    r2, u2 = oracle.hydro(f)
    assert np.allclose(r2, rho, rtol=1e-14)
    assert np.allclose(u2, u, rtol=1e-12, atol=1e-15)


def test_collision_conserves_mass_and_momentum(oracle):
    rng = np.random.default_rng(0)
    M, _ = oracle.mode_tables()
    for _ in range(50):
        f = 0.05 + 0.05 * rng.random(15)
        g = oracle.collide_cell(f, 1.3, 0.8)
        assert np.allclose(M[:4] @ g, M[:4] @ f, rtol=1e-14, atol=1e-16)
        # ghost modes are relaxed to zero
        assert np.allclose(M[10:] @ g, 0.0, atol=1e-15)


def test_periodic_step_conserves_mass(oracle):
    nx, ny, nz = 9, 6, 7
    rho_c, u_c = smooth_random(nx, ny, nz, seed=11)
    rho, u = oracle.c_to_fab(nx, ny, nz, rho_c, u_c)
    f = oracle.equilibrium(rho, u)
    m0 = oracle.mass_momentum(f)
    oracle.step(f, 0.6, 0.6, 30, nthreads=2)
    m1 = oracle.mass_momentum(f)
    assert abs(m1[0] - m0[0]) < 1e-12 * m0[0]
    assert np.allclose(m1[1:], m0[1:], atol=1e-12)


# ---- multi-level oracle ----------------------------------------------------

def _amr(oracle, dims, tau, mode, max_level=1):
    nx, ny, nz = dims
    o = oracle.AmrOracle(nx, ny, nz, max_level, tau, tau, mode)
    rho_c, u_c = smooth_random(nx, ny, nz, seed=2)
    o.init(rho_c, u_c)
    return o


def test_amr_level_timing_and_tau(oracle):
    """catch2AMRTests.cpp:341-354: dt_l = 2^-l, tau_l = r(tau_{l-1} - 1/2) + 1/2."""
    o = _amr(oracle, (16, 12, 8), 0.8, mode=0)
    o.refine(0, (4, 3, 2), (11, 8, 5))
    t1 = o.time(1)
    assert t1["dt"] == 0.5
    assert t1["tau_s"] == pytest.approx(2 * (0.8 - 0.5) + 0.5)
    assert o.extent(1) == ((8, 6, 4), (23, 17, 11))
    o.iterate(3)
    assert o.time(0)["step"] == 3 and o.time(1)["step"] == 6
    assert o.time(1)["time"] == pytest.approx(3.0)


def test_amr_new_level_is_piecewise_constant(oracle):
    """MakeNewLevelFromCoarse: fine cells copy their parent (PCInterp)."""
    o = _amr(oracle, (8, 8, 8), 0.7, mode=0)
    o.refine(0, (2, 2, 2), (5, 5, 5))
    fc, ff = o.f(0), o.f(1)
    for q in (0, 3, 9):
        np.testing.assert_array_equal(ff[q][::2, ::2, ::2], fc[q][2:6, 2:6, 2:6])
        np.testing.assert_array_equal(ff[q][1::2, 1::2, 1::2], fc[q][2:6, 2:6, 2:6])


def test_amr_conservative_mass_is_conserved(oracle):
    o = _amr(oracle, (16, 16, 16), 0.8, mode=1)
    o.refine(0, (4, 5, 6), (11, 10, 12))
    m0 = o.mass()
    o.iterate(12)
    m1 = o.mass()
    assert abs(m1 - m0) < 1e-12 * m0


def test_amr_three_levels_conservative(oracle):
    o = _amr(oracle, (16, 16, 16), 0.8, mode=1, max_level=2)
    o.refine(0, (4, 4, 4), (11, 11, 11))
    o.refine(1, (12, 12, 12), (19, 19, 19))
    assert o.finest() == 2
    m0 = o.mass()
    o.iterate(4)
    assert abs(o.mass() - m0) < 1e-12 * m0
    assert o.time(2)["step"] == 16


def test_amr_three_levels_faithful_recursion(oracle):
    """RohdeCycle recurses into the next level twice per coarse step when the
    fine level is not the finest (src/AmrSim.cpp:444-455); per-level dt and
    tau follow ComputeDt (src/AmrSim.cpp:297-322) on every level."""
    o = _amr(oracle, (16, 16, 16), 0.8, mode=0, max_level=2)
    o.refine(0, (4, 4, 4), (11, 11, 11))
    o.refine(1, (12, 12, 12), (19, 19, 19))
    assert o.finest() == 2
    assert o.extent(2) == ((24, 24, 24), (39, 39, 39))
    tau = 0.8
    for L in range(3):
        t = o.time(L)
        assert t["dt"] == 0.5 ** L
        assert t["tau_s"] == pytest.approx(tau) and t["tau_b"] == pytest.approx(tau)
        tau = 2 * (tau - 0.5) + 0.5
    o.iterate(3)
    for L in range(3):
        assert o.time(L)["step"] == 3 * 2 ** L
        assert o.time(L)["time"] == pytest.approx(3.0)
        assert np.isfinite(o.f(L)).all()


def test_amr_faithful_whole_domain_patch_runs(oracle):
    """ml_pulse set-up (catch2RegressionTests.cpp:95-152): the fine level is
    the whole periodic domain and starts as a copy of the coarse one."""
    nx, ny, nz, tau, rho_c, u_c = pulse_problem()
    o = oracle.AmrOracle(nx, ny, nz, 1, tau, tau, 0)
    o.init(rho_c, u_c)
    o.refine(0, (0, 0, 0), (nx - 1, ny - 1, nz - 1))
    r0, _ = o.hydro(0)
    r1, _ = o.hydro(1)
    np.testing.assert_allclose(r1[::2, ::2, ::2], r0, rtol=1e-14)
    o.iterate(2)
    assert np.isfinite(o.f(0)).all() and np.isfinite(o.f(1)).all()


@pytest.mark.parametrize("mode", [0, 1])
def test_ml_pulse_level_creation_catch2(oracle, mode):
    """ml_pulse (catch2RegressionTests.cpp:95-152) at t = 0: after the whole
    domain is refined, both levels (the fine one sampled at every second
    cell, as the reference test does) pass the reference's Approx rule
    against the single-level golden density and velocity.  The test's later
    checks (t = 100, 200) compare a refined run with single-level golden
    values; the faithful restatement does not meet them (its coarse level
    gains mass through the covered-cell mask) and the conservative scheme
    resolves the pulse at twice the resolution, so only level creation is
    pinned here."""
    golden = parse_pulse_header(reference_file("tests/pulseRegression.h"))
    nx, ny, nz, tau, rho_c, u_c = pulse_problem()
    o = oracle.AmrOracle(nx, ny, nz, 1, tau, tau, mode)
    o.init(rho_c, u_c)
    o.refine(0, (0, 0, 0), (nx - 1, ny - 1, nz - 1))
    for lev in (0, 1):
        r, u = o.hydro(lev)
        s = (slice(None, None, 2),) * 3 if lev else (slice(None),) * 3
        assert catch2_approx(r[s].reshape(-1), golden["RHO_t0"]).all()
        assert catch2_approx(np.moveaxis(u[(slice(None),) + s], 0, -1).reshape(-1),
                             golden["VEL_t0"]).all()


def _ml_pulse_errors(oracle, readings):
    """ml_pulse (catch2RegressionTests.cpp:95-196) under one reading of the
    AMReX behaviour: the largest relative density error of the coarse level
    at t = 100 and t = 200 and of the fine level (every second cell) at
    t = 200 against the single-level golden data, and the fine density."""
    golden = parse_pulse_header(reference_file("tests/pulseRegression.h"))
    nx, ny, nz, tau, rho_c, u_c = pulse_problem()
    o = oracle.AmrOracle(nx, ny, nz, 1, tau, tau, 0, readings=readings)
    o.init(rho_c, u_c)
    o.refine(0, (0, 0, 0), (nx - 1, ny - 1, nz - 1))
    rel = lambda a, key: float(np.max(np.abs(a.reshape(-1) - golden[key]) / golden[key]))
    o.iterate(100)
    c100 = rel(o.hydro(0)[0], "RHO_t100")
    o.iterate(100)
    c200 = rel(o.hydro(0)[0], "RHO_t200")
    r1 = o.hydro(1)[0]
    f200 = rel(r1[::2, ::2, ::2], "RHO_t200")
    return c100, c200, f200, r1


def test_ml_pulse_readings_table(oracle):
    """The readings of AMReX's behaviour behind the faithful cycle against the
    later checks of ml_pulse.  The refined level covers the whole periodic
    domain, so it fills its ghost cells from itself and does not depend on
    any reading: it lands 8.7e-5 from the golden t = 200 density under every
    reading, and an exact periodic run on the fine grid lands 8.9e-5 from it,
    both beyond the test's 100*FLT_EPSILON.  No reading can pass those checks.
    The coarse level does depend on them: the default readings (the mask the
    reference's code builds, AMReX's average over the coarsened fine box
    grown by one, zero fresh memory) gain mass without bound; the intended
    mask with the ghost ring left out of the restriction is the best reading
    and stays bounded, 0.43 from the golden values (its domain-face cells
    also receive the periodic ghost copies the coarse fill made before the
    masked collide).  The figures are the measured ones, held here."""
    best = oracle.READ_MASK_FINE | oracle.READ_GROW0
    c100, c200, f200, fine_default = _ml_pulse_errors(oracle, 0)
    assert c100 > 1e10 and c200 > 1e60                     # measured 4.6e10, 1.9e71
    assert 8.68e-5 < f200 < 8.69e-5                        # measured 8.685e-5
    b100, b200, bf200, fine_best = _ml_pulse_errors(oracle, best)
    assert 0.430 < b100 < 0.431 and 0.430 < b200 < 0.431  # measured 0.4305, 0.4306
    assert bf200 == f200
    assert np.array_equal(fine_best, fine_default)         # the fine level ignores the readings
    # the best any coupling can do for the fine level: an exact periodic run
    # of the piecewise-constant refinement on the fine grid
    golden = parse_pulse_header(reference_file("tests/pulseRegression.h"))
    nx, ny, nz, tau, rho_c, u_c = pulse_problem()
    f = oracle.equilibrium(*oracle.c_to_fab(nx, ny, nz, rho_c, u_c))
    ff = np.ascontiguousarray(np.repeat(np.repeat(np.repeat(f, 2, 1), 2, 2), 2, 3))
    oracle.step(ff, tau, tau, 400, nthreads=4, style=1)
    r = oracle.hydro(ff)[0][::2, ::2, ::2].reshape(-1)
    exact = float(np.max(np.abs(r - golden["RHO_t200"]) / golden["RHO_t200"]))
    assert 8.88e-5 < exact < 8.89e-5                       # measured 8.887e-5
    assert not catch2_approx(r, golden["RHO_t200"]).all()


@pytest.mark.parametrize("readings", [1, 2, 8])
def test_ml_pulse_other_readings_diverge(oracle, readings):
    """The x8 sum, the ungrown restriction and stale fresh memory, each with
    the reference's own mask, all leave the coarse level unbounded."""
    c100, _, _, _ = _ml_pulse_errors(oracle, readings)
    assert c100 > 1e7                                      # measured 4.5e10, 3.8e8, 5.1e12


def test_rescaled_coupling_keeps_rest_state(oracle):
    """Mode 2 (non-equilibrium rescaling, ghost data interpolated in time):
    a uniform rest state is a fixed point of the collision at every rate, so
    the explosion, the fine steps and the restriction leave both levels at
    it (to round-off)."""
    o = oracle.AmrOracle(16, 16, 16, 1, 0.7, 0.9, 2)
    o.init(np.full(16 ** 3, 1.02), np.zeros(3 * 16 ** 3))
    o.refine(0, (4, 4, 4), (11, 11, 11))
    g0 = o.f(0)[:, 0, 0, 0]
    o.iterate(5)
    for L in (0, 1):
        f = o.f(L).reshape(15, -1)
        assert np.max(np.abs(f - g0[:, None]) / g0[:, None]) < 1e-14
    assert o.time(1)["tau_s"] == pytest.approx(1.4) and o.time(1)["step"] == 10


def test_rescaled_coupling_accuracy_against_uniform_fine(oracle):
    """The two-level pulse on a 32^3 coarse level refined over [8,23]^3
    (tau 0.8, rho 1.05 on the plane x = 16) after 40 coarse steps, against a
    uniformly fine 64^3 run of the same populations (tau 1.6, 80 steps):
    largest fine-level density error in units of the uniform run's pulse
    amplitude.  Rescaled: 2.2 % (measured), mass drift 6.6e-6; conservative:
    11.6x the amplitude at the patch boundary, mass exact."""
    import bench
    n, tau, lo, hi, rho_c, u_c = bench.config2_problem(32)
    f = oracle.equilibrium(*oracle.c_to_fab(n, n, n, rho_c, u_c))
    ff = np.ascontiguousarray(np.repeat(np.repeat(np.repeat(f, 2, 1), 2, 2), 2, 3))
    oracle.step(ff, 2 * tau, 2 * tau, 80, nthreads=4, style=1)
    ru = oracle.hydro(ff)[0]
    amp = np.max(np.abs(ru - 1))
    fl, fh = 2 * lo[0], 2 * hi[0] + 1
    err, drift = {}, {}
    for mode in (1, 2):
        o = oracle.AmrOracle(n, n, n, 1, tau, tau, mode)
        o.init(rho_c, u_c)
        o.refine(0, lo, hi)
        m0 = o.mass()
        o.iterate(40)
        err[mode] = np.max(np.abs(o.hydro(1)[0] - ru[fl:fh + 1, fl:fh + 1, fl:fh + 1])) / amp
        drift[mode] = (o.mass() - m0) / m0
    assert err[2] <= 0.025 and abs(drift[2]) <= 1e-5       # measured 0.0223, 6.6e-6
    assert err[1] >= 10 * err[2] and abs(drift[1]) <= 1e-13  # measured 11.6, -3.8e-15


# ---- reads of unwritten memory (fresh ghost-cell storage poisoned with NaN)

def _poisoned(oracle, on, run):
    oracle.set_poison(on)
    try:
        return run()
    finally:
        oracle.set_poison(False)


def test_single_level_reads_only_written_memory(oracle):
    """The reference-style step (ghost-cell FABs, periodic fill, stream into
    a fresh buffer) gives the same bits when fresh storage is NaN."""
    nx, ny, nz = 12, 10, 8
    rho, u = oracle.c_to_fab(nx, ny, nz, *smooth_random(nx, ny, nz, seed=3))

    def run():
        f = oracle.equilibrium(rho, u)
        oracle.step(f, 0.8, 0.9, 5, nthreads=1, style=0)
        return f

    clean, poisoned = _poisoned(oracle, False, run), _poisoned(oracle, True, run)
    assert np.isfinite(poisoned).all() and np.array_equal(clean, poisoned)


def _two_level(oracle, mode):
    o = oracle.AmrOracle(16, 12, 10, 1, 0.8, 0.8, mode)
    o.init(*smooth_random(16, 12, 10, seed=4))
    o.refine(0, (4, 4, 2), (11, 7, 7))
    o.iterate(3)
    return o.f(0), o.f(1)


def test_conservative_amr_reads_only_written_memory(oracle):
    """Explosion, patch sub-steps, coalescence and restriction read nothing
    they did not write: the same bits with NaN-filled fresh storage."""
    clean = _poisoned(oracle, False, lambda: _two_level(oracle, 1))
    poisoned = _poisoned(oracle, True, lambda: _two_level(oracle, 1))
    for a, b in zip(clean, poisoned):
        assert np.isfinite(b).all() and np.array_equal(a, b)


def test_faithful_amr_reads_fresh_memory(oracle):
    """The reference's Rohde cycle streams the fine level into a freshly
    allocated buffer and reads its outer ghost ring (uninitialised in the
    reference, zero in this restatement): with NaN-filled fresh storage the
    NaN reaches the levels' valid cells.  This is the reference's quirk,
    kept in faithful mode; the conservative scheme has no such read."""
    f0, f1 = _poisoned(oracle, True, lambda: _two_level(oracle, 0))
    assert not (np.isfinite(f0).all() and np.isfinite(f1).all())
