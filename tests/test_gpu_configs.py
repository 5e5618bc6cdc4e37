"""GPU parity at the stated configurations' own geometry and step counts.

Configuration 2: coarse 64^3 periodic, the fine level refining [16,47]^3
(64^3 fine cells), tau_c 0.8, rho = 1.05 on the coarse plane x = 32, u = 0,
200 coarse steps; both couplings in FP64 and in the paired-FP32 collision
against the oracle (every f_i of both levels), the FP32 store against the
FP64 oracle, and the conservative coupling's composite mass.  The faithful
cycle is unstable on this geometry (the reference's covered-cell mask feeds
the fine average back into cells that also collide): its populations grow
from 0.47 to 31 in 8 coarse steps and to 1e5 in 12, and every rounding
difference grows with them (GPU against oracle, measured: 1.3e-13 after 5
steps, 9e-11 after 8, O(1) after 12, in FP64 and paired alike).  Its parity
is therefore held after 5 coarse steps, while the run is still bounded.

Configuration 4: the 64-box draw of the batched ensemble (per-axis sizes from
{16, ..., 128}, tau U[0.6, 1.5], plane pulses), 1000 steps in FP64 and FP32:
the eight smallest boxes against the oracle and every box of the FP32 run
against the FP64 run.
"""
import numpy as np
import pytest

import bench

pytestmark = pytest.mark.gpu
RTOL = 1e-12
STEPS2 = {"conservative": 200, "faithful": 5}


def rel(a, b):
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-300)))


@pytest.fixture(scope="module")
def config2_oracle(oracle):
    """Oracle state of configuration 2 after 200 coarse steps, per coupling."""
    n, tau, lo, hi, rho_c, u_c = bench.config2_problem()
    out = {}
    for mode, code in (("faithful", 0), ("conservative", 1)):
        o = oracle.AmrOracle(n, n, n, 1, tau, tau, code)
        o.init(rho_c, u_c)
        o.refine(0, lo, hi)
        m0 = o.mass()
        o.iterate(STEPS2[mode])
        out[mode] = dict(f=[o.f(0), o.f(1)], rho=[o.hydro(0)[0], o.hydro(1)[0]], m0=m0,
                         m1=o.mass())
    return out


def run_config2(lbx, mode, precision):
    n, tau, lo, hi, rho_c, u_c = bench.config2_problem()
    sim = lbx.AmrSim(n, n, n, 1, [1, 1, 1], tau, tau, precision=precision, amr_mode=mode)
    sim.SetInitialDensity(rho_c)
    sim.SetInitialVelocity(0.0)
    sim.InitFromScratch(0.0)
    sim.SetStaticRefinement(0, lo, hi)
    assert sim.GetExtent(1) == ([32, 32, 32], [95, 95, 95])
    m0 = sim.total_mass()
    steps = STEPS2[mode]
    sim.Iterate(steps)
    assert sim.GetTimeStep(0) == steps and sim.GetTimeStep(1) == 2 * steps
    return sim, m0


@pytest.mark.parametrize("precision", ["f64", "f64p"])
@pytest.mark.parametrize("mode", ["conservative", "faithful"])
def test_config2_parity(gpu_lib, config2_oracle, mode, precision):
    """Every f_i of both levels within 1e-12 of the oracle: the conservative
    coupling after 200 coarse steps, the faithful cycle after 5 (see the
    module docstring).  The faithful cycle zeroes populations, so its zero
    entries are held absolutely and the others relatively."""
    sim, m0 = run_config2(gpu_lib, mode, precision)
    ref = config2_oracle[mode]
    for L in (0, 1):
        got, want = sim.copy_f(L), ref["f"][L]
        nz = want != 0
        assert rel(got[nz], want[nz]) <= RTOL, (L, rel(got[nz], want[nz]))
        assert np.all(got[~nz] == 0) or np.max(np.abs(got[~nz])) <= RTOL * np.max(np.abs(want))
    if mode == "conservative":
        assert m0 == pytest.approx(ref["m0"], rel=1e-14)
        assert abs(sim.total_mass() - m0) <= 1e-12 * m0   # measured -1.2e-14 (FP64)
    sim.close()


def test_config2_f32_against_f64_oracle(gpu_lib, config2_oracle):
    """FP32 shifted store, conservative coupling: rho of both levels within
    1e-5 relative of the FP64 oracle after 200 coarse steps; composite mass
    within 1e-6."""
    sim, m0 = run_config2(gpu_lib, "conservative", "f32s")
    ref = config2_oracle["conservative"]
    for L in (0, 1):
        sim.CalcHydroVars(L)
        r = sim.density_field(L)
        assert np.max(np.abs(r - ref["rho"][L]) / ref["rho"][L]) <= 1e-5
    assert abs(sim.total_mass() - ref["m1"]) <= 1e-6 * ref["m1"]
    sim.close()


ENS_STEPS = 1000


@pytest.fixture(scope="module")
def ensemble_runs(gpu_lib):
    dims, taus, inputs = bench.ensemble_draw()
    out = {}
    for prec in ("f64", "f32s"):
        e = gpu_lib.Ensemble(dims, taus, precision=prec)
        for b in range(len(dims)):
            e.init_box(b, *inputs[b])
        e.autotune(trial_steps=4)      # state is saved and restored around the trials
        e.iterate(ENS_STEPS)
        out[prec] = [e.copy_f(b) for b in range(len(dims))]
        e.close()
    return dims, taus, inputs, out


def test_config4_smallest_boxes_against_oracle(ensemble_runs, oracle):
    """The eight smallest boxes of the 64-box draw after 1000 steps: FP64
    every f_i within 1e-12 of the oracle; FP32 rho within 1e-5 relative and
    u within 1e-5 of the box's velocity scale."""
    dims, taus, inputs, out = ensemble_runs
    order = np.argsort([int(np.prod(d)) for d in dims])[:8]
    for b in order:
        nx, ny, nz = dims[b]
        f = oracle.equilibrium(*oracle.c_to_fab(nx, ny, nz, *inputs[b]))
        oracle.step(f, taus[b], taus[b], ENS_STEPS, nthreads=8, style=1)
        got64 = out["f64"][b].reshape(f.shape)
        assert rel(got64, f) <= RTOL, (b, rel(got64, f))
        r_ref, u_ref = oracle.hydro(f)
        r32, u32 = oracle.hydro(np.ascontiguousarray(out["f32s"][b].reshape(f.shape)))
        assert np.max(np.abs(r32 - r_ref) / r_ref) <= 1e-5, b
        assert np.max(np.abs(u32 - u_ref)) <= 1e-5 * max(np.max(np.abs(u_ref)), 1e-30), b


def test_config4_f32_against_f64_every_box(ensemble_runs, oracle):
    """All 64 boxes: the FP32 run's rho within 1e-5 relative of the FP64
    run's after 1000 steps."""
    dims, _, _, out = ensemble_runs
    for b, d in enumerate(dims):
        shape = (15, d[2], d[1], d[0])
        r64, _ = oracle.hydro(np.ascontiguousarray(out["f64"][b].reshape(shape)))
        r32, _ = oracle.hydro(np.ascontiguousarray(out["f32s"][b].reshape(shape)))
        assert np.max(np.abs(r32 - r64) / r64) <= 1e-5, b
