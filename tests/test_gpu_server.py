"""GPU tests of the continuous-batching server: every request gives the same
result alone and in a mix, matches the single-simulation conservative path
and (FP64) the CPU oracle, conserves mass, and waits for HBM budget."""
import numpy as np
import pytest

from golden_util import plane_pulse

pytestmark = pytest.mark.gpu

GB = 1 << 30
A = dict(levels=2, dims=(32, 32, 48), steps=14, tau=0.7, pulse_axis=0, pulse_index=16, amplitude=0.05)
B = dict(levels=1, dims=(48, 32, 32), steps=9, tau=1.1, pulse_axis=1, pulse_index=3, amplitude=0.02)
C = dict(levels=3, dims=(32, 48, 32), steps=11, tau=0.9, pulse_axis=2, pulse_index=20, amplitude=0.08)


def serve(lbx, reqs, precision="f32s", budget=8 * GB, max_active=8, stagger=False):
    s = lbx.Server(budget, max_active=max_active, precision=precision)
    ids = []
    for r in reqs:
        ids.append(s.submit(**r))
        if stagger:
            s.pump(3)  # later requests join while earlier ones run
    s.run_until_done(ids, quantum=4)
    out = []
    for i in ids:
        done, mass, probe = s.poll(i)
        out.append((mass, probe, s.take(i)))
    return out, s


def single(lbx, r, precision="f32s"):
    nx, ny, nz = r["dims"]
    sim = lbx.AmrSim(nx, ny, nz, r["levels"] - 1, [1, 1, 1], r["tau"], r["tau"], precision=precision,
                     amr_mode="conservative")
    sim.SetInitialDensity(plane_pulse(nx, ny, nz, r["pulse_axis"], r["pulse_index"], r["amplitude"]))
    sim.SetInitialVelocity(0.0)
    sim.InitFromScratch(0.0)
    lo, hi = [0, 0, 0], [nx - 1, ny - 1, nz - 1]
    for L in range(r["levels"] - 1):
        n = [hi[d] - lo[d] + 1 for d in range(3)]
        tlo = [lo[d] + n[d] // 4 for d in range(3)]
        thi = [tlo[d] + n[d] // 2 - 1 for d in range(3)]
        sim.SetStaticRefinement(L, tlo, thi)
        lo, hi = [2 * t for t in tlo], [2 * t + 1 for t in thi]
    sim.Iterate(r["steps"])
    sim.CalcHydroVars(0)
    return sim.density_field(0), sim.total_mass()


def test_alone_equals_mix(gpu_lib):
    alone = [serve(gpu_lib, [r])[0][0] for r in (A, B, C)]
    mix, _ = serve(gpu_lib, [A, B, C], stagger=True)
    for (m1, p1, r1), (m2, p2, r2) in zip(alone, mix):
        np.testing.assert_array_equal(r1, r2)
        assert m1 == m2 and p1 == p2


@pytest.mark.parametrize("req", [A, B, C])
def test_server_matches_single_simulation(gpu_lib, req):
    (mass, probe, rho), = serve(gpu_lib, [req])[0]
    rho_ref, mass_ref = single(gpu_lib, req)
    np.testing.assert_allclose(rho, rho_ref, rtol=1e-6)
    assert mass == pytest.approx(mass_ref, rel=1e-9)


def refinements(r):
    """The server's level boxes: each level refines the centred half of its
    parent."""
    lo, hi = [0, 0, 0], [d - 1 for d in r["dims"]]
    out = []
    for _ in range(r["levels"] - 1):
        n = [hi[d] - lo[d] + 1 for d in range(3)]
        tlo = [lo[d] + n[d] // 4 for d in range(3)]
        thi = [tlo[d] + n[d] // 2 - 1 for d in range(3)]
        out.append((tuple(tlo), tuple(thi)))
        lo, hi = [2 * t for t in tlo], [2 * t + 1 for t in thi]
    return out


@pytest.mark.parametrize("req", [A, C], ids=["two_levels", "three_levels"])
def test_server_f64_matches_oracle(gpu_lib, oracle, req):
    r = dict(req, steps=6)
    (mass, probe, rho), = serve(gpu_lib, [r], precision="f64")[0]
    nx, ny, nz = r["dims"]
    o = oracle.AmrOracle(nx, ny, nz, r["levels"] - 1, r["tau"], r["tau"], 1)
    o.init(plane_pulse(nx, ny, nz, r["pulse_axis"], r["pulse_index"], r["amplitude"]),
           np.zeros(3 * nx * ny * nz))
    for L, (lo, hi) in enumerate(refinements(r)):
        o.refine(L, lo, hi)
    o.iterate(6)
    rho_ref, _ = o.hydro(0)
    np.testing.assert_allclose(rho, rho_ref, rtol=1e-12)
    assert mass == pytest.approx(o.mass(), rel=1e-13)


@pytest.mark.parametrize("req", [A, B, C], ids=["two_levels", "one_level", "three_levels"])
def test_server_pull_form_equals_push_form(gpu_lib, req):
    """The server steps its levels in the pull form; the single-simulation
    conservative path steps the same scheme in the push form.  In FP64 the
    two give the same density field and mass, bit for bit."""
    (mass, probe, rho), = serve(gpu_lib, [req], precision="f64")[0]
    rho_ref, mass_ref = single(gpu_lib, req, precision="f64")
    np.testing.assert_array_equal(rho, rho_ref)


def test_mass_conserved_in_mix(gpu_lib):
    out, _ = serve(gpu_lib, [A, B, C], stagger=True)
    for (mass, probe, rho), r in zip(out, (A, B, C)):
        nx, ny, nz = r["dims"]
        m0 = nx * ny * nz * 1.0 + r["amplitude"] * (nx * ny * nz // r["dims"][r["pulse_axis"]])
        assert abs(mass - m0) <= 2e-6 * m0


def test_budget_admission_queues(gpu_lib):
    # one 64^3 two-level FP32 request holds ~69 MB of stores
    s = gpu_lib.Server(int(0.1 * GB), max_active=8)
    big = dict(A, dims=(64, 64, 64), steps=6)
    i1 = s.submit(**big)
    i2 = s.submit(**big)
    active, queued = s.pump(2)
    assert (active, queued) == (1, 1)  # only one fits the budget
    s.run_until_done([i1, i2], quantum=4)
    assert s.poll(i1)[0] and s.poll(i2)[0]
    with pytest.raises(gpu_lib.LbxError):
        s.submit(**dict(A, dims=(256, 256, 256)))  # can never fit


def test_oversized_box_rejected_at_submission(gpu_lib):
    """A request whose box exceeds the batch engine's index limits (2^23 cells
    per box) is refused when submitted, so it never blocks the queue."""
    s = gpu_lib.Server(8 * GB, max_active=8)
    with pytest.raises(gpu_lib.LbxError) as e:
        s.submit(**dict(B, dims=(256, 256, 256)))
    assert e.value.status == 5  # LBX_ERR_UNSUPPORTED
    i = s.submit(**dict(B, dims=(48, 32, 32), steps=2))
    s.run_until_done([i], quantum=4)
    assert s.poll(i)[0]
    s.close()
