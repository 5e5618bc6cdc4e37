"""GPU tests of tagging and regridding through the C ABI.

ErrorEst follows the reference's rule (src/AmrSim.cpp:633-663 with TagCell
:413-417): every cell CLEAR without a static tag box (the reference's own
check, tests/catch2AMRTests.cpp:24-52 and :209-230), SET exactly inside it
with one.  The density criterion (the bounding box of the cells whose
density leaves the level's mean by more than a threshold) is checked
against numpy on the density field, and a run that refines to the tagged
box, steps, tags again and regrids (RemakeLevel) is checked against the
oracle given the same boxes: every f_i within 1e-12."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
RTOL = 1e-12


def bump(nx, ny, nz, centre, sigma, amplitude):
    """C-order density 1 + amplitude exp(-|x - centre|^2 / sigma^2)."""
    i, j, k = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    r2 = (i - centre[0]) ** 2 + (j - centre[1]) ** 2 + (k - centre[2]) ** 2
    return (1.0 + amplitude * np.exp(-r2 / sigma ** 2)).reshape(-1)


def numpy_tags(rho_fab, threshold):
    """(lo, hi, count) of |rho - mean| > threshold on a (z, y, x) field."""
    d = np.abs(rho_fab - rho_fab.mean())
    z, y, x = np.nonzero(d > threshold)
    if x.size == 0:
        return None, None, 0
    return [x.min(), y.min(), z.min()], [x.max(), y.max(), z.max()], x.size


def clear_threshold(rho_fab, target):
    """A threshold near target that no cell's |rho - mean| lies close to, so
    that the library's mean (from its mass reduction) and numpy's agree on
    every tag."""
    d = np.sort(np.abs(rho_fab - rho_fab.mean()).ravel())
    i = np.searchsorted(d, target)
    i = min(max(i, 1), d.size - 1)
    while i < d.size - 1 and d[i] - d[i - 1] < 1e-9:
        i += 1
    return 0.5 * (d[i - 1] + d[i])


def test_error_est_follows_the_static_tags(gpu_lib):
    nx, ny, nz = 24, 20, 16
    sim = gpu_lib.AmrSim(nx, ny, nz, 2, [1, 1, 1], 0.8, 0.8, precision="f64",
                         amr_mode="conservative")
    sim.SetInitialDensity(0.5)
    sim.SetInitialVelocity(0.2)
    sim.InitFromScratch(0.0)
    assert not sim.ErrorEst(0).any()  # catch2AMRTests.cpp:24-52
    lo, hi = (5, 4, 3), (14, 11, 9)
    sim.SetStaticRefinement(0, lo, hi)
    tags = sim.ErrorEst(0).reshape(nz, ny, nx)
    want = np.zeros((nz, ny, nx), dtype=np.uint8)
    want[lo[2]:hi[2] + 1, lo[1]:hi[1] + 1, lo[0]:hi[0] + 1] = 1
    np.testing.assert_array_equal(tags, want)
    assert not sim.ErrorEst(1).any()  # the finest level has no tag box
    lo1, hi1 = (12, 10, 8), (21, 17, 13)
    sim.SetStaticRefinement(1, lo1, hi1)
    flo, fhi = sim.GetExtent(1)
    t1 = sim.ErrorEst(1).reshape(fhi[2] - flo[2] + 1, fhi[1] - flo[1] + 1, fhi[0] - flo[0] + 1)
    assert t1.sum() == np.prod([hi1[d] - lo1[d] + 1 for d in range(3)])
    assert t1[lo1[2] - flo[2], lo1[1] - flo[1], lo1[0] - flo[0]] == 1
    sim.UnsetStaticRefinement(1)
    assert not sim.ErrorEst(1).any()
    sim.UnsetStaticRefinement(0)
    assert not sim.ErrorEst(0).any()  # catch2AMRTests.cpp:209-230


@pytest.mark.parametrize("precision", ["f64", "f32s"])
def test_tag_density_matches_numpy(gpu_lib, precision):
    nx, ny, nz = 40, 32, 24
    rho_c = bump(nx, ny, nz, (18, 14, 11), 4.0, 0.05)
    sim = gpu_lib.AmrSim(nx, ny, nz, 0, [1, 1, 1], 0.7, 0.7, precision=precision)
    sim.SetInitialDensity(rho_c)
    sim.SetInitialVelocity(0.0)
    sim.InitFromScratch(0.0)
    for steps in (0, 7):
        sim.Iterate(steps)
        sim.CalcHydroVars(0)
        rho = sim.density_field(0).copy()
        thr = clear_threshold(rho, 0.004)
        lo, hi, n = sim.TagDensity(0, thr)
        rlo, rhi, rn = numpy_tags(rho, thr)
        assert (lo, hi, n) == (rlo, rhi, rn), (steps, thr)
        assert n > 0
    assert sim.TagDensity(0, 1.0) == (None, None, 0)


# FP64 to the parity bar; the FP32 store against the FP64 oracle: its AMR
# bound in every f_i (the shifted store keeps ~1e-7 of f per rounding)
REGRID_BOUND = {"f64": RTOL, "f32s": 1e-6}


@pytest.mark.parametrize("precision", ["f64", "f32s"])
def test_regrid_to_tagged_boxes_matches_oracle(gpu_lib, oracle, precision):
    """Tag, refine, step, tag again and regrid to the grown box (RemakeLevel:
    the new box takes the old fine data where it exists, its parents'
    elsewhere), step: the conservative coupling against the FP64 oracle
    given the same boxes."""
    nx, ny, nz, tau = 32, 32, 32, 0.8
    rho_c = bump(nx, ny, nz, (15, 16, 17), 3.0, 0.04)
    u_c = np.zeros(3 * nx * ny * nz)
    sim = gpu_lib.AmrSim(nx, ny, nz, 1, [1, 1, 1], tau, tau, precision=precision,
                         amr_mode="conservative")
    sim.SetInitialDensity(rho_c)
    sim.SetInitialVelocity(u_c)
    sim.InitFromScratch(0.0)
    o = oracle.AmrOracle(nx, ny, nz, 1, tau, tau, 1)
    o.init(rho_c, u_c)
    boxes = []
    for threshold, steps in ((0.01, 4), (0.002, 4)):
        lo, hi, n = sim.TagDensity(0, threshold)
        assert n > 0
        boxes.append((lo, hi))
        sim.SetStaticRefinement(0, lo, hi)
        o.refine(0, lo, hi)
        assert sim.GetExtent(1) == ([2 * v for v in lo], [2 * v + 1 for v in hi])
        sim.Iterate(steps)
        o.iterate(steps)
        for L in (0, 1):
            a, b = sim.copy_f(L), o.f(L)
            err = float(np.max(np.abs(a - b) / np.abs(b)))
            assert err <= REGRID_BOUND[precision], (threshold, L, err)
    # the second box grew around the spreading pulse
    (lo0, hi0), (lo1, hi1) = boxes
    assert all(lo1[d] <= lo0[d] and hi1[d] >= hi0[d] for d in range(3))
    assert boxes[0] != boxes[1]
    assert sim.total_mass() == pytest.approx(o.mass(), rel=1e-13 if precision == "f64" else 1e-7)
