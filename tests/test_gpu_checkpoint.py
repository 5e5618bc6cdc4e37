"""Checkpoint / restart through the C ABI (lbx_checkpoint_write / _read):
a restored simulation continues bit for bit, with the same times and step
counters, in every precision and coupling mode."""
import numpy as np
import pytest

from golden_util import smooth_random

pytestmark = pytest.mark.gpu

CASES = [("f64", "conservative", 0), ("f32s", "conservative", 0), ("f64p", "conservative", 0),
         ("f64", "conservative", 1), ("f32s", "conservative", 2), ("f64", "faithful", 1)]


@pytest.mark.parametrize("precision,mode,levels", CASES)
def test_restart_continues_bit_for_bit(gpu_lib, tmp_path, precision, mode, levels):
    dims = (16, 12, 12)
    rho_c, u_c = smooth_random(*dims, seed=77)
    a = gpu_lib.AmrSim(*dims, levels, [1, 1, 1], 0.9, 0.7, precision=precision, amr_mode=mode)
    a.SetInitialDensity(rho_c)
    a.SetInitialVelocity(u_c)
    a.InitFromScratch(0.0)
    if levels >= 1:
        a.SetStaticRefinement(0, (4, 3, 3), (11, 8, 8))
    if levels >= 2:
        a.SetStaticRefinement(1, (10, 8, 8), (17, 13, 13))
    a.Iterate(7)
    path = str(tmp_path / "state.lbx")
    a.checkpoint(path)
    b = gpu_lib.AmrSim.from_checkpoint(path)
    assert b.finestLevel() == a.finestLevel() and b.GetDims() == a.GetDims()
    for sim in (a, b):
        sim.Iterate(6)
        sim.Iterate(1)
    for lev in range(levels + 1):
        assert np.array_equal(a.copy_f(lev), b.copy_f(lev), equal_nan=True), lev
        assert a.GetTime(lev) == b.GetTime(lev) and a.GetTimeStep(lev) == b.GetTimeStep(lev)
        assert a.GetTau(lev) == b.GetTau(lev)
    a.CalcHydroVars(0)
    b.CalcHydroVars(0)
    assert np.array_equal(a.density_field(0), b.density_field(0), equal_nan=True)


def test_corrupt_checkpoint_is_rejected(gpu_lib, tmp_path):
    p = tmp_path / "bad.lbx"
    p.write_bytes(b"LBXCKPT1" + bytes(7))
    with pytest.raises(gpu_lib.LbxError) as e:
        gpu_lib.AmrSim.from_checkpoint(str(p))
    assert e.value.status == 9
