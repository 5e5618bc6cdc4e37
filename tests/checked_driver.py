"""Drives every device path of the library once on small cases and prints
the bounds counters as one JSON line.  Run by tests/test_gpu_checked.py in a
subprocess with LBX_LIBRARY=checked (the bounds-checked debug build)."""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, HERE)

from golden_util import smooth_random  # noqa: E402
from lambrex_gb300 import lbx  # noqa: E402


def single_level(dims, precision):
    nx, ny, nz = dims
    rho, u = smooth_random(nx, ny, nz, seed=nx + ny + nz)
    s = lbx.AmrSim(nx, ny, nz, 0, [1, 1, 1], 0.7, 1.1, precision=precision)
    s.SetInitialDensity(rho)
    s.SetInitialVelocity(u)
    s.InitFromScratch(0.0)
    s.Iterate(3)
    s.CalcHydroVars(0)
    f = s.copy_f(0)
    s.set_f(0, f)
    s.Iterate(2)
    s.CalcHydroVars(0)   # stepped on after a readout: the readout runs the next step
    s.Iterate(2)         # and this takes it
    s.mass_momentum(0)
    s.TagDensity(0, 1e-3)
    s.CalcEquilibriumDist(0)
    s.Iterate(1)
    s.total_mass()
    s.close()


def amr(mode, precision, levels):
    dims = (16, 12, 10)
    rho, u = smooth_random(*dims, seed=5)
    s = lbx.AmrSim(*dims, levels - 1, [1, 1, 1], 0.8, 0.8, precision=precision, amr_mode=mode)
    s.SetInitialDensity(rho)
    s.SetInitialVelocity(u)
    s.InitFromScratch(0.0)
    s.SetStaticRefinement(0, (4, 3, 2), (11, 8, 7))
    if levels > 2:
        s.SetStaticRefinement(1, (10, 8, 6), (17, 13, 11))
    s.Iterate(2)
    for lev in range(levels):
        s.CalcHydroVars(lev)
        s.copy_f(lev)
        s.mass_momentum(lev)
        s.TagDensity(lev, 1e-3)
        s.ErrorEst(lev)
    s.total_mass()
    s.UnsetStaticRefinement(0)
    s.Iterate(1)
    s.SetStaticRefinement(0, (0, 0, 0), (5, 4, 3))  # touches the periodic faces
    s.Iterate(2)
    s.copy_f(1)
    s.close()


def ensemble():
    dims = [(16, 8, 8), (5, 7, 3), (24, 16, 12), (1, 4, 2)]
    e = lbx.Ensemble(dims, [0.7, 0.9, 1.2, 0.6], precision="f32s")
    for b, d in enumerate(dims):
        rho, u = smooth_random(*d, seed=b)
        e.init_box(b, rho, u)
    e.iterate(3)
    e.autotune(trial_steps=2)
    e.iterate(4)
    for b in range(len(dims)):
        e.copy_f(b)
        e.hydro(b)
    e.close()


def server(precision):
    srv = lbx.Server(2 << 30, max_active=8, precision=precision)
    ids = [srv.submit(1, (16, 12, 8), 6, 0.8, 0, 3, 0.02),
           srv.submit(2, (32, 16, 16), 4, 0.9, 1, 5, 0.05),
           srv.submit(3, (32, 32, 32), 2, 1.1, 2, 7, 0.01, keep_field=False)]
    srv.run_until_done(ids, quantum=3)
    for i in ids:
        srv.take(i)
    srv.close()


def main():
    lbx.lambrexInit()
    lbx.debug_bounds(reset=True)
    cases = 0
    for dims in [(5, 7, 3), (1, 3, 2), (11, 13, 7)]:
        for prec in ("f64", "f64p", "f32s"):
            single_level(dims, prec)
            cases += 1
    for mode, prec, levels in [("faithful", "f64", 2), ("conservative", "f64", 2),
                               ("conservative", "f32s", 2), ("conservative", "f64", 3),
                               ("faithful", "f64p", 2), ("conservative", "f64p", 3),
                               ("rescaled", "f64", 2), ("rescaled", "f64p", 3),
                               ("rescaled", "f32s", 2)]:
        amr(mode, prec, levels)
        cases += 1
    ensemble()
    cases += 1
    for prec in ("f32s", "f64"):
        server(prec)
        cases += 1
    count, first = lbx.debug_bounds()
    print(json.dumps({"variant": lbx.LIB_VARIANT, "cases": cases, "count": count, "first": first}))


if __name__ == "__main__":
    main()
