"""Generate tests/golden/pulse_oracle.json.

Reads the reference's known-answer data (tests/pulseRegression.h of LAMBReX,
driven by tests/catch2RegressionTests.cpp:6-93), runs the CPU oracle on the
same pulse problem, checks every value with the reference's own Catch2
``Approx`` rule (relative epsilon 100*FLT_EPSILON, margin 0), and writes the
SHA-256 digests of the oracle's outputs together with the check record.  The
digests pin the oracle on machines that do not hold the reference (the
oracle is compiled with -ffp-contract=off and is bit-reproducible across
hosts).  The reference's data itself is not copied.

usage: python tests/golden/make_golden.py <reference_dir>   (or LBX_REFERENCE_DIR)
"""
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from oracle import oracle as O  # noqa: E402

sys.path.insert(0, os.path.dirname(HERE))
from golden_util import (catch2_approx, config1_problem, parse_pulse_header,  # noqa: E402
                         pulse_problem)


def digest(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<f8").tobytes()).hexdigest()


def main():
    ref_dir = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("LBX_REFERENCE_DIR")
    if not ref_dir:
        raise SystemExit("usage: make_golden.py <LAMBReX source dir> (or set LBX_REFERENCE_DIR)")
    header = os.path.join(ref_dir, "tests", "pulseRegression.h")
    golden = parse_pulse_header(header)
    nx, ny, nz, tau, rho_c, u_c = pulse_problem()
    rho, u = O.c_to_fab(nx, ny, nz, rho_c, u_c)
    f = O.equilibrium(rho, u)
    out = {"problem": "pulse 10x10x50, tau 0.5, amplitude 0.01 (catch2RegressionTests.cpp:6-93)",
           "checkpoints": {}}
    step_done = 0
    for tag, t in (("t0", 0), ("t100", 100), ("t200", 200)):
        O.step(f, tau, tau, t - step_done, nthreads=4, style=1)
        step_done = t
        r, v = O.hydro(f) if t else (rho, u)
        r_flat = r.reshape(-1)                      # golden order: k, j, i
        v_flat = np.moveaxis(v, 0, -1).reshape(-1)  # n innermost
        ok_r = catch2_approx(r_flat, golden["RHO_" + tag])
        ok_v = catch2_approx(v_flat, golden["VEL_" + tag])
        if not (ok_r.all() and ok_v.all()):
            raise SystemExit("oracle fails the reference's Catch2 check at %s" % tag)
        out["checkpoints"][tag] = {
            "step": t,
            "sha256_f": digest(f),
            "sha256_rho": digest(r),
            "sha256_u": digest(v),
            "catch2_checks_passed": int(ok_r.size + ok_v.size),
            "mass": float(O.mass_momentum(f)[0]),
        }
    # config 1 of the benchmark plan: 32^3 plane pulse, tau 1.0, 100 steps
    nx, ny, nz, tau, steps, rho_c, u_c = config1_problem()
    rho, u = O.c_to_fab(nx, ny, nz, rho_c, u_c)
    f = O.equilibrium(rho, u)
    O.step(f, tau, tau, steps, nthreads=4, style=1)
    out["config1"] = {"problem": "32^3, tau 1.0, rho 1.1 on plane x=16, 100 steps",
                      "sha256_f": digest(f), "mass": float(O.mass_momentum(f)[0])}
    with open(os.path.join(HERE, "pulse_oracle.json"), "w") as fh:
        json.dump(out, fh, indent=1, sort_keys=True)
    print("wrote pulse_oracle.json")


if __name__ == "__main__":
    main()
