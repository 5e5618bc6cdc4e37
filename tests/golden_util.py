"""Problem set-ups and comparison rules shared by the tests.

The pulse problem restates tests/catch2RegressionTests.cpp:8-40 of the
reference; ``catch2_approx`` restates Catch2 v2's ``Approx`` (relative
epsilon 100*FLT_EPSILON, margin 0, scale 0).
"""
import re

import numpy as np

CATCH2_EPS = float(np.finfo(np.float32).eps) * 100


def catch2_approx(actual, expected):
    """Elementwise ``actual == Approx(expected)``."""
    actual = np.asarray(actual, dtype=np.float64)
    expected = np.asarray(expected, dtype=np.float64)
    m = CATCH2_EPS * np.abs(expected)
    return (actual + m >= expected) & (expected + m >= actual)


def pulse_problem():
    """10x10x50 plane pulse, tau 0.5 (catch2RegressionTests.cpp:8-40)."""
    NX, NY, NZ = 10, 10, 50
    N = NX * NY * NZ
    rho = np.ones(N)
    k = NZ // 2
    for i in range(NX):
        for j in range(NY):
            rho[i * NY * NZ + j * NZ + k - 1] += 0.01
    z_mean = sum(rho[(N + NY * NZ) // 2 + kk] for kk in range(NZ)) / NZ
    rho /= z_mean
    return NX, NY, NZ, 0.5, rho, np.zeros(3 * N)


def config1_problem():
    """32^3 periodic, tau 1.0, rho 1.1 on the plane x = 16, u = 0, 100 steps."""
    n = 32
    rho = np.ones((n, n, n))  # C order: [i][j][k]
    rho[16, :, :] = 1.1
    return n, n, n, 1.0, 100, rho.reshape(-1), np.zeros(3 * n ** 3)


def plane_pulse(nx, ny, nz, axis, index, amplitude):
    """C-order density with rho = 1 + amplitude on one plane."""
    rho = np.ones((nx, ny, nz))
    sl = [slice(None)] * 3
    sl[axis] = index
    rho[tuple(sl)] += amplitude
    return rho.reshape(-1)


def smooth_random(nx, ny, nz, seed, amp_rho=0.02, amp_u=0.01):
    """Seeded smooth-ish random C-order rho, u (box-filtered noise)."""
    rng = np.random.default_rng(seed)
    g = rng.standard_normal((nx, ny, nz))
    for ax in range(3):
        g = (np.roll(g, 1, ax) + g + np.roll(g, -1, ax)) / 3.0
    rho = 1.0 + amp_rho * g / max(np.abs(g).max(), 1e-30)
    u = rng.uniform(-amp_u, amp_u, size=(nx, ny, nz, 3))
    return rho.reshape(-1), u.reshape(-1)


def parse_pulse_header(path):
    """Arrays RHO_t0.. VEL_t200 from the reference's pulseRegression.h."""
    src = open(path).read()
    out = {}
    for name in ("RHO_t0", "RHO_t100", "RHO_t200", "VEL_t0", "VEL_t100", "VEL_t200"):
        m = re.search(name + r"\s*=\s*\{([^}]*)\}", src)
        out[name] = np.array([float(t) for t in m.group(1).split(",")])
    return out


def parse_mode_tables(path):
    """MODE_MATRIX and MODE_MATRIX_INVERSE from the reference's AmrSim.cpp."""
    from fractions import Fraction
    src = open(path).read()

    def table(name):
        blk = src.split(name + "[NMODES][NMODES] =")[1].split("};")[0]
        rows = re.findall(r"\{([^{}]*)\}", blk)
        res = []
        for r in rows:
            vals = []
            for t in r.split(","):
                t = t.strip().replace("./", "/").rstrip(".")
                vals.append(float(Fraction(t.replace(".", ""))) if "/" in t else float(t))
            res.append(vals)
        return np.array(res)

    return table("MODE_MATRIX"), table("MODE_MATRIX_INVERSE")
