"""The pulse example (examples/amr_pulse.cpp of the reference) built against
the drop-in headers: compiles on any host; on a GPU it prints the same
numbers as the oracle at 6 significant digits."""
import os
import re
import subprocess

import numpy as np
import pytest

from golden_util import pulse_problem

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def build_example(tmp_path):
    from lambrex_gb300 import build as B
    B.build()
    exe = str(tmp_path / "amr_pulse")
    cmd = ["g++", "-std=c++17", "-Wall", "-Werror", "-I" + os.path.join(ROOT, "include"),
           os.path.join(ROOT, "examples", "amr_pulse.cpp"), "-L" + os.path.join(ROOT, "lambrex_gb300"),
           "-llbx_cuda", "-Wl,-rpath," + os.path.join(ROOT, "lambrex_gb300"), "-o", exe]
    subprocess.run(cmd, check=True)
    return exe


def test_example_compiles(tmp_path):
    assert os.path.exists(build_example(tmp_path))


@pytest.mark.gpu
def test_example_output_matches_oracle(tmp_path, oracle):
    exe = build_example(tmp_path)
    out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    blocks = re.findall(r"\{ (.*?) \};", out, flags=re.S)
    assert len(blocks) == 6  # density and velocity at t = 0, 100, 200
    assert "Time: 200" in out and "Time step: 200" in out
    nx, ny, nz, tau, rho_c, u_c = pulse_problem()
    rho, u = oracle.c_to_fab(nx, ny, nz, rho_c, u_c)
    f = oracle.equilibrium(rho, u)
    for b, t in enumerate((0, 100, 200)):
        if t:
            oracle.step(f, tau, tau, 100, nthreads=4)
            rho, u = oracle.hydro(f)
        dens = np.array([float(x) for x in blocks[2 * b].split(",")])
        vel = np.array([float(x) for x in blocks[2 * b + 1].split(",")])
        np.testing.assert_allclose(dens, rho.reshape(-1), rtol=1e-5)
        vz = vel.reshape(-1, 3)[:, 2]
        np.testing.assert_allclose(vz, u[2].reshape(-1), rtol=1e-5, atol=1e-14)
