"""ctypes loader and builder for the CPU oracle (oracle/lbx_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()``
and by bench.py's CPU-baseline leg.  The shipped library never imports it.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "liblbx_oracle.so")
SRC = os.path.join(HERE, "lbx_oracle.cpp")
HDR = os.path.join(HERE, "lbx_oracle.h")

NV = 15

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)


def build(force: bool = False) -> str:
    """Compile the oracle with g++ (-O3, OpenMP, no FP contraction)."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    if (not force and os.path.exists(LIB_PATH)
            and os.path.getmtime(LIB_PATH) >= max(os.path.getmtime(SRC), os.path.getmtime(HDR))):
        return LIB_PATH
    tmp = LIB_PATH + ".tmp%d" % os.getpid()
    cmd = ["g++", "-std=c++17", "-O3", "-fopenmp", "-ffp-contract=off", "-fno-fast-math",
           "-fPIC", "-shared", SRC, "-o", tmp]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        path = build()
        L = ctypes.CDLL(path)
        L.orc_set_poison.argtypes = [ctypes.c_int]
        L.orc_mode_tables.argtypes = [_dp, _dp]
        L.orc_collide_cell.argtypes = [_dp, ctypes.c_double, ctypes.c_double]
        L.orc_c_to_fab.argtypes = [ctypes.c_int] * 3 + [_dp, ctypes.c_size_t, _dp, ctypes.c_size_t, _dp, _dp]
        L.orc_c_to_fab.restype = ctypes.c_int
        L.orc_equilibrium.argtypes = [ctypes.c_int] * 3 + [_dp, _dp, _dp]
        L.orc_step.argtypes = [ctypes.c_int] * 3 + [_dp, ctypes.c_double, ctypes.c_double,
                                                     ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.orc_step.restype = ctypes.c_int
        L.orc_hydro.argtypes = [ctypes.c_int] * 3 + [_dp, _dp, _dp]
        L.orc_mass_momentum.argtypes = [ctypes.c_int] * 3 + [_dp, _dp]
        L.orc_amr_create.argtypes = [ctypes.c_int] * 4 + [ctypes.c_double, ctypes.c_double, ctypes.c_int]
        L.orc_amr_create.restype = ctypes.c_void_p
        L.orc_amr_destroy.argtypes = [ctypes.c_void_p]
        L.orc_amr_set_readings.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.orc_amr_set_readings.restype = ctypes.c_int
        L.orc_amr_init.argtypes = [ctypes.c_void_p, _dp, ctypes.c_size_t, _dp, ctypes.c_size_t, ctypes.c_double]
        L.orc_amr_refine.argtypes = [ctypes.c_void_p, ctypes.c_int, _ip, _ip]
        L.orc_amr_unrefine.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.orc_amr_iterate.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.orc_amr_finest.argtypes = [ctypes.c_void_p]
        L.orc_amr_extent.argtypes = [ctypes.c_void_p, ctypes.c_int, _ip, _ip]
        L.orc_amr_copy_f.argtypes = [ctypes.c_void_p, ctypes.c_int, _dp]
        L.orc_amr_copy_f_grown.argtypes = [ctypes.c_void_p, ctypes.c_int, _dp]
        L.orc_amr_calc_hydro.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.orc_amr_get_hydro.argtypes = [ctypes.c_void_p, ctypes.c_int, _dp, _dp]
        L.orc_amr_time.argtypes = [ctypes.c_void_p, ctypes.c_int, _dp, _dp, _ip, _dp, _dp]
        L.orc_amr_mass.argtypes = [ctypes.c_void_p]
        L.orc_amr_mass.restype = ctypes.c_double
        _lib = L
    return _lib


def _p(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_dp)


def set_poison(on: bool):
    """Fresh ghost-cell storage NaN (True) or zero (False, the default)."""
    lib().orc_set_poison(1 if on else 0)


def mode_tables():
    M = np.zeros((NV, NV))
    Mi = np.zeros((NV, NV))
    lib().orc_mode_tables(_p(M), _p(Mi))
    return M, Mi


def collide_cell(f15, omega_s, omega_b):
    f = np.ascontiguousarray(f15, dtype=np.float64).copy()
    lib().orc_collide_cell(_p(f), omega_s, omega_b)
    return f


def c_to_fab(nx, ny, nz, rho_c, u_c):
    rho_c = np.ascontiguousarray(rho_c, dtype=np.float64)
    u_c = np.ascontiguousarray(u_c, dtype=np.float64)
    rho = np.zeros((nz, ny, nx))
    u = np.zeros((3, nz, ny, nx))
    rc = lib().orc_c_to_fab(nx, ny, nz, _p(rho_c), rho_c.size, _p(u_c), u_c.size, _p(rho), _p(u))
    if rc:
        raise IndexError("initial vector shorter than the domain")
    return rho, u


def equilibrium(rho, u):
    rho = np.ascontiguousarray(rho, dtype=np.float64)
    u = np.ascontiguousarray(u, dtype=np.float64)
    nz, ny, nx = rho.shape
    f = np.zeros((NV, nz, ny, nx))
    lib().orc_equilibrium(nx, ny, nz, _p(rho), _p(u), _p(f))
    return f


def step(f, tau_s, tau_b, nsteps, nthreads=1, style=1):
    """Advance FAB-order f (modified in place) by nsteps periodic steps."""
    assert f.dtype == np.float64 and f.flags.c_contiguous and f.shape[0] == NV
    _, nz, ny, nx = f.shape
    rc = lib().orc_step(nx, ny, nz, _p(f), tau_s, tau_b, nsteps, nthreads, style)
    assert rc == 0
    return f


def hydro(f):
    _, nz, ny, nx = f.shape
    rho = np.zeros((nz, ny, nx))
    u = np.zeros((3, nz, ny, nx))
    lib().orc_hydro(nx, ny, nz, _p(np.ascontiguousarray(f)), _p(rho), _p(u))
    return rho, u


def mass_momentum(f):
    _, nz, ny, nx = f.shape
    out = np.zeros(4)
    lib().orc_mass_momentum(nx, ny, nz, _p(np.ascontiguousarray(f)), _p(out))
    return out


# readings of the AMReX behaviour behind the faithful cycle (lbx_oracle.h)
READ_SUM8, READ_GROW0, READ_MASK_FINE, READ_RING2_STALE = 1, 2, 4, 8


class AmrOracle:
    """Multi-level oracle.  mode 0 = reference-faithful Rohde cycle,
    mode 1 = the library's conservative volumetric scheme, mode 2 = the
    library's rescaled coupling (non-equilibrium rescaling, time-interpolated
    ghost data).  ``readings`` (mode 0) flips READ_* readings of AMReX's
    behaviour; 0 = the defaults."""

    def __init__(self, nx, ny, nz, max_level, tau_s, tau_b, mode=0, readings=0):
        self.L = lib()
        self.h = self.L.orc_amr_create(nx, ny, nz, max_level, tau_s, tau_b, mode)
        if not self.h:
            raise ValueError("bad oracle arguments")
        self.dims = (nx, ny, nz)
        if readings and self.L.orc_amr_set_readings(self.h, readings):
            raise ValueError("unknown readings %r" % readings)

    def __del__(self):
        if getattr(self, "h", None):
            self.L.orc_amr_destroy(self.h)
            self.h = None

    def init(self, rho_c, u_c, time=0.0):
        rho_c = np.ascontiguousarray(rho_c, dtype=np.float64)
        u_c = np.ascontiguousarray(u_c, dtype=np.float64)
        if self.L.orc_amr_init(self.h, _p(rho_c), rho_c.size, _p(u_c), u_c.size, time):
            raise IndexError("initial vector shorter than the domain")

    def refine(self, level, lo, hi):
        lo = (ctypes.c_int * 3)(*lo)
        hi = (ctypes.c_int * 3)(*hi)
        if self.L.orc_amr_refine(self.h, level, lo, hi):
            raise ValueError("refinement rejected")

    def unrefine(self, level):
        self.L.orc_amr_unrefine(self.h, level)

    def iterate(self, n):
        assert self.L.orc_amr_iterate(self.h, n) == 0

    def finest(self):
        return self.L.orc_amr_finest(self.h)

    def extent(self, level):
        lo = (ctypes.c_int * 3)()
        hi = (ctypes.c_int * 3)()
        if self.L.orc_amr_extent(self.h, level, lo, hi):
            raise ValueError("no such level")
        return tuple(lo), tuple(hi)

    def f(self, level):
        lo, hi = self.extent(level)
        n = [hi[d] - lo[d] + 1 for d in range(3)]
        out = np.zeros((NV, n[2], n[1], n[0]))
        self.L.orc_amr_copy_f(self.h, level, _p(out))
        return out

    def f_grown(self, level):
        lo, hi = self.extent(level)
        n = [hi[d] - lo[d] + 5 for d in range(3)]
        out = np.zeros((NV, n[2], n[1], n[0]))
        self.L.orc_amr_copy_f_grown(self.h, level, _p(out))
        return out

    def hydro(self, level):
        lo, hi = self.extent(level)
        n = [hi[d] - lo[d] + 1 for d in range(3)]
        self.L.orc_amr_calc_hydro(self.h, level)
        rho = np.zeros((n[2], n[1], n[0]))
        u = np.zeros((3, n[2], n[1], n[0]))
        self.L.orc_amr_get_hydro(self.h, level, _p(rho), _p(u))
        return rho, u

    def time(self, level):
        t = ctypes.c_double()
        dt = ctypes.c_double()
        st = ctypes.c_int()
        ts = ctypes.c_double()
        tb = ctypes.c_double()
        self.L.orc_amr_time(self.h, level, ctypes.byref(t), ctypes.byref(dt), ctypes.byref(st),
                            ctypes.byref(ts), ctypes.byref(tb))
        return dict(time=t.value, dt=dt.value, step=st.value, tau_s=ts.value, tau_b=tb.value)

    def mass(self):
        return self.L.orc_amr_mass(self.h)
