"""Python mirror of LAMBReX's ``AmrSim`` / ``lambrex.h`` API over liblbx_cuda.so.

Method names, argument meaning and error behaviour follow the reference
(include/AmrSim.h:127-155, include/lambrex.h:6-7):

* ``SetInitialDensity`` / ``SetInitialVelocity`` take a scalar or a C-order
  vector (``rho[(i*NY + j)*NZ + k]``, ``u[((i*NY + j)*NZ + k)*3 + n]``);
* ``Iterate`` does not refresh density/velocity; call ``CalcHydroVars``;
* getters return the reference's sentinels (-1 and -3e8) for points that are
  not on the level;
* where the reference calls ``amrex::Abort`` this raises :class:`LbxError`.

The compute path is the CUDA library only: if ``liblbx_cuda.so`` is missing
the import fails loudly; there is no CPU fallback.  With the environment
variable ``LBX_LIBRARY=checked`` the process loads the bounds-checked debug
build ``liblbx_cuda_checked.so`` instead (same API; see :func:`debug_bounds`).
"""
from __future__ import annotations

import ctypes
import os
from typing import Sequence

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_VARIANT = os.environ.get("LBX_LIBRARY", "release")
if LIB_VARIANT not in ("release", "checked"):
    raise ImportError("LBX_LIBRARY must be 'release' or 'checked', not %r" % LIB_VARIANT)
LIB_PATH = os.path.join(_HERE, "liblbx_cuda.so" if LIB_VARIANT == "release"
                        else "liblbx_cuda_checked.so")

NV = 15
# AmrSim prints its extents on construction as the reference's constructor
# does (src/AmrSim.cpp:776); a program whose stdout carries data sets this False
ANNOUNCE = True
LBX_OK = 0
LBX_ERR_NOT_FOUND = 8
F64 = 0
F32_SHIFTED = 1
AMR_FAITHFUL = 0
AMR_CONSERVATIVE = 1
AMR_RESCALED = 2

_c_int_p = ctypes.POINTER(ctypes.c_int)
_c_dbl_p = ctypes.POINTER(ctypes.c_double)


class LbxError(RuntimeError):
    def __init__(self, status: int, where: str):
        self.status = status
        super().__init__("%s failed: %s (status %d)" % (where, _lib().lbx_status_string(status).decode(), status))


_LIB = None


def _lib():
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError("%s is not built (run lambrex_gb300.build.build(%s)); there is no "
                              "CPU fallback" % (os.path.basename(LIB_PATH),
                                                "" if LIB_VARIANT == "release" else "'checked'"))
        L = ctypes.CDLL(LIB_PATH)
        L.lbx_status_string.restype = ctypes.c_char_p
        L.lbx_status_string.argtypes = [ctypes.c_int]
        L.lbx_nl_density.restype = ctypes.c_double
        L.lbx_nl_velocity.restype = ctypes.c_double
        vp = ctypes.c_void_p
        L.lbx_create.argtypes = [ctypes.c_int] * 4 + [_c_int_p, ctypes.c_double, ctypes.c_double,
                                                      ctypes.c_int, ctypes.c_int, ctypes.POINTER(vp)]
        L.lbx_destroy.argtypes = [vp]
        L.lbx_set_initial_density.argtypes = [vp, _c_dbl_p, ctypes.c_size_t]
        L.lbx_set_initial_velocity.argtypes = [vp, _c_dbl_p, ctypes.c_size_t]
        L.lbx_init_from_scratch.argtypes = [vp, ctypes.c_double]
        L.lbx_set_static_refinement.argtypes = [vp, ctypes.c_int, _c_int_p, _c_int_p]
        L.lbx_unset_static_refinement.argtypes = [vp, ctypes.c_int]
        L.lbx_iterate.argtypes = [vp, ctypes.c_int]
        L.lbx_calc_hydro.argtypes = [vp, ctypes.c_int]
        L.lbx_calc_equilibrium.argtypes = [vp, ctypes.c_int]
        L.lbx_get_density.argtypes = [vp] + [ctypes.c_int] * 4 + [_c_dbl_p]
        L.lbx_get_velocity.argtypes = [vp] + [ctypes.c_int] * 5 + [_c_dbl_p]
        L.lbx_get_density_field.argtypes = [vp, ctypes.c_int, _c_dbl_p, ctypes.c_size_t]
        L.lbx_get_velocity_field.argtypes = [vp, ctypes.c_int, _c_dbl_p, ctypes.c_size_t]
        L.lbx_get_time.argtypes = [vp, ctypes.c_int, _c_dbl_p]
        L.lbx_get_time_step.argtypes = [vp, ctypes.c_int, _c_int_p]
        L.lbx_get_dt.argtypes = [vp, ctypes.c_int, _c_dbl_p]
        L.lbx_get_tau.argtypes = [vp, ctypes.c_int, _c_dbl_p, _c_dbl_p]
        L.lbx_get_dims.argtypes = [vp, _c_int_p]
        L.lbx_max_level.argtypes = [vp, _c_int_p]
        L.lbx_finest_level.argtypes = [vp, _c_int_p]
        L.lbx_ref_ratio.argtypes = [vp, ctypes.c_int, _c_int_p]
        L.lbx_get_extent.argtypes = [vp, ctypes.c_int, _c_int_p, _c_int_p]
        L.lbx_error_est.argtypes = [vp, ctypes.c_int, ctypes.c_void_p, ctypes.c_size_t]
        L.lbx_tag_density.argtypes = [vp, ctypes.c_int, ctypes.c_double, _c_int_p, _c_int_p,
                                      ctypes.POINTER(ctypes.c_longlong)]
        L.lbx_copy_f.argtypes = [vp, ctypes.c_int, _c_dbl_p, ctypes.c_size_t]
        L.lbx_set_f.argtypes = [vp, ctypes.c_int, _c_dbl_p, ctypes.c_size_t]
        L.lbx_reduce_mass_momentum.argtypes = [vp, ctypes.c_int, _c_dbl_p]
        L.lbx_total_mass.argtypes = [vp, _c_dbl_p]
        L.lbx_synchronize.argtypes = [vp]
        L.lbx_iterate_timed.argtypes = [vp, ctypes.c_int, _c_dbl_p]
        L.lbx_launch_count.argtypes = [vp, ctypes.POINTER(ctypes.c_longlong)]
        L.lbx_get_stream.argtypes = [vp, ctypes.POINTER(vp)]
        L.lbx_get_device_f.argtypes = [vp, ctypes.c_int, ctypes.POINTER(vp), _c_int_p, _c_int_p, _c_int_p]
        L.lbx_debug_bounds.argtypes = [ctypes.POINTER(ctypes.c_longlong),
                                       ctypes.POINTER(ctypes.c_longlong), ctypes.c_int]
        L.lbx_checkpoint_write.argtypes = [vp, ctypes.c_char_p]
        L.lbx_checkpoint_read.argtypes = [ctypes.c_char_p, ctypes.POINTER(vp)]
        _LIB = L
    return _LIB


def lib():
    """The loaded liblbx_cuda.so (ctypes handle)."""
    return _lib()


def _check(status: int, where: str):
    if status != LBX_OK:
        raise LbxError(status, where)


def _dptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_c_dbl_p)


def lambrexInit():
    """lambrexInit (src/lambrex.cpp:4-9): bring up the CUDA device."""
    _check(_lib().lbx_init(), "lambrexInit")


def lambrexFinalise():
    """lambrexFinalise (src/lambrex.cpp:11-14)."""
    _check(_lib().lbx_finalize(), "lambrexFinalise")


def set_device(device: int):
    """Select the GPU used by handles created afterwards in this thread."""
    _check(_lib().lbx_set_device(device), "set_device")


def debug_bounds(reset: bool = False):
    """(count, first bad index) of the out-of-range global memory accesses
    that the checked build caught and skipped on the current GPU; ``reset``
    clears the counters.  The release library raises LbxError (unsupported)."""
    n, first = ctypes.c_longlong(), ctypes.c_longlong()
    _check(_lib().lbx_debug_bounds(ctypes.byref(n), ctypes.byref(first), int(reset)), "debug_bounds")
    return n.value, first.value


F64_PAIRED = 2
_PREC = {"f64": F64, "fp64": F64, F64: F64, "f32s": F32_SHIFTED, "f32-shifted": F32_SHIFTED,
         F32_SHIFTED: F32_SHIFTED, "f64p": F64_PAIRED, "f64-paired": F64_PAIRED,
         F64_PAIRED: F64_PAIRED}
_MODE = {"faithful": AMR_FAITHFUL, AMR_FAITHFUL: AMR_FAITHFUL, "conservative": AMR_CONSERVATIVE,
         AMR_CONSERVATIVE: AMR_CONSERVATIVE, "rescaled": AMR_RESCALED, AMR_RESCALED: AMR_RESCALED}


class AmrSim:
    """``AmrSim(nx, ny, nz, max_ref_level, periodicity, tau_s, tau_b)``
    (include/AmrSim.h:128-129) on the GPU.

    Extra keyword arguments select the store precision (``"f64"`` or
    ``"f32s"``, FP32 shifted populations) and the multi-level coupling
    (``"faithful"`` reproduces the reference's Rohde cycle, ``"conservative"``
    is the library's mass-conserving scheme, ``"rescaled"`` the coupling with
    non-equilibrium rescaling and time-interpolated ghost data)."""

    NL_DENSITY = -1.0
    NL_VELOCITY = -3e8

    def __init__(self, nx: int, ny: int, nz: int, max_ref_level: int, periodicity: Sequence[int],
                 tau_s: float, tau_b: float, precision="f64", amr_mode="faithful"):
        L = _lib()
        self._L = L
        self._h = ctypes.c_void_p()
        per = (ctypes.c_int * 3)(*[int(p) for p in periodicity])
        _check(L.lbx_create(nx, ny, nz, max_ref_level, per, tau_s, tau_b, _PREC[precision],
                            _MODE[amr_mode], ctypes.byref(self._h)), "AmrSim")
        self.NX, self.NY, self.NZ = nx, ny, nz
        if ANNOUNCE:
            print("NX: %d NY: %d NZ: %d" % (nx, ny, nz))  # src/AmrSim.cpp:776

    @classmethod
    def from_checkpoint(cls, path: str) -> "AmrSim":
        """A new simulation restored from a file of :meth:`checkpoint`
        (lbx_checkpoint_read): it continues bit for bit."""
        L = _lib()
        obj = cls.__new__(cls)
        obj._L = L
        obj._h = ctypes.c_void_p()
        _check(L.lbx_checkpoint_read(os.fsencode(path), ctypes.byref(obj._h)), "from_checkpoint")
        d = (ctypes.c_int * 3)()
        _check(L.lbx_get_dims(obj._h, d), "GetDims")
        obj.NX, obj.NY, obj.NZ = d[0], d[1], d[2]
        return obj

    def checkpoint(self, path: str):
        """Save the whole state (lbx_checkpoint_write)."""
        _check(self._L.lbx_checkpoint_write(self._h, os.fsencode(path)), "checkpoint")

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            self._L.lbx_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def handle(self):
        return self._h

    # ---- setup ----
    def SetInitialDensity(self, rho):
        a = np.ascontiguousarray(np.atleast_1d(np.asarray(rho, dtype=np.float64)))
        _check(self._L.lbx_set_initial_density(self._h, _dptr(a), a.size), "SetInitialDensity")

    def SetInitialVelocity(self, u):
        a = np.ascontiguousarray(np.atleast_1d(np.asarray(u, dtype=np.float64)))
        _check(self._L.lbx_set_initial_velocity(self._h, _dptr(a), a.size), "SetInitialVelocity")

    def InitFromScratch(self, time: float = 0.0):
        _check(self._L.lbx_init_from_scratch(self._h, time), "InitFromScratch")

    def SetStaticRefinement(self, level: int, lo: Sequence[int], hi: Sequence[int]):
        _check(self._L.lbx_set_static_refinement(self._h, level, (ctypes.c_int * 3)(*lo),
                                                 (ctypes.c_int * 3)(*hi)), "SetStaticRefinement")

    def UnsetStaticRefinement(self, level: int):
        _check(self._L.lbx_unset_static_refinement(self._h, level), "UnsetStaticRefinement")

    # ---- stepping and fields ----
    def Iterate(self, nsteps: int):
        _check(self._L.lbx_iterate(self._h, nsteps), "Iterate")

    def iterate_timed(self, nsteps: int) -> float:
        """Iterate bracketed by CUDA events on the sim's stream; device ms."""
        ms = ctypes.c_double()
        _check(self._L.lbx_iterate_timed(self._h, nsteps, ctypes.byref(ms)), "iterate_timed")
        return ms.value

    def launch_count(self) -> int:
        n = ctypes.c_longlong()
        _check(self._L.lbx_launch_count(self._h, ctypes.byref(n)), "launch_count")
        return n.value

    def CalcHydroVars(self, level: int):
        _check(self._L.lbx_calc_hydro(self._h, level), "CalcHydroVars")

    def CalcEquilibriumDist(self, level: int):
        _check(self._L.lbx_calc_equilibrium(self._h, level), "CalcEquilibriumDist")

    def GetDensity(self, i: int, j: int, k: int, level: int) -> float:
        out = ctypes.c_double()
        self._L.lbx_get_density(self._h, i, j, k, level, ctypes.byref(out))
        return out.value

    def GetVelocity(self, i: int, j: int, k: int, n: int, level: int) -> float:
        out = ctypes.c_double()
        self._L.lbx_get_velocity(self._h, i, j, k, n, level, ctypes.byref(out))
        return out.value

    def OnProcessDensity(self, rho: float) -> bool:
        return rho != self.NL_DENSITY

    def OnProcessVelocity(self, u: float) -> bool:
        return u != self.NL_VELOCITY

    def GetTime(self, level: int) -> float:
        t = ctypes.c_double()
        _check(self._L.lbx_get_time(self._h, level, ctypes.byref(t)), "GetTime")
        return t.value

    def GetTimeStep(self, level: int) -> int:
        t = ctypes.c_int()
        _check(self._L.lbx_get_time_step(self._h, level, ctypes.byref(t)), "GetTimeStep")
        return t.value

    def GetDt(self, level: int) -> float:
        t = ctypes.c_double()
        _check(self._L.lbx_get_dt(self._h, level, ctypes.byref(t)), "GetDt")
        return t.value

    def GetTau(self, level: int):
        a, b = ctypes.c_double(), ctypes.c_double()
        _check(self._L.lbx_get_tau(self._h, level, ctypes.byref(a), ctypes.byref(b)), "GetTau")
        return a.value, b.value

    def GetDims(self):
        d = (ctypes.c_int * 3)()
        _check(self._L.lbx_get_dims(self._h, d), "GetDims")
        return [d[0], d[1], d[2]]

    def GetExtent(self, level: int):
        lo, hi = (ctypes.c_int * 3)(), (ctypes.c_int * 3)()
        _check(self._L.lbx_get_extent(self._h, level, lo, hi), "GetExtent")
        return [lo[0], lo[1], lo[2]], [hi[0], hi[1], hi[2]]

    def ErrorEst(self, level: int) -> np.ndarray:
        """ErrorEst (src/AmrSim.cpp:633-663): the level's tags in FAB order,
        1 (SET) inside its static tag box, 0 (CLEAR) elsewhere."""
        lo, hi = self.GetExtent(level)
        n = int(np.prod([hi[d] - lo[d] + 1 for d in range(3)]))
        tags = np.zeros(n, dtype=np.uint8)
        _check(self._L.lbx_error_est(self._h, level, tags.ctypes.data, n), "ErrorEst")
        return tags

    def TagDensity(self, level: int, threshold: float):
        """Bounding box (lo, hi, in the level's cells) of the cells whose
        density differs from the level's mean by more than threshold, and
        their number; (None, None, 0) when there are none."""
        lo, hi = (ctypes.c_int * 3)(), (ctypes.c_int * 3)()
        n = ctypes.c_longlong()
        _check(self._L.lbx_tag_density(self._h, level, float(threshold), lo, hi,
                                       ctypes.byref(n)), "TagDensity")
        if n.value == 0:
            return None, None, 0
        return [lo[0], lo[1], lo[2]], [hi[0], hi[1], hi[2]], n.value

    def maxLevel(self) -> int:
        o = ctypes.c_int()
        _check(self._L.lbx_max_level(self._h, ctypes.byref(o)), "maxLevel")
        return o.value

    def finestLevel(self) -> int:
        o = ctypes.c_int()
        _check(self._L.lbx_finest_level(self._h, ctypes.byref(o)), "finestLevel")
        return o.value

    def refRatio(self, level: int):
        r = (ctypes.c_int * 3)()
        _check(self._L.lbx_ref_ratio(self._h, level, r), "refRatio")
        return [r[0], r[1], r[2]]

    # ---- bulk access (FAB order, i fastest) ----
    def _shape(self, level):
        lo, hi = self.GetExtent(level)
        return [hi[d] - lo[d] + 1 for d in range(3)]

    @staticmethod
    def _out(out, shape):
        """A new array, or the caller's C-contiguous float64 buffer of that
        size (reused buffers skip the first-touch cost of fresh pages)."""
        if out is None:
            return np.empty(shape)
        if (not isinstance(out, np.ndarray) or out.dtype != np.float64
                or not out.flags.c_contiguous or out.size != int(np.prod(shape))):
            raise ValueError("out must be a C-contiguous float64 array of %d elements"
                             % int(np.prod(shape)))
        return out.reshape(shape)

    def density_field(self, level: int, out: np.ndarray = None) -> np.ndarray:
        n = self._shape(level)
        out = self._out(out, (n[2], n[1], n[0]))
        _check(self._L.lbx_get_density_field(self._h, level, _dptr(out), out.size), "density_field")
        return out

    def velocity_field(self, level: int, out: np.ndarray = None) -> np.ndarray:
        n = self._shape(level)
        out = self._out(out, (3, n[2], n[1], n[0]))
        _check(self._L.lbx_get_velocity_field(self._h, level, _dptr(out), out.size), "velocity_field")
        return out

    def copy_f(self, level: int = 0) -> np.ndarray:
        n = self._shape(level)
        out = np.empty((NV, n[2], n[1], n[0]))
        _check(self._L.lbx_copy_f(self._h, level, _dptr(out), out.size), "copy_f")
        return out

    def set_f(self, level: int, f: np.ndarray):
        a = np.ascontiguousarray(f, dtype=np.float64)
        _check(self._L.lbx_set_f(self._h, level, _dptr(a), a.size), "set_f")

    def mass_momentum(self, level: int = 0) -> np.ndarray:
        out = np.zeros(4)
        _check(self._L.lbx_reduce_mass_momentum(self._h, level, _dptr(out)), "mass_momentum")
        return out

    def total_mass(self) -> float:
        out = ctypes.c_double()
        _check(self._L.lbx_total_mass(self._h, ctypes.byref(out)), "total_mass")
        return out.value

    def synchronize(self):
        _check(self._L.lbx_synchronize(self._h), "synchronize")


class Request(ctypes.Structure):
    """lbx_request: a 1..3 level periodic pulse simulation to serve."""
    _fields_ = [("levels", ctypes.c_int), ("nx", ctypes.c_int), ("ny", ctypes.c_int),
                ("nz", ctypes.c_int), ("steps", ctypes.c_int), ("tau", ctypes.c_double),
                ("pulse_axis", ctypes.c_int), ("pulse_index", ctypes.c_int),
                ("amplitude", ctypes.c_double), ("keep_field", ctypes.c_int)]


class Server:
    """Continuous-batching serving loop (lbx_server_*)."""

    def __init__(self, hbm_budget_bytes, max_active=64, precision="f32s"):
        L = _lib()
        self._L = L
        vp = ctypes.c_void_p
        L.lbx_server_create.argtypes = [ctypes.c_size_t, ctypes.c_int, ctypes.c_int, ctypes.POINTER(vp)]
        L.lbx_server_destroy.argtypes = [vp]
        L.lbx_server_submit.argtypes = [vp, ctypes.POINTER(Request), ctypes.POINTER(ctypes.c_longlong)]
        L.lbx_server_pump.argtypes = [vp, ctypes.c_int, _c_int_p, _c_int_p]
        L.lbx_server_poll.argtypes = [vp, ctypes.c_longlong, _c_int_p, _c_dbl_p, _c_dbl_p]
        L.lbx_server_take.argtypes = [vp, ctypes.c_longlong, _c_dbl_p, ctypes.c_size_t]
        L.lbx_server_stats.argtypes = [vp, ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_size_t),
                                       ctypes.POINTER(ctypes.c_longlong)]
        self._h = vp()
        self._dims = {}
        _check(L.lbx_server_create(int(hbm_budget_bytes), max_active, _PREC[precision],
                                   ctypes.byref(self._h)), "server_create")

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            self._L.lbx_server_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, levels, dims, steps, tau, pulse_axis, pulse_index, amplitude,
               keep_field=True) -> int:
        r = Request(levels, dims[0], dims[1], dims[2], steps, tau, pulse_axis, pulse_index, amplitude,
                    1 if keep_field else 0)
        rid = ctypes.c_longlong()
        _check(self._L.lbx_server_submit(self._h, ctypes.byref(r), ctypes.byref(rid)), "server_submit")
        self._dims[rid.value] = (tuple(dims), bool(keep_field))
        return rid.value

    def pump(self, quantum=16):
        a, q = ctypes.c_int(), ctypes.c_int()
        _check(self._L.lbx_server_pump(self._h, quantum, ctypes.byref(a), ctypes.byref(q)), "server_pump")
        return a.value, q.value

    def poll(self, rid):
        d, m, p = ctypes.c_int(), ctypes.c_double(), ctypes.c_double()
        _check(self._L.lbx_server_poll(self._h, rid, ctypes.byref(d), ctypes.byref(m), ctypes.byref(p)),
               "server_poll")
        return bool(d.value), m.value, p.value

    def take(self, rid):
        """Level-0 density of a finished request (None unless it was
        submitted with keep_field); the server then forgets the request."""
        (nx, ny, nz), keep = self._dims.pop(rid)
        if not keep:
            _check(self._L.lbx_server_take(self._h, rid, None, 0), "server_take")
            return None
        rho = np.empty((nz, ny, nx))
        _check(self._L.lbx_server_take(self._h, rid, _dptr(rho), rho.size), "server_take")
        return rho

    def stats(self):
        c, b, l = ctypes.c_longlong(), ctypes.c_size_t(), ctypes.c_longlong()
        _check(self._L.lbx_server_stats(self._h, ctypes.byref(c), ctypes.byref(b), ctypes.byref(l)), "stats")
        return dict(cell_updates=c.value, bytes_in_use=b.value, launches=l.value)

    def set_config(self, tile_cells, block, cells_per_thread):
        self._L.lbx_server_set_config.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        _check(self._L.lbx_server_set_config(self._h, tile_cells, block, cells_per_thread), "set_config")

    def timing(self):
        t = (ctypes.c_double * 4)()
        self._L.lbx_server_timing.argtypes = [ctypes.c_void_p, _c_dbl_p]
        _check(self._L.lbx_server_timing(self._h, t), "timing")
        return dict(admit_s=t[0], finish_s=t[1], tables_s=t[2], step_s=t[3])

    def run_until_done(self, ids, quantum=16, max_pumps=100000):
        for _ in range(max_pumps):
            active, queued = self.pump(quantum)
            if all(self.poll(i)[0] for i in ids):
                return
        raise RuntimeError("requests did not finish")


class Ensemble:
    """Batched ensemble of independent periodic boxes (lbx_ensemble_*): one
    persistent launch per step for all boxes, graph-replayed steps."""

    def __init__(self, dims, taus, precision="f32s"):
        L = _lib()
        self._L = L
        vp = ctypes.c_void_p
        L.lbx_ensemble_create.argtypes = [ctypes.c_int, _c_int_p, _c_dbl_p, ctypes.c_int, ctypes.POINTER(vp)]
        for name in ("destroy", "synchronize"):
            getattr(L, "lbx_ensemble_" + name).argtypes = [vp]
        L.lbx_ensemble_init_box.argtypes = [vp, ctypes.c_int, _c_dbl_p, ctypes.c_size_t, _c_dbl_p, ctypes.c_size_t]
        L.lbx_ensemble_autotune.argtypes = [vp, ctypes.c_int, _c_int_p]
        L.lbx_ensemble_set_config.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.lbx_ensemble_iterate.argtypes = [vp, ctypes.c_int]
        L.lbx_ensemble_iterate_timed.argtypes = [vp, ctypes.c_int, _c_dbl_p]
        L.lbx_ensemble_copy_f.argtypes = [vp, ctypes.c_int, _c_dbl_p, ctypes.c_size_t]
        L.lbx_ensemble_hydro.argtypes = [vp, ctypes.c_int, _c_dbl_p, _c_dbl_p, ctypes.c_size_t]
        L.lbx_ensemble_launches.argtypes = [vp, ctypes.POINTER(ctypes.c_longlong)]
        self.dims = [tuple(int(v) for v in d) for d in dims]
        flat = (ctypes.c_int * (3 * len(self.dims)))(*[v for d in self.dims for v in d])
        t = np.ascontiguousarray(taus, dtype=np.float64)
        self._h = vp()
        _check(L.lbx_ensemble_create(len(self.dims), flat, _dptr(t), _PREC[precision],
                                     ctypes.byref(self._h)), "ensemble_create")

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            self._L.lbx_ensemble_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def init_box(self, b, rho_c, u_c):
        r = np.ascontiguousarray(rho_c, dtype=np.float64)
        u = np.ascontiguousarray(u_c, dtype=np.float64)
        _check(self._L.lbx_ensemble_init_box(self._h, b, _dptr(r), r.size, _dptr(u), u.size), "init_box")

    def autotune(self, trial_steps=6):
        c = (ctypes.c_int * 3)()
        _check(self._L.lbx_ensemble_autotune(self._h, trial_steps, c), "autotune")
        return tuple(c)

    def set_config(self, tile_cells, block, cells_per_thread):
        _check(self._L.lbx_ensemble_set_config(self._h, tile_cells, block, cells_per_thread), "set_config")

    def iterate(self, n):
        _check(self._L.lbx_ensemble_iterate(self._h, n), "ensemble_iterate")

    def iterate_timed(self, n) -> float:
        ms = ctypes.c_double()
        _check(self._L.lbx_ensemble_iterate_timed(self._h, n, ctypes.byref(ms)), "iterate_timed")
        return ms.value

    def launches(self) -> int:
        n = ctypes.c_longlong()
        _check(self._L.lbx_ensemble_launches(self._h, ctypes.byref(n)), "launches")
        return n.value

    def copy_f(self, b):
        nx, ny, nz = self.dims[b]
        out = np.empty((NV, nz, ny, nx))
        _check(self._L.lbx_ensemble_copy_f(self._h, b, _dptr(out), out.size), "ensemble_copy_f")
        return out

    def hydro(self, b):
        nx, ny, nz = self.dims[b]
        rho = np.empty((nz, ny, nx))
        u = np.empty((3, nz, ny, nx))
        _check(self._L.lbx_ensemble_hydro(self._h, b, _dptr(rho), _dptr(u), rho.size), "ensemble_hydro")
        return rho, u

    def synchronize(self):
        _check(self._L.lbx_ensemble_synchronize(self._h), "ensemble_synchronize")
