"""CPU tests of the C ABI: the library loads, exports every function that
include/lbx.h declares, and rejects bad arguments without touching a GPU."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def L():
    from lambrex_gb300 import build as B
    path = B.build()
    return ctypes.CDLL(path)


def declared_functions():
    src = open(os.path.join(ROOT, "include", "lbx.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"\b(lbx_[a-z0-9_]+)\s*\(", src)
    return sorted(set(names))


def test_header_declares_functions():
    names = declared_functions()
    assert "lbx_create" in names and "lbx_iterate" in names
    assert len(names) > 30


@pytest.mark.parametrize("name", declared_functions())
def test_symbol_exported(L, name):
    assert hasattr(L, name), name


@pytest.fixture(scope="module")
def L_checked():
    from lambrex_gb300 import build as B
    return ctypes.CDLL(B.build("checked"))


def test_checked_variant_exports_the_same_api(L_checked):
    missing = [n for n in declared_functions() if not hasattr(L_checked, n)]
    assert not missing


def test_checkpoint_read_rejects_missing_and_foreign_files(L, tmp_path):
    """Header validation happens before any device work."""
    h = ctypes.c_void_p()
    L.lbx_checkpoint_read.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_void_p)]
    assert L.lbx_checkpoint_read(str(tmp_path / "none.lbx").encode(), ctypes.byref(h)) == 9
    bad = tmp_path / "bad.lbx"
    bad.write_bytes(b"NOTACKPT" + bytes(200))
    assert L.lbx_checkpoint_read(str(bad).encode(), ctypes.byref(h)) == 9
    assert h.value is None
    L.lbx_status_string.restype = ctypes.c_char_p
    assert b"checkpoint" in L.lbx_status_string(9)


def _ckpt_header(levels, n=(16, 16, 16), amr_mode=1, max_level=2):
    """Checkpoint header and level records as lbx_checkpoint_write lays them
    out (little-endian): magic, version, precision, coupling mode, extents,
    max level, finest level, rates and shift; per level its valid box, time,
    dt, rates, mass and step.  No population data follows."""
    import struct
    out = struct.pack("<8s8i3d", b"LBXCKPT1", 1, 0, amr_mode, *n, max_level,
                      len(levels) - 1, 0.8, 0.8, 0.0)
    for lo, hi in levels:
        out += struct.pack("<6i5dq", *lo, *hi, 0.0, 1.0, 0.8, 0.8, 1.0, 0)
    return out


def test_checkpoint_read_validates_fine_levels(L, tmp_path):
    """A fine level must be the refinement of a tag box that
    lbx_set_static_refinement would accept; anything else is LBX_ERR_IO
    before any device work."""
    import torch
    L.lbx_checkpoint_read.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_void_p)]
    dom = ((0, 0, 0), (15, 15, 15))
    lev1 = ((8, 8, 8), (23, 23, 23))  # refine([4, 11]^3)
    cases = {
        "odd corner": [dom, ((9, 8, 8), (23, 23, 23))],
        "exchange ring wraps": [dom, ((0, 0, 0), (29, 29, 29))],  # refine([0, 14]^3)
        "no parent margin": [dom, lev1, ((16, 16, 16), (47, 47, 47))],  # refine([8, 23]^3)
        "outside the parent": [dom, lev1, ((4, 20, 20), (43, 43, 43))],
    }
    h = ctypes.c_void_p()
    for name, levels in cases.items():
        p = tmp_path / (name.replace(" ", "_") + ".lbx")
        p.write_bytes(_ckpt_header(levels))
        assert L.lbx_checkpoint_read(str(p).encode(), ctypes.byref(h)) == 9, name
        assert h.value is None
    if not torch.cuda.is_available():  # an acceptable layout gets as far as the device
        p = tmp_path / "nested.lbx"
        p.write_bytes(_ckpt_header([dom, lev1, ((20, 20, 20), (43, 43, 43))]))
        assert L.lbx_checkpoint_read(str(p).encode(), ctypes.byref(h)) == 3  # LBX_ERR_CUDA


def test_debug_bounds_is_unsupported_in_release(L):
    n, first = ctypes.c_longlong(7), ctypes.c_longlong(7)
    assert L.lbx_debug_bounds(ctypes.byref(n), ctypes.byref(first), 0) == 5  # LBX_ERR_UNSUPPORTED
    assert n.value == 0 and first.value == -1
    assert L.lbx_debug_bounds(None, ctypes.byref(first), 0) == 1


def test_status_strings(L):
    L.lbx_status_string.restype = ctypes.c_char_p
    for st in range(0, 9):
        assert L.lbx_status_string(st)
    assert L.lbx_status_string(0) == b"ok"


def test_sentinels(L):
    L.lbx_nl_density.restype = ctypes.c_double
    L.lbx_nl_velocity.restype = ctypes.c_double
    assert L.lbx_nl_density() == -1.0   # include/AmrSim.h:35
    assert L.lbx_nl_velocity() == -3e8  # include/AmrSim.h:36


def test_create_rejects_bad_arguments(L):
    h = ctypes.c_void_p()
    per = (ctypes.c_int * 3)(1, 1, 1)
    L.lbx_create.argtypes = [ctypes.c_int] * 4 + [ctypes.POINTER(ctypes.c_int), ctypes.c_double,
                                                  ctypes.c_double, ctypes.c_int, ctypes.c_int,
                                                  ctypes.POINTER(ctypes.c_void_p)]
    assert L.lbx_create(0, 4, 4, 0, per, 1.0, 1.0, 0, 0, ctypes.byref(h)) == 1   # LBX_ERR_ARG
    assert L.lbx_create(4, 4, 4, 0, per, 1.0, 1.0, 7, 0, ctypes.byref(h)) == 1
    # coupling modes 0 (faithful), 1 (conservative), 2 (rescaled); 3 is not one:
    # rejected before any device work, the valid ones pass the argument checks
    assert L.lbx_create(4, 4, 4, 1, per, 1.0, 1.0, 0, 3, ctypes.byref(h)) == 1
    nonper = (ctypes.c_int * 3)(1, 0, 1)
    for mode in (0, 1, 2):
        assert L.lbx_create(4, 4, 4, 1, nonper, 1.0, 1.0, 0, mode, ctypes.byref(h)) == 5
    # only periodic boundaries (src/AmrSim.cpp:795)
    assert L.lbx_create(4, 4, 4, 0, nonper, 1.0, 1.0, 0, 0, ctypes.byref(h)) == 5
    assert not h.value


def test_null_handles_are_rejected(L):
    L.lbx_iterate.argtypes = [ctypes.c_void_p, ctypes.c_int]
    assert L.lbx_iterate(None, 1) == 1
    L.lbx_destroy.argtypes = [ctypes.c_void_p]
    assert L.lbx_destroy(None) == 0
    # the tagging entry points (ErrorEst, the density criterion)
    tags = (ctypes.c_ubyte * 8)()
    L.lbx_error_est.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_size_t]
    assert L.lbx_error_est(None, 0, tags, 8) == 1
    lo, hi, n = (ctypes.c_int * 3)(), (ctypes.c_int * 3)(), ctypes.c_longlong(7)
    L.lbx_tag_density.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_double,
                                  ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    assert L.lbx_tag_density(None, 0, 0.01, lo, hi, ctypes.byref(n)) == 1
    assert n.value == 7  # untouched on an error


def test_python_binding_has_reference_method_names():
    from lambrex_gb300 import lbx
    for m in ("SetInitialDensity", "SetInitialVelocity", "InitFromScratch", "Iterate",
              "CalcHydroVars", "CalcEquilibriumDist", "GetDensity", "GetVelocity", "GetTime",
              "GetTimeStep", "GetDims", "OnProcessDensity", "OnProcessVelocity",
              "SetStaticRefinement", "UnsetStaticRefinement", "GetExtent", "ErrorEst", "maxLevel",
              "finestLevel", "refRatio"):
        assert hasattr(lbx.AmrSim, m), m
