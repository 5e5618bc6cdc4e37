"""In-tree build of liblbx_cuda.so for sm_103a (nvcc, no cmake).

Each translation unit is compiled in its own nvcc process (in parallel), then
linked into ``lambrex_gb300/liblbx_cuda.so`` with the static CUDA runtime.
``build("checked")`` makes the debug variant ``liblbx_cuda_checked.so``:
the same sources with LBX_CHECKED, which bounds-checks every global load and
store of the kernels (csrc/checked.cuh).
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
VARIANTS = {
    "release": ([], os.path.join(PKG, "_build"), os.path.join(PKG, "liblbx_cuda.so")),
    "checked": (["-DLBX_CHECKED"], os.path.join(PKG, "_build_checked"),
                os.path.join(PKG, "liblbx_cuda_checked.so")),
}
OBJ = VARIANTS["release"][1]
LIB = VARIANTS["release"][2]

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              "-I" + INCLUDE, "-I" + CSRC]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build liblbx_cuda.so")


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def _headers():
    return (glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h"))
            + glob.glob(os.path.join(INCLUDE, "*.h")))


def _newest(paths):
    return max((os.path.getmtime(p) for p in paths), default=0.0)


def _compile(src: str, hdr_time: float, objdir: str, defines) -> str:
    obj = os.path.join(objdir, os.path.basename(src)[:-3] + ".o")
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(src), hdr_time):
        return obj
    tmp = obj + ".tmp%d" % os.getpid()
    cmd = [nvcc()] + ARCH + NVCC_FLAGS + list(defines) + ["-c", src, "-o", tmp]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, res.stdout, res.stderr))
    os.replace(tmp, obj)
    return obj


def build(variant: str = "release", force: bool = False, jobs: int | None = None) -> str:
    """Compile and link the library variant ("release" or "checked");
    returns its path."""
    if variant not in VARIANTS:
        raise ValueError("unknown library variant %r" % variant)
    defines, objdir, lib = VARIANTS[variant]
    os.makedirs(objdir, exist_ok=True)
    srcs = _sources()
    hdr_time = _newest(_headers())
    if force:
        for o in glob.glob(os.path.join(objdir, "*.o")):
            os.remove(o)
    jobs = jobs or min(len(srcs), os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        objs = list(ex.map(lambda s: _compile(s, hdr_time, objdir, defines), srcs))
    if os.path.exists(lib) and os.path.getmtime(lib) >= _newest(objs) and not force:
        return lib
    tmp = lib + ".tmp%d" % os.getpid()
    cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-cudart", "static"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (res.stdout, res.stderr))
    os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    print(build())
