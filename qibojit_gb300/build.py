"""Build the engine library ``qibojit_gb300/libqibojit_gb300.so`` for sm_103a.

Each ``csrc/*.cu`` translation unit is compiled in parallel with nvcc (one
``-gencode``, ``-lineinfo``) and linked into one shared library with a plain C ABI
(declared in ``include/qibojit_gb300.h``).  The library is built in-tree so the
Python layer (and any process using the engine) loads it from the package folder.
No cmake; host code is portable C++17 (the same recipe builds on x86_64 and
aarch64).
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libqibojit_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the engine library cannot be built")


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def _deps():
    return _sources() + glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(INCLUDE, "*.h"))


def up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(d) <= t for d in _deps())


def _embed_device_header() -> None:
    """The run-time pass specialiser compiles generated kernels together with
    ``csrc/sv_device.cuh``; its text goes into the library as a C string."""
    with open(os.path.join(CSRC, "sv_device.cuh")) as f:
        text = f.read()
    delim = "SVDEVICE"
    assert f"){delim}\"" not in text
    out = os.path.join(BUILD, "sv_device_text.inc")
    body = f'static const char kDeviceHeaderText[] = R"{delim}({text}){delim}";\n'
    if not os.path.exists(out) or open(out).read() != body:
        with open(out, "w") as f:
            f.write(body)


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and up_to_date():
        return LIB
    nvcc = _nvcc()
    os.makedirs(BUILD, exist_ok=True)
    _embed_device_header()
    common = ["-std=c++17", "-O3", "-lineinfo", *ARCH, "-Xcompiler", "-fPIC", f"-I{INCLUDE}", f"-I{CSRC}", f"-I{BUILD}"]

    def compile_one(src):
        obj = os.path.join(BUILD, os.path.basename(src)[:-3] + ".o")
        cmd = [nvcc, *common, "-c", src, "-o", obj]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {os.path.basename(src)}:\n{r.stdout}\n{r.stderr}")
        return obj

    srcs = _sources()
    with cf.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = LIB + ".tmp"
    cmd = [nvcc, *ARCH, "-shared", "-cudart", "static", "-o", tmp, *objs, "-ldl"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
