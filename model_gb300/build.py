"""Build the in-tree CUDA library model_gb300/libga_anelastic.so for sm_103a.

Three translation units compiled in parallel with nvcc, then linked:
  ga_f64.cu  FP64 engine, --fmad=false (no contraction: the parity path)
  ga_f32.cu  FP32 engine
  ga_api.cu  the extern "C" boundary of include/ga_anelastic.h
  ga_noalloc.cu  FP64 pressure solve with file-scope scratch (no allocation)
and the run driver model_gb300/ga_driver (csrc/ga_driver.cpp, host C++ on the
C ABI, linked against the library).
Objects go to model_gb300/_build/ (git-ignored).  A rebuild happens only
when a source is newer than the library.
"""
from __future__ import annotations

import glob
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libga_anelastic.so")
DRIVER = os.path.join(PKG, "ga_driver")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# -ffp-contract=off for host code too: the host builds the sponge, Rayleigh and
# spectral tables, and GCC on Arm would otherwise fuse their multiply-adds
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
          "-Xcompiler", "-ffp-contract=off",
          "-I" + os.path.join(ROOT, "include")]
UNITS = {
    "ga_f64": ["--fmad=false"],
    "ga_f32": [],
    "ga_api": [],
    "ga_noalloc": ["--fmad=false"],
}


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found")
    return cand


def _sources():
    return glob.glob(os.path.join(CSRC, "*")) + [os.path.join(ROOT, "include", "ga_anelastic.h"),
                                                 os.path.abspath(__file__)]


def up_to_date() -> bool:
    if not os.path.exists(LIB) or not os.path.exists(DRIVER):
        return False
    t = min(os.path.getmtime(LIB), os.path.getmtime(DRIVER))
    return all(os.path.getmtime(s) <= t for s in _sources())


def build_driver() -> str:
    """The C++ run driver on the C ABI (links the library by $ORIGIN)."""
    cxx = shutil.which("g++") or "g++"
    tmp = DRIVER + ".tmp"
    cmd = [cxx, "-O2", "-std=c++17", "-I" + os.path.join(ROOT, "include"), os.path.join(CSRC, "ga_driver.cpp"),
           "-L" + PKG, "-lga_anelastic", "-Wl,-rpath,$ORIGIN", "-o", tmp]
    subprocess.run(cmd, check=True)
    os.replace(tmp, DRIVER)
    return DRIVER


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and up_to_date():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    nv = nvcc()
    procs = []
    for unit, extra in UNITS.items():
        src = os.path.join(CSRC, unit + ".cu")
        obj = os.path.join(BUILD, unit + ".o")
        cmd = [nv, *ARCH, *COMMON, *extra, "-c", src, "-o", obj]
        if verbose:
            print(" ".join(cmd))
        procs.append((unit, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    failed = []
    for unit, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            failed.append((unit, out.decode(errors="replace")))
        elif verbose and out:
            print(out.decode(errors="replace"))
    if failed:
        msg = "\n".join(f"--- {u}\n{o}" for u, o in failed)
        raise RuntimeError("nvcc failed:\n" + msg)
    objs = [os.path.join(BUILD, u + ".o") for u in UNITS]
    tmp = LIB + ".tmp"
    cmd = [nv, *ARCH, "-shared", "-o", tmp, *objs]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    build_driver()
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
