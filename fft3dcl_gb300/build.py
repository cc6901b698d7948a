"""Build recipe of the CUDA engine library (sm_103a) and its plugin.

    python -m fft3dcl_gb300.build          # or __graft_entry__.build()

Compiles the translation units under csrc/ in parallel with nvcc
(-gencode arch=compute_103a,code=sm_103a) into _build/, links
lib/libfft3d_gb300.so (the C ABI of include/fft3d_gb300.h) and, when the
VapourSynth API-4 headers can be found, lib/libfft3dcl.so (the VapourSynth
plugin exporting VapourSynthPluginInit2). Objects are rebuilt only when a
source or header is newer. Cross-compiles without a GPU.
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
INC = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "_build")
LIBDIR = os.path.join(PKG, "lib")
LIB = os.path.join(LIBDIR, "libfft3d_gb300.so")
PLUGIN = os.path.join(LIBDIR, "libfft3dcl.so")
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
EXACT_BW = (4, 8, 16, 32, 64)

NVCC_COMMON = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                      "-I", INC, "-I", CSRC, "--expt-relaxed-constexpr"]
# Exact form: no fused multiply-add, IEEE division and square root, no
# flush-to-zero -- every fp32 operation rounds like the reference CPU code.
NVCC_EXACT = ["--fmad=false", "-prec-div=true", "-prec-sqrt=true", "-ftz=false"]
# Fast and tensor-core forms: FMA and the hardware reciprocal / square root.
NVCC_FAST = ["--fmad=true", "-ftz=true", "-prec-div=false", "-prec-sqrt=false"]
# Host code builds the tables the kernels read; GCC fuses multiply-adds in
# C++ by default on aarch64, which would change their last bits there.
HOST_CXX = ["-std=c++17", "-O2", "-fPIC", "-Wall", "-ffp-contract=off"]


def _units():
    """(object, command, sources the object depends on) for every unit."""
    headers = glob.glob(os.path.join(CSRC, "*.hpp")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        glob.glob(os.path.join(INC, "*.h"))
    units = []
    src = os.path.join(CSRC, "f3d_k_exact.cu")
    for bw in EXACT_BW:
        obj = os.path.join(BUILD, f"f3d_k_exact_bw{bw}.o")
        units.append((obj, [NVCC] + NVCC_COMMON + NVCC_EXACT + [f"-DF3D_BW={bw}", "-c", src, "-o", obj],
                       [src] + headers))
    for name, extra in (("f3d_k_common.cu", NVCC_EXACT), ("f3d_k_big.cu", NVCC_EXACT), ("f3d_k_fast.cu", NVCC_FAST),
                        ("f3d_k_sweep.cu", NVCC_FAST), ("f3d_k_tc.cu", NVCC_FAST + ["-Xcompiler", "-ffp-contract=off"]),
                        ("f3d_noalloc.cu", NVCC_EXACT + ["-Xcompiler", "-ffp-contract=off"])):
        src = os.path.join(CSRC, name)
        if not os.path.exists(src):
            continue
        obj = os.path.join(BUILD, name.replace(".cu", ".o"))
        units.append((obj, [NVCC] + NVCC_COMMON + extra + ["-c", src, "-o", obj], [src] + headers))
    for name in ("f3d_engine.cpp", "f3d_batch.cpp", "f3d_serve.cpp"):
        src = os.path.join(CSRC, name)
        if not os.path.exists(src):
            continue
        obj = os.path.join(BUILD, name.replace(".cpp", ".o"))
        units.append((obj, ["g++"] + HOST_CXX + ["-I", INC, "-I", CSRC,
                            "-I", os.path.join(CUDA, "include"), "-c", src, "-o", obj], [src] + headers))
    return units


def _stale(obj, deps):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build step failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return r.stderr


VS_HEADERS = ("VapourSynth4.h", "VSHelper4.h")
VS_CACHE = os.path.join(BUILD, "vsinclude")


def _has_vs_headers(d: str) -> bool:
    return bool(d) and all(os.path.exists(os.path.join(d, h)) for h in VS_HEADERS)


def vs_include_dir():
    """Directory holding the VapourSynth API-4 headers (VapourSynth4.h,
    VSHelper4.h; LGPL, not part of this repository), or None.

    Looked up in $VAPOURSYNTH_INCLUDE, the usual system locations and
    _build/vsinclude. Headers found elsewhere are copied into _build/vsinclude
    (git-ignored), so that a build from a copy of this working tree on another
    machine finds them too."""
    for c in (os.environ.get("VAPOURSYNTH_INCLUDE", ""), "/usr/include/vapoursynth",
              "/usr/local/include/vapoursynth"):
        if _has_vs_headers(c):
            os.makedirs(VS_CACHE, exist_ok=True)
            for h in VS_HEADERS:
                dst = os.path.join(VS_CACHE, h)
                if not os.path.exists(dst) or os.path.getmtime(dst) < os.path.getmtime(os.path.join(c, h)):
                    shutil.copy(os.path.join(c, h), dst)
            return c
    return VS_CACHE if _has_vs_headers(VS_CACHE) else None


def build(verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    units = _units()
    todo = [(o, c) for (o, c, d) in units if _stale(o, d)]
    jobs = max(2, min(len(todo), os.cpu_count() or 4))
    if todo:
        with cf.ThreadPoolExecutor(jobs) as ex:
            for out in ex.map(lambda oc: _run(oc[1]), todo):
                if verbose and out:
                    print(out, file=sys.stderr)
    objs = [o for (o, c, d) in units]
    if _stale(LIB, objs):
        _run([NVCC] + ARCH + ["-shared", "-o", LIB] + objs + ["-lpthread"])
    vsinc = vs_include_dir()
    psrc = os.path.join(CSRC, "f3d_plugin.cpp")
    if not vsinc:
        print("fft3dcl_gb300.build: VapourSynth API-4 headers not found ($VAPOURSYNTH_INCLUDE); "
              "the plugin library is not built", file=sys.stderr)
    if vsinc and os.path.exists(psrc):
        pobj = os.path.join(BUILD, "f3d_plugin.o")
        if _stale(pobj, [psrc] + glob.glob(os.path.join(CSRC, "*.hpp"))):
            _run(["g++"] + HOST_CXX + ["-I", INC, "-I", CSRC, "-I", vsinc,
                  "-c", psrc, "-o", pobj])
        if _stale(PLUGIN, [pobj] + objs):
            _run([NVCC] + ARCH + ["-shared", "-o", PLUGIN, pobj] + objs + ["-lpthread"])
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
