"""Builds the engine library libgbhsolve.so in-tree for sm_103a (GB300).

The CUDA/C++ translation units are compiled in parallel:
  gbh_k64.cu    FP64 kernels, --fmad=false (bit-level parity with the CPU solver)
  gbh_k32.cu    mixed-precision kernels (FP32 gates), contraction allowed
  gbh_adjoint.cu adjoint (gradient) kernels of the FP64 form, --fmad=false
  gbh_engine.cu host layout, launches and the C ABI
  gbh_decode.cpp ops[]/funcs[] decoder
  gbh_hsolve.cpp hsolve-level ABI: many hsolves in one batch engine
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(ROOT, "csrc")
REPO = os.path.dirname(ROOT)
INCLUDE = os.path.join(REPO, "include")
OUT_DIR = os.path.join(PKG, "_lib")
LIB = os.path.join(OUT_DIR, "libgbhsolve.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _sources():
    return [os.path.join(CSRC, f) for f in sorted(os.listdir(CSRC))
            if f.endswith((".cu", ".cpp", ".cuh", ".h"))] + [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]


def up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(s) <= t for s in _sources())


JIT_HEADERS = ["gbh_internal.h", "gbh_df.cuh", "gbh_devfn.cuh"]
STDINT_STUB = ("typedef signed char int8_t; typedef short int16_t; typedef int int32_t; "
               "typedef long long int64_t; typedef unsigned char uint8_t; typedef unsigned short uint16_t; "
               "typedef unsigned int uint32_t; typedef unsigned long long uint64_t;")


def _write_jit_sources(path):
    """Embeds the device headers the runtime compiler needs as C string literals."""
    lines = ["// generated by gbhsolve/build.py: device headers for the runtime compiler", "#pragma once"]
    for h in JIT_HEADERS:
        text = open(os.path.join(CSRC, h)).read()
        name = "kSrc_" + h.replace(".", "_")
        lines.append('static const char %s[] = R"GBHSRC(%s)GBHSRC";' % (name, text))
    lines.append('static const char kStdintStub[] = "%s";' % STDINT_STUB)
    new = "\n".join(lines) + "\n"
    if not os.path.exists(path) or open(path).read() != new:
        with open(path, "w") as f:
            f.write(new)


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and up_to_date():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    obj_dir = os.path.join(OUT_DIR, "obj")
    os.makedirs(obj_dir, exist_ok=True)
    cc = nvcc()
    common = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2",
                     "-I" + CSRC, "-I" + INCLUDE]
    gen_dir = os.path.join(OUT_DIR, "gen")
    os.makedirs(gen_dir, exist_ok=True)
    _write_jit_sources(os.path.join(gen_dir, "gbh_jit_sources.h"))
    common = common + ["-I" + gen_dir]
    units = [
        ("gbh_k64.cu", ["--fmad=false", "-Xptxas", "-v"] if verbose else ["--fmad=false"]),
        ("gbh_k32.cu", ["-Xptxas", "-v"] if verbose else []),
        ("gbh_adjoint.cu", ["--fmad=false", "-Xptxas", "-v"] if verbose else ["--fmad=false"]),
        ("gbh_engine.cu", []),
        ("gbh_noalloc.cu", []),
        ("gbh_decode.cpp", []),
        ("gbh_hsolve.cpp", []),
        ("gbh_jit.cu", []),
    ]

    def compile_unit(u):
        src, extra = u
        obj = os.path.join(obj_dir, src.rsplit(".", 1)[0] + ".o")
        cmd = [cc] + common + extra + ["-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd), r.stderr))
        return obj, r.stderr

    with ThreadPoolExecutor(max_workers=len(units)) as ex:
        results = list(ex.map(compile_unit, units))
    if verbose:
        for _, log in results:
            if log:
                print(log)
    objs = [o for o, _ in results]
    tmp = LIB + ".tmp"
    cmd = [cc] + ARCH + ["-shared", "-o", tmp] + objs + ["-ldl"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s" % r.stderr)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
