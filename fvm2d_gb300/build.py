"""Build the C-ABI shared library ``_build/libfvm2d_gb300.so`` in-tree.

Every translation unit is compiled in parallel:
  * CUDA kernels for sm_103a only (``-gencode arch=compute_103a,code=sm_103a``);
    the FP64 kernels and the set-up kernels with ``--fmad=false`` so their
    arithmetic is rounded exactly as written; the FP32 kernels with
    contraction allowed, approximate division and square root (a few ulp)
    and subnormals flushed to zero (the FP32 path is checked against the
    FP64 oracle by tolerance);
  * host C++ with ``-ffp-contract=off`` (the driver-side geometry must equal
    the serial FP64 arithmetic on x86 and on Arm alike).
No CPU fallback is built: without this library the package refuses to run.

A second library, ``libfvm2d_gb300_fp64fma.so``, differs only in its FP64
kernels, compiled with FMA contraction: the FP64 method rounded as the
compiler pleases, not bitwise the reference, and faster on this GPU's FP64
pipe.  It is the fair FP64 baseline for speed comparisons; the package
loads it instead of the main library when FVM_LIB_VARIANT=fp64fma.
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import platform
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
INC = os.path.join(os.path.dirname(HERE), "include")
# FVM_BUILD_TAG / FVM_FP32_FLAGS / FVM_CXX_FLAGS select an alternative build
# (own directory)
TAG = os.environ.get("FVM_BUILD_TAG", "")
OUT = os.path.join(HERE, "_build", platform.machine() + (("-" + TAG) if TAG else ""))
LIB = os.path.join(OUT, "libfvm2d_gb300.so")
LIB_FP64FMA = os.path.join(OUT, "libfvm2d_gb300_fp64fma.so")

CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_COMMON = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                      "-Xcompiler", "-ffp-contract=off", "--expt-relaxed-constexpr",
                      f"-I{INC}", f"-I{SRC}"]
CXX_COMMON = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-Wextra",
              "-Wno-unused-parameter", f"-I{CUDA_HOME}/include", f"-I{INC}", f"-I{SRC}"]

UNITS = [
    ("fvm_kernels_fp64.cu", "nvcc", ["--fmad=false"]),
    ("fvm_kernels_fp64.cu@fma", "nvcc", ["--fmad=true"]),   # the FMA library only
    ("fvm_kernels_fp32.cu", "nvcc", os.environ.get(
        "FVM_FP32_FLAGS", "-prec-div=false -prec-sqrt=false -ftz=true").split()),
    ("fvm_setup.cu", "nvcc", ["--fmad=false"]),
    ("fvm_noalloc.cu", "nvcc", ["--fmad=false"]),
    ("fvm_geom_gpu.cu", "nvcc", ["--fmad=false"]),
    ("fvm_batch.cpp", "cxx", []),
    ("fvm_serve.cpp", "cxx", []),
    ("fvm_layout.cpp", "cxx", []),
    ("fvm_geometry.cpp", "cxx", []),
]


def _headers_digest() -> str:
    h = hashlib.sha256()
    for d in (SRC, INC):
        for n in sorted(os.listdir(d)):
            if n.endswith((".h", ".cuh")):
                with open(os.path.join(d, n), "rb") as f:
                    h.update(n.encode() + f.read())
    return h.hexdigest()


def _compile(unit, kind, extra, digest, verbose):
    src = os.path.join(SRC, unit.split("@")[0])
    obj = os.path.join(OUT, unit.replace("@", "_") + ".o")
    stamp = obj + ".stamp"
    with open(src, "rb") as f:
        key = hashlib.sha256(f.read() + digest.encode() + " ".join(extra).encode()).hexdigest()
    if os.path.exists(obj) and os.path.exists(stamp) and open(stamp).read() == key:
        return obj, ""
    # an alternative build reuses the main build's object of an unchanged unit
    base = os.path.join(os.path.dirname(OUT), platform.machine())
    bobj = os.path.join(base, os.path.basename(obj))
    if TAG and os.path.exists(bobj + ".stamp") and open(bobj + ".stamp").read() == key:
        shutil.copyfile(bobj, obj)
        with open(stamp, "w") as f:
            f.write(key)
        return obj, ""
    if kind == "nvcc":
        cmd = [NVCC] + NVCC_COMMON + extra + ["-c", src, "-o", obj]
    else:
        cmd = ([os.environ.get("CXX", "g++")] + CXX_COMMON + extra +
               os.environ.get("FVM_CXX_FLAGS", "").split() + ["-c", src, "-o", obj])
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    with open(stamp, "w") as f:
        f.write(key)
    return obj, (r.stderr if verbose else "")


def build(verbose: bool = False, ptxas_info: bool = False) -> str:
    """Compile and link the library; returns its path."""
    if not os.path.exists(NVCC):
        raise RuntimeError(f"nvcc not found at {NVCC}")
    os.makedirs(OUT, exist_ok=True)
    digest = _headers_digest()
    units = []
    for unit, kind, extra in UNITS:
        e = list(extra)
        if ptxas_info and kind == "nvcc":
            e += ["-Xptxas", "-v"]
        units.append((unit, kind, e))
    with cf.ThreadPoolExecutor(max_workers=len(units)) as ex:
        futs = [ex.submit(_compile, u, k, e, digest, verbose or ptxas_info) for u, k, e in units]
        objs = {}
        for (u, _, _), f in zip(units, futs):
            obj, log = f.result()
            objs[u] = obj
            if log:
                sys.stderr.write(log)
    main = [o for u, o in objs.items() if u != "fvm_kernels_fp64.cu@fma"]
    fma = [objs["fvm_kernels_fp64.cu@fma"] if u == "fvm_kernels_fp64.cu" else o
           for u, o in objs.items() if u != "fvm_kernels_fp64.cu@fma"]
    for lib, group in ((LIB, main), (LIB_FP64FMA, fma)):
        newest = max(os.path.getmtime(o) for o in group)
        if os.path.exists(lib) and os.path.getmtime(lib) >= newest:
            continue
        tmp = lib + ".tmp"
        cmd = [NVCC] + ARCH + ["-shared", "-o", tmp] + group + ["-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        shutil.move(tmp, lib)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, ptxas_info="--ptxas" in sys.argv))
