"""Build recipe for the engine's shared library (sm_103a only).

Compiles every ``csrc/*.cu`` translation unit in parallel with nvcc and links
``_build/libknngb300.so`` (C ABI: include/knn_gb300.h and include/cuknns.h).
No cmake, no torch extension machinery: plain ``nvcc -shared``.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libknngb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    p = shutil.which("nvcc")
    if p:
        return p
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found")


def _flags(extra=()):
    return (ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O3", "--expt-relaxed-constexpr",
                    "-I", os.path.join(HERE, "..", "include")] + list(extra))


def _compile(src: str, verbose_ptxas: bool) -> str:
    obj = os.path.join(BUILD, os.path.basename(src)[:-3] + ".o")
    deps = [src] + glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h")) + \
        glob.glob(os.path.join(HERE, "..", "include", "*.h"))
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(d) for d in deps):
        return obj
    extra = ["-Xptxas", "-v"] if verbose_ptxas else []
    cmd = [nvcc(), "-c", src, "-o", obj] + _flags(extra)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    if verbose_ptxas:
        sys.stderr.write(r.stderr)
    return obj


LIB_F64 = os.path.join(BUILD, "libknngb300_double.so")
CSRC_F64 = os.path.join(HERE, "csrc_f64")
# the double library exports the reference's names with double arguments and its own status API only
F64_EXPORTS = ["gpuknnsBitonic", "gpuknnsHeap", "knnsplan", "knnsexecute", "knns_search_device_f64",
               "knns_search_host_f64", "knns_f64_last_error"]


def _compile_f64(src: str, verbose_ptxas: bool) -> str:
    obj = os.path.join(BUILD, "f64_" + os.path.basename(src)[:-3] + ".o")
    deps = [src] + glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h")) + \
        glob.glob(os.path.join(HERE, "..", "include", "*.h"))
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(d) for d in deps):
        return obj
    extra = (["-Xptxas", "-v"] if verbose_ptxas else []) + ["-D__DOUBLE__", "-I", CSRC]
    cmd = [nvcc(), "-c", src, "-o", obj] + _flags(extra)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def build_f64(float_objs, verbose_ptxas: bool = False) -> str:
    """libknngb300_double.so: the double drop-in plus the engine objects (its float shortlist stage)."""
    srcs = sorted(glob.glob(os.path.join(CSRC_F64, "*.cu")))
    objs = [_compile_f64(s, verbose_ptxas) for s in srcs]
    engine = [o for o in float_objs if os.path.basename(o) != "dropin.o"]
    allo = objs + engine
    if os.path.exists(LIB_F64) and os.path.getmtime(LIB_F64) >= max(os.path.getmtime(o) for o in allo):
        return LIB_F64
    vs = os.path.join(BUILD, "f64.version")
    with open(vs, "w") as f:
        f.write("{ global: " + " ".join(n + ";" for n in F64_EXPORTS) + " local: *; };\n")
    tmp = LIB_F64 + ".tmp"
    cmd = [nvcc(), "-shared", "-o", tmp] + allo + ARCH + ["-Xcompiler", "-fPIC",
                                                          "-Xlinker", "--version-script=" + vs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link (double) failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB_F64)
    return LIB_F64


APPS = os.path.join(HERE, "apps")


def build_apps() -> list:
    """knn_test / knn_test_double: the reference's file-based driver (src/knnTest.cu) over the libraries."""
    out = []
    inc = os.path.join(HERE, "..", "include")
    for name, lib, extra in (("knn_test", "knngb300", []), ("knn_test_double", "knngb300_double", ["-D__DOUBLE__"])):
        src = os.path.join(APPS, "knn_test.cpp")
        exe = os.path.join(BUILD, name)
        libf = os.path.join(BUILD, "lib" + lib + ".so")
        if os.path.exists(exe) and os.path.getmtime(exe) >= max(os.path.getmtime(src), os.path.getmtime(libf)):
            out.append(exe)
            continue
        cmd = ["g++", "-O2", "-std=c++17", "-I", inc] + extra + [src, "-o", exe, "-L", BUILD, "-l" + lib,
                                                                 "-Wl,-rpath," + BUILD]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"g++ failed for {name}:\n{r.stdout}\n{r.stderr}")
        out.append(exe)
    return out


def build(force: bool = False, verbose_ptxas: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    if force:
        for f in glob.glob(os.path.join(BUILD, "*.o")):
            os.remove(f)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose_ptxas), srcs))
    build_f64(objs, verbose_ptxas)
    if not (os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(o) for o in objs)):
        tmp = LIB + ".tmp"
        cmd = [nvcc(), "-shared", "-o", tmp] + objs + ARCH + ["-Xcompiler", "-fPIC"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB)
    build_apps()
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose_ptxas="-v" in sys.argv))
