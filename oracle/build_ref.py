"""Recipe for oracle/_ref: the reference's own code, compiled from its sources.

Test infrastructure only (the checker, never the product).  The library
oracle/_ref/libref_merge.so holds the reference's float path as the reference
builds it (src/cuknnBitonic.cu and src/cuknnHeap.cu, Makefile:53-56):

* the host merges of per-stream results, mergeResBitonic
  (src/cuknnBitonic.cu:381-417) and mergeResHeap (src/cuknnHeap.cu:26-59),
  exposed under C names by oracle/ref_merge_bitonic.cu and
  oracle/ref_merge_heap.cu (each includes the reference file it names);
* the reference's drivers gpuknnsBitonic (src/cuknnBitonic.cu:422-618) and
  gpuknnsHeap (src/cuknnHeap.cu:394-575), exported by those files themselves.

tests/test_oracle.py pins the oracle's merge restatement against the merges on
the CPU; tests/golden/make_ref_fixtures.py runs the drivers on a GB300 to write
the reference's own answers for the 65,536 x 128 and 1,000,000 x 128 workloads
(tests/golden/ref_*.npz), which the GPU tests hold the engine to.

Where the reference sources are read from (first that exists):
  1. $KNN_REFERENCE_DIR;
  2. /root/reference, the read-only mount of the reference project;
  3. oracle/_ref/src, an unmodified copy of the five files the build needs,
     staged from (1) or (2) by ``stage()`` so that the recipe also runs on a
     machine without the mount.  oracle/_ref is git-ignored: the copy is never
     committed.
oracle/ref_shim/cublas.h empties the legacy cuBLAS header, which current cuBLAS
refuses beside cublas_v2.h (src/cuknnBitonic.cu:6-7, src/cuknnHeap.cu:5-6).
"""
import os
import shutil
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
MOUNT = "/root/reference"
OUT = os.path.join(ROOT, "oracle", "_ref")
STAGED = os.path.join(OUT, "src")
LIB = "libref_merge.so"
UNITS = (("ref_merge_bitonic.cu", "src/cuknnBitonic.cu"), ("ref_merge_heap.cu", "src/cuknnHeap.cu"))
# every file the two units read (includes are relative to src/ and include/)
FILES = ("src/cuknnBitonic.cu", "src/cuknnHeap.cu", "include/cuknns.h", "include/utils.h",
         "include/shared_functions.h")


def _complete(d: str) -> bool:
    return bool(d) and all(os.path.exists(os.path.join(d, f)) for f in FILES)


def mounted_dir():
    """The reference project as mounted (environment variable, then the usual mount), or None."""
    for d in (os.environ.get("KNN_REFERENCE_DIR", ""), MOUNT):
        if _complete(d):
            return d
    return None


def source_dir():
    """Where the build reads the reference sources: the mount, else the staged copy, else None."""
    d = mounted_dir()
    if d:
        return d
    return STAGED if _complete(STAGED) else None


def available() -> bool:
    return source_dir() is not None


def lib_path() -> str:
    return os.path.join(OUT, LIB)


def stage() -> bool:
    """Copy the files the build needs, unmodified, from the mount into oracle/_ref/src."""
    src = mounted_dir()
    if not src:
        return False
    for f in FILES:
        dst = os.path.join(STAGED, f)
        os.makedirs(os.path.dirname(dst), exist_ok=True)
        if not (os.path.exists(dst) and os.path.getmtime(dst) >= os.path.getmtime(os.path.join(src, f))):
            shutil.copyfile(os.path.join(src, f), dst)
    return True


def build_if_available() -> bool:
    """Build oracle/_ref/libref_merge.so; False when no reference sources are at hand."""
    stage()
    ref = source_dir()
    if ref is None:
        return False
    out = lib_path()
    deps = [os.path.join(ROOT, "oracle", w) for w, _ in UNITS] + [os.path.join(ref, f) for f in FILES]
    deps.append(os.path.join(ROOT, "oracle", "ref_shim", "cublas.h"))
    if os.path.exists(out) and all(os.path.getmtime(out) >= os.path.getmtime(d) for d in deps):
        return True
    os.makedirs(OUT, exist_ok=True)
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    tmp = out + ".tmp"
    cmd = [nvcc, "-shared", "-Xcompiler", "-fPIC", "-O2", "-w",
           "-gencode", "arch=compute_103a,code=sm_103a",
           "-D", "CUARCH=103",  # the reference's build passes its target as CUARCH (Makefile:53-56)
           "-I", os.path.join(ROOT, "oracle", "ref_shim"),
           "-I", os.path.join(ref, "src"), "-I", os.path.join(ref, "include")]
    cmd += [os.path.join(ROOT, "oracle", w) for w, _ in UNITS] + ["-o", tmp, "-lcublas", "-lcuda"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("building oracle/_ref/%s failed:\n%s" % (LIB, (r.stdout + r.stderr)[-4000:]))
    os.replace(tmp, out)
    return True


def load():
    """Load the reference library.  Its search entry points call the CUDA driver API
    (cuStreamCreate, cuMemGetInfo, ...); where no driver is installed the toolkit's
    link stub provides the symbols, which is enough for the merges (they never call it)."""
    import ctypes
    if not os.path.exists(lib_path()):
        raise FileNotFoundError(lib_path())
    try:
        ctypes.CDLL("libcuda.so.1", mode=ctypes.RTLD_GLOBAL)
    except OSError:
        for d in (os.environ.get("CUDA_HOME", ""), "/usr/local/cuda"):
            stub = os.path.join(d, "lib64", "stubs", "libcuda.so")
            if d and os.path.exists(stub):
                ctypes.CDLL(stub, mode=ctypes.RTLD_GLOBAL)
                break
    return ctypes.CDLL(lib_path())


if __name__ == "__main__":
    if "--stage" in sys.argv:
        print("staged" if stage() else "reference sources absent: nothing staged")
    else:
        print("built" if build_if_available() else "reference sources absent: nothing built")
