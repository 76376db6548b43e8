"""Recipe for oracle/_ref: the reference's own host merges, compiled from its sources.

Test infrastructure only (the checker, never the product): the two host-side merges
of per-stream results on the reference's path -- mergeResBitonic
(src/cuknnBitonic.cu:381-417) and mergeResHeap (src/cuknnHeap.cu:26-59) -- are plain
host functions.  Each is compiled from the reference's source file where it lies,
through a wrapper that includes that file and exposes the merge under a C name
(oracle/ref_merge_bitonic.cu, oracle/ref_merge_heap.cu); the two units are linked into
one library as the reference links them (cuknnBitonic.cu launches kernels that
cuknnHeap.cu defines through include/utils.h).  oracle/ref_shim/cublas.h empties the
legacy cuBLAS header, which current cuBLAS refuses beside cublas_v2.h.  The device code
is compiled but never run: the merges need no GPU, so tests/test_oracle.py pins the
oracle's merge restatement against them on the CPU.

Runs only where the reference sources are mounted; elsewhere (the GPU host) it does
nothing and the pinning test skips.
"""
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = "/root/reference"
OUT = os.path.join(ROOT, "oracle", "_ref")
LIB = "libref_merge.so"
UNITS = (("ref_merge_bitonic.cu", "src/cuknnBitonic.cu"), ("ref_merge_heap.cu", "src/cuknnHeap.cu"))


def available() -> bool:
    return all(os.path.exists(os.path.join(REF, src)) for _, src in UNITS)


def lib_path() -> str:
    return os.path.join(OUT, LIB)


def build_if_available() -> bool:
    """Build oracle/_ref/libref_merge.so from the mounted reference sources; False when absent."""
    if not available():
        return False
    out = lib_path()
    deps = [os.path.join(ROOT, "oracle", w) for w, _ in UNITS] + [os.path.join(REF, s_) for _, s_ in UNITS]
    deps.append(os.path.join(ROOT, "oracle", "ref_shim", "cublas.h"))
    if os.path.exists(out) and all(os.path.getmtime(out) >= os.path.getmtime(d) for d in deps):
        return True
    os.makedirs(OUT, exist_ok=True)
    cmd = ["nvcc", "-shared", "-Xcompiler", "-fPIC", "-O2", "-w",
           "-gencode", "arch=compute_103a,code=sm_103a",
           "-D", "CUARCH=103",  # the reference's build passes its target as CUARCH (Makefile:53-56)
           "-I", os.path.join(ROOT, "oracle", "ref_shim"),
           "-I", os.path.join(REF, "src"), "-I", os.path.join(REF, "include")]
    cmd += [os.path.join(ROOT, "oracle", w) for w, _ in UNITS] + ["-o", out, "-lcublas"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("building oracle/_ref/%s failed:\n%s" % (LIB, (r.stdout + r.stderr)[-4000:]))
    return True


def load():
    """Load the merge library.  The reference's files also call the CUDA driver API
    (cuStreamCreate, cuMemGetInfo, ... in their search entry points); the merges never
    do, so where no driver is installed the toolkit's link stub provides the symbols."""
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
    print("built" if build_if_available() else "reference sources absent: nothing built")
