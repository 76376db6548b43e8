"""Golden answers of the reference's own CUDA library, for the GPU parity tests.

Run on a machine with a GB300 (the reference's drivers need a GPU) after
``oracle/build_ref.py`` has built oracle/_ref/libref_merge.so from the
reference's sources (the read-only mount, or the unmodified copy staged in
oracle/_ref/src):

    python tests/golden/make_ref_fixtures.py OUT_DIR

It calls the reference's heap driver exactly as its own C API does
(knnsexecute -> plan.pt2Function, src/knnsexecute.cu:14), with numStreams = 1:

* gpuknnsHeap (src/cuknnHeap.cu:394-575) on the 65,536 x 128 uniform [0,1)
  corpus with its 1,024 queries, k = 16, seed 0 -- the whole workload;
* gpuknnsHeap on the 1,000,000 x 128 integer-descriptor corpus, seed 1,
  k = 128 (its heap holds 2^floor(log2 k) entries, so k must be a power of
  two; the tests truncate to k = 100), in chunks of 250 queries: the driver
  sizes its N x Q distance buffer with int arithmetic
  (src/cuknnHeap.cu:476-496), and with more than 256 queries (BLOCKSIZE) its
  norm-add kernel pdot_v2 (include/utils.h:463-483, launched at :917-926) has
  no bound on the corpus row, which for 1,000,000 rows (not a multiple of its
  62 rows per block) runs past the distance buffer; at 250 queries it takes the
  bounded pdot (:442-461).  All forty chunks are run and timed; the answers of
  the first four (queries 0..999) are stored.

The reference's other driver, gpuknnsBitonic, is not called: its selection
kernels execute __syncthreads() inside `if (threadIdx.x < obj)`
(bitonic_shared, src/cuknnBitonic.cu:99-107; bitonic_shared2, :168-175), a
barrier that half of the block skips from the second merge round on.  That is
undefined on GPUs with independent thread scheduling, and on a GB300 the call
ran until its time limit.

Inputs are regenerated from the seeded generators of cuknns.synth and their
SHA-256 is stored beside the answers, so a test can check it holds the same
inputs.  The reference's outputs are stored as it returns them: k-leading
[query][rank] in its own (unsorted) order, distances with ||q||^2 added,
indices as 0-based floats (converted to int32 after an exactness check).

Environment: NVIDIA_TF32_OVERRIDE=0, so cuBLAS runs the reference's SGEMM in
plain FP32 (the reference never asks for TF32).  As in the reference's own
file driver (src/knnTest.cu:78-80), the inputs are page-locked host buffers,
allocated before the first call -- which also creates the CUDA context that the
drivers' first driver-API call (cuMemGetInfo, src/cuknnBitonic.cu:437) needs.
Before each call the script restates the driver's device-memory sizing
(src/cuknnBitonic.cu:519-536, src/cuknnHeap.cu:476-486) and refuses a call
whose corpus would not fit one block or whose N x Q int products reach 2^31.
"""
import ctypes
import hashlib
import json
import os
import sys
import time

os.environ["NVIDIA_TF32_OVERRIDE"] = "0"

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for p in (os.path.join(ROOT, "knn-toolbox_gb300"), os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)

import numpy as np  # noqa: E402

C2_CHUNK = 250
C2_KEEP = 1000


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def driver(lib, name):
    f = getattr(lib, name)
    fp = ctypes.POINTER(ctypes.c_float)
    f.argtypes = [fp, fp, fp, fp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int]
    f.restype = ctypes.c_double
    return f


def check_sizing(heap, N, Q, D, k):
    """The driver's block sizing from the free device memory it will see: one block of the whole
    corpus, and every int product of the sizes below 2^31."""
    import math
    import torch
    free, _ = torch.cuda.mem_get_info()
    if heap:
        qk = int(math.log(float(k)) / math.log(2.0)) + 1
        req = (Q + D + (1 << qk) - 1) * 4
    else:
        req = (4 * Q + D) * 4
    max_obj = int(math.ceil(free * 0.9 / req))
    max_obj = 1 << int(math.floor(math.log(max_obj) / math.log(2)))
    assert max_obj >= N, f"corpus of {N} rows would be split into blocks of {max_obj}"
    assert N * Q < 2 ** 31 and N * D < 2 ** 31, "int overflow in the driver's sizes"


def run(fn, corpus, queries, k, heap=False):
    """One driver call; returns (dist [Q, k] float32, idx [Q, k] int32, seconds reported, wall seconds)."""
    fp = ctypes.POINTER(ctypes.c_float)
    Q, D = queries.shape
    N = corpus.shape[0]
    check_sizing(heap, N, Q, D, k)
    vals = np.zeros(Q * k, np.float32)
    idxf = np.zeros(Q * k, np.float32)
    t0 = time.perf_counter()
    sec = fn(queries.ctypes.data_as(fp), corpus.ctypes.data_as(fp), vals.ctypes.data_as(fp),
             idxf.ctypes.data_as(fp), N, Q, D, k, 1)
    wall = time.perf_counter() - t0
    assert np.array_equal(idxf, np.rint(idxf)) and idxf.min() >= 0 and idxf.max() < N, "reference indices"
    return vals.reshape(Q, k), idxf.astype(np.int32).reshape(Q, k), float(sec), wall


def main(out_dir: str) -> int:
    import build_ref
    import torch
    import cuknns.synth as S
    if not build_ref.build_if_available():
        print("reference sources absent (neither mounted nor staged in oracle/_ref/src)")
        return 2
    torch.cuda.init()
    torch.empty(1, device="cuda")  # the context the drivers' driver-API calls run in
    lib = build_ref.load()
    keep = []

    def pinned(a):
        t = torch.from_numpy(np.ascontiguousarray(a)).pin_memory()
        keep.append(t)
        return t.numpy()
    heap = driver(lib, "gpuknnsHeap")
    os.makedirs(out_dir, exist_ok=True)
    log = {}

    def say(msg):
        print(msg, flush=True)

    # ---- 65,536 x 128 uniform, 1,024 queries, k = 16
    corpus, queries = S.uniform(65_536, 128, seed=0, nq=1_024)
    corpus, queries = pinned(corpus), pinned(queries)
    say("uniform64k: warm-up call (64 queries)")
    run(heap, corpus, pinned(queries[:64]), 16, heap=True)  # warms cuBLAS
    say("uniform64k: 1,024 queries")
    hd, hi, hs, hw = run(heap, corpus, queries, 16, heap=True)
    np.savez_compressed(os.path.join(out_dir, "ref_uniform64k.npz"), heap_dist=hd, heap_idx=hi,
                        corpus_sha256=sha(corpus), queries_sha256=sha(queries),
                        N=65_536, D=128, Q=1_024, k=16, seed=0)
    log["uniform64k"] = {"heap_s": hs, "heap_wall_s": hw}
    say(json.dumps(log["uniform64k"]))

    # ---- 1,000,000 x 128 integer descriptors, 10,000 queries in chunks of 1,000, k = 128
    corpus, queries = S.int_descriptor(1_000_000, 128, seed=1, nq=10_000)
    corpus = pinned(corpus)
    secs, walls, kept = [], [], []
    for c0 in range(0, queries.shape[0], C2_CHUNK):
        d, i, s_, w = run(heap, corpus, pinned(queries[c0:c0 + C2_CHUNK]), 128, heap=True)
        say(f"int1m: queries {c0}..{c0 + C2_CHUNK - 1}: {s_:.3f} s reported, {w:.3f} s wall")
        secs.append(s_)
        walls.append(w)
        if c0 < C2_KEEP:
            kept.append((d, i))
            if c0 + C2_CHUNK == C2_KEEP:
                np.savez_compressed(os.path.join(out_dir, "ref_int1m_q1000.npz"),
                                    heap_dist=np.concatenate([x[0] for x in kept]),
                                    heap_idx=np.concatenate([x[1] for x in kept]),
                                    corpus_sha256=sha(corpus), queries_sha256=sha(queries[:C2_KEEP]),
                                    N=1_000_000, D=128, Q=C2_KEEP, k=128, seed=1)
    log["int1m"] = {"chunk_queries": C2_CHUNK, "chunks": len(secs), "reported_s": secs, "wall_s": walls,
                    "queries_per_s_reported": queries.shape[0] / sum(secs),
                    "queries_per_s_wall": queries.shape[0] / sum(walls)}
    with open(os.path.join(out_dir, "ref_fixtures_log.json"), "w") as f:
        json.dump(log, f, indent=1)
    print(json.dumps(log))
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv[1] if len(sys.argv) > 1 else os.path.join(ROOT, "gpurun_out", "ref_fixtures")))
