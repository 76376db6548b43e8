#!/usr/bin/env python3
"""Benchmark of the brute-force squared-L2 kNN hot path on GB300.

Default workload (one GB300): corpus 1,000,000 x 128 float32 holding integers
clip(round(|N(0,40)|),0,255) with 8% of each row's coordinates zeroed,
10,000 queries from the same generator, k = 100, seed 1.  A step is one
search of the whole query batch against the whole corpus.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                    [--workload int1m|uniform64k|mix4m|aniso8m|serve2m|...]
                    [--precision exact|bf16|fp8] [--shortlist C]

Prints one JSON line (rank 0).  `value` is queries/s with the corpus and the
queries resident in HBM; `e2e` is the same metric through the drop-in C ABI
(gpuknnsBitonic; knns_search_host for the precision forms) from pinned host
buffers, host<->device copies included.
`--impl reference` times the reference's CPU path (demo/knn.m, restated in C
in oracle/knn_oracle.c) on the host cores, on whole query batches where the
step budget allows (the default run times the full 10,000-query batch).

The plain-form line also carries `accuracy` (recall@k and the largest relative
distance error against the FP64 oracle on a query sample, outside the timed
region) and `forms`: the same workload through the BF16 shortlist form (c from
the autotuner) and through the plain form on 3xTF32 keys (`tf32_only`), each
timed like the headline and checked against the same FP64 sample.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (os.path.join(ROOT, "knn-toolbox_gb300"), os.path.join(ROOT, "oracle")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

WORKLOADS = {
    "int1m": dict(desc="int-descriptor corpus 1,000,000 x 128 (clip(round(|N(0,40)|),0,255), 8% of coords "
                       "zeroed), 10,000 queries, k=100, seed 1",
                  gen="int_descriptor", N=1_000_000, D=128, Q=10_000, k=100, seed=1),
    "uniform64k": dict(desc="uniform [0,1) corpus 65,536 x 128, 1,024 queries, k=16, seed 0",
                       gen="uniform", N=65_536, D=128, Q=1_024, k=16, seed=0),
    "mix4m": dict(desc="Gaussian mixture corpus 4,000,000 x 96 (1,024 centres N(0,1), sigma 0.15, rows "
                       "L2-normalised), 10,000 queries, k=10, seed 2",
                  gen="gauss_mixture", N=4_000_000, D=96, Q=10_000, k=10, seed=2),
    # profiling-sized cut of mix4m for ncu captures of the 3xTF32 scan (corpus still larger than L2)
    "mix1m": dict(desc="Gaussian mixture corpus 1,000,000 x 96 (1,024 centres N(0,1), sigma 0.15, rows "
                       "L2-normalised), 2,500 queries, k=10, seed 2",
                  gen="gauss_mixture", N=1_000_000, D=96, Q=2_500, k=10, seed=2),
    # serving form: resident corpus, Poisson arrivals of requests of uneven size and k
    "serve2m": dict(desc="serving: int-descriptor corpus 2,000,000 x 128 resident (FP32 + BF16 + TF32 copies), "
                         "Poisson arrivals, request sizes log-uniform on [1,512], k in {1,10,100}, seed 1",
                    gen="int_descriptor", N=2_000_000, D=128, Q=0, k=0, seed=1, serve=True),
    # precision form with E4M3 keys: anisotropic Gaussian N(0, diag(1/sqrt(1+j)))
    "aniso8m": dict(desc="anisotropic Gaussian corpus 8,000,000 x 256 (coordinate j ~ N(0, 1/sqrt(1+j))), "
                         "16,384 queries, k=32, seed 3",
                    gen="anisotropic", N=8_000_000, D=256, Q=16_384, k=32, seed=3),
    # profiling-sized cut of aniso8m for ncu captures of the E4M3 scan (corpus still larger than L2)
    "aniso1m": dict(desc="anisotropic Gaussian corpus 1,000,000 x 256, 4,096 queries, k=32, seed 3",
                    gen="anisotropic", N=1_000_000, D=256, Q=4_096, k=32, seed=3),
    # profiling cut of int1m: full corpus (same candidate density per corpus row), a quarter of the queries
    "int1m_q2500": dict(desc="int-descriptor corpus 1,000,000 x 128, 2,500 queries, k=100, seed 1",
                        gen="int_descriptor", N=1_000_000, D=128, Q=2_500, k=100, seed=1),
    # profiling-sized cut of int1m (corpus still larger than L2) for ncu captures
    "int256k": dict(desc="int-descriptor corpus 262,144 x 128, 10,000 queries, k=100, seed 1",
                    gen="int_descriptor", N=262_144, D=128, Q=10_000, k=100, seed=1),
}
METRIC = "queries/s (exact squared-L2 kNN, plain FP32 form)"


def gen_data(w, rank=0):
    import cuknns.synth as S
    fn = getattr(S, w["gen"])
    corpus, queries = fn(w["N"], w["D"], seed=w["seed"], nq=w["Q"])
    if rank:
        _, queries = fn(w["Q"], w["D"], seed=w["seed"] + 1000 * rank, nq=w["Q"])
    return corpus, queries


def reduce_max(x, dist, device):
    """Max of a float over the ranks (dist = torch.distributed or None; device = where the
    backend's tensors live: the rank's GPU for NCCL, the CPU for gloo)."""
    if dist is None:
        return float(x)
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f), "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


# DRAM traffic per launch of the dominant kernel, from one ncu capture of each workload
# (dram__bytes_read.sum + dram__bytes_write.sum; the summaries under profiles/ give the
# command and, where the capture ran on a cut of the workload, the scaling).
NCU_TRAFFIC = {
    ("scan_kernel", "int1m"): 398.3e6,
    ("scan_kernel", "aniso8m"): 2537.0e6,
    ("tscan_kernel", "uniform64k"): 69.9e6,
    ("tscan_kernel", "mix4m"): 3405.0e6,
}


def tf32_peak_live():
    """Dense TF32 rate of cuBLAS on this GPU (torch.matmul on FP32 with TF32 allowed, 8192^3, best of
    5), TFLOP/s, as the roofline denominator of the 3xTF32 kernels; None when unavailable."""
    import torch
    n = 8192
    old = torch.backends.cuda.matmul.allow_tf32
    try:
        torch.backends.cuda.matmul.allow_tf32 = True
        a = torch.randn(n, n, device="cuda")
        b = torch.randn(n, n, device="cuda")
        for _ in range(3):
            a @ b
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        best = 1e9
        for _ in range(5):
            e0.record()
            a @ b
            e1.record()
            e1.synchronize()
            best = min(best, e0.elapsed_time(e1))
        del a, b
        torch.cuda.empty_cache()
        return 2 * n ** 3 / (best / 1e3) / 1e12
    except Exception:
        return None
    finally:
        torch.backends.cuda.matmul.allow_tf32 = old


def fp8_peak_live():
    """Dense FP8 E4M3 rate of cuBLASLt on this GPU (torch._scaled_mm, 8192^3, best of 5), TFLOP/s,
    as the roofline denominator of the E4M3 scan; None when the GEMM is unavailable."""
    import torch
    n = 8192
    try:
        dev = torch.device("cuda")
        a8 = torch.randn(n, n, device=dev).to(torch.float8_e4m3fn)
        b8 = torch.randn(n, n, device=dev).to(torch.float8_e4m3fn).t().contiguous().t()
        one = torch.tensor(1.0, device=dev)

        def fn():
            return torch._scaled_mm(a8, b8, scale_a=one, scale_b=one, out_dtype=torch.bfloat16)
        for _ in range(3):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        best = 1e9
        for _ in range(5):
            e0.record()
            fn()
            e1.record()
            e1.synchronize()
            best = min(best, e0.elapsed_time(e1))
        del a8, b8
        torch.cuda.empty_cache()
        return 2 * n ** 3 / (best / 1e3) / 1e12
    except Exception:
        return None


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index):
        self.dev = device_index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.dev), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, ValueError):
            self.proc = None
        return self

    def __exit__(self, *a):
        self.out = ""
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                self.out, _ = self.proc.communicate()

    def summary(self):
        rows = []
        for line in (self.out or "").splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                rows.append((float(f[1]), float(f[2]), f[5:9]))
            except ValueError:
                continue
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[j] for _, _, r in rows for j, v in enumerate(r) if v.lower() == "active"})
        return {"sm_mhz": statistics.median(r[0] for r in rows), "sm_max_mhz": max(r[1] for r in rows),
                "reasons": reasons, "samples": len(rows)}


def path_of(st, bf16_keys):
    """(path, dominant kernel) of a search from its statistics: bf16_keys when its keys are BF16 /
    E4M3 (a precision form, or BF16-exact data in the exact form)."""
    import cuknns
    keys = st.get("scan_keys", 0)
    if keys & 1 and (bf16_keys or not keys & 2):
        return "threshold scan (BF16 / E4M3 keys)", "scan_kernel"
    if keys & 2:
        return "threshold scan (3xTF32 keys)", "tscan_kernel"
    if st["algo"] == cuknns.ALGO_TC:
        return "shortlist kernel (tcgen05)", "tc_kernel"
    return "shortlist kernel (CUDA cores)", "simt_kernel"


def lo_tile_fraction(x, rows=128):
    """Fraction of 128-row tiles whose TF32 low part (x - tf32(x), rounded to TF32) is nonzero.

    The tensor-core kernel runs the two correction products of 3xTF32 only on
    such tiles, so this sets the executed tensor work.
    """
    def tf32(a):
        u = a.view(np.uint32).astype(np.uint64)
        u = (u + 0xFFF + ((u >> 13) & 1)) & 0xFFFFE000
        return u.astype(np.uint32).view(np.float32)
    hits = []
    for s in range(0, x.shape[0], 1 << 16):
        blk = x[s:s + (1 << 16)]
        lo = tf32((blk - tf32(blk)).astype(np.float32))
        row = (lo != 0).any(axis=1)
        pad = (-len(row)) % rows
        hits.append(np.concatenate([row, np.zeros(pad, bool)]).reshape(-1, rows).any(axis=1))
    h = np.concatenate(hits)
    return float(h.mean()) if h.size else 0.0


def cpu_baseline(corpus, queries, k, budget_s=12.0):
    """demo/knn.m restated in C (oracle), all host threads, on a bounded query sample."""
    import oracle
    oracle.build()
    threads = oracle.max_threads()
    # grow the sample until one timed call takes at least half the budget (a small call is
    # dominated by the per-call corpus sweep, so a single probe underestimates the rate)
    m = max(1, threads)
    while True:
        t0 = time.perf_counter()
        oracle.knn_gemm(corpus, queries[:m], k, nthreads=threads)
        el = time.perf_counter() - t0
        if el >= 0.5 * budget_s or m >= len(queries):
            break
        m = int(min(len(queries), max(2 * m, m * budget_s / max(el, 1e-3))))
    return {"value": m / el, "unit": "queries/s", "cores": threads, "kind": "port",
            "sample": f"first {m} of {len(queries)} queries against the full corpus, "
                      f"{el:.1f} s on {threads} host threads (demo/knn.m restated in C, oracle/knn_oracle.c)"}


def run_reference(args, w):
    """The reference's CPU path on the host cores: demo/knn.m restated in C (oracle/knn_oracle.c),
    every host thread.  Each timed step searches a contiguous block of the workload's queries
    against the whole corpus: the full batch when the steps fit a budget of about three
    minutes, else the largest block that does (sized from a 1,000-query probe, large enough
    that the per-call corpus sweep does not dominate)."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    import oracle
    oracle.build()
    corpus, queries = gen_data(w)
    threads = oracle.max_threads()
    k, Q = w["k"], len(queries)
    probe = min(Q, 1000)
    t0 = time.perf_counter()
    oracle.knn_gemm(corpus, queries[:probe], k, nthreads=threads)
    per_q = (time.perf_counter() - t0) / probe
    budget = 180.0 / max(1, args.steps)
    m = int(max(probe, min(Q, budget / max(per_q, 1e-9))))
    for _ in range(args.warmup):  # untimed; a small block each
        oracle.knn_gemm(corpus, queries[:min(m, 256)], k, nthreads=threads)
    t0 = time.perf_counter()
    for s_ in range(args.steps):
        lo = (s_ * m) % max(1, Q - m + 1)
        oracle.knn_gemm(corpus, queries[lo:lo + m], k, nthreads=threads)
    el = time.perf_counter() - t0
    value = m * args.steps / el
    sample = (f"{m} of {Q} queries per step against the full {w['N']} x {w['D']} corpus, "
              f"{threads} host threads, demo/knn.m restated in C (oracle/knn_oracle.c)")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "queries/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": el / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": w["desc"], "N": w["N"], "Q": w["Q"], "D": w["D"], "k": w["k"],
                       "queries_per_step": m},
            "cpu_baseline": {"value": value, "unit": "queries/s", "cores": threads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": value, "unit": "queries/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def run_e2e(corpus_np, queries_np, k, Q, world, steps, barrier, dist, dev, prec_opts=None):
    """Same metric through the reference-facing C ABI with host buffers (copies timed).

    The plain form goes through the drop-in gpuknnsBitonic; the precision forms,
    which the reference API cannot select, through knns_search_host.
    """
    import torch
    import cuknns
    hc = torch.from_numpy(corpus_np).pin_memory().numpy()
    hq = torch.from_numpy(queries_np).pin_memory().numpy()
    if prec_opts:
        def call():
            return cuknns.search_host(hc, hq, k, **prec_opts)
        api = "knns_search_host (include/knn_gb300.h)"
    else:
        def call():
            return cuknns.gpuknnsBitonic(hq, hc, k, 1)[:2]
        api = "gpuknnsBitonic (include/cuknns.h)"
    call()  # warm (staging buffers)
    barrier()
    t0 = time.perf_counter()
    for _ in range(steps):
        vals, idxf = call()
    e2e_s = (time.perf_counter() - t0) / steps
    e2e_s = reduce_max(e2e_s, dist, dev)
    return {"value": Q * world / e2e_s, "unit": "queries/s", "h2d_bytes_per_step": int(hc.nbytes + hq.nbytes),
            "d2h_bytes_per_step": int(vals.nbytes + idxf.nbytes), "api": api,
            "host_buffers": "pinned inputs, pageable outputs", "steps": steps}


def run_gb300(args, w):
    import torch
    import cuknns

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    split_corpus = args.split == "corpus" and world > 1
    # replicas: the same corpus and this rank's own queries; corpus split: this rank's shard of
    # the corpus and everybody's queries (rank 0's)
    corpus_np, queries_np = gen_data(w, 0 if split_corpus else rank)
    N, D, Q, k = w["N"], w["D"], w["Q"], w["k"]
    if split_corpus:
        from cuknns import shard as SH
        r0, r1 = SH.shard_bounds(N, world, rank)
        c = torch.from_numpy(corpus_np[r0:r1]).to(dev)
    else:
        c = torch.from_numpy(corpus_np).to(dev)
    q = torch.from_numpy(queries_np).to(dev)
    dist_out = torch.empty((Q, k), dtype=torch.float32, device=dev)
    idx_out = torch.empty((Q, k), dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream(dev)

    prec = {"exact": cuknns.PREC_EXACT, "bf16": cuknns.PREC_BF16, "fp8": cuknns.PREC_FP8}[args.precision]
    scan_mode = {"auto": cuknns.SCAN_AUTO, "on": cuknns.SCAN_ON, "off": cuknns.SCAN_OFF,
                 "tf32": cuknns.SCAN_TF32}[args.scan]

    def autotune(p):
        """Shortlist factor c of a precision form: recall@k against the exact form on 256 queries."""
        t0 = time.perf_counter()
        ix = cuknns.Index(c, fp8=p == cuknns.PREC_FP8)
        cf, rec = ix.autotune_shortlist(q[:256].contiguous(), k, target=0.999, precision=p)
        ix.close()
        torch.cuda.empty_cache()
        return cf, {"shortlist_c": cf, "sample_recall": rec, "sample_queries": 256, "target": 0.999,
                    "seconds": time.perf_counter() - t0}

    tuned = None
    if prec != cuknns.PREC_EXACT and args.shortlist == 0:
        args.shortlist, tuned = autotune(prec)

    def barrier():
        if dist is not None:
            dist.barrier()

    def timed(step, steps):
        """W untimed steps, then `steps` steps between two CUDA events on the launching stream."""
        for _ in range(args.warmup):
            step(False)
        rc_ = cuknns.lib().knns_check_device(None)
        if rc_ != 0:
            raise RuntimeError(cuknns.last_error())
        st_ = cuknns.last_stats()
        cuknns.timing_collect5()  # drop anything recorded so far
        barrier()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            step(True)
        e1.record(stream)
        torch.cuda.synchronize()
        barrier()
        stages = cuknns.timing_collect5()
        rc_ = cuknns.lib().knns_check_device(None)
        if rc_ != 0:
            raise RuntimeError(cuknns.last_error())
        return reduce_max(e0.elapsed_time(e1), dist, dev), stages, st_

    def search_step(p, shortlist, tf32_only=False, single_stream=False):
        if split_corpus:
            def step(timing):
                # this rank's shard, then the all-gather of every rank's Q x k list and the merge
                d_, i_ = SH.sharded_search(c, r0, q, k, stream=stream, check=False, timing=timing, precision=p,
                                           shortlist=shortlist, scan=scan_mode, scan_boxes=args.scan_boxes,
                                           tf32_only=tf32_only, scan_accs=args.scan_accs,
                                           single_stream=single_stream, splits=args.splits)
                dist_out.copy_(d_)
                idx_out.copy_(i_)
            return step

        def step(timing):
            cuknns.search(c, q, k, dist=dist_out, idx=idx_out, stream=stream, check=False, timing=timing,
                          precision=p, shortlist=shortlist, scan=scan_mode, scan_boxes=args.scan_boxes,
                          tf32_only=tf32_only, scan_accs=args.scan_accs, single_stream=single_stream,
                          splits=args.splits)
        return step

    # ---- headline: the requested form, inputs resident in HBM
    with ClockSampler(local) as clk:
        el_ms, hl_stages, st = timed(search_step(prec, args.shortlist, single_stream=args.single_stream),
                                     args.steps)
    # the path that ran: the exact form decides between BF16 and 3xTF32 keys on the device (BF16
    # keys when every corpus and query value is exact in BF16); the data tell which
    bf16_exact = bool(((corpus_np.view(np.uint32) & 0xFFFF) == 0).all() and
                      ((queries_np.view(np.uint32) & 0xFFFF) == 0).all())
    path, kern = path_of(st, args.precision != "exact" or bf16_exact)
    # whole-job throughput: replicas search world x Q queries; a corpus split searches Q
    value = Q * args.steps * (1 if split_corpus else world) / (el_ms / 1e3)
    # stage times and the dominant kernel's launch time: the same search with every kernel on the
    # search stream (by default the threshold scan overlaps the corpus preparation with the seeding
    # and scans the corpus in blocks on two more streams, which no single stage event brackets)
    if args.single_stream:
        ss_ms, (prep_ms, seed_ms, fused_ms, select_ms, fix_ms, nt) = el_ms, hl_stages
    else:
        ss_ms, (prep_ms, seed_ms, fused_ms, select_ms, fix_ms, nt), _ = timed(
            search_step(prec, args.shortlist, single_stream=True), args.steps)
    single_stream_qps = Q * args.steps * (1 if split_corpus else world) / (ss_ms / 1e3)

    # ---- accuracy against the FP64 oracle on a query sample (outside every timed region)
    nrq = args.recall_queries if args.recall_queries else 100
    sub = np.linspace(0, Q - 1, min(nrq, Q)).astype(np.int64)
    exact64 = None
    if rank == 0 and nrq:
        import oracle
        oracle.build()
        exact64 = oracle.knn_f64(corpus_np, queries_np[sub], k)

    def accuracy_now():
        """recall@k and the largest relative distance error of idx_out / dist_out on the sample."""
        if exact64 is None:
            return None
        import oracle
        ii = torch.from_numpy(sub).to(dev)
        got_i = idx_out[ii].cpu().numpy()
        got_d = dist_out[ii].cpu().numpy()
        d64 = oracle.pair_dist_f64(corpus_np, queries_np[sub], got_i)
        return {"queries": int(len(sub)), "recall_at_k": oracle.recall_at_k(got_i, exact64[1]),
                "max_dist_rel_err": float((np.abs(got_d - d64) / np.maximum(d64, 1e-30)).max()),
                "oracle": "FP64 direct difference (oracle/knn_oracle.c)"}

    accuracy = accuracy_now()

    # ---- the other forms on the same workload (plain form only): BF16 shortlist, 3xTF32 keys
    forms = None
    if prec == cuknns.PREC_EXACT and not args.no_forms and not split_corpus:
        forms = {"exact": {"queries_per_s": value, "accuracy": accuracy, "path": path}}
        cf, tuned_bf = autotune(cuknns.PREC_BF16)
        f_ms, f_stages, f_st = timed(search_step(cuknns.PREC_BF16, cf), args.steps)
        forms["bf16_shortlist"] = {"queries_per_s": Q * args.steps * world / (f_ms / 1e3),
                                   "ms_per_step": f_ms / args.steps, "shortlist": f_st["kp"], "autotune": tuned_bf,
                                   "accuracy": accuracy_now()}
        t_steps = max(3, min(args.steps, 20))
        t_ms, t_stages, t_st = timed(search_step(cuknns.PREC_EXACT, 0, tf32_only=True, single_stream=True), t_steps)
        f_c, f_q = lo_tile_fraction(corpus_np), lo_tile_fraction(queries_np)
        t_path, t_kern = path_of(t_st, False)
        t_scan = t_kern == "tscan_kernel"
        # the TF32 scan's main pass is its own stage; the shortlist kernel's stage includes its pilot
        t_fused = (t_stages[2] if t_scan else t_stages[1] + t_stages[2]) / max(1, t_stages[5])
        products = 1.0 + f_c + f_q
        t_flops = products * 2.0 * N * Q * D * (1.0 + (1.0 / 16.0 if t_st["pilot"] and not t_scan else 0.0))
        tf32_peak = tf32_peak_live()
        forms["tf32_plain"] = {"queries_per_s": Q * t_steps * world / (t_ms / 1e3), "ms_per_step": t_ms / t_steps,
                               "steps": t_steps, "kernel": f"{t_kern} (3xTF32)", "path": t_path,
                               "products_per_useful_product": products,
                               "note": "3xTF32 keys; a correction product is skipped where the TF32 low part of the "
                                       "corpus tile or query tile is zero (exact zeros), as on integer data",
                               "fused_ms": t_fused,
                               "tf32_tflops_executed": t_flops / (t_fused / 1e3) / 1e12,
                               "tf32_peak_measured": tf32_peak,
                               "accuracy": accuracy_now()}
        forms["bf16_over_tf32"] = forms["bf16_shortlist"]["queries_per_s"] / forms["tf32_plain"]["queries_per_s"]
        # leave the headline's answers in the output buffers
        search_step(prec, args.shortlist)(False)

    # ---- end to end through the drop-in C ABI from pinned host buffers
    e2e = None
    e2e_steps = 0 if (args.no_e2e or split_corpus) else max(1, min(args.steps, 20))
    if e2e_steps:
        popts = None if prec == cuknns.PREC_EXACT else {"precision": prec, "shortlist": args.shortlist}
        e2e = run_e2e(corpus_np, queries_np, k, Q, world, e2e_steps, barrier, dist, dev, popts)

    # ---- roofline of the dominant kernel (the main fused distance pass)
    peaks, peak_kind = measured_peaks()
    on_scan = kern == "scan_kernel"
    # shortlist kernels: the fused stage includes their pilot pass; the scans' seeding passes are
    # their own stage
    fused_avg_ms = (fused_ms if kern in ("scan_kernel", "tscan_kernel") else seed_ms + fused_ms) / max(1, nt)
    if on_scan:
        # the main pass alone is timed (seeding passes are their own stage); one product per pair
        flops = 2.0 * N * Q * D
        if args.precision == "fp8":
            row_bytes = -(-D // 128) * 128
            live = fp8_peak_live()
            if live is not None:
                peak, peak_src = live, "cuBLASLt FP8 E4M3 8192^3 GEMM burst, measured in this run"
            else:
                peak, peak_src = 2.0 * peaks["bf16_tflops"], f"2 x {peak_kind} bf16 dense burst"
            mma = f"e4m3 (kind::f8f6f4, M128 N{96 if args.scan_accs == 4 else (224 if row_bytes <= 256 else 192)})"
            padded_k = row_bytes
        else:
            padded_k = -(-D // 64) * 64
            peak, peak_src = peaks["bf16_tflops"], f"{peak_kind} bf16 dense burst"
            mma = f"bf16 (kind::f16, M128 N{96 if args.scan_accs == 4 else (224 if padded_k <= 128 else 192)})"
        roof = {"bound": "tensor", "achieved": flops / (fused_avg_ms / 1e3) / 1e12, "peak": peak,
                "unit": "TFLOP/s", "peak_source": peak_src, "mma_kind": mma, "products_per_useful_product": 1.0,
                "flops_per_launch": flops, "padded_k": int(padded_k)}
    elif st["algo"] == cuknns.ALGO_TC:
        # executed tensor work of the fused stage (main pass + the 1/16-sample pilot pass of the
        # shortlist kernel; the TF32 scan's main pass alone)
        pilot_f = 1.0 + (1.0 / 16.0 if st["pilot"] and kern == "tc_kernel" else 0.0)
        if args.precision != "exact" or bf16_exact:
            kind, products, peak = ("bf16 shortlist" if args.precision != "exact" else "bf16 (data BF16-exact)",
                                    1.0, peaks["bf16_tflops"])
            peak_src = f"{peak_kind} bf16 dense burst"
        else:
            # 3xTF32 issues hi.hi always and the two correction products only for
            # tiles whose TF32 low part is nonzero (corpus tile / query tile)
            f_c, f_q = lo_tile_fraction(corpus_np), lo_tile_fraction(queries_np)
            kind, products = "3xTF32", 1.0 + f_c + f_q
            live = tf32_peak_live()
            if live is not None:
                peak, peak_src = live, "cuBLAS TF32 8192^3 GEMM burst, measured in this run"
            else:
                peak, peak_src = peaks["bf16_tflops"] / 2.0, f"{peak_kind} bf16 dense burst / 2 (nominal TF32 rate)"
        flops = products * 2.0 * N * Q * D * pilot_f
        roof = {"bound": "tensor", "achieved": flops / (fused_avg_ms / 1e3) / 1e12, "peak": peak,
                "unit": "TFLOP/s", "peak_source": peak_src, "mma_kind": kind,
                "products_per_useful_product": products, "pilot_pass_included": pilot_f > 1.0}
    else:
        flops = 2.0 * N * Q * D
        peak = 152 * 128 * 2 * 2.07e9 / 1e12
        roof = {"bound": "fp32-simt", "achieved": flops / (fused_avg_ms / 1e3) / 1e12, "peak": peak,
                "unit": "TFLOP/s", "peak_source": "nominal FP32 FMA rate at max SM clock"}
    roof["frac"] = roof["achieved"] / roof["peak"]
    if on_scan and args.precision == "fp8":
        # the same achieved rate against twice the BF16 peak (the nominal FP8:BF16 ratio)
        roof["frac_vs_2x_bf16"] = roof["achieved"] / (2.0 * peaks["bf16_tflops"])
    roof["traffic"] = NCU_TRAFFIC.get((kern, args.workload))
    roof["kernel"] = kern
    roof["kernel_ms"] = fused_avg_ms
    roof["effective_fp32_tflops"] = 2.0 * N * Q * D / (fused_avg_ms / 1e3) / 1e12

    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return 0
    cpu = cpu_baseline(corpus_np, queries_np, k) if world == 1 and not args.no_cpu_baseline else None
    line = {"metric": METRIC, "value": value, "unit": "queries/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": el_ms / args.steps, "higher_is_better": True,
            "scaling": "strong" if split_corpus else "weak", "vs_baseline": None,
            "dtype": {"exact": "f32", "bf16": "bf16 keys, f32 re-rank", "fp8": "e4m3 keys, f32 re-rank"}[args.precision],
            "data": "synthetic",
            "config": {"workload": w["desc"], "N": N, "Q": Q, "D": D, "k": k,
                       "parallelism": (f"corpus split x{world} (contiguous shards, all-gather of Q x k lists, "
                                       f"device merge)" if split_corpus else
                                       f"replicas x{world} (queries sharded, corpus replicated)"),
                       "l2": f"inputs larger than L2 ({N * D * 4 / 1e6:.0f} MB FP32 corpus)" if N * D * 4 > 129e6
                       else "working set within L2 (65,536 x 128 corpus)",
                       "algo": {1: "tcgen05", 2: "CUDA-core FP32"}[st["algo"]], "precision": args.precision,
                       "pilot": st["pilot"], "splits": st["scan_splits"] if on_scan else st["splits"],
                       "shortlist": st["kp"], "path": path,
                       "scan_cap": st["scan_cap"], "scan_ring": st["scan_ring"], "stages": st["stages"]},
            "stage_ms": {"prep": prep_ms / max(1, nt), "seed": seed_ms / max(1, nt), "fused": fused_ms / max(1, nt),
                         "select": select_ms / max(1, nt), "fixup": fix_ms / max(1, nt),
                         "note": "every kernel on the search stream (single_stream); the headline value runs the "
                                 "default overlapped schedule"},
            "single_stream_queries_per_s": single_stream_qps,
            "roofline": roof, "cpu_baseline": cpu, "e2e": e2e, "accuracy": accuracy, "forms": forms,
            "autotune": tuned, "gpu_launches": st["launches"] * args.steps,
            "clocks": clk.summary()}
    print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()
    return 0


def run_serve(args, w):
    """Serving form: a request server over a resident index under Poisson load."""
    import queue
    import threading
    import torch
    import cuknns
    import cuknns.synth as S

    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    torch.cuda.set_device(0)
    rng = np.random.default_rng(w["seed"] + 7)
    n_req = args.requests
    sizes = np.minimum(512, np.exp(rng.uniform(0.0, np.log(512.0), n_req)).astype(np.int64) + 0)
    sizes = np.maximum(sizes, 1)
    ks = rng.choice([1, 10, 100], n_req)
    corpus_np, queries_np = S.int_descriptor(w["N"], w["D"], seed=w["seed"], nq=int(sizes.sum()))
    c = torch.from_numpy(corpus_np).cuda()
    ix = cuknns.Index(c)
    prec = cuknns.PREC_BF16 if args.precision == "bf16" else cuknns.PREC_EXACT
    srv = cuknns.Server(ix, slots=2, max_batch=1024, precision=prec, shortlist=args.shortlist, autotune=True)
    t0 = time.perf_counter()
    srv.warmup([32, 64, 128, 256, 512, 1024], [1, 10, 100])
    warm_s = time.perf_counter() - t0
    offs = np.concatenate([[0], np.cumsum(sizes)])
    arrivals = np.cumsum(rng.exponential(1.0 / args.rate, n_req))
    ids = queue.Queue()
    lat = [0.0] * n_req
    res = [None] * n_req

    def waiter():
        while True:
            item = ids.get()
            if item is None:
                return
            j, rid = item
            d, i, ms = srv.wait(rid)
            lat[j] = ms
            res[j] = i

    pool = [threading.Thread(target=waiter) for _ in range(8)]
    for t in pool:
        t.start()
    with ClockSampler(0) as clk:
        start = time.perf_counter()
        for j in range(n_req):
            dt = arrivals[j] - (time.perf_counter() - start)
            if dt > 0:
                time.sleep(dt)
            ids.put((j, srv.submit(queries_np[offs[j]:offs[j + 1]], int(ks[j]))))
        for _ in pool:
            ids.put(None)
        for t in pool:
            t.join()
        wall = time.perf_counter() - start
    st = srv.stats()
    # every request's answer is the one the same request gets alone: spot-check a sample
    checked = 0
    for j in np.linspace(0, n_req - 1, 16).astype(int):
        q = torch.from_numpy(queries_np[offs[j]:offs[j + 1]]).cuda()
        _, i0 = ix.search(q, int(ks[j]), precision=prec, shortlist=args.shortlist)
        checked += int(np.array_equal(res[j], i0.cpu().numpy()))
    srv.close()
    ix.close()
    lat_a = np.array(lat)
    total_q = int(sizes.sum())
    line = {"metric": "queries/s and p50/p99 request latency, serving form (continuous batching)",
            "value": total_q / wall, "unit": "queries/s", "n_gpus": 1, "steps": n_req, "warmup": 0,
            "ms_per_step": wall * 1e3 / n_req, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32" if prec == cuknns.PREC_EXACT else "bf16 keys, f32 re-rank", "data": "synthetic",
            "config": {"workload": w["desc"], "N": w["N"], "D": w["D"], "requests": n_req,
                       "offered_rate_rps": args.rate, "mean_request_queries": float(sizes.mean()),
                       "slots": 2, "max_batch": 1024, "graph_warmup_s": warm_s},
            "latency_ms": {"p50": float(np.percentile(lat_a, 50)), "p99": float(np.percentile(lat_a, 99)),
                           "mean": float(lat_a.mean()), "max": float(lat_a.max())},
            "served": {"launches": st["launches"], "queries_per_launch": st["queries"] / max(1, st["launches"]),
                       "graphs": st["graphs"], "achieved_rate_rps": n_req / wall,
                       "answers_equal_alone": f"{checked}/16 sampled requests"},
            "clocks": clk.summary()}
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="int1m", choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true", help="skip the host-buffer leg (profiling runs)")
    ap.add_argument("--precision", default="exact", choices=["exact", "bf16", "fp8"],
                    help="exact: FP32-accurate keys (plain form); bf16 / fp8: BF16 or E4M3 (per-row scales) "
                         "shortlist + exact re-rank")
    ap.add_argument("--shortlist", type=int, default=0,
                    help="bf16 / fp8: shortlist factor c (0 = chosen by the autotuner)")
    ap.add_argument("--scan", default="auto", choices=["auto", "on", "off", "tf32"],
                    help="threshold scan (auto: BF16 keys for BF16-exact data and 3xTF32 keys otherwise from "
                         "131,072 rows, 3xTF32 keys from 16,384; on: the pair from 16,384; tf32: 3xTF32 alone)")
    ap.add_argument("--scan-boxes", type=int, default=0, help="threshold scan: K boxes per ring slot (0 = auto)")
    ap.add_argument("--single-stream", action="store_true",
                    help="the headline search with every kernel on one stream (a fixed launch order for "
                         "profiler captures)")
    ap.add_argument("--scan-accs", type=int, default=0, choices=[0, 2, 4],
                    help="threshold scan: tensor-memory accumulators (0 = auto)")
    ap.add_argument("--splits", type=int, default=0, help="corpus splits of the main scan (0 = auto)")
    ap.add_argument("--rate", type=float, default=4000.0, help="serving: offered requests per second")
    ap.add_argument("--requests", type=int, default=4000, help="serving: requests in the timed run")
    ap.add_argument("--recall-queries", type=int, default=0,
                    help="queries of the FP64-oracle accuracy sample (0 = 100)")
    ap.add_argument("--no-forms", action="store_true",
                    help="plain form: skip the BF16-shortlist and 3xTF32 comparison runs")
    ap.add_argument("--split", default="queries", choices=["queries", "corpus"],
                    help="N > 1 GPUs: replicas with their own queries (weak scaling), or one query batch "
                         "against a corpus split across the GPUs (strong scaling: all-gather + merge)")
    args = ap.parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        # one process per GPU: launch the ranks ourselves
        import socket
        with socket.socket() as sk:
            sk.bind(("127.0.0.1", 0))
            port = sk.getsockname()[1]
        cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", str(args.gpus),
               "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.abspath(__file__)] + sys.argv[1:]
        return subprocess.call(cmd)
    if world != args.gpus:
        print(f"bench.py: --gpus {args.gpus} but WORLD_SIZE={world}", file=sys.stderr)
        return 2
    if args.warmup < 3:
        args.warmup = 3
    w = WORKLOADS[args.workload]
    if args.impl == "reference":
        return run_reference(args, w)
    if w.get("serve"):
        return run_serve(args, w)
    return run_gb300(args, w)


if __name__ == "__main__":
    sys.exit(main())
