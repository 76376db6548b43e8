// engine.cu -- host engine and the status-returning C ABI (include/knn_gb300.h).
//
// One engine per CUDA device holds a grow-only workspace (norms, TF32 hi/lo
// copies of the corpus, per-split shortlists, staging for host calls) so a
// search allocates nothing once warm.  It replaces the reference's per-call
// set-up in gpuknnsBitonic / gpuknnsHeap (src/cuknnBitonic.cu:422-547,
// src/cuknnHeap.cu:394-505): cublasCreate, stream creation, cudaMalloc of
// N*Q-sized distance buffers, and the corpus blocking by free memory.  The
// corpus stays resident; the work is split across CTAs instead of streams.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <tuple>

#include <cuda.h>
#include <cuda_runtime.h>

#include "knn_gb300.h"
#include "engine.h"
#include "kernels.h"

namespace knn {

static thread_local std::string g_last_error;
static thread_local knns_stats g_last_stats;
static thread_local bool g_have_stats = false;

int set_error(int code, const char* fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return code;
}

void clear_error() { g_last_error.clear(); }

#define KNN_CUDA(call)                                                                              \
    do {                                                                                            \
        cudaError_t e_ = (call);                                                                    \
        if (e_ != cudaSuccess)                                                                      \
            return set_error(KNNS_ERR_CUDA, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), \
                             __FILE__, __LINE__);                                                   \
    } while (0)

int DevBuf::ensure(size_t bytes)
{
    if (bytes <= cap) return KNNS_OK;
    if (p) {
        cudaFree(p);
        p = nullptr;
        cap = 0;
    }
    size_t want = std::max(bytes, (size_t)256);
    cudaError_t e = cudaMalloc(&p, want);
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        p = nullptr;
        return set_error(KNNS_ERR_NOMEM, "cudaMalloc(%zu) failed: %s", want, cudaGetErrorString(e));
    }
    cap = want;
    return KNNS_OK;
}

void DevBuf::release()
{
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
}

// ---------------------------------------------------------------- engine registry
static std::mutex g_reg_mu;
static std::map<int, std::unique_ptr<Engine>> g_engines;

int get_engine(Engine** out)
{
    int dev = 0;
    KNN_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(g_reg_mu);
    auto it = g_engines.find(dev);
    if (it != g_engines.end()) {
        *out = it->second.get();
        return KNNS_OK;
    }
    std::unique_ptr<Engine> e(new Engine());
    e->device = dev;
    KNN_CUDA(cudaDeviceGetAttribute(&e->sms, cudaDevAttrMultiProcessorCount, dev));
    int major = 0, minor = 0;
    KNN_CUDA(cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev));
    KNN_CUDA(cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev));
    e->cc = major * 10 + minor;
    KNN_CUDA(cudaEventCreateWithFlags(&e->last_done, cudaEventDisableTiming));
    int rc = e->err.ensure(sizeof(int));
    if (rc) return rc;
    KNN_CUDA(cudaMemset(e->err.p, 0, sizeof(int)));
    *out = e.get();
    g_engines[dev] = std::move(e);
    return KNNS_OK;
}

// ---------------------------------------------------------------- tensor maps
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static int get_encode_fn(EncodeTiledFn* fn)
{
    static EncodeTiledFn cached = nullptr;
    static std::mutex mu;
    std::lock_guard<std::mutex> lk(mu);
    if (!cached) {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q);
        if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !p)
            return set_error(KNNS_ERR_CUDA, "cuTensorMapEncodeTiled entry point unavailable");
        cached = (EncodeTiledFn)p;
    }
    *fn = cached;
    return KNNS_OK;
}

// 2-D fp32 matrix [rows][cols] (cols contiguous, rows `pitch` elements apart),
// box {32 cols, 128 rows}, 128B swizzle
static int encode_rows(CUtensorMap* m, const float* base, int64_t rows, int64_t cols, int64_t pitch = 0)
{
    EncodeTiledFn fn;
    int rc = get_encode_fn(&fn);
    if (rc) return rc;
    cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)(pitch > 0 ? pitch : cols) * sizeof(float)};
    cuuint32_t box[2] = {(cuuint32_t)kChunkK, (cuuint32_t)kTileN};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, (void*)base, dims, strides, box, estr,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return set_error(KNNS_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
    return KNNS_OK;
}

// 2-D bf16 matrix [rows][cols] (rows `pitch` elements apart), box {64 cols (128 B), 128 rows}, 128B swizzle
static int encode_rows_bf16(CUtensorMap* m, const void* base, int64_t rows, int64_t cols, int64_t pitch = 0)
{
    EncodeTiledFn fn;
    int rc = get_encode_fn(&fn);
    if (rc) return rc;
    cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)(pitch > 0 ? pitch : cols) * 2};
    cuuint32_t box[2] = {64u, (cuuint32_t)kTileN};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box, estr,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return set_error(KNNS_ERR_CUDA, "cuTensorMapEncodeTiled (bf16) failed (%d)", (int)r);
    return KNNS_OK;
}

// ---------------------------------------------------------------- planning
static inline int64_t cdiv(int64_t a, int64_t b) { return (a + b - 1) / b; }
static inline int round32(int x) { return (x + 31) & ~31; }
static inline int round16(int x) { return (x + 15) & ~15; }

// Shortlist length: k plus a re-rank margin of max(8, k/8), in multiples of 16.
int auto_kp(int k, int rerank)
{
    int kp = rerank ? round16(k + std::max(8, k / 8)) : round16(k);
    return std::max(kp, 32);
}

// Corpus splits: minimise (waves of CTAs) x (tiles per split), with a small
// charge per split for the shortlist warm-up and the merge.
int auto_splits(int64_t qtiles, int64_t tiles, int sms, int max_splits)
{
    int best = 1;
    double best_cost = 1e300;
    int lim = (int)std::min<int64_t>(tiles, max_splits);
    for (int S = 1; S <= lim; ++S) {
        double waves = (double)cdiv(qtiles * S, sms);
        double cost = waves * (double)cdiv(tiles, S) * (1.0 + 0.004 * S);
        if (cost < best_cost - 1e-9) {
            best_cost = cost;
            best = S;
        }
    }
    return best;
}

int resolve_config(const Engine& E, int64_t N, int64_t Q, int D, int k, const knns_options& o, Config* c)
{
    c->rerank = o.rerank ? 1 : 0;
    c->pilot = o.pilot != 0;
    c->precision = o.precision;
    if (o.precision == KNNS_PREC_BF16) {
        // BF16 keys rank a shortlist of c*k; the exact re-rank picks the k
        if (!o.rerank) return set_error(KNNS_ERR_INVALID, "BF16 precision needs the exact re-rank");
        if (E.cc < 100) return set_error(KNNS_ERR_UNSUPPORTED, "BF16 precision needs sm_100+");
        if (o.algo == KNNS_ALGO_SIMT) return set_error(KNNS_ERR_UNSUPPORTED, "BF16 precision runs on tensor cores");
        const int dpb = (D + 63) & ~63;
        if (dpb / 2 > kMaxDpTC) return set_error(KNNS_ERR_UNSUPPORTED, "BF16 precision needs D <= %d", 2 * kMaxDpTC);
        const int cf = o.shortlist > 0 ? o.shortlist : 4;
        c->kp = o.kp > 0 ? o.kp : std::max(32, round16(k * cf));
        if (c->kp % 16 != 0 || c->kp < k || c->kp > kMaxKpTC)
            return set_error(KNNS_ERR_UNSUPPORTED, "BF16 shortlist of %d entries (k=%d) outside [k, %d]", c->kp, k,
                             kMaxKpTC);
        c->algo = KNNS_ALGO_TC;
        c->dp = kChunkK;  // TF32 operands unused
        c->dpb = dpb;
        c->stages = std::min(4, tc_max_stages(c->kp));
        c->qtile = kTileQ;
        const int64_t tiles = cdiv(N, kTileN);
        int S = o.splits > 0 ? o.splits : auto_splits(cdiv(Q, kTileQ), tiles, E.sms, 64);
        S = (int)std::max<int64_t>(1, std::min<int64_t>(S, tiles));
        c->split_len = cdiv(tiles, S) * kTileN;
        c->splits = (int)cdiv(N, c->split_len);
        return KNNS_OK;
    } else if (o.precision != KNNS_PREC_EXACT) {
        return set_error(KNNS_ERR_INVALID, "unknown precision %d", o.precision);
    }
    c->kp = o.kp > 0 ? o.kp : auto_kp(k, c->rerank);
    if (o.kp <= 0 && c->kp > 512 && k <= 512) c->kp = std::max(round16(k), 32);  // no margin at the limit
    if (c->kp % 16 != 0 || c->kp < k || c->kp < 32)
        return set_error(KNNS_ERR_INVALID, "shortlist length %d must be a multiple of 16, >= 32 and >= k=%d", c->kp,
                         k);
    int algo = o.algo;
    const int dp = (int)round32(D);
    const bool tc_ok = E.cc >= 100 && dp <= kMaxDpTC;
    if (algo == KNNS_ALGO_AUTO) {
        if (tc_ok && c->kp > kMaxKpTC && round16(k) <= kMaxKpTC && o.kp <= 0) c->kp = std::max(round16(k), 32);
        algo = (tc_ok && c->kp <= kMaxKpTC) ? KNNS_ALGO_TC : KNNS_ALGO_SIMT;
    }
    if (algo == KNNS_ALGO_TC) {
        if (!tc_ok) return set_error(KNNS_ERR_UNSUPPORTED, "tensor-core path needs sm_100+ and D <= %d", kMaxDpTC);
        if (c->kp > kMaxKpTC)
            return set_error(KNNS_ERR_UNSUPPORTED, "tensor-core path holds at most %d shortlist entries", kMaxKpTC);
        c->dp = dp;
        c->dpb = (D + 63) & ~63;
        c->stages = std::min(4, tc_max_stages(c->kp));
        c->qtile = kTileQ;
    } else if (algo == KNNS_ALGO_SIMT) {
        if (c->kp > 512) return set_error(KNNS_ERR_UNSUPPORTED, "shortlist of %d entries exceeds 512", c->kp);
        c->qtile = c->kp <= 128 ? 128 : 32;
        c->dp = D;
        c->stages = 0;
    } else {
        return set_error(KNNS_ERR_INVALID, "unknown algo %d", algo);
    }
    c->algo = algo;
    const int tile_n = algo == KNNS_ALGO_TC ? kTileN : kSimtTileN;
    const int64_t tiles = cdiv(N, tile_n);
    const int64_t qtiles = cdiv(Q, c->qtile);
    int S = o.splits > 0 ? o.splits : auto_splits(qtiles, tiles, E.sms, 64);
    S = (int)std::max<int64_t>(1, std::min<int64_t>(S, tiles));
    int64_t per = cdiv(tiles, S) * tile_n;
    if (algo == KNNS_ALGO_TC && per % kTileN) per = cdiv(per, kTileN) * kTileN;
    c->split_len = per;
    c->splits = (int)cdiv(N, per);
    return KNNS_OK;
}

// ---------------------------------------------------------------- search
int run_search(Engine& E, const float* corpus, int64_t N, int64_t ldc, const float* queries, int64_t Q, int64_t ldq,
               int D, int k, float* dist, int32_t* idx, float* idx_f, const knns_options& o, cudaStream_t s,
               knns_stats* st)
{
    if (N <= 0 || D <= 0 || k <= 0 || Q < 0) return set_error(KNNS_ERR_INVALID, "invalid sizes N=%lld Q=%lld D=%d k=%d",
                                                               (long long)N, (long long)Q, D, k);
    if (k > N) return set_error(KNNS_ERR_INVALID, "k=%d exceeds the corpus size N=%lld", k, (long long)N);
    if (N > 0x7fffffffLL) return set_error(KNNS_ERR_UNSUPPORTED, "corpus larger than 2^31-1 rows");
    if (ldc < D || ldq < D) return set_error(KNNS_ERR_INVALID, "row pitch smaller than D");
    if (!corpus || (!queries && Q > 0)) return set_error(KNNS_ERR_INVALID, "null input pointer");
    Config c;
    int rc = resolve_config(E, N, Q, D, k, o, &c);
    if (rc) return rc;
    if (Q == 0) {
        if (st) *st = knns_stats{c.algo, c.splits, c.kp, c.stages, 0, 0, 0};
        return KNNS_OK;
    }

    const int64_t n_pad = cdiv(N, 128) * 128;
    size_t ws = 0;
    rc = E.cn.ensure(n_pad * sizeof(float));
    if (rc) return rc;
    ws += E.cn.cap;
    rc = E.part.ensure((size_t)c.splits * Q * c.kp * sizeof(uint64_t));
    if (rc) return rc;
    ws += E.part.cap;
    rc = E.thr.ensure(Q * sizeof(uint32_t));
    if (rc) return rc;
    ws += E.thr.cap;
    // Threshold seeding: a pilot pass over every s-th corpus row gives each
    // query the key of a conservatively high rank r of its sample shortlist;
    // the main pass drops candidates above it from the first tile on.  Exact:
    // a query whose merged shortlist ends up with fewer than min(kp, N)
    // entries is redone (its whole query tile) without the seed.
    const int sample_stride = 16;
    const bool pilot = c.pilot && N >= (int64_t)sample_stride * 4096;
    const int qt = (int)cdiv(Q, c.qtile);
    const int tile_n = c.algo == KNNS_ALGO_TC ? kTileN : kSimtTileN;
    int64_t ns = 0, ns_pad = 0, split_len1 = 0;
    int rank = 0, kp1 = 0, stages1 = 0, splits1 = 0;
    if (pilot) {
        ns = (N - 1) / sample_stride + 1;
        ns_pad = cdiv(ns, 128) * 128;
        const double per = (double)c.kp / sample_stride;
        rank = (int)std::ceil(2.0 * per + 3.0 * std::sqrt(per)) + 1;
        kp1 = std::max(32, round16(rank));
        stages1 = c.algo == KNNS_ALGO_TC ? std::min(4, tc_max_stages(kp1)) : 0;
        const int64_t tiles1 = cdiv(ns, tile_n);
        // at most one wave of CTAs: every extra split pays its own shortlist warm-up
        splits1 = (int)std::max<int64_t>(1, std::min<int64_t>(tiles1, E.sms / std::max(1, qt)));
        split_len1 = cdiv(tiles1, splits1) * tile_n;
        splits1 = (int)cdiv(ns, split_len1);
        rc = E.cn_s.ensure((size_t)ns_pad * sizeof(float));
        if (!rc) rc = E.thr2.ensure(Q * sizeof(uint32_t));
        if (!rc) rc = E.redo.ensure((size_t)qt * sizeof(uint32_t));
        if (!rc) rc = E.part.ensure((size_t)splits1 * Q * kp1 * sizeof(uint64_t));
        if (rc) return rc;
        ws += E.cn_s.cap + E.thr2.cap + E.redo.cap;
    }
    if (!c.rerank) {
        rc = E.qn.ensure(Q * sizeof(float));
        if (rc) return rc;
        ws += E.qn.cap;
    }
    const bool bf16_only = c.precision == KNNS_PREC_BF16;
    if (c.algo == KNNS_ALGO_TC) {
        if (!bf16_only) {
            rc = E.hi.ensure((size_t)N * c.dp * sizeof(float));
            if (!rc) rc = E.lo.ensure((size_t)N * c.dp * sizeof(float));
            if (rc) return rc;
        }
        rc = E.bf.ensure((size_t)N * c.dpb * 2);
        if (rc) return rc;
        rc = E.loflags.ensure(((size_t)cdiv(N, 128) + 2) * sizeof(uint32_t));
        if (rc) return rc;
        ws += E.hi.cap + E.lo.cap + E.bf.cap + E.loflags.cap;
    }

    KNN_CUDA(cudaStreamWaitEvent(s, E.last_done, 0));
    cudaEvent_t tv[4] = {nullptr, nullptr, nullptr, nullptr};
    if (o.timing && E.timing_slot(tv) != KNNS_OK) return KNNS_ERR_CUDA;
    if (tv[0]) KNN_CUDA(cudaEventRecord(tv[0], s));
    int launches = 0;
    float* cn = (float*)E.cn.p;
    KNN_CUDA(launch_norms(corpus, N, ldc, D, cn, n_pad, s));
    ++launches;
    if (!c.rerank) {
        KNN_CUDA(launch_norms(queries, Q, ldq, D, (float*)E.qn.p, Q, s));
        ++launches;
    }
    uint64_t* part = (uint64_t*)E.part.p;
    uint32_t* thr_g = (uint32_t*)E.thr.p;
    uint32_t* flags = nullptr;
    uint32_t* any_lo = nullptr;
    uint32_t* not_exact = nullptr;
    if (c.algo == KNNS_ALGO_TC) {
        flags = (uint32_t*)E.loflags.p;
        any_lo = flags + cdiv(N, 128);
        not_exact = any_lo + 1;
        KNN_CUDA(cudaMemsetAsync(any_lo, 0, 2 * sizeof(uint32_t), s));
        if (bf16_only) {
            // BF16 keys whatever the data: the "not exact" word stays 0 (the
            // conversion reports into the unused any_lo word instead)
            KNN_CUDA(launch_bf16(corpus, N, ldc, D, c.dpb, E.bf.p, any_lo, s));
            launches += 1;
        } else {
            // BF16 copy of the corpus and the exactness test of corpus and queries;
            // the TF32 split then runs only for data that is not BF16-exact
            KNN_CUDA(launch_bf16(corpus, N, ldc, D, c.dpb, E.bf.p, not_exact, s));
            KNN_CUDA(launch_bf16(queries, Q, ldq, D, c.dpb, nullptr, not_exact, s));
            KNN_CUDA(launch_split(corpus, N, ldc, D, c.dp, (float*)E.hi.p, (float*)E.lo.p, flags, any_lo, not_exact,
                                  s));
            launches += 3;
        }
    }
    if (tv[1]) KNN_CUDA(cudaEventRecord(tv[1], s));

    // One fused pass over a corpus view: rows 0, stride, 2*stride, ... (nview of them).
    auto fused_pass = [&](int64_t nview, int64_t stride, const float* cn_view, int kp, int stages, int splits,
                          int64_t split_len, uint32_t* thr, const uint32_t* redo, bool tile_flags) -> int {
        if (c.algo == KNNS_ALGO_TC) {
            TcArgs a;
            memset(&a, 0, sizeof(a));
            int r = 0;
            if (!bf16_only) {
                r = encode_rows(&a.tm_hi, (const float*)E.hi.p, nview, c.dp, stride * c.dp);
                if (!r) r = encode_rows(&a.tm_lo, (const float*)E.lo.p, nview, c.dp, stride * c.dp);
            }
            if (!r) r = encode_rows_bf16(&a.tm_bf, E.bf.p, nview, c.dpb, stride * c.dpb);
            if (r) return r;
            a.not_exact = not_exact;
            a.tile_redo = redo;
            a.dpb = c.dpb;
            a.cn = cn_view;
            a.queries = queries;
            a.Q = Q;
            a.ldq = ldq;
            a.N = nview;
            a.split_len = split_len;
            a.part = part;
            a.thr_g = thr;
            a.lo_flags = tile_flags ? flags : nullptr;
            a.corpus_any_lo = tile_flags ? any_lo : nullptr;
            a.dump = nullptr;
            a.err = (int*)E.err.p;
            a.D = D;
            a.dp = c.dp;
            a.kp = kp;
            a.stages = stages;
            // both precisions are launched; the one that does not match the data returns at once
            if (!bf16_only) {
                KNN_CUDA(launch_tc(a, splits, false, s));
                ++launches;
            }
            KNN_CUDA(launch_tc(a, splits, true, s));
            ++launches;
        } else {
            KNN_CUDA(launch_simt(corpus, nview, ldc * stride, cn_view, queries, Q, ldq, D, kp, c.qtile, split_len,
                                 splits, part, thr, s, redo));
            ++launches;
        }
        return KNNS_OK;
    };

    if (pilot) {
        float* cn_s = (float*)E.cn_s.p;
        KNN_CUDA(launch_gather_norms(cn, ns, sample_stride, cn_s, ns_pad, s));
        KNN_CUDA(cudaMemsetAsync(thr_g, 0xFF, Q * sizeof(uint32_t), s));
        rc = fused_pass(ns, sample_stride, cn_s, kp1, stages1, splits1, split_len1, thr_g, nullptr, false);
        if (rc) return rc;
        SelectExtra ex;
        ex.thr_out = thr_g;
        ex.thr_rank = rank;
        ex.qtile = c.qtile;
        KNN_CUDA(launch_select(part, splits1, Q, kp1, std::min(kp1, (int)ns), corpus, ldc, queries, ldq, D, 0,
                               nullptr, nullptr, nullptr, nullptr, s, ex));
        launches += 2;
    } else {
        KNN_CUDA(cudaMemsetAsync(thr_g, 0xFF, Q * sizeof(uint32_t), s));
    }
    rc = fused_pass(N, 1, cn, c.kp, c.stages, c.splits, c.split_len, thr_g, nullptr, true);
    if (rc) return rc;
    if (tv[2]) KNN_CUDA(cudaEventRecord(tv[2], s));
    SelectExtra ex;
    ex.qtile = c.qtile;
    uint32_t* redo = (uint32_t*)E.redo.p;
    if (pilot) {
        KNN_CUDA(cudaMemsetAsync(redo, 0, qt * sizeof(uint32_t), s));
        ex.redo_out = redo;
        ex.need = (int)std::min<int64_t>(c.kp, N);
    }
    KNN_CUDA(launch_select(part, c.splits, Q, c.kp, k, corpus, ldc, queries, ldq, D, c.rerank,
                           c.rerank ? nullptr : (const float*)E.qn.p, dist, idx, idx_f, s, ex));
    ++launches;
    if (pilot) {
        // fix-up: flagged query tiles again, unseeded (CTAs of other tiles return at once)
        uint32_t* thr2 = (uint32_t*)E.thr2.p;
        KNN_CUDA(cudaMemsetAsync(thr2, 0xFF, Q * sizeof(uint32_t), s));
        rc = fused_pass(N, 1, cn, c.kp, c.stages, c.splits, c.split_len, thr2, redo, true);
        if (rc) return rc;
        SelectExtra ex2;
        ex2.qtile = c.qtile;
        ex2.redo_in = redo;
        KNN_CUDA(launch_select(part, c.splits, Q, c.kp, k, corpus, ldc, queries, ldq, D, c.rerank,
                               c.rerank ? nullptr : (const float*)E.qn.p, dist, idx, idx_f, s, ex2));
        ++launches;
    }
    if (tv[3]) KNN_CUDA(cudaEventRecord(tv[3], s));
    KNN_CUDA(cudaEventRecord(E.last_done, s));
    if (st) *st = knns_stats{c.algo, c.splits, c.kp, c.stages, launches, pilot ? 1 : 0, (int64_t)ws};
    return KNNS_OK;
}

int check_device_error(Engine& E, cudaStream_t s)
{
    KNN_CUDA(cudaStreamSynchronize(s));
    int code = 0;
    KNN_CUDA(cudaMemcpy(&code, E.err.p, sizeof(int), cudaMemcpyDeviceToHost));
    if (code != 0) {
        KNN_CUDA(cudaMemset(E.err.p, 0, sizeof(int)));
        return set_error(KNNS_ERR_DEVICE_TIMEOUT, "kernel gave up a bounded wait (code %d) and wound down", code);
    }
    return KNNS_OK;
}

int search_host(const float* corpus, int64_t N, const float* queries, int64_t Q, int D, int k, float* dist,
                int32_t* idx, float* idx_f_host, const knns_options& o, double* seconds, knns_stats* st)
{
    if (N <= 0 || D <= 0 || k <= 0 || Q < 0) return set_error(KNNS_ERR_INVALID, "invalid sizes");
    if (!corpus || (!queries && Q > 0)) return set_error(KNNS_ERR_INVALID, "null input pointer");
    Engine* E = nullptr;
    int rc = get_engine(&E);
    if (rc) return rc;
    std::lock_guard<std::mutex> lk(E->mu);
    cudaStream_t s = E->host_stream();
    if (!s) return set_error(KNNS_ERR_CUDA, "stream creation failed");
    const size_t cb = (size_t)N * D * sizeof(float), qb = (size_t)Q * D * sizeof(float);
    const size_t ob = (size_t)Q * k;
    if ((rc = E->in_corpus.ensure(cb))) return rc;
    if ((rc = E->in_queries.ensure(std::max(qb, (size_t)4)))) return rc;
    if ((rc = E->out_dist.ensure(std::max(ob * 4, (size_t)4)))) return rc;
    if ((rc = E->out_idx.ensure(std::max(ob * 4, (size_t)4)))) return rc;
    cudaEvent_t t0 = E->t0(), t1 = E->t1();
    KNN_CUDA(cudaEventRecord(t0, s));
    KNN_CUDA(cudaMemcpyAsync(E->in_corpus.p, corpus, cb, cudaMemcpyHostToDevice, s));
    if (qb) KNN_CUDA(cudaMemcpyAsync(E->in_queries.p, queries, qb, cudaMemcpyHostToDevice, s));
    rc = run_search(*E, (const float*)E->in_corpus.p, N, D, (const float*)E->in_queries.p, Q, D, D, k,
                    dist ? (float*)E->out_dist.p : nullptr, idx ? (int32_t*)E->out_idx.p : nullptr,
                    idx_f_host ? (float*)E->out_idx.p : nullptr, o, s, st);
    if (rc) return rc;
    if (dist && ob) KNN_CUDA(cudaMemcpyAsync(dist, E->out_dist.p, ob * 4, cudaMemcpyDeviceToHost, s));
    if (idx && ob) KNN_CUDA(cudaMemcpyAsync(idx, E->out_idx.p, ob * 4, cudaMemcpyDeviceToHost, s));
    if (idx_f_host && ob) KNN_CUDA(cudaMemcpyAsync(idx_f_host, E->out_idx.p, ob * 4, cudaMemcpyDeviceToHost, s));
    KNN_CUDA(cudaEventRecord(t1, s));
    rc = check_device_error(*E, s);
    if (rc) return rc;
    float ms = 0.f;
    KNN_CUDA(cudaEventElapsedTime(&ms, t0, t1));
    if (seconds) *seconds = ms / 1000.0;
    return KNNS_OK;
}

int Engine::timing_slot(cudaEvent_t out[4])
{
    const size_t need = (size_t)(tcount + 1) * 4;
    while (tev.size() < need) {
        cudaEvent_t e;
        KNN_CUDA(cudaEventCreate(&e));
        tev.push_back(e);
    }
    for (int i = 0; i < 4; ++i) out[i] = tev[(size_t)tcount * 4 + i];
    ++tcount;
    return KNNS_OK;
}

cudaStream_t Engine::host_stream()
{
    if (!stream_) {
        if (cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking) != cudaSuccess) stream_ = nullptr;
    }
    return stream_;
}

cudaEvent_t Engine::t0()
{
    if (!ev0_) cudaEventCreate(&ev0_);
    return ev0_;
}

cudaEvent_t Engine::t1()
{
    if (!ev1_) cudaEventCreate(&ev1_);
    return ev1_;
}

void remember_stats(const knns_stats& st)
{
    g_last_stats = st;
    g_have_stats = true;
}

}  // namespace knn

using namespace knn;

extern "C" {

void knns_default_options(knns_options* opt)
{
    if (!opt) return;
    memset(opt, 0, sizeof(*opt));
    opt->algo = KNNS_ALGO_AUTO;
    opt->splits = 0;
    opt->rerank = 1;
    opt->kp = 0;
    opt->timing = 0;
    opt->pilot = 1;
    opt->precision = KNNS_PREC_EXACT;
    opt->shortlist = 0;
}

int knns_search_device(const float* corpus, int64_t N, int64_t ldc, const float* queries, int64_t Q, int64_t ldq,
                       int D, int k, float* dist, int32_t* idx, const knns_options* opt, void* stream)
{
    clear_error();
    knns_options o;
    if (opt) o = *opt;
    else knns_default_options(&o);
    Engine* E = nullptr;
    int rc = get_engine(&E);
    if (rc) return rc;
    std::lock_guard<std::mutex> lk(E->mu);
    knns_stats st;
    rc = run_search(*E, corpus, N, ldc, queries, Q, ldq, D, k, dist, idx, nullptr, o, (cudaStream_t)stream, &st);
    if (rc == KNNS_OK) remember_stats(st);
    return rc;
}

int knns_search_host(const float* corpus, int64_t N, const float* queries, int64_t Q, int D, int k, float* dist,
                     int32_t* idx, const knns_options* opt)
{
    clear_error();
    knns_options o;
    if (opt) o = *opt;
    else knns_default_options(&o);
    knns_stats st;
    int rc = search_host(corpus, N, queries, Q, D, k, dist, idx, nullptr, o, nullptr, &st);
    if (rc == KNNS_OK) remember_stats(st);
    return rc;
}

int knns_check_device(void* stream)
{
    clear_error();
    Engine* E = nullptr;
    int rc = get_engine(&E);
    if (rc) return rc;
    return check_device_error(*E, (cudaStream_t)stream);
}

const char* knns_last_error(void) { return g_last_error.c_str(); }

int knns_last_stats(knns_stats* out)
{
    if (!out) return KNNS_ERR_INVALID;
    if (!g_have_stats) return set_error(KNNS_ERR_INVALID, "no search has completed on this thread");
    *out = g_last_stats;
    return KNNS_OK;
}

int knns_version(void) { return 100; }

int knns_timing_collect(double ms[3], int* count)
{
    clear_error();
    if (!ms) return set_error(KNNS_ERR_INVALID, "null output");
    Engine* E = nullptr;
    int rc = get_engine(&E);
    if (rc) return rc;
    std::lock_guard<std::mutex> lk(E->mu);
    ms[0] = ms[1] = ms[2] = 0.0;
    for (int i = 0; i < E->tcount; ++i) {
        cudaEvent_t* ev = &E->tev[(size_t)i * 4];
        KNN_CUDA(cudaEventSynchronize(ev[3]));
        for (int j = 0; j < 3; ++j) {
            float t = 0.f;
            KNN_CUDA(cudaEventElapsedTime(&t, ev[j], ev[j + 1]));
            ms[j] += t;
        }
    }
    if (count) *count = E->tcount;
    E->tcount = 0;
    return KNNS_OK;
}

int knns_debug_tc_dot_tile(const float* corpus, int64_t N, const float* queries, int64_t Q, int D, float* dump)
{
    clear_error();
    if (!corpus || !queries || !dump || N <= 0 || Q <= 0 || D <= 0) return set_error(KNNS_ERR_INVALID, "bad args");
    Engine* E = nullptr;
    int rc = get_engine(&E);
    if (rc) return rc;
    std::lock_guard<std::mutex> lk(E->mu);
    if (E->cc < 100) return set_error(KNNS_ERR_UNSUPPORTED, "needs sm_100+");
    const int dp = (D + 31) & ~31;
    const int dpb = (D + 63) & ~63;
    if (dp > kMaxDpTC) return set_error(KNNS_ERR_UNSUPPORTED, "D > %d", kMaxDpTC);
    const int64_t n_use = std::min<int64_t>(N, kTileN);
    const int64_t n_pad = 128;
    cudaStream_t s = E->host_stream();
    if ((rc = E->cn.ensure(n_pad * 4))) return rc;
    if ((rc = E->hi.ensure((size_t)n_use * dp * 4))) return rc;
    if ((rc = E->lo.ensure((size_t)n_use * dp * 4))) return rc;
    if ((rc = E->bf.ensure((size_t)n_use * dpb * 2))) return rc;
    if ((rc = E->loflags.ensure(4 * sizeof(uint32_t)))) return rc;
    if ((rc = E->part.ensure((size_t)std::min<int64_t>(Q, kTileQ) * 32 * 8))) return rc;
    KNN_CUDA(cudaStreamWaitEvent(s, E->last_done, 0));
    KNN_CUDA(launch_norms(corpus, n_use, D, D, (float*)E->cn.p, n_pad, s));
    uint32_t* not_exact = (uint32_t*)E->loflags.p;
    const int64_t q_use = std::min<int64_t>(Q, kTileQ);
    KNN_CUDA(cudaMemsetAsync(not_exact, 0, sizeof(uint32_t), s));
    KNN_CUDA(launch_bf16(corpus, n_use, D, D, dpb, E->bf.p, not_exact, s));
    KNN_CUDA(launch_bf16(queries, q_use, D, D, dpb, nullptr, not_exact, s));
    KNN_CUDA(launch_split(corpus, n_use, D, D, dp, (float*)E->hi.p, (float*)E->lo.p, nullptr, nullptr, nullptr, s));
    TcArgs a;
    memset(&a, 0, sizeof(a));
    if ((rc = encode_rows(&a.tm_hi, (const float*)E->hi.p, n_use, dp))) return rc;
    if ((rc = encode_rows(&a.tm_lo, (const float*)E->lo.p, n_use, dp))) return rc;
    if ((rc = encode_rows_bf16(&a.tm_bf, E->bf.p, n_use, dpb))) return rc;
    a.not_exact = not_exact;
    a.dpb = dpb;
    a.cn = (const float*)E->cn.p;
    a.queries = queries;
    a.Q = std::min<int64_t>(Q, kTileQ);
    a.ldq = D;
    a.N = n_use;
    a.split_len = kTileN;
    a.part = (uint64_t*)E->part.p;
    a.thr_g = nullptr;
    a.lo_flags = nullptr;
    a.corpus_any_lo = nullptr;
    a.dump = dump;
    a.err = (int*)E->err.p;
    a.D = D;
    a.dp = dp;
    a.kp = 32;
    a.stages = std::min(4, tc_max_stages(32));
    KNN_CUDA(cudaMemsetAsync(dump, 0, (size_t)kTileQ * kTileN * 4, s));
    KNN_CUDA(launch_tc(a, 1, false, s));
    KNN_CUDA(launch_tc(a, 1, true, s));
    KNN_CUDA(cudaEventRecord(E->last_done, s));
    return check_device_error(*E, s);
}

}  // extern "C"
