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
#include <atomic>
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
// test hook (knns_debug_stall_next_search): wait bound of the next search's shortlist kernels,
// whose producers then issue no copy; 0 = off
static std::atomic<uint64_t> g_test_stall_ns{0};
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

// 2-D bf16 matrix [rows][cols] (rows `pitch` elements apart), box {64 cols (128 B), box_rows rows},
// 128B swizzle
static int encode_rows_bf16(CUtensorMap* m, const void* base, int64_t rows, int64_t cols, int64_t pitch = 0,
                            int box_rows = kTileN)
{
    EncodeTiledFn fn;
    int rc = get_encode_fn(&fn);
    if (rc) return rc;
    cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)(pitch > 0 ? pitch : cols) * 2};
    cuuint32_t box[2] = {64u, (cuuint32_t)box_rows};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box, estr,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return set_error(KNNS_ERR_CUDA, "cuTensorMapEncodeTiled (bf16) failed (%d)", (int)r);
    return KNNS_OK;
}

// Norm parts [rows][kNormParts] BF16 (rows `pitch` elements apart), box {kNormParts, box_rows},
// 32B swizzle (one 32-byte row per corpus row, the BF16 scan's last K step)
static int encode_np(CUtensorMap* m, const void* base, int64_t rows, int64_t pitch, int box_rows)
{
    EncodeTiledFn fn;
    int rc = get_encode_fn(&fn);
    if (rc) return rc;
    cuuint64_t dims[2] = {(cuuint64_t)kNormParts, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)pitch * 2};
    cuuint32_t box[2] = {(cuuint32_t)kNormParts, (cuuint32_t)box_rows};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box, estr,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_32B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return set_error(KNNS_ERR_CUDA, "cuTensorMapEncodeTiled (norm parts) failed (%d)", (int)r);
    return KNNS_OK;
}

// ---------------------------------------------------------------- planning
// smallest corpus the threshold scan runs on when asked to (KNNS_SCAN_ON, long shortlists)
constexpr int64_t kScanMinRowsForced = 16384;
// Corpus size from which the BF16 / E4M3 threshold scan runs by default; below it the exact
// form runs the 3xTF32 threshold scan (from kScanMinRowsForced rows) for data of any kind.
constexpr int64_t kScanMinRowsAuto = 131072;
// accumulators of the threshold scan when the options leave it open
constexpr int kScanAccsAuto = 2;
// widest rows the 3xTF32 scan takes: its K loop has no limit, the selection's re-rank stages
// candidate rows in shared memory (four rows of 2048 values per warp)
constexpr int kTscanMaxDp = 2048;
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
    if (o.precision == KNNS_PREC_BF16 || o.precision == KNNS_PREC_FP8) {
        // BF16 (or E4M3) keys rank a shortlist of c*k; the exact re-rank picks the k.
        // E4M3 keys run on the threshold scan; the fix-up of its rare failed queries
        // (and corpora too small for the scan) use BF16 keys.
        const char* name = o.precision == KNNS_PREC_FP8 ? "FP8" : "BF16";
        if (!o.rerank) return set_error(KNNS_ERR_INVALID, "%s precision needs the exact re-rank", name);
        if (E.cc < 100) return set_error(KNNS_ERR_UNSUPPORTED, "%s precision needs sm_100+", name);
        if (o.algo == KNNS_ALGO_SIMT) return set_error(KNNS_ERR_UNSUPPORTED, "%s precision runs on tensor cores", name);
        const int dpb = (D + 63) & ~63;
        if (dpb / 2 > kMaxDpTC) return set_error(KNNS_ERR_UNSUPPORTED, "%s precision needs D <= %d", name, 2 * kMaxDpTC);
        c->fp8 = o.precision == KNNS_PREC_FP8;
        c->dpf = c->fp8 ? ((D + 127) & ~127) / 2 : 0;
        const int cf = o.shortlist > 0 ? o.shortlist : 4;
        c->kp = o.kp > 0 ? o.kp : std::max(32, round16(k * cf));
        if (c->kp % 16 != 0 || c->kp < k || c->kp > kMaxKpScan)
            return set_error(KNNS_ERR_UNSUPPORTED, "%s shortlist of %d entries (k=%d) outside [k, %d]", name, c->kp, k,
                             kMaxKpScan);
        // shortlists above kMaxKpTC live only on the threshold scan (global candidate segments)
        if (c->kp > kMaxKpTC && (N < kScanMinRowsForced || o.scan == KNNS_SCAN_OFF))
            return set_error(KNNS_ERR_UNSUPPORTED,
                             "%s shortlist of %d entries needs the threshold scan (N >= %d, scan not off); "
                             "at most %d entries otherwise", name, c->kp, kScanMinRowsForced, kMaxKpTC);
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
    // The 3xTF32 threshold scan alone (no BF16 path beside it) on corpora large enough to seed
    // its thresholds: rows wider than 128 or k above 128 (the shortlist kernel's limits),
    // corpora below the BF16 scan's default size, or on request
    const bool wide = dp > kMaxDpTC || round16(k) > kMaxKpTC;
    const bool small = o.scan == KNNS_SCAN_AUTO && N < kScanMinRowsAuto && c->rerank;
    const bool tscan_ok = E.cc >= 100 && o.scan != KNNS_SCAN_OFF && N >= kScanMinRowsForced && dp <= kTscanMaxDp &&
                          c->kp <= kMaxKpScan && (wide || small || o.scan == KNNS_SCAN_TF32);
    if ((algo == KNNS_ALGO_AUTO || algo == KNNS_ALGO_TC) && tscan_ok) {
        c->algo = KNNS_ALGO_TC;
        c->tscan = true;
        c->dp = dp;
        c->dpb = (D + 63) & ~63;
        c->qtile = kTileQ;
        c->stages = 0;
        c->splits = 0;  // planned by the scan
        c->split_len = 0;
        return KNNS_OK;
    }
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

// ---------------------------------------------------------------- threshold-scan plan
// Seeding: the main scan needs, per query, a threshold T with at least kp keys
// below it (then every top-kp candidate is collected) and few more.  Nested
// corpus samples give it, coarse to fine: level l keeps every stride_l-th row
// (stride s for the finest level -- seed_stride below --, kSeedRatio x more per coarser level, the
// coarsest small enough to keep every key).  Each level collects the keys below
// the previous level's threshold and picks the key of rank j_l as its own.  With
// m = j_next / kSeedRatio (the expected rank, in this level's sample, of the key of
// rank j_next in the next one; m = kp / s for the finest level)
// j = 2m + 4 sqrt(m) + 1 leaves a chance of roughly 1e-5 that fewer than j_next
// keys fall below the threshold at the next level.  Queries for which that
// happens in the main pass (and any whose segments overflow) are found by the
// selection and searched again without a threshold, so results never depend
// on the seeds.
constexpr int kMaxSeedLevels = 6;
// Finest sampling stride: a coarser sample makes seeding cheaper (its cost grows with N / stride)
// and the main pass and its selection handle more candidates (about 2 kp + 4 sqrt(kp * stride)
// per query, whatever N).  Per search: 1M x 128, 2.429 ms with 32 against 2.447 with 64; 4M x 96
// (BF16 keys) 7.32 against 7.31; 8M x 256 (E4M3 keys) 32.4 against 31.7 (seeding 1.34 against
// 0.80 ms).  So 64 from 6M corpus rows on.  Long shortlists take a finer stride,
// so that a query's main-pass candidates (mean + six standard deviations) still fit the
// selection's buffer.
constexpr int64_t kSeedStride = 32;
constexpr int64_t kSeedStrideWide = 64;
constexpr int64_t kSeedStrideWideRows = 6000000;
// Stride ratio of neighbouring levels.  32 would leave two levels for a million rows where 16
// needs three, but its coarser thresholds cost more than the level they save: seeding 0.46
// against 0.37 ms on the 1M x 128 integer workload, and on the 4M x 96 mixture (BF16 keys) a
// main pass of 7.7 against 6.8 ms with 0.85 against 0.03 ms of fix-up.
constexpr int64_t kSeedRatio = 16;
// Rows of the coarsest sample, whose keys are all kept: at most what the threshold selection ranks
// in registers (32 lanes x 8 keys).  With 1,024 the 4M-row corpora kept 489 keys per query there:
// that level and its selection took 82 + 82 us on the 4M x 96 mixture (seeding 1.27 ms, 1.19 with
// one more level of 31 rows; 8M x 256: 1.64 against 1.36 ms).
constexpr int64_t kSeedCoarsest = 256;

static int64_t seed_stride(int kp, int64_t N)
{
    int64_t s = N >= kSeedStrideWideRows ? kSeedStrideWide : kSeedStride;
    while (s > 4) {
        const double mean = 2.0 * kp + 4.0 * std::sqrt((double)kp * s), spread = 6.0 * std::sqrt(2.0 * kp * s);
        if (mean + spread + 64.0 <= (double)kCandMax) break;
        s /= 2;
    }
    return s;
}

struct ScanLevel {
    int64_t n = 0, stride = 1, len = 0, n_pad = 0;
    int j = 0, S = 1, cap = 0;
};

struct ScanPlan {
    int bps = 0, ring = 0, accs = 2;
    int64_t stride0 = 0;  // finest seeding stride
    int levels = 0;
    ScanLevel lv[kMaxSeedLevels];
    int64_t len = 0;
    int S = 1, cap = 0;
    int sel_words = 0;  // bound on one query's stored main-pass candidates (selection buffer)
    int64_t fixA_rows = 0, fixA_len = 0, fixB_rows = 0, fixB_len = 0;
    int fixA_S = 1, fixB_S = 1;
    bool simt_fix = false;  // the fix-up runs on the CUDA-core kernel (shortlist above kMaxKpTC)
    size_t cand_words = 0, cnt_words = 0, part_words = 0, norm_words = 0;
};

// Split count of a seeding pass: few tiles per CTA, so each CTA's fixed cost (setup, the
// queries into tensor memory, the first corpus copies, the drain; about 8 tiles' worth)
// counts beside the waves x tiles of auto_splits.  (The main pass keeps auto_splits: there
// the model moved it to more splits, a slower scan and a slower selection.)
static int seed_splits(int64_t qtiles, int64_t tiles, int sms, int max_splits)
{
    constexpr double kFixedTiles = 8.0;
    int best = 1;
    double best_cost = 1e300;
    const int lim = (int)std::min<int64_t>(tiles, max_splits);
    for (int S = 1; S <= lim; ++S) {
        const double waves = (double)cdiv(qtiles * S, sms);
        const double cost = waves * ((double)cdiv(tiles, S) + kFixedTiles);
        if (cost < best_cost - 1e-9) {
            best_cost = cost;
            best = S;
        }
    }
    return best;
}

static int seg_cap(double per_seg, double sigmas)
{
    return round16((int)std::ceil(sigmas * per_seg + 8.0 * std::sqrt(per_seg) + 16.0));
}

static int seed_rank(double m) { return (int)std::ceil(2.0 * m + 4.0 * std::sqrt(m)) + 1; }

// tf32: the plan of the 3xTF32 scan (tiles of 128 rows, 32 columns per segment; fix-up on the
// CUDA-core kernel); otherwise of the BF16 / E4M3 scan of row width dpb.
static int plan_scan(const Engine& E, int64_t N, int64_t Q, int dpb, int kp, const knns_options& o, ScanPlan* P,
                     bool fp8, bool tf32 = false)
{
    if (o.scan_accs != 0 && o.scan_accs != 2 && o.scan_accs != 4)
        return set_error(KNNS_ERR_INVALID, "threshold scan: %d accumulators (2 or 4)", o.scan_accs);
    int tn = 128, pc = 32;
    if (tf32) {
        P->accs = 4;
        P->ring = tscan_ring(dpb <= 128);  // rows of up to 128 columns: queries in tensor memory
    } else {
        P->accs = o.scan_accs ? o.scan_accs : kScanAccsAuto;
        if (scan_plan(dpb, o.scan_boxes, &P->bps, &P->ring, fp8, P->accs) != 0)
            return set_error(KNNS_ERR_UNSUPPORTED,
                             "threshold scan: no ring geometry for %d BF16 columns with %d boxes per slot", dpb,
                             o.scan_boxes);
        tn = scan_tile_rows(dpb, P->accs);
        pc = scan_part_cols(dpb, P->accs);  // segment columns per tile
    }
    const int64_t qt = cdiv(Q, kTileQ);  // query tiles
    // levels, finest first: strides s, kSeedRatio s, ... until the sample is small enough to keep
    // every key (kSeedCoarsest rows)
    P->stride0 = seed_stride(kp, N);
    int64_t st[kMaxSeedLevels];
    int L = 0;
    for (int64_t stride = P->stride0;; stride *= kSeedRatio) {
        if (L == kMaxSeedLevels) return set_error(KNNS_ERR_UNSUPPORTED, "threshold scan: corpus too large to seed");
        st[L++] = stride;
        if (cdiv(N, stride) <= kSeedCoarsest) break;
    }
    P->levels = L;
    // level index 0 = coarsest
    for (int l = 0; l < L; ++l) {
        ScanLevel& v = P->lv[l];
        v.stride = st[L - 1 - l];
        v.n = cdiv(N, v.stride);
        v.n_pad = cdiv(v.n, kScanTileN) * kScanTileN + kScanTileN;  // >= one tile past the view
    }
    // ranks, finest to coarsest
    double m = (double)kp / (double)P->stride0;
    for (int l = L - 1; l >= 0; --l) {
        ScanLevel& v = P->lv[l];
        v.j = std::min<int>((int)v.n, seed_rank(m));
        if (l > 0) m = (double)v.j * (double)P->lv[l - 1].n / (double)v.n;
    }
    if (P->lv[L - 1].j > kCandMax / 2 || P->lv[L - 1].n < 4 * P->lv[L - 1].j)
        return set_error(KNNS_ERR_UNSUPPORTED, "threshold scan: shortlist of %d too long for N=%lld", kp, (long long)N);
    P->cand_words = 0;
    P->cnt_words = 0;
    P->norm_words = 0;
    for (int l = 0; l < L; ++l) {
        ScanLevel& v = P->lv[l];
        const int64_t tiles = cdiv(v.n, tn);
        if (l == 0) {
            // every key kept: at most two splits, each segment holds all its columns
            v.S = (int)std::min<int64_t>(2, tiles);
            v.len = cdiv(tiles, v.S) * tn;
            v.S = (int)cdiv(v.n, v.len);
            v.cap = (int)(v.len / tn * pc);
        } else {
            v.S = seed_splits(qt, tiles, E.sms, kScanMaxSegs / kScanParts);
            v.len = cdiv(tiles, v.S) * tn;
            v.S = (int)cdiv(v.n, v.len);
            const double hits = (double)P->lv[l - 1].j * (double)v.n / (double)P->lv[l - 1].n;
            v.cap = std::min<int>((int)(v.len / tn * pc), seg_cap(hits * pc / ((double)tn * v.S), 3.0));
        }
        P->cand_words = std::max(P->cand_words, (size_t)kScanParts * v.S * Q * v.cap);
        P->cnt_words = std::max(P->cnt_words, (size_t)kScanParts * v.S * Q);
        P->norm_words += (size_t)v.n_pad;
    }
    // main pass
    const int64_t tiles = cdiv(N, tn);
    const int max_splits = kScanMaxSegs / kScanParts;
    P->S = o.splits > 0 ? std::min<int>(std::min(o.splits, max_splits), (int)tiles)
                        : auto_splits(qt, tiles, E.sms, max_splits);
    P->len = cdiv(tiles, P->S) * tn;
    P->S = (int)cdiv(N, P->len);
    const double hm = (double)P->lv[L - 1].j * (double)P->lv[L - 1].stride;
    P->cap = std::min<int>((int)(P->len / tn * pc), seg_cap(hm * pc / ((double)tn * P->S), 2.0));
    // a query's main-pass count is about stride x (a Gamma(j) variable): hm + 6 stride sqrt(j)
    // bounds it but for queries whose strided sample misrepresents them (those fail over to
    // the fix-up either way); the selection buffer is sized to it, not to its ceiling
    P->sel_words = (int)std::min<double>(
        (double)kCandMax, std::ceil((hm + 6.0 * (double)P->lv[L - 1].stride * std::sqrt((double)P->lv[L - 1].j) + 64.0) / 32.0) * 32.0);
    P->cand_words = std::max(P->cand_words, (size_t)kScanParts * P->S * Q * P->cap);
    P->cnt_words = std::max(P->cnt_words, (size_t)kScanParts * P->S * Q);
    // fix-up of failed queries: up to 512 on a full wave, the rest (rare) on 8 splits; shortlists
    // above the tensor-core kernel's kMaxKpTC go to the CUDA-core kernel in tiles of 32 queries
    // (exact FP32 keys): the first 32 failed queries on a wave of splits, the rest on 8
    P->simt_fix = kp > kMaxKpTC || tf32;
    const int ft = P->simt_fix ? kSimtTileN : kTileN;
    const int fq = P->simt_fix ? 32 : kTileQ;
    const int64_t tilesF = cdiv(N, ft);
    P->fixA_rows = std::min<int64_t>(Q, P->simt_fix ? fq : 4 * kTileQ);
    P->fixA_S = (int)std::max<int64_t>(1, std::min<int64_t>(tilesF, E.sms / cdiv(P->fixA_rows, fq)));
    P->fixA_len = cdiv(tilesF, P->fixA_S) * ft;
    P->fixA_S = (int)cdiv(N, P->fixA_len);
    P->fixB_rows = Q - P->fixA_rows;
    P->fixB_S = (int)std::min<int64_t>(tilesF, 8);
    P->fixB_len = cdiv(tilesF, P->fixB_S) * ft;
    P->fixB_S = (int)cdiv(N, P->fixB_len);
    P->part_words = std::max((size_t)P->fixA_S * P->fixA_rows * kp, (size_t)P->fixB_S * P->fixB_rows * kp);
    return KNNS_OK;
}

// ---------------------------------------------------------------- 3xTF32 threshold scan
// The stages of the 3xTF32 threshold scan over prepared corpus operands (norms, TF32 hi / lo
// copies and their tile flags) and query norms: the queries' TF32 split, threshold seeding over
// nested corpus samples, the main scan, the selection with the exact re-rank, and the CUDA-core
// fix-up of the queries the scan could not answer.  With run_if set, every kernel that writes
// thresholds, candidates or results returns at once unless *run_if != 0 (the exact form's
// device-side choice between BF16 and TF32 keys); its failed-query list is its own (fail), so
// the other path's fix-up never sees it.
struct TscanStages {
    Engine& E;
    const Config& c;
    const ScanPlan& sp;
    const float* corpus;
    int64_t N, ldc;
    const float* queries;
    int64_t Q, ldq;
    int D, k;
    const float* cn;
    const float* hi;
    const float* lo;
    const uint32_t* cflags;
    const float* qn;
    float* dist;
    int32_t* idx;
    float* idx_f;
    const uint32_t* run_if;
    uint32_t* q_any_lo;  // a word the queries' split ORs its low-part flag into
    DevBuf& fail;
    DevBuf& thr2;        // fix-up thresholds
    cudaStream_t s;
    int launches = 0;
    TscanArgs a;
    const float* T = nullptr;

    // buffers of the queries and of the plan (the corpus side is the caller's)
    int ensure()
    {
        const int dp = c.dp;
        int rc = E.qhi.ensure((size_t)Q * dp * sizeof(float));
        if (!rc) rc = E.qlo.ensure((size_t)Q * dp * sizeof(float));
        if (!rc) rc = E.qlof.ensure(((size_t)cdiv(Q, 128) + 4) * sizeof(uint32_t));
        if (!rc) rc = E.tq.ensure((size_t)2 * Q * sizeof(float));
        if (!rc) rc = E.cand.ensure(sp.cand_words * sizeof(uint64_t));
        if (!rc) rc = E.cnt.ensure(sp.cnt_words * sizeof(uint32_t));
        if (!rc) rc = E.cnv.ensure(sp.norm_words * sizeof(float));
        if (!rc) rc = fail.ensure((size_t)(Q + 1) * sizeof(uint32_t));
        if (!rc) rc = E.part.ensure(sp.part_words * sizeof(uint64_t));
        if (!rc) rc = thr2.ensure(Q * sizeof(uint32_t));
        return rc;
    }
    size_t workspace() const
    {
        return E.qhi.cap + E.qlo.cap + E.qlof.cap + E.tq.cap + E.cand.cap + E.cnt.cap + E.cnv.cap + fail.cap +
               E.part.cap + thr2.cap;
    }
    // the queries' TF32 hi / lo copies and the tensor maps of the scan's query operand
    int split_queries()
    {
        memset(&a, 0, sizeof(a));
        if (c.dp <= 128) {
            // the kernel splits the queries into tensor memory itself
            a.tmem_a = 1;
            a.queries = queries;
            a.ldq = ldq;
            a.D = D;
        } else {
            KNN_CUDA(launch_split(queries, Q, ldq, D, c.dp, (float*)E.qhi.p, (float*)E.qlo.p, (uint32_t*)E.qlof.p,
                                  q_any_lo, run_if, s));
            ++launches;
            int rc = encode_rows(&a.tm_qhi, (const float*)E.qhi.p, Q, c.dp, c.dp);
            if (!rc) rc = encode_rows(&a.tm_qlo, (const float*)E.qlo.p, Q, c.dp, c.dp);
            if (rc) return rc;
            a.qlo_flags = (const uint32_t*)E.qlof.p;
        }
        a.cand = (uint64_t*)E.cand.p;
        a.cnt = (uint32_t*)E.cnt.p;
        a.err = (int*)E.err.p;
        a.Q = Q;
        a.dp = c.dp;
        a.ring = sp.ring;
        a.run_if = run_if;
        return KNNS_OK;
    }
    // one scan over rows 0, stride, 2*stride, ... of the corpus (nview of them)
    int pass(int64_t nview, int64_t stride, const float* cn_view, const float* thr, int splits, int64_t split_len,
             int cap, const uint32_t* flags)
    {
        int r = encode_rows(&a.tm_chi, hi, nview, c.dp, stride * c.dp);
        if (!r) r = encode_rows(&a.tm_clo, lo, nview, c.dp, stride * c.dp);
        if (r) return r;
        a.cn = cn_view;
        a.thr = thr;
        a.N = nview;
        a.split_len = split_len;
        a.cap = cap;
        a.clo_flags = flags;
        KNN_CUDA(launch_tscan(a, splits, s));
        ++launches;
        return KNNS_OK;
    }
    CandSelect cand_select() const
    {
        CandSelect cs;
        cs.cand = (const uint64_t*)E.cand.p;
        cs.cnt = (const uint32_t*)E.cnt.p;
        cs.Q = Q;
        cs.D = D;
        cs.skip_if_zero = run_if;
        return cs;
    }
    // seeding, coarse to fine: level l keeps the keys below the previous level's threshold (the
    // coarsest keeps every key) and yields the key of rank j_l
    int seed()
    {
        float* Tbuf[2] = {(float*)E.tq.p, (float*)E.tq.p + Q};
        float* cnv = (float*)E.cnv.p;
        CandSelect cs = cand_select();
        T = nullptr;
        for (int l = 0; l < sp.levels; ++l) {
            const ScanLevel& v = sp.lv[l];
            KNN_CUDA(launch_gather_norms(cn, v.n, v.stride, cnv, v.n_pad, s, std::numeric_limits<float>::infinity(), run_if));
            int rc = pass(v.n, v.stride, cnv, T, v.S, v.len, v.cap, nullptr);
            if (rc) return rc;
            cs.nseg = kScanParts * v.S;
            cs.cap = v.cap;
            cs.thr_out = Tbuf[l & 1];
            cs.thr_rank = v.j;
            cs.thr_fallback = T;
            KNN_CUDA(launch_select_cand(cs, s));
            launches += 2;
            T = Tbuf[l & 1];
            cnv += v.n_pad;
        }
        return KNNS_OK;
    }
    int main_pass() { return pass(N, 1, cn, T, sp.S, sp.len, sp.cap, cflags); }
    int select()
    {
        uint32_t* fail_cnt = (uint32_t*)fail.p;
        KNN_CUDA(cudaMemsetAsync(fail_cnt, 0, sizeof(uint32_t), s));
        CandSelect cs = cand_select();
        cs.nseg = kScanParts * sp.S;
        cs.cap = sp.cap;
        cs.kp = c.kp;
        cs.k = k;
        cs.need = (int)std::min<int64_t>(c.kp, N);
        cs.buf_words = sp.sel_words;
        cs.rerank = c.rerank;
        cs.corpus = corpus;
        cs.ldc = ldc;
        cs.queries = queries;
        cs.ldq = ldq;
        cs.qn = qn;
        cs.out_dist = dist;
        cs.out_idx = idx;
        cs.out_idx_f = idx_f;
        cs.fail_idx = (int32_t*)fail.p + 1;
        cs.fail_cnt = fail_cnt;
        KNN_CUDA(launch_select_cand(cs, s));
        ++launches;
        return KNNS_OK;
    }
    // fix-up: the queries the scan could not answer, on the CUDA-core kernel (exact FP32 keys),
    // compacted; launches whose rows are all past the failure count return at once
    int fix_pass(int64_t qbase, int64_t rows, int splits, int64_t split_len)
    {
        if (rows <= 0) return KNNS_OK;
        uint32_t* fail_cnt = (uint32_t*)fail.p;
        int32_t* fail_idx = (int32_t*)fail.p + 1;
        uint32_t* t2 = (uint32_t*)thr2.p;
        KNN_CUDA(cudaMemsetAsync(t2, 0xFF, rows * sizeof(uint32_t), s));
        KNN_CUDA(launch_simt(corpus, N, ldc, cn, queries, rows, ldq, D, c.kp, 32, split_len, splits,
                             (uint64_t*)E.part.p, t2, s, nullptr, fail_idx, fail_cnt, qbase));
        SelectExtra ex;
        ex.qmap = fail_idx;
        ex.qcount = fail_cnt;
        ex.qbase = qbase;
        KNN_CUDA(launch_select((const uint64_t*)E.part.p, splits, rows, c.kp, k, corpus, ldc, queries, ldq, D,
                               c.rerank, c.rerank ? nullptr : qn, dist, idx, idx_f, s, ex));
        launches += 2;
        return KNNS_OK;
    }
    int fix()
    {
        int rc = fix_pass(0, sp.fixA_rows, sp.fixA_S, sp.fixA_len);
        if (!rc) rc = fix_pass(sp.fixA_rows, sp.fixB_rows, sp.fixB_S, sp.fixB_len);
        return rc;
    }
};

// The exact form on TF32 keys alone (rows wider than 128, k above 128, corpora below the BF16
// scan's size, or on request): corpus and query norms and TF32 copies, then the stages above.
static int run_tscan(Engine& E, const Config& c, const float* corpus, int64_t N, int64_t ldc, const float* queries,
                     int64_t Q, int64_t ldq, int D, int k, float* dist, int32_t* idx, float* idx_f,
                     const knns_options& o, cudaStream_t s, knns_stats* st, const PreparedCorpus* pc, bool capture)
{
    ScanPlan sp;
    int rc = plan_scan(E, N, Q, c.dpb, c.kp, o, &sp, false, true);
    if (rc) return rc;
    const int dp = c.dp;
    if (pc && (!pc->tf32 || pc->dp != dp))
        return set_error(KNNS_ERR_INVALID, "the exact form needs an index prepared with TF32 copies of this width");
    const int64_t n_pad = cdiv(N, kScanTileN) * kScanTileN + kScanTileN;
    if (!pc) {
        rc = E.cn.ensure(n_pad * sizeof(float));
        if (!rc) rc = E.hi.ensure((size_t)N * dp * sizeof(float));
        if (!rc) rc = E.lo.ensure((size_t)N * dp * sizeof(float));
        if (!rc) rc = E.loflags.ensure(((size_t)cdiv(N, 128) + 4) * sizeof(uint32_t));
        if (rc) return rc;
    }
    rc = E.qn.ensure(Q * sizeof(float));
    if (!rc) rc = E.words.ensure(8 * sizeof(uint32_t));
    if (rc) return rc;
    uint32_t* words = (uint32_t*)E.words.p;
    float* cn = (float*)(pc ? pc->cn.p : E.cn.p);
    uint32_t* cflags = (uint32_t*)(pc ? pc->tiles.p : E.loflags.p);
    TscanStages ts{E, c, sp, corpus, N, ldc, queries, Q, ldq, D, k, cn,
                   (const float*)(pc ? pc->hi.p : E.hi.p), (const float*)(pc ? pc->lo.p : E.lo.p), cflags,
                   (const float*)E.qn.p, dist, idx, idx_f, nullptr, words + 1, E.fail, E.thr2, s};
    if ((rc = ts.ensure())) return rc;
    const size_t ws = (pc ? 0 : E.cn.cap + E.hi.cap + E.lo.cap + E.loflags.cap) + E.qn.cap + ts.workspace();

    if (!capture) KNN_CUDA(cudaStreamWaitEvent(s, E.last_done, 0));
    cudaEvent_t tv[Engine::kTimingEvents] = {};
    if (o.timing && E.timing_slot(tv) != KNNS_OK) return KNNS_ERR_CUDA;
    auto mark = [&](int i) -> int {
        if (tv[i]) KNN_CUDA(cudaEventRecord(tv[i], s));
        return KNNS_OK;
    };
    if ((rc = mark(0))) return rc;
    KNN_CUDA(cudaMemsetAsync(words, 0, 4 * sizeof(uint32_t), s));
    if (!pc) {
        KNN_CUDA(launch_prep_rows(corpus, N, ldc, D, 0, nullptr, cn, n_pad, nullptr, s));
        KNN_CUDA(launch_split(corpus, N, ldc, D, dp, (float*)E.hi.p, (float*)E.lo.p, cflags, words, nullptr, s));
        ts.launches += 2;
    }
    KNN_CUDA(launch_prep_rows(queries, Q, ldq, D, 0, nullptr, (float*)E.qn.p, Q, nullptr, s));
    ++ts.launches;
    if ((rc = ts.split_queries())) return rc;
    if ((rc = mark(1))) return rc;
    if ((rc = ts.seed())) return rc;
    if ((rc = mark(2))) return rc;
    if ((rc = ts.main_pass())) return rc;
    if ((rc = mark(3))) return rc;
    if ((rc = ts.select())) return rc;
    if ((rc = mark(4))) return rc;
    if ((rc = ts.fix())) return rc;
    if ((rc = mark(5))) return rc;
    if (!capture) KNN_CUDA(cudaEventRecord(E.last_done, s));
    if (st)
        *st = knns_stats{c.algo, sp.S, c.kp, 0, ts.launches, 1, (int64_t)ws, 1, sp.S, sp.cap, 100 * sp.ring, 2};
    return KNNS_OK;
}

// ---------------------------------------------------------------- search
int run_search(Engine& E, const float* corpus, int64_t N, int64_t ldc, const float* queries, int64_t Q, int64_t ldq,
               int D, int k, float* dist, int32_t* idx, float* idx_f, const knns_options& o, cudaStream_t s,
               knns_stats* st, const PreparedCorpus* pc, bool capture, const float* host_corpus)
{
    if (N <= 0 || D <= 0 || k <= 0 || Q < 0) return set_error(KNNS_ERR_INVALID, "invalid sizes N=%lld Q=%lld D=%d k=%d",
                                                               (long long)N, (long long)Q, D, k);
    if (k > N) return set_error(KNNS_ERR_INVALID, "k=%d exceeds the corpus size N=%lld", k, (long long)N);
    if (N > 0x7fffffffLL) return set_error(KNNS_ERR_UNSUPPORTED, "corpus larger than 2^31-1 rows");
    if (ldc < D || ldq < D) return set_error(KNNS_ERR_INVALID, "row pitch smaller than D");
    if (!corpus || (!queries && Q > 0)) return set_error(KNNS_ERR_INVALID, "null input pointer");
    if (o.scan < KNNS_SCAN_AUTO || o.scan > KNNS_SCAN_TF32) return set_error(KNNS_ERR_INVALID, "unknown scan mode %d", o.scan);
    Config c;
    int rc = resolve_config(E, N, Q, D, k, o, &c);
    if (rc) return rc;
    if (Q == 0) {
        if (st) *st = knns_stats{c.algo, c.splits, c.kp, c.stages, 0, 0, 0, 0, 0, 0, 0, 0};
        return KNNS_OK;
    }
    // the precision forms: BF16 / E4M3 keys only, always re-ranked
    const bool bf16_only = c.precision == KNNS_PREC_BF16 || c.precision == KNNS_PREC_FP8;
    const uint64_t stall_ns = capture ? 0 : g_test_stall_ns.exchange(0);
    if (host_corpus != nullptr && (pc != nullptr || capture || ldc != D))
        return set_error(KNNS_ERR_INVALID, "a corpus streamed from the host needs pitch D and no prepared index");
    if (c.tscan) {
        if (host_corpus != nullptr) {
            // the whole corpus lands before the search starts (no overlap on this path)
            cudaStream_t cs_ = E.copy_stream();
            cudaEvent_t e0 = E.order_event(0), e1 = E.order_event(1);
            if (!cs_ || !e0 || !e1) return set_error(KNNS_ERR_CUDA, "stream or event creation failed");
            KNN_CUDA(cudaStreamWaitEvent(s, E.last_done, 0));
            KNN_CUDA(cudaEventRecord(e0, s));
            KNN_CUDA(cudaStreamWaitEvent(cs_, e0, 0));
            KNN_CUDA(cudaMemcpyAsync(const_cast<float*>(corpus), host_corpus, (size_t)N * D * sizeof(float),
                                     cudaMemcpyHostToDevice, cs_));
            KNN_CUDA(cudaEventRecord(e1, cs_));
            KNN_CUDA(cudaStreamWaitEvent(s, e1, 0));
        }
        return run_tscan(E, c, corpus, N, ldc, queries, Q, ldq, D, k, dist, idx, idx_f, o, s, st, pc, capture);
    }

    // The threshold scan serves BF16 keys on large corpora: always in the BF16
    // precision form, and in the exact form when the data turn out BF16-exact; otherwise the
    // exact form runs the 3xTF32 threshold scan (decided on the device: the kernels of the path
    // that does not match the data return at once).
    ScanPlan sp, sp_tf;
    bool scan = false;
    if (c.algo == KNNS_ALGO_TC && o.scan != KNNS_SCAN_OFF && E.cc >= 100 && c.dpb <= 256 && c.rerank) {
        const int64_t min_n = (o.scan == KNNS_SCAN_ON || c.kp > kMaxKpTC) ? kScanMinRowsForced : kScanMinRowsAuto;
        if (N >= min_n) {
            rc = plan_scan(E, N, Q, c.fp8 ? c.dpf : c.dpb, c.kp, o, &sp, c.fp8);
            if (rc) return rc;
            scan = true;
        }
    }
    // E4M3 keys exist only on the scan: without it the form falls back to BF16 keys
    const bool f8 = scan && c.fp8;
    // beside the BF16 scan, the exact form's TF32 keys run on the 3xTF32 scan; without the scan,
    // on the shortlist kernel
    const bool tf_scan = scan && !bf16_only;
    const bool run_old = !scan;
    if (tf_scan && (rc = plan_scan(E, N, Q, c.dpb, c.kp, o, &sp_tf, false, true))) return rc;
    if (pc != nullptr) {
        // (the CUDA-core kernel uses the index's norms only)
        if (pc->corpus != corpus || pc->N != N || pc->ldc != ldc || pc->D != D ||
            (c.algo == KNNS_ALGO_TC && pc->dpb != c.dpb))
            return set_error(KNNS_ERR_INVALID, "prepared corpus does not match the search's corpus");
        if (f8 && !pc->fp8) return set_error(KNNS_ERR_INVALID, "the FP8 form needs an index prepared with E4M3 copies");
        if (c.algo == KNNS_ALGO_TC && !bf16_only && !pc->tf32)
            return set_error(KNNS_ERR_INVALID, "the exact form needs an index prepared with TF32 copies");
        if (c.algo == KNNS_ALGO_TC && !bf16_only && pc->dp != c.dp)
            return set_error(KNNS_ERR_INVALID, "prepared corpus has TF32 copies of another width");
    }

    // norms padded with +inf at least one tile (of any kernel) past the corpus
    const int64_t n_pad = cdiv(N, kScanTileN) * kScanTileN + kScanTileN;
    size_t ws = 0;
    if (!pc) {
        rc = E.cn.ensure(n_pad * sizeof(float));
        if (rc) return rc;
        ws += E.cn.cap;
    }
    rc = E.words.ensure(8 * sizeof(uint32_t));
    if (rc) return rc;
    rc = E.thr.ensure(Q * sizeof(uint32_t));
    if (rc) return rc;
    ws += E.thr.cap;
    if (run_old) {
        rc = E.part.ensure((size_t)c.splits * Q * c.kp * sizeof(uint64_t));
        if (rc) return rc;
    }
    // Threshold seeding of the shortlist path: a pilot pass over every s-th
    // corpus row gives each query the key of a conservatively high rank r of
    // its sample shortlist; the main pass drops candidates above it from the
    // first tile on.  Exact: a query whose merged shortlist ends up with fewer
    // than min(kp, N) entries is redone (its whole query tile) without the seed.
    const int sample_stride = 16;
    const bool pilot = run_old && c.pilot && N >= (int64_t)sample_stride * 4096;
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
        ws += E.cn_s.cap + E.redo.cap;
    }
    if (!c.rerank || scan) {
        rc = E.qn.ensure(Q * sizeof(float));
        if (rc) return rc;
        ws += E.qn.cap;
    }
    if (c.algo == KNNS_ALGO_TC && !pc) {
        if (!bf16_only) {
            rc = E.hi.ensure((size_t)N * c.dp * sizeof(float));
            if (!rc) rc = E.lo.ensure((size_t)N * c.dp * sizeof(float));
            if (rc) return rc;
        }
        rc = E.bf.ensure((size_t)N * c.dpb * 2);
        if (rc) return rc;
        rc = E.loflags.ensure(((size_t)cdiv(N, 128) + 4) * sizeof(uint32_t));
        if (rc) return rc;
        ws += E.hi.cap + E.lo.cap + E.bf.cap + E.loflags.cap;
        if (f8) {
            rc = E.f8.ensure((size_t)N * c.dpf * 2);
            if (!rc) rc = E.cs.ensure(n_pad * sizeof(float));
            if (rc) return rc;
            ws += E.f8.cap + E.cs.cap;
        }
        if (scan && !f8) {
            // BF16 keys: the norms as BF16 parts, added inside the scan's MMA
            rc = E.np.ensure((size_t)N * kNormParts * 2);
            if (rc) return rc;
            ws += E.np.cap;
        }
    }
    if (f8) {
        rc = E.qs.ensure(Q * sizeof(float));
        if (!rc) rc = E.csv.ensure(sp.norm_words * sizeof(float));
        if (rc) return rc;
        ws += E.qs.cap + E.csv.cap;
    }
    // corpus-side buffers: the index's, or this engine's
    const void* bf_p = pc ? pc->bf.p : E.bf.p;
    const float* hi_p = (const float*)(pc ? pc->hi.p : E.hi.p);
    const float* lo_p = (const float*)(pc ? pc->lo.p : E.lo.p);
    const void* f8_p = pc ? pc->f8.p : E.f8.p;
    const float* cs_p = (const float*)(pc ? pc->cs.p : E.cs.p);
    // BF16 keys on the scan: the corpus norm parts (the scan's last K step)
    const bool np_keys = scan && !f8;
    const void* np_p = pc ? pc->np.p : E.np.p;
    // the scan's operand row width in 16-bit units
    const int sdp = f8 ? c.dpf : c.dpb;
    if (scan) {
        rc = E.qbf.ensure((size_t)Q * sdp * 2);
        if (!rc) rc = E.cand.ensure(sp.cand_words * sizeof(uint64_t));
        if (!rc) rc = E.cnt.ensure(sp.cnt_words * sizeof(uint32_t));
        if (!rc) rc = E.tq.ensure((size_t)2 * Q * sizeof(float));
        if (!rc) rc = E.cnv.ensure(sp.norm_words * sizeof(float));
        if (!rc) rc = E.fail.ensure((size_t)(Q + 1) * sizeof(uint32_t));
        if (!rc) rc = E.part.ensure(sp.part_words * sizeof(uint64_t));
        if (!rc) rc = E.thr2.ensure(Q * sizeof(uint32_t));
        if (rc) return rc;
        ws += E.qbf.cap + E.cand.cap + E.cnt.cap + E.tq.cap + E.cnv.cap + E.fail.cap;
    }
    ws += E.part.cap + E.thr2.cap;
    // the 3xTF32 scan beside the BF16 one (its buffers are shared with it but for its queries'
    // TF32 copies and its failed-query list: only one of the two paths runs)
    const float* cn_ts = (const float*)(pc ? pc->cn.p : E.cn.p);
    TscanStages ts{E, c, sp_tf, corpus, N, ldc, queries, Q, ldq, D, k, cn_ts,
                   (const float*)(pc ? pc->hi.p : E.hi.p), (const float*)(pc ? pc->lo.p : E.lo.p),
                   (const uint32_t*)(pc ? pc->tiles.p : E.loflags.p), (const float*)E.qn.p, dist, idx, idx_f,
                   (const uint32_t*)E.words.p + 1, (uint32_t*)E.words.p + 5, E.tfail, E.tthr2, s};
    if (tf_scan) {
        if ((rc = ts.ensure())) return rc;
        ws += E.qhi.cap + E.qlo.cap + E.qlof.cap + E.tfail.cap + E.tthr2.cap;
    }
    // Resident corpora (one stream otherwise): the 3xTF32 scan runs on a side stream beside the
    // BF16 path, so that the launches of whichever path does not match the data (they return at
    // once) overlap the other path's kernels instead of adding to the search.  The two paths
    // share no buffer that both write: candidates, thresholds and results are written by the
    // path that runs only; failed-query lists and fix-up thresholds are their own.
    const bool ts_side = tf_scan && !host_corpus && !capture && !o.single_stream;
    cudaStream_t ts_stream = ts_side ? E.worker_stream(0) : nullptr;
    if (ts_side && (!ts_stream || !E.order_event(1)))
        return set_error(KNNS_ERR_CUDA, "stream or event creation failed");
    // Blocked mode (threshold scan on a corpus still in host memory, not under capture): the
    // seeding sample (every sp.stride0-th row, the rows the seeding levels read) is prepared first
    // and the seeding passes run while the corpus is copied in blocks (of whole main-scan splits)
    // on the copy stream and prepared block by block, as each lands, on the engine's preparation
    // stream; each block is scanned, on one of two worker streams, once it is prepared and the
    // thresholds are seeded.  A resident corpus is searched on the search's stream alone: there
    // the blocks' partial waves and the preparation beside the scans cost more than the overlap
    // gives (4M x 96 mixture, BF16 keys: 10.8 against 8.3 ms).  Without the scan a host corpus
    // is copied whole before the search starts.
    const bool blocked = scan && !pc && !capture && !o.single_stream && host_corpus != nullptr;
    const bool streamed = blocked;
    const int64_t smp_n = blocked ? cdiv(N, sp.stride0) : 0;
    const int64_t smp_pad = cdiv(smp_n, kScanTileN) * kScanTileN + kScanTileN;
    // where the sample rows are read: page-locked host memory in place (it is mapped into the
    // device's address space); otherwise a device copy gathered by a 2-D copy
    const float* smp_src = nullptr;
    int64_t smp_ld = 0;
    bool smp_copy = false;
    if (streamed) {
        cudaPointerAttributes pa;
        if (cudaPointerGetAttributes(&pa, host_corpus) == cudaSuccess && pa.type == cudaMemoryTypeHost &&
            pa.devicePointer != nullptr) {
            smp_src = (const float*)pa.devicePointer;
            smp_ld = sp.stride0 * D;
        } else {
            (void)cudaGetLastError();
            smp_copy = true;
            smp_ld = D;
        }
    }
    if (blocked) {
        rc = smp_copy ? E.smp.ensure((size_t)smp_n * D * sizeof(float)) : KNNS_OK;
        if (!rc) rc = E.smp_cn.ensure((size_t)smp_pad * sizeof(float));
        if (!rc) rc = E.smp_bf.ensure((size_t)smp_n * c.dpb * 2);
        if (!rc && f8) rc = E.smp_f8.ensure((size_t)smp_n * c.dpf * 2);
        if (!rc && f8) rc = E.smp_cs.ensure((size_t)smp_pad * sizeof(float));
        if (!rc && np_keys) rc = E.smp_np.ensure((size_t)smp_n * kNormParts * 2);
        if (rc) return rc;
        if (smp_copy) smp_src = (const float*)E.smp.p;
    }
    constexpr int kBlocks = 8;
    const int blk_splits = blocked ? (int)cdiv(sp.S, std::min(sp.S, kBlocks)) : 0;  // main-scan splits per block
    const int nblk = blocked ? (int)cdiv(sp.S, blk_splits) : 0;
    auto blk_rows = [&](int b, int64_t* r0, int64_t* r1) {
        *r0 = (int64_t)b * blk_splits * sp.len;
        *r1 = std::min(N, *r0 + blk_splits * sp.len);
    };

    if (!capture) KNN_CUDA(cudaStreamWaitEvent(s, E.last_done, 0));
    // ordering events: [0] start, [1] sample landed, [2 + b] block b landed, [2 + nblk + b]
    // block b prepared, [2 + 2 nblk + b] block b scanned, [2 + 3 nblk] flag words cleared,
    // [3 + 3 nblk] thresholds seeded, [4 + 3 nblk] the TF32 scan done
    auto oev = [&](int i) -> cudaEvent_t { return E.order_event(i); };
    if (host_corpus != nullptr || blocked) {
        if (!oev(5 + 3 * nblk) || !E.copy_stream() || (blocked && (!E.prep_stream() || !E.worker_stream(0) ||
                                                                   !E.worker_stream(Engine::kScanWorkers - 1))))
            return set_error(KNNS_ERR_CUDA, "stream or event creation failed");
    }
    if (host_corpus != nullptr) {
        cudaStream_t cs_ = E.copy_stream();
        // the copies overwrite the device corpus only once the previous search is done with it
        KNN_CUDA(cudaEventRecord(oev(0), s));
        KNN_CUDA(cudaStreamWaitEvent(cs_, oev(0), 0));
        if (streamed) {
            if (smp_copy)
                KNN_CUDA(cudaMemcpy2DAsync(E.smp.p, (size_t)D * sizeof(float), host_corpus,
                                           (size_t)sp.stride0 * D * sizeof(float), (size_t)D * sizeof(float),
                                           (size_t)smp_n, cudaMemcpyHostToDevice, cs_));
            KNN_CUDA(cudaEventRecord(oev(1), cs_));
            for (int b = 0; b < nblk; ++b) {
                int64_t r0, r1;
                blk_rows(b, &r0, &r1);
                KNN_CUDA(cudaMemcpyAsync(const_cast<float*>(corpus) + r0 * D, host_corpus + r0 * D,
                                         (size_t)(r1 - r0) * D * sizeof(float), cudaMemcpyHostToDevice, cs_));
                KNN_CUDA(cudaEventRecord(oev(2 + b), cs_));
            }
        } else {
            KNN_CUDA(cudaMemcpyAsync(const_cast<float*>(corpus), host_corpus, (size_t)N * D * sizeof(float),
                                     cudaMemcpyHostToDevice, cs_));
            KNN_CUDA(cudaEventRecord(oev(2), cs_));
            KNN_CUDA(cudaStreamWaitEvent(s, oev(2), 0));
        }
    }
    cudaEvent_t tv[Engine::kTimingEvents] = {};
    if (o.timing && E.timing_slot(tv) != KNNS_OK) return KNNS_ERR_CUDA;
    auto mark = [&](int i) -> int {
        if (tv[i]) KNN_CUDA(cudaEventRecord(tv[i], s));
        return KNNS_OK;
    };
    if ((rc = mark(0))) return rc;
    int launches = 0;
    float* cn = (float*)(pc ? pc->cn.p : E.cn.p);
    float* qn = (!c.rerank || scan) ? (float*)E.qn.p : nullptr;
    uint64_t* part = (uint64_t*)E.part.p;
    uint32_t* thr_g = (uint32_t*)E.thr.p;
    // flag words of this search: [0] TF32 low part in the corpus, [1] corpus or queries not
    // BF16-exact, [2..3] integrality / max |x| of corpus and queries, [4] always zero
    uint32_t* words = (uint32_t*)E.words.p;
    uint32_t* any_lo = words;
    uint32_t* not_exact = words + 1;
    uint32_t* int_stats = words + 2;
    const uint32_t* zero_word = words + 4;
    uint32_t* flags = c.algo == KNNS_ALGO_TC ? (uint32_t*)(pc ? pc->tiles.p : E.loflags.p) : nullptr;
    if (pc) {
        KNN_CUDA(cudaMemcpyAsync(words, pc->words.p, 4 * sizeof(uint32_t), cudaMemcpyDeviceToDevice, s));
        KNN_CUDA(cudaMemsetAsync(words + 4, 0, 2 * sizeof(uint32_t), s));
    } else {
        KNN_CUDA(cudaMemsetAsync(words, 0, 6 * sizeof(uint32_t), s));
    }
    // 3xTF32 keys on request: the data count as not BF16-exact (the preparation only ORs into the word)
    if (o.tf32_only && !bf16_only) KNN_CUDA(cudaMemsetAsync(words + 1, 0x01, 1, s));
    if (blocked) {
        // the corpus blocks, prepared on the preparation stream as they land (their flag words
        // only OR into the words just cleared)
        cudaStream_t ps = E.prep_stream();
        KNN_CUDA(cudaEventRecord(oev(2 + 3 * nblk), s));
        KNN_CUDA(cudaStreamWaitEvent(ps, oev(2 + 3 * nblk), 0));
        const int64_t ld = streamed ? D : ldc;
        for (int b = 0; b < nblk; ++b) {
            int64_t r0, r1;
            blk_rows(b, &r0, &r1);
            if (streamed) KNN_CUDA(cudaStreamWaitEvent(ps, oev(2 + b), 0));
            KNN_CUDA(launch_prep_rows(corpus + r0 * ld, r1 - r0, ld, D, c.dpb, (char*)E.bf.p + (size_t)r0 * c.dpb * 2,
                                      cn + r0, b == nblk - 1 ? n_pad - r0 : r1 - r0, not_exact, ps, int_stats,
                                      f8 ? (char*)E.f8.p + (size_t)r0 * c.dpf * 2 : nullptr, 2 * c.dpf,
                                      f8 ? (float*)E.cs.p + r0 : nullptr,
                                      np_keys ? (char*)E.np.p + (size_t)r0 * kNormParts * 2 : nullptr));
            ++launches;
            KNN_CUDA(cudaEventRecord(oev(2 + nblk + b), ps));
        }
    }
    if (c.algo == KNNS_ALGO_TC) {
        // one pass per input: BF16 copy, exactness test, integrality, norms (blocked mode: the
        // corpus block by block, above)
        if (!pc && !blocked) {
            KNN_CUDA(launch_prep_rows(corpus, N, ldc, D, c.dpb, E.bf.p, cn, n_pad, not_exact, s, int_stats,
                                      f8 ? E.f8.p : nullptr, 2 * c.dpf, f8 ? (float*)E.cs.p : nullptr,
                                      np_keys ? E.np.p : nullptr));
            ++launches;
        }
        if (f8)
            KNN_CUDA(launch_prep_rows(queries, Q, ldq, D, c.dpb, nullptr, qn, Q, not_exact, s, int_stats, E.qbf.p,
                                      2 * c.dpf, (float*)E.qs.p));
        else
            KNN_CUDA(launch_prep_rows(queries, Q, ldq, D, c.dpb, scan ? E.qbf.p : nullptr, qn, Q, not_exact, s,
                                      int_stats));
        ++launches;
        if (!bf16_only && !pc && !blocked) {
            // the TF32 split runs only for data that is not BF16-exact
            KNN_CUDA(launch_split(corpus, N, ldc, D, c.dp, (float*)E.hi.p, (float*)E.lo.p, flags, any_lo, not_exact,
                                  s));
            ++launches;
        }
        if (tf_scan && !blocked && (rc = ts.split_queries())) return rc;
    } else {
        if (!pc) {
            KNN_CUDA(launch_prep_rows(corpus, N, ldc, D, 0, nullptr, cn, n_pad, nullptr, s));
            ++launches;
        }
        if (qn) {
            KNN_CUDA(launch_prep_rows(queries, Q, ldq, D, 0, nullptr, qn, Q, nullptr, s));
            ++launches;
        }
    }
    // gate of the BF16 kernels: in the BF16 form they always run
    const uint32_t* bf_gate = bf16_only ? zero_word : not_exact;
    if ((rc = mark(1))) return rc;

    // One shortlist pass over a corpus view: rows 0, stride, 2*stride, ... (nview
    // of them); runs only without the threshold scan.
    auto fused_pass = [&](int64_t nview, int64_t stride, const float* cn_view, int kp, int stages, int splits,
                          int64_t split_len, uint32_t* thr, const uint32_t* redo, bool tile_flags) -> int {
        if (c.algo == KNNS_ALGO_TC) {
            TcArgs a;
            memset(&a, 0, sizeof(a));
            int r = 0;
            if (!bf16_only) {
                r = encode_rows(&a.tm_hi, hi_p, nview, c.dp, stride * c.dp);
                if (!r) r = encode_rows(&a.tm_lo, lo_p, nview, c.dp, stride * c.dp);
            }
            if (!r) r = encode_rows_bf16(&a.tm_bf, bf_p, nview, c.dpb, stride * c.dpb);
            if (r) return r;
            a.not_exact = bf_gate;
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
            a.timeout_ns = stall_ns;
            a.test_stall = stall_ns != 0;
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
    // The shortlist path (corpora below the threshold scan's size, or the scan off): TF32 and
    // BF16 variants, the one that does not match the data returning at once.
    auto old_path = [&]() -> int {
        if (!run_old) return KNNS_OK;
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
        return KNNS_OK;
    };
    if (run_old && (rc = old_path())) return rc;

    if (!scan) {
        for (int i = 2; i <= 5; ++i)
            if ((rc = mark(i))) return rc;
    } else {
        // ---------------------------------------------------------------- threshold scan
        // (runs when *scan_gate == 0: always in the BF16 form, for BF16-exact data in the exact form)
        const uint32_t* scan_gate = bf16_only ? nullptr : not_exact;
        float* Tbuf[2] = {(float*)E.tq.p, (float*)E.tq.p + Q};
        uint32_t* fail_cnt = (uint32_t*)E.fail.p;
        int32_t* fail_idx = (int32_t*)E.fail.p + 1;
        ScanArgs a;
        memset(&a, 0, sizeof(a));
        a.qbf = E.qbf.p;
        a.skip_if = scan_gate;
        a.cand = (uint64_t*)E.cand.p;
        a.cnt = (uint32_t*)E.cnt.p;
        a.err = (int*)E.err.p;
        a.Q = Q;
        a.dpb = sdp;
        a.ksteps = f8 ? (D + 31) / 32 : (D + 15) / 16;
        a.bps = sp.bps;
        a.ring = sp.ring;
        a.accs = sp.accs;
        a.fp8 = f8 ? 1 : 0;
        a.qs = f8 ? (const float*)E.qs.p : nullptr;
        // one scan over rows 0, stride, 2*stride, ... (nview of them) of the operand copy at src;
        // grid rows are the splits split0 .. split0 + splits - 1, launched on stream ls
        auto scan_pass = [&](const void* src, const void* np_src, int64_t nview, int64_t stride, const float* cn_view,
                             const float* cs_view, const float* thr, int splits, int64_t split_len, int cap,
                             int split0 = 0, cudaStream_t ls = nullptr) -> int {
            // the map moves bytes: E4M3 rows are described as rows of 16-bit units
            int r = encode_rows_bf16(&a.tm_c, src, nview, sdp, stride * sdp, scan_box_rows(sdp, sp.accs));
            if (!r && np_keys) r = encode_np(&a.tm_np, np_src, nview, stride * kNormParts, scan_box_rows(sdp, sp.accs));
            if (r) return r;
            a.cn = cn_view;
            a.cs = cs_view;
            a.thr = thr;
            a.N = nview;
            a.split_len = split_len;
            a.cap = cap;
            a.split0 = split0;
            KNN_CUDA(launch_scan(a, splits, ls ? ls : s));
            ++launches;
            return KNNS_OK;
        };
        CandSelect cs;
        cs.cand = (const uint64_t*)E.cand.p;
        cs.cnt = (const uint32_t*)E.cnt.p;
        cs.Q = Q;
        cs.skip_if = scan_gate;
        cs.D = D;
        // seeding, coarse to fine: level l keeps the keys below the previous level's
        // threshold (the coarsest keeps every key) and yields the key of rank j_l
        // (blocked mode: the levels read the sample prepared ahead of the corpus, whose row r is
        // corpus row sp.stride0 * r -- the same rows, prepared by the same pass)
        const void* key_src = f8 ? f8_p : bf_p;
        const float* lv_cn = cn;
        const float* lv_cs = cs_p;
        const void* lv_np = np_p;
        int64_t lv_div = 1;
        if (blocked) {
            if (smp_copy) KNN_CUDA(cudaStreamWaitEvent(s, oev(1), 0));
            KNN_CUDA(launch_prep_rows(smp_src, smp_n, smp_ld, D, c.dpb, E.smp_bf.p, (float*)E.smp_cn.p, smp_pad,
                                      not_exact, s, int_stats, f8 ? E.smp_f8.p : nullptr, 2 * c.dpf,
                                      f8 ? (float*)E.smp_cs.p : nullptr, np_keys ? E.smp_np.p : nullptr));
            ++launches;
            key_src = f8 ? E.smp_f8.p : E.smp_bf.p;
            lv_cn = (const float*)E.smp_cn.p;
            lv_cs = (const float*)E.smp_cs.p;
            lv_np = E.smp_np.p;
            lv_div = sp.stride0;
        }
        float* cnv = (float*)E.cnv.p;
        float* csv = f8 ? (float*)E.csv.p : nullptr;
        const float* T = nullptr;
        for (int l = 0; l < sp.levels; ++l) {
            const ScanLevel& v = sp.lv[l];
            if (f8) {
                // norms and scales of the sample rows: 0 scales for padding, whose +inf norms keep
                // their keys at +inf (BF16 keys take the norm parts in place)
                KNN_CUDA(launch_gather_norms(lv_cn, v.n, v.stride / lv_div, cnv, v.n_pad, s));
                KNN_CUDA(launch_gather_norms(lv_cs, v.n, v.stride / lv_div, csv, v.n_pad, s, 0.f));
                launches += 2;
            }
            if ((rc = scan_pass(key_src, lv_np, v.n, v.stride / lv_div, cnv, csv, T, v.S, v.len, v.cap))) return rc;
            cs.nseg = kScanParts * v.S;
            cs.cap = v.cap;
            cs.thr_out = Tbuf[l & 1];
            cs.thr_rank = v.j;
            cs.thr_fallback = T;  // a level that fails keeps the previous threshold
            KNN_CUDA(launch_select_cand(cs, s));
            ++launches;
            T = Tbuf[l & 1];
            cnv += v.n_pad;
            if (csv) csv += v.n_pad;
        }
        // (the TF32 scan's seeding reuses the sample norms and threshold buffers: the BF16
        // levels, run or skipped, are done with them)
        if (ts_side) {
            // the whole TF32 scan on the side stream, from the prepared inputs on
            KNN_CUDA(cudaEventRecord(E.order_event(0), s));
            KNN_CUDA(cudaStreamWaitEvent(ts_stream, E.order_event(0), 0));
            ts.s = ts_stream;
            if ((rc = ts.seed()) || (rc = ts.main_pass()) || (rc = ts.select()) || (rc = ts.fix())) return rc;
            KNN_CUDA(cudaEventRecord(E.order_event(1), ts_stream));
        } else if (tf_scan && !blocked && (rc = ts.seed())) {
            return rc;
        }
        if ((rc = mark(2))) return rc;
        // main pass
        if (!blocked) {
            if ((rc = scan_pass(f8 ? f8_p : bf_p, np_p, N, 1, cn, cs_p, T, sp.S, sp.len, sp.cap))) return rc;
            if (tf_scan && !ts_side && (rc = ts.main_pass())) return rc;
        } else {
            // block by block on the worker streams (blocks scanned on the two workers overlap each
            // other's tails), each once prepared and once the thresholds are seeded
            KNN_CUDA(cudaEventRecord(oev(3 + 3 * nblk), s));
            for (int b = 0; b < nblk; ++b) {
                cudaStream_t w = E.worker_stream(b % Engine::kScanWorkers);
                KNN_CUDA(cudaStreamWaitEvent(w, oev(2 + nblk + b), 0));
                KNN_CUDA(cudaStreamWaitEvent(w, oev(3 + 3 * nblk), 0));
                const int sb = std::min(blk_splits, sp.S - b * blk_splits);
                if ((rc = scan_pass(f8 ? f8_p : bf_p, np_p, N, 1, cn, cs_p, T, sb, sp.len, sp.cap, b * blk_splits, w)))
                    return rc;
                KNN_CUDA(cudaEventRecord(oev(2 + 2 * nblk + b), w));
            }
            // What needs the whole corpus, the TF32 copies and the TF32 scan (gated on the data's
            // BF16-exactness in the exact form), runs on the preparation stream: the copies (their own
            // buffers) once the last block is prepared, the flag then final; the scan, which writes
            // the thresholds and candidate segments the BF16 path also uses, once every block is
            // scanned (a block scanned before a later block cleared the flag ran its BF16 scan), beside
            // the BF16 selection and fix-up on the search's stream: one of the two paths returns at once.
            for (int b = 0; b < nblk; ++b) KNN_CUDA(cudaStreamWaitEvent(s, oev(2 + 2 * nblk + b), 0));
            if (tf_scan) {
                cudaStream_t ps = E.prep_stream();
                KNN_CUDA(launch_split(corpus, N, ldc, D, c.dp, (float*)E.hi.p, (float*)E.lo.p, flags, any_lo,
                                      not_exact, ps));
                ++launches;
                ts.s = ps;
                if ((rc = ts.split_queries())) return rc;
                for (int b = 0; b < nblk; ++b) KNN_CUDA(cudaStreamWaitEvent(ps, oev(2 + 2 * nblk + b), 0));
                if ((rc = ts.seed()) || (rc = ts.main_pass()) || (rc = ts.select()) || (rc = ts.fix())) return rc;
                KNN_CUDA(cudaEventRecord(oev(4 + 3 * nblk), ps));
            }
        }
        if ((rc = mark(3))) return rc;
        KNN_CUDA(cudaMemsetAsync(fail_cnt, 0, sizeof(uint32_t), s));
        cs.nseg = kScanParts * sp.S;
        cs.cap = sp.cap;
        cs.thr_out = nullptr;
        cs.thr_fallback = nullptr;
        cs.kp = c.kp;
        cs.k = k;
        cs.need = (int)std::min<int64_t>(c.kp, N);
        cs.buf_words = sp.sel_words;
        cs.rerank = c.rerank;
        cs.corpus = corpus;
        cs.ldc = ldc;
        cs.queries = queries;
        cs.ldq = ldq;
        cs.qn = qn;
        // E4M3 keys are never exact: always re-ranked
        cs.int_stats = f8 ? nullptr : int_stats;
        cs.bf16_inexact = not_exact;
        cs.out_dist = dist;
        cs.out_idx = idx;
        cs.out_idx_f = idx_f;
        cs.fail_idx = fail_idx;
        cs.fail_cnt = fail_cnt;
        KNN_CUDA(launch_select_cand(cs, s));
        ++launches;
        if (tf_scan && !ts_side && !blocked && (rc = ts.select())) return rc;
        if ((rc = mark(4))) return rc;
        // fix-up: failed queries, compacted, through the shortlist kernel without a threshold
        // (launches whose rows are all past the failure count return at once)
        auto fix_pass = [&](int64_t qbase, int64_t rows, int splits, int64_t split_len) -> int {
            if (rows <= 0) return KNNS_OK;
            if (sp.simt_fix) {
                // long shortlists: the CUDA-core kernel with exact FP32 keys, compacted rows
                uint32_t* thr2 = (uint32_t*)E.thr2.p;
                KNN_CUDA(cudaMemsetAsync(thr2, 0xFF, rows * sizeof(uint32_t), s));
                KNN_CUDA(launch_simt(corpus, N, ldc, cn, queries, rows, ldq, D, c.kp, 32, split_len, splits, part,
                                     thr2, s, nullptr, fail_idx, fail_cnt, qbase));
                SelectExtra ex;
                ex.qmap = fail_idx;
                ex.qcount = fail_cnt;
                ex.qbase = qbase;
                KNN_CUDA(launch_select(part, splits, rows, c.kp, k, corpus, ldc, queries, ldq, D, c.rerank,
                                       c.rerank ? nullptr : (const float*)E.qn.p, dist, idx, idx_f, s, ex));
                launches += 2;
                return KNNS_OK;
            }
            TcArgs t;
            memset(&t, 0, sizeof(t));
            int r = encode_rows_bf16(&t.tm_bf, bf_p, N, c.dpb, c.dpb);
            if (r) return r;
            uint32_t* thr2 = (uint32_t*)E.thr2.p;
            KNN_CUDA(cudaMemsetAsync(thr2, 0xFF, rows * sizeof(uint32_t), s));
            t.not_exact = bf_gate;  // the BF16 variant runs when the data are BF16 (always in the BF16 form)
            t.dpb = c.dpb;
            t.cn = cn;
            t.queries = queries;
            t.Q = rows;
            t.ldq = ldq;
            t.N = N;
            t.split_len = split_len;
            t.part = part;
            t.thr_g = thr2;
            t.qmap = fail_idx;
            t.qcount = fail_cnt;
            t.qbase = qbase;
            t.err = (int*)E.err.p;
            t.D = D;
            t.dp = kChunkK;
            t.kp = c.kp;
            t.stages = std::min(4, tc_max_stages(c.kp));
            KNN_CUDA(launch_tc(t, splits, true, s));
            SelectExtra ex;
            ex.qmap = fail_idx;
            ex.qcount = fail_cnt;
            ex.qbase = qbase;
            KNN_CUDA(launch_select(part, splits, rows, c.kp, k, corpus, ldc, queries, ldq, D, c.rerank,
                                   c.rerank ? nullptr : (const float*)E.qn.p, dist, idx, idx_f, s, ex));
            launches += 2;
            return KNNS_OK;
        };
        if ((rc = fix_pass(0, sp.fixA_rows, sp.fixA_S, sp.fixA_len))) return rc;
        if ((rc = fix_pass(sp.fixA_rows, sp.fixB_rows, sp.fixB_S, sp.fixB_len))) return rc;
        if (tf_scan && !ts_side && !blocked && (rc = ts.fix())) return rc;
        if (ts_side) KNN_CUDA(cudaStreamWaitEvent(s, E.order_event(1), 0));
        if (tf_scan && blocked) KNN_CUDA(cudaStreamWaitEvent(s, oev(4 + 3 * nblk), 0));
        if ((rc = mark(5))) return rc;
    }
    launches += ts.launches;
    if (!capture) KNN_CUDA(cudaEventRecord(E.last_done, s));
    if (st)
        *st = knns_stats{c.algo, c.splits, c.kp, c.stages, launches, (pilot || scan) ? 1 : 0, (int64_t)ws,
                         scan ? 1 : 0, scan ? sp.S : 0, scan ? sp.cap : 0, scan ? 100 * sp.ring + sp.bps : 0,
                         (scan ? 1 : 0) | (tf_scan ? 2 : 0)};
    return KNNS_OK;
}

void PreparedCorpus::release()
{
    cn.release();
    bf.release();
    hi.release();
    lo.release();
    tiles.release();
    words.release();
    f8.release();
    cs.release();
    np.release();
}

int prepare_corpus(Engine& E, PreparedCorpus* pc, const float* corpus, int64_t N, int64_t ldc, int D, bool tf32,
                   cudaStream_t s, bool fp8)
{
    if (!pc || !corpus || N <= 0 || D <= 0 || ldc < D) return set_error(KNNS_ERR_INVALID, "invalid corpus");
    if (N > 0x7fffffffLL) return set_error(KNNS_ERR_UNSUPPORTED, "corpus larger than 2^31-1 rows");
    if (E.cc < 100) return set_error(KNNS_ERR_UNSUPPORTED, "a prepared corpus needs sm_100+");
    const int dpb = (D + 63) & ~63, dp = (D + 31) & ~31;
    if (dpb > 256) return set_error(KNNS_ERR_UNSUPPORTED, "a prepared corpus needs D <= 256");
    const int64_t n_pad = cdiv(N, kScanTileN) * kScanTileN + kScanTileN;
    int rc = pc->cn.ensure(n_pad * sizeof(float));
    if (!rc) rc = pc->bf.ensure((size_t)N * dpb * 2);
    if (!rc) rc = pc->words.ensure(8 * sizeof(uint32_t));
    if (!rc) rc = pc->tiles.ensure(((size_t)cdiv(N, 128) + 1) * sizeof(uint32_t));
    if (!rc && tf32) rc = pc->hi.ensure((size_t)N * dp * sizeof(float));
    if (!rc && tf32) rc = pc->lo.ensure((size_t)N * dp * sizeof(float));
    const int dpf = ((D + 127) & ~127) / 2;
    if (!rc && fp8) rc = pc->f8.ensure((size_t)N * dpf * 2);
    if (!rc && fp8) rc = pc->cs.ensure(n_pad * sizeof(float));
    if (!rc) rc = pc->np.ensure((size_t)N * kNormParts * 2);
    if (rc) return rc;
    uint32_t* w = (uint32_t*)pc->words.p;
    KNN_CUDA(cudaMemsetAsync(w, 0, 8 * sizeof(uint32_t), s));
    KNN_CUDA(launch_prep_rows(corpus, N, ldc, D, dpb, pc->bf.p, (float*)pc->cn.p, n_pad, w + 1, s, w + 2,
                              fp8 ? pc->f8.p : nullptr, 2 * dpf, fp8 ? (float*)pc->cs.p : nullptr, pc->np.p));
    if (tf32)
        KNN_CUDA(launch_split(corpus, N, ldc, D, dp, (float*)pc->hi.p, (float*)pc->lo.p, (uint32_t*)pc->tiles.p, w,
                              nullptr, s));
    pc->corpus = corpus;
    pc->N = N;
    pc->ldc = ldc;
    pc->D = D;
    pc->dpb = dpb;
    pc->dpf = dpf;
    pc->fp8 = fp8;
    pc->dp = dp;
    pc->tf32 = tf32;
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

// Corpus rows per device block of a host-buffer search: the requested count, or
// (requested 0) the whole corpus when its copies fit in about 60 % of the free
// device memory (the engine's own cached corpus buffers counted as free), else as
// many rows as do, rounded down to 4096.  0 when not even k rows fit.
static int64_t host_block_rows(Engine& E, int64_t N, int64_t Q, int D, int k, int requested)
{
    if (requested > 0) return std::max<int64_t>(std::min<int64_t>(requested, N), std::min<int64_t>(k, N));
    size_t fr = 0, tot = 0;
    if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) return N;
    const double avail = 0.6 * (double)(fr + E.in_corpus.cap + E.bf.cap + E.hi.cap + E.lo.cap + E.cn.cap);
    // FP32 input, BF16 copy, TF32 hi/lo, norms and flags per row; query-side workspace
    const double per_row = (double)D * (4 + 2 + 8) + 32;
    const double fixed = (double)Q * ((double)D * 8 + 8192) + 256.0 * (1 << 20);
    const double rows = (avail - fixed) / per_row;
    if (rows >= (double)N) return N;
    const int64_t r = (int64_t)rows / 4096 * 4096;
    return r >= k ? r : 0;
}

// Host-buffer search over a corpus streamed in blocks of br rows: each block is
// copied, searched for its top-min(k, rows) and merged into the running top-k
// (src/cuknnBitonic.cu:550-589).  Per-pair arithmetic does not depend on the
// blocking, so the result is the one search over the whole corpus gives.
static int search_host_blocked(Engine& E, cudaStream_t s, const float* corpus, int64_t N, const float* queries,
                               int64_t Q, int D, int k, float* dist, int32_t* idx, float* idx_f_host,
                               const knns_options& o, int64_t br, double* seconds, knns_stats* st)
{
    if (N > 0x7fffffffLL) return set_error(KNNS_ERR_UNSUPPORTED, "corpus larger than 2^31-1 rows");
    const size_t qb = (size_t)Q * D * sizeof(float), ob = (size_t)Q * k;
    int rc = E.in_corpus.ensure((size_t)br * D * sizeof(float));
    if (!rc) rc = E.in_queries.ensure(std::max(qb, (size_t)4));
    if (!rc) rc = E.out_dist.ensure(std::max(ob * 4, (size_t)4));
    if (!rc) rc = E.out_idx.ensure(std::max(ob * 4, (size_t)4));
    if (!rc) rc = E.mrg.ensure(std::max(ob * 20, (size_t)20));
    if (rc) return rc;
    // two running lists (distances, indices) and the float indices of the drop-in output
    float* rd[2] = {(float*)E.mrg.p, (float*)E.mrg.p + ob};
    int32_t* ri[2] = {(int32_t*)E.mrg.p + 2 * ob, (int32_t*)E.mrg.p + 3 * ob};
    float* fidx = (float*)E.mrg.p + 4 * ob;
    cudaEvent_t t0 = E.t0(), t1 = E.t1();
    KNN_CUDA(cudaEventRecord(t0, s));
    if (qb) KNN_CUDA(cudaMemcpyAsync(E.in_queries.p, queries, qb, cudaMemcpyHostToDevice, s));
    int have = 0, cur = 0;
    for (int64_t b0 = 0; b0 < N; b0 += br) {
        const int64_t nb = std::min<int64_t>(br, N - b0);
        const int kb = (int)std::min<int64_t>(k, nb);
        KNN_CUDA(cudaMemcpyAsync(E.in_corpus.p, corpus + b0 * D, (size_t)nb * D * sizeof(float),
                                 cudaMemcpyHostToDevice, s));
        rc = run_search(E, (const float*)E.in_corpus.p, nb, D, (const float*)E.in_queries.p, Q, D, D, kb,
                        (float*)E.out_dist.p, (int32_t*)E.out_idx.p, nullptr, o, s, st);
        if (rc) return rc;
        const bool last = b0 + nb >= N;
        KNN_CUDA(launch_merge_topk(rd[cur], ri[cur], have, (const float*)E.out_dist.p, (const int32_t*)E.out_idx.p,
                                   kb, (int32_t)b0, Q, k, rd[cur ^ 1], ri[cur ^ 1],
                                   (last && idx_f_host) ? fidx : nullptr, s));
        have = (int)std::min<int64_t>(k, have + kb);
        cur ^= 1;
    }
    // the final lists: rd[cur], ri[cur]; float indices (drop-in) in fidx
    if (dist && ob) KNN_CUDA(cudaMemcpyAsync(dist, rd[cur], ob * 4, cudaMemcpyDeviceToHost, s));
    if (idx && ob) KNN_CUDA(cudaMemcpyAsync(idx, ri[cur], ob * 4, cudaMemcpyDeviceToHost, s));
    if (idx_f_host && ob) KNN_CUDA(cudaMemcpyAsync(idx_f_host, fidx, ob * 4, cudaMemcpyDeviceToHost, s));
    KNN_CUDA(cudaEventRecord(t1, s));
    rc = check_device_error(E, s);
    if (rc) return rc;
    float ms = 0.f;
    KNN_CUDA(cudaEventElapsedTime(&ms, t0, t1));
    if (seconds) *seconds = ms / 1000.0;
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
    if (k > N) return set_error(KNNS_ERR_INVALID, "k=%d exceeds the corpus size N=%lld", k, (long long)N);
    if (o.block_rows < 0) return set_error(KNNS_ERR_INVALID, "negative block_rows");
    const int64_t br = host_block_rows(*E, N, Q, D, k, o.block_rows);
    if (br <= 0) return set_error(KNNS_ERR_NOMEM, "no corpus block of at least %d rows fits in device memory", k);
    if (br < N) return search_host_blocked(*E, s, corpus, N, queries, Q, D, k, dist, idx, idx_f_host, o, br, seconds, st);
    const size_t cb = (size_t)N * D * sizeof(float), qb = (size_t)Q * D * sizeof(float);
    const size_t ob = (size_t)Q * k;
    if ((rc = E->in_corpus.ensure(cb))) return rc;
    if ((rc = E->in_queries.ensure(std::max(qb, (size_t)4)))) return rc;
    if ((rc = E->out_dist.ensure(std::max(ob * 4, (size_t)4)))) return rc;
    if ((rc = E->out_idx.ensure(std::max(ob * 4, (size_t)4)))) return rc;
    cudaEvent_t t0 = E->t0(), t1 = E->t1();
    KNN_CUDA(cudaEventRecord(t0, s));
    if (qb) KNN_CUDA(cudaMemcpyAsync(E->in_queries.p, queries, qb, cudaMemcpyHostToDevice, s));
    // the corpus is copied by the search itself, in blocks that overlap its computation
    rc = run_search(*E, (const float*)E->in_corpus.p, N, D, (const float*)E->in_queries.p, Q, D, D, k,
                    dist ? (float*)E->out_dist.p : nullptr, idx ? (int32_t*)E->out_idx.p : nullptr,
                    idx_f_host ? (float*)E->out_idx.p : nullptr, o, s, st, nullptr, false, corpus);
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

int Engine::timing_slot(cudaEvent_t out[kTimingEvents])
{
    const size_t need = (size_t)(tcount + 1) * kTimingEvents;
    while (tev.size() < need) {
        cudaEvent_t e;
        KNN_CUDA(cudaEventCreate(&e));
        tev.push_back(e);
    }
    for (int i = 0; i < kTimingEvents; ++i) out[i] = tev[(size_t)tcount * kTimingEvents + i];
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

cudaStream_t Engine::copy_stream()
{
    if (!copy_) {
        if (cudaStreamCreateWithFlags(&copy_, cudaStreamNonBlocking) != cudaSuccess) copy_ = nullptr;
    }
    return copy_;
}

cudaStream_t Engine::prep_stream()
{
    if (!prep_) {
        if (cudaStreamCreateWithFlags(&prep_, cudaStreamNonBlocking) != cudaSuccess) prep_ = nullptr;
    }
    return prep_;
}

cudaStream_t Engine::worker_stream(int i)
{
    if (i < 0 || i >= kScanWorkers) return nullptr;
    if (!workers_[i]) {
        if (cudaStreamCreateWithFlags(&workers_[i], cudaStreamNonBlocking) != cudaSuccess) workers_[i] = nullptr;
    }
    return workers_[i];
}

cudaEvent_t Engine::order_event(int i)
{
    while ((int)order_.size() <= i) {
        cudaEvent_t e = nullptr;
        if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return nullptr;
        order_.push_back(e);
    }
    return order_[(size_t)i];
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
    opt->scan = KNNS_SCAN_AUTO;
    opt->scan_boxes = 0;
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

int knns_last_fixups(int64_t* out)
{
    if (!out) return KNNS_ERR_INVALID;
    if (!g_have_stats) return set_error(KNNS_ERR_INVALID, "no search has completed on this thread");
    *out = 0;
    if (!g_last_stats.scan) return KNNS_OK;
    Engine* E = nullptr;
    int rc = get_engine(&E);
    if (rc) return rc;
    std::lock_guard<std::mutex> lk(E->mu);
    if (!E->fail.p) return KNNS_OK;
    uint32_t n = 0;
    KNN_CUDA(cudaDeviceSynchronize());
    KNN_CUDA(cudaMemcpy(&n, E->fail.p, sizeof n, cudaMemcpyDeviceToHost));
    *out = (int64_t)n;
    return KNNS_OK;
}

int knns_version(void) { return 100; }

int knns_merge_topk(const float* run_d, const int32_t* run_i, int have, const float* blk_d, const int32_t* blk_i,
                    int kb, int32_t offset, int64_t Q, int k, float* out_d, int32_t* out_i, void* stream)
{
    clear_error();
    if (Q < 0 || k < 1 || have < 0 || have > k || kb < 0 || kb > k)
        return set_error(KNNS_ERR_INVALID, "merge: bad sizes Q=%lld k=%d have=%d kb=%d", (long long)Q, k, have, kb);
    if (Q > 0 && (!out_d || !out_i || (have > 0 && (!run_d || !run_i)) || (kb > 0 && (!blk_d || !blk_i))))
        return set_error(KNNS_ERR_INVALID, "merge: null pointer");
    KNN_CUDA(launch_merge_topk(run_d, run_i, have, blk_d, blk_i, kb, offset, Q, k, out_d, out_i, nullptr,
                               (cudaStream_t)stream));
    return KNNS_OK;
}

int knns_debug_stall_next_search(int64_t timeout_us)
{
    clear_error();
    if (timeout_us <= 0 || timeout_us > 10000000) return set_error(KNNS_ERR_INVALID, "timeout outside (0, 10 s]");
    g_test_stall_ns.store((uint64_t)timeout_us * 1000u);
    return KNNS_OK;
}

static int timing_collect(double ms[Engine::kTimingEvents - 1], int* count)
{
    Engine* E = nullptr;
    int rc = get_engine(&E);
    if (rc) return rc;
    std::lock_guard<std::mutex> lk(E->mu);
    const int ne = Engine::kTimingEvents;
    for (int j = 0; j < ne - 1; ++j) ms[j] = 0.0;
    for (int i = 0; i < E->tcount; ++i) {
        cudaEvent_t* ev = &E->tev[(size_t)i * ne];
        KNN_CUDA(cudaEventSynchronize(ev[ne - 1]));
        for (int j = 0; j < ne - 1; ++j) {
            float t = 0.f;
            KNN_CUDA(cudaEventElapsedTime(&t, ev[j], ev[j + 1]));
            ms[j] += t;
        }
    }
    if (count) *count = E->tcount;
    E->tcount = 0;
    return KNNS_OK;
}

int knns_timing_collect(double ms[3], int* count)
{
    clear_error();
    if (!ms) return set_error(KNNS_ERR_INVALID, "null output");
    double m5[5];
    int rc = timing_collect(m5, count);
    if (rc) return rc;
    ms[0] = m5[0];
    ms[1] = m5[1] + m5[2];
    ms[2] = m5[3] + m5[4];
    return KNNS_OK;
}

int knns_timing_collect5(double ms[5], int* count)
{
    clear_error();
    if (!ms) return set_error(KNNS_ERR_INVALID, "null output");
    return timing_collect(ms, count);
}

int knns_index_create(const float* corpus, int64_t N, int64_t ldc, int D, int flags, knns_index** out, void* stream)
{
    clear_error();
    if (!out) return set_error(KNNS_ERR_INVALID, "null output");
    *out = nullptr;
    Engine* E = nullptr;
    int rc = get_engine(&E);
    if (rc) return rc;
    std::lock_guard<std::mutex> lk(E->mu);
    std::unique_ptr<knns_index> ix(new knns_index());
    ix->device = E->device;
    cudaStream_t s = (cudaStream_t)stream;
    rc = prepare_corpus(*E, &ix->pc, corpus, N, ldc, D, (flags & KNNS_INDEX_TF32) != 0, s,
                        (flags & KNNS_INDEX_FP8) != 0);
    if (rc) {
        ix->pc.release();
        return rc;
    }
    // the first search on any stream sees the prepared buffers
    KNN_CUDA(cudaStreamSynchronize(s));
    *out = ix.release();
    return KNNS_OK;
}

int knns_index_search(knns_index* ix, const float* queries, int64_t Q, int64_t ldq, int k, float* dist, int32_t* idx,
                      const knns_options* opt, void* stream)
{
    clear_error();
    if (!ix) return set_error(KNNS_ERR_INVALID, "null index");
    knns_options o;
    if (opt) o = *opt;
    else knns_default_options(&o);
    Engine* E = nullptr;
    int rc = get_engine(&E);
    if (rc) return rc;
    if (E->device != ix->device) return set_error(KNNS_ERR_INVALID, "index built on device %d", ix->device);
    std::lock_guard<std::mutex> lk(E->mu);
    knns_stats st;
    rc = run_search(*E, ix->pc.corpus, ix->pc.N, ix->pc.ldc, queries, Q, ldq, ix->pc.D, k, dist, idx, nullptr, o,
                    (cudaStream_t)stream, &st, &ix->pc);
    if (rc == KNNS_OK) remember_stats(st);
    return rc;
}

int knns_autotune_shortlist(knns_index* ix, const float* queries, int64_t Q, int64_t ldq, int k, int precision,
                            double target, int* c_out, double* recall_out, void* stream)
{
    clear_error();
    if (!ix || !queries || Q <= 0 || k <= 0 || !c_out) return set_error(KNNS_ERR_INVALID, "bad arguments");
    if (precision != KNNS_PREC_BF16 && precision != KNNS_PREC_FP8)
        return set_error(KNNS_ERR_INVALID, "the shortlist factor belongs to the BF16 and FP8 forms");
    Engine* E = nullptr;
    int rc = get_engine(&E);
    if (rc) return rc;
    std::lock_guard<std::mutex> lk(E->mu);
    cudaStream_t s = (cudaStream_t)stream;
    const PreparedCorpus& P = ix->pc;
    const size_t n = (size_t)Q * k;
    float* d_dist = nullptr;
    int32_t* d_idx = nullptr;
    KNN_CUDA(cudaMalloc(&d_dist, n * 4));
    if (cudaMalloc(&d_idx, n * 4 * 4) != cudaSuccess) {
        cudaFree(d_dist);
        return set_error(KNNS_ERR_NOMEM, "autotune buffers");
    }
    std::vector<int32_t> exact(n), got(n);
    auto run = [&](int precision, int c, std::vector<int32_t>& out) -> int {
        knns_options o;
        knns_default_options(&o);
        o.precision = precision;
        o.shortlist = c;
        int r = run_search(*E, P.corpus, P.N, P.ldc, queries, Q, ldq, P.D, k, d_dist, d_idx, nullptr, o, s, nullptr,
                           &P);
        if (r) return r;
        r = check_device_error(*E, s);
        if (r) return r;
        if (cudaMemcpy(out.data(), d_idx, n * 4, cudaMemcpyDeviceToHost) != cudaSuccess)
            return set_error(KNNS_ERR_CUDA, "autotune copy");
        return KNNS_OK;
    };
    // ground truth: the exact form (needs the index's TF32 copies unless the data are BF16-exact)
    rc = run(KNNS_PREC_EXACT, 0, exact);
    int best = 0;
    double best_recall = 0.0, last_recall = 0.0;
    int last_c = 0;
    for (int c : {2, 4, 8}) {
        if (rc) break;
        if ((int64_t)c * k > kMaxKpScan && c != 2) break;  // the shortlist holds at most kMaxKpScan entries
        rc = run(precision, c, got);
        if (rc) break;
        int64_t hit = 0;
        for (int64_t q = 0; q < Q; ++q) {
            std::vector<int32_t> a(exact.begin() + q * k, exact.begin() + (q + 1) * k);
            std::sort(a.begin(), a.end());
            for (int j = 0; j < k; ++j) hit += std::binary_search(a.begin(), a.end(), got[q * k + j]) ? 1 : 0;
        }
        last_recall = (double)hit / (double)n;
        last_c = c;
        if (last_recall >= target) {
            best = c;
            best_recall = last_recall;
            break;
        }
    }
    cudaFree(d_dist);
    cudaFree(d_idx);
    if (rc) return rc;
    if (!best) {  // no factor reached the target: the largest one tried
        best = last_c;
        best_recall = last_recall;
    }
    *c_out = best;
    if (recall_out) *recall_out = best_recall;
    return KNNS_OK;
}

void knns_index_destroy(knns_index* ix)
{
    if (!ix) return;
    cudaDeviceSynchronize();
    ix->pc.release();
    delete ix;
}

int knns_debug_prep(const float* x, int64_t n, int64_t ld, int D, float* norms, void* bf16, void* f8, float* scales,
                    uint32_t* words, void* norm_parts)
{
    clear_error();
    if (!x || !norms || !bf16 || !f8 || !scales || !words || n <= 0 || D <= 0 || D > kPrepMaxD || ld < D)
        return set_error(KNNS_ERR_INVALID, "bad args");
    Engine* E = nullptr;
    int rc = get_engine(&E);
    if (rc) return rc;
    std::lock_guard<std::mutex> lk(E->mu);
    cudaStream_t s = E->host_stream();
    KNN_CUDA(cudaMemsetAsync(words, 0, 3 * sizeof(uint32_t), s));
    KNN_CUDA(launch_prep_rows(x, n, ld, D, (D + 63) & ~63, bf16, norms, n, words, s, words + 1, f8, (D + 127) & ~127,
                              scales, norm_parts));
    KNN_CUDA(cudaStreamSynchronize(s));
    return KNNS_OK;
}

int knns_debug_scan_plan(int64_t N, int64_t Q, int D, int k, int sms, int tf32, knns_scan_plan_info* out)
{
    clear_error();
    static_assert(KNNS_MAX_SEED_LEVELS == kMaxSeedLevels, "seeding levels of the plan record");
    if (!out || N < 1 || Q < 1 || D < 1 || k < 1 || k > 512 || sms < 1) return set_error(KNNS_ERR_INVALID, "bad args");
    // the planner reads only the SM count of the engine: a host-only engine stands in for the GPU's
    Engine E;
    E.sms = sms;
    knns_options o;
    knns_default_options(&o);
    int kp = auto_kp(k, 1);
    if (kp > 512) kp = std::max(round16(k), 32);  // no margin at the limit (as resolve_config)
    ScanPlan P;
    const int rc = plan_scan(E, N, Q, (D + 63) & ~63, kp, o, &P, false, tf32 != 0);
    if (rc) return rc;
    memset(out, 0, sizeof(*out));
    out->kp = kp;
    out->tile_rows = tf32 ? 128 : scan_tile_rows((D + 63) & ~63, P.accs);
    out->levels = P.levels;
    for (int l = 0; l < P.levels; ++l) {
        out->level_rows[l] = P.lv[l].n;
        out->level_stride[l] = P.lv[l].stride;
        out->level_rank[l] = P.lv[l].j;
        out->level_splits[l] = P.lv[l].S;
        out->level_cap[l] = P.lv[l].cap;
    }
    out->splits = P.S;
    out->split_len = P.len;
    out->cap = P.cap;
    out->sel_words = P.sel_words;
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
