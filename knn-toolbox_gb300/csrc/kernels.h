// kernels.h -- launchers of the engine's CUDA kernels (internal interface).
#pragma once

#include <cstdint>
#include <limits>
#include <cuda.h>
#include <cuda_runtime.h>

namespace knn {

// Tile geometry shared by host and device.
constexpr int kTileQ = 128;       // queries per CTA (tensor-core M, TMEM lanes)
constexpr int kTileN = 128;       // corpus rows per tile (tensor-core N)
constexpr int kChunkK = 32;       // fp32 elements per 128-byte swizzle row
constexpr int kMaxDpTC = 128;     // A hi + lo must fit next to two accumulators in TMEM
constexpr int kMaxKpTC = 128;     // shortlist entries per query held in shared memory
constexpr int kSimtTileN = 64;

// error codes written by kernels into the device error word
enum DeviceError : int {
    kDevOk = 0,
    kDevTimeoutProducer = 1,
    kDevTimeoutMma = 2,
    kDevTimeoutEpilogue = 3,
    kDevTimeoutAload = 4,
    kDevMisaligned = 5,
};

cudaError_t launch_norms(const float* x, int64_t n, int64_t ld, int D, float* out, int64_t n_pad,
                         cudaStream_t s);
// TF32 hi/lo split into [n][dp] arrays; lo_flags[tile of 128 rows] = any lo != 0 (may be null);
// *any_lo (zeroed by the caller, may be null) becomes 1 when some tile has a low part.  When
// skip_unless is given and *skip_unless == 0 at run time, the kernel does nothing.
cudaError_t launch_split(const float* x, int64_t n, int64_t ld, int D, int dp, float* hi, float* lo,
                         uint32_t* lo_flags, uint32_t* any_lo, const uint32_t* skip_unless, cudaStream_t s);
// BF16 copy into [n][dpb] (out may be null: check only); *not_exact |= 1 when some element
// is not exactly representable in BF16.
cudaError_t launch_bf16(const float* x, int64_t n, int64_t ld, int D, int dpb, void* out, uint32_t* not_exact,
                        cudaStream_t s);

// One pass over a row-major matrix: optional BF16 copy out[n][dpb] (dpb = 0: none)
// with the exactness flag, optional norms[0..n_pad) (+inf padding), same
// conventions as launch_norms / launch_bf16.  Rows wider than kPrepMaxD fall
// back to those two kernels.
constexpr int kPrepMaxD = 384;
// int_stats (optional, 2 words, zeroed by the caller): [0] |= 1 when some value is not an
// integer, [1] = max |x| as float bits.
// f8 / scales (optional): E4M3 copy [n][f8_bytes] (f8_bytes a multiple of 128, zero padded) with
// per-row absmax scales (row = scale * codes; scales[n..n_pad) = 0); needs D <= kPrepMaxD.
// np (optional): norm parts [n][kNormParts] BF16, (n1, n2, n3, 0, ...) with n1 + n2 + n3 equal
// to the row's FP32 norm; needs D <= kPrepMaxD.
constexpr int kNormParts = 16;
cudaError_t launch_prep_rows(const float* x, int64_t n, int64_t ld, int D, int dpb, void* out, float* norms,
                             int64_t n_pad, uint32_t* not_exact, cudaStream_t s, uint32_t* int_stats = nullptr,
                             void* f8 = nullptr, int f8_bytes = 0, float* scales = nullptr, void* np = nullptr);

// CUDA-core FP32 fused distance + shortlist.  qpb in {32, 128}.
size_t simt_smem_bytes(int qpb, int kp);
// tile_redo (optional): a CTA runs only when tile_redo[blockIdx.x] != 0.
// qmap / qcount / qbase (optional, together): compacted rows, as for TcArgs -- row r of the
// launch (r < Q) is query qmap[qbase + r], present only when qbase + r < *qcount.
cudaError_t launch_simt(const float* corpus, int64_t N, int64_t ldc, const float* cn,
                        const float* queries, int64_t Q, int64_t ldq, int D, int kp, int qpb,
                        int64_t split_len, int splits, uint64_t* part, uint32_t* thr_g, cudaStream_t s,
                        const uint32_t* tile_redo = nullptr, const int32_t* qmap = nullptr,
                        const uint32_t* qcount = nullptr, int64_t qbase = 0);

// Tensor-core 3xTF32 fused distance + shortlist (tcgen05, TMA, TMEM).
struct TcArgs {
    CUtensorMap tm_hi;        // corpus hi  [N][dp] fp32, box {32, 128}, 128B swizzle
    CUtensorMap tm_lo;        // corpus lo
    CUtensorMap tm_bf;        // corpus bf16 [N][dpb], box {64, 128}, 128B swizzle
    const float* cn;          // [>= roundup(N,128)] corpus norms, +inf padding
    const float* queries;     // [Q][ldq]
    int64_t Q;
    int64_t ldq;
    int64_t N;
    int64_t split_len;        // corpus rows per split, multiple of kTileN
    uint64_t* part;           // [splits][Q][kp]
    uint32_t* thr_g;          // [Q] shared per-query threshold (order-mapped key), or null
    const uint32_t* lo_flags; // [ceil(N/128)] 1 when the corpus tile has a nonzero TF32 low part, or null
    const uint32_t* corpus_any_lo;  // 1 when any corpus tile has a low part (null: assume so)
    const uint32_t* not_exact;      // 0 when corpus and queries are BF16-exact (null: TF32 path only)
    const uint32_t* tile_redo;      // optional: a CTA runs only when tile_redo[blockIdx.x] != 0
    // optional compacted-query mode: row r of this launch (r < Q) is query qmap[qbase + r],
    // present only when qbase + r < *qcount; part / thr_g rows are indexed by r
    const int32_t* qmap;
    const uint32_t* qcount;
    int64_t qbase;
    float* dump;              // optional: raw dot tile of CTA (0,0), tile 0, [128][128]
    int* err;                 // device error word
    int D;
    int dp;                   // D rounded up to kChunkK
    int dpb;                  // D rounded up to 64 (BF16 boxes)
    int kp;
    int stages;
    uint64_t timeout_ns;      // bound of every barrier wait (0: 4 s)
    int test_stall;           // test hook: the producer issues no copy, so the waits run out
};
size_t tc_smem_bytes(int kp, int stages);
int tc_max_stages(int kp);
// Launches the BF16 (bf16 = true) or TF32 variant; each returns at once unless
// *a.not_exact selects it (BF16: inputs exact in BF16; TF32: otherwise).
cudaError_t launch_tc(const TcArgs& a, int splits, bool bf16, cudaStream_t s);

// Tensor-core BF16 threshold scan (csrc/scan_bf16.cu): 128 queries x 256-row
// corpus tiles; every key strictly below the query's threshold is appended to
// the query's segment cand[(split*kScanParts + part)][q][0..cap) (part = the
// tile's 64-column quarter; in increasing corpus index), as (raw float bits of
// the key) << 32 | index; cnt[(split*kScanParts + part)][q] = keys found (may
// exceed cap: overflow).
constexpr int kScanTileN = 256;
constexpr int kScanParts = 4;
constexpr int kScanMaxRing = 8;
constexpr size_t kScanSmemLimit = 232448;
// Row width of the scan's operands in 16-bit units (dpb below): D rounded up to
// 64 for BF16 keys; for E4M3 keys the row's bytes (D rounded up to 128) / 2,
// so both key types share one tile geometry per 128-byte K box.
struct ScanArgs {
    CUtensorMap tm_c;          // corpus [N][dpb] 16-bit units (view), box {64, scan_box_rows(dpb)}, 128B swizzle
    CUtensorMap tm_np;         // BF16 keys: norm parts of the view [N][kNormParts] BF16, box {16, tile rows},
                               // 32B swizzle (E4M3 keys: unused)
    const void* qbf;           // queries [Q][dpb] 16-bit units (BF16, or E4M3 bytes)
    const float* cn;           // fp8: [>= N + scan_tile_rows(dpb)] corpus norms of the view, +inf padding
    const float* cs;           // fp8: corpus row scales of the view (same padding, 0 there)
    const float* qs;           // fp8: query row scales [Q]
    const float* thr;          // [Q] thresholds (null: +inf, every key collected)
    const uint32_t* skip_if;   // optional: the kernel returns at once when *skip_if != 0
    uint64_t* cand;            // [splits*kScanParts][Q][cap]
    uint32_t* cnt;             // [splits*kScanParts][Q]
    int* err;                  // device error word
    int64_t Q;
    int64_t N;
    int64_t split_len;         // multiple of scan_tile_rows(dpb)
    int cap;
    int dpb;                   // row width in 16-bit units, multiple of 64, <= 256
    int ksteps;                // MMA K steps holding data (32 bytes each): ceil(D / 16) BF16, ceil(D / 32) E4M3
    int bps;                   // K-boxes per ring slot (divides dpb/64)
    int ring;                  // ring slots
    int fp8;                   // keys from E4M3 operands with per-row scales
    int split0;                // first split of this launch (grid row y is split split0 + y)
    int accs;                  // TMEM accumulators: 2 (tiles of 224 / 192 rows) or 4 (tiles of 96)
};
// corpus rows per tile (MMA N): with 2 accumulators 224 for dpb <= 128, 192 for dpb <= 256;
// with 4 accumulators 96
int scan_tile_rows(int dpb, int accs);
// rows of the corpus tensor map's box (one whole tile)
int scan_box_rows(int dpb, int accs);
// most columns of one tile that a single candidate segment (epilogue part) collects
int scan_part_cols(int dpb, int accs);
size_t scan_smem_bytes(int dpb, int bps, int ring, bool fp8, int accs);
// Ring geometry for dpb (want_bps = 0: automatic).  Returns 0 on success.
int scan_plan(int dpb, int want_bps, int* bps, int* ring, bool fp8, int accs);
cudaError_t launch_scan(const ScanArgs& a, int splits, cudaStream_t s);

// Tensor-core 3xTF32 threshold scan (csrc/scan_tf32.cu): 128 queries x 128-row corpus
// tiles, K in chunks of 32 FP32 columns, both operands from shared memory (any D, a
// multiple of 32 after padding); the candidate segments are those of the BF16 scan
// (kScanParts per split, 32 columns of every tile each).
struct TscanArgs {
    CUtensorMap tm_qhi, tm_qlo;   // queries hi / lo [Q][dp] fp32, box {32, 128}, 128B swizzle
    CUtensorMap tm_chi, tm_clo;   // corpus hi / lo view [N][dp] fp32, same boxes
    const float* cn;              // [>= N + 128] corpus norms of the view, +inf padding
    const float* thr;             // [Q] thresholds (null: +inf, every key collected)
    const uint32_t* qlo_flags;    // [query tiles] 1 when the tile has a nonzero low part (null: all)
    const uint32_t* clo_flags;    // [128-row tiles of the view] same for the corpus (null: all)
    uint64_t* cand;               // [splits*kScanParts][Q][cap]
    uint32_t* cnt;                // [splits*kScanParts][Q]
    int* err;                     // device error word
    int64_t Q;
    int64_t N;
    int64_t split_len;            // multiple of 128
    int cap;
    int dp;                       // D rounded up to 32
    int split0;                   // first split of this launch
    int ring;                     // ring slots (tscan_ring())
    const uint32_t* run_if;       // optional: the kernel returns at once when *run_if == 0
    // dp <= 128: the queries' TF32 hi / lo parts in tensor memory, split by the kernel from the
    // FP32 queries (tm_qhi, tm_qlo, qlo_flags unused); the ring carries corpus chunks only
    int tmem_a;
    const float* queries;         // [Q][ldq] fp32 (tmem_a)
    int64_t ldq;
    int D;
};
size_t tscan_smem_bytes(int ring, bool tmem_a);
int tscan_ring(bool tmem_a);
cudaError_t launch_tscan(const TscanArgs& a, int splits, cudaStream_t s);

// Merge of the per-split shortlists, optional exact re-rank, final top-k.
// Extra modes (all optional):
//  * thr_out: instead of results, write the order-mapped key of the merged
//    shortlist's entry thr_rank (1-based; all ones when missing) per query;
//  * redo_out / need: when the merged shortlist holds fewer than `need` real
//    entries, set redo_out[q / qtile] = 1 and write no result for q;
//  * redo_in: process only queries whose tile has redo_in[q / qtile] != 0.
//  * skip_if_zero: the kernel does nothing when *skip_if_zero == 0 (device-side path choice);
//  * qmap / qcount / qbase: compacted rows, as for TcArgs: part row r is query
//    qmap[qbase + r], present when qbase + r < *qcount; results go to that query's row.
struct SelectExtra {
    uint32_t* thr_out = nullptr;
    int thr_rank = 0;
    uint32_t* redo_out = nullptr;
    int need = 0;
    const uint32_t* redo_in = nullptr;
    int qtile = 128;
    const uint32_t* skip_if_zero = nullptr;
    const int32_t* qmap = nullptr;
    const uint32_t* qcount = nullptr;
    int64_t qbase = 0;
};
size_t select_smem_bytes(int kp, int D, int rerank);
cudaError_t launch_select(const uint64_t* part, int splits, int64_t Q, int kp, int k,
                          const float* corpus, int64_t ldc, const float* queries, int64_t ldq,
                          int D, int rerank, const float* qn, float* out_dist, int32_t* out_idx,
                          float* out_idx_f, cudaStream_t s, const SelectExtra& ex = SelectExtra());

// Selection over the threshold scan's candidate segments (one warp per query).
// The candidates of query q are the first min(cnt, cap) words of its nseg
// segments; total = sum of cnt (the number of keys below the threshold).
//  * thr_out (threshold mode): thr_out[q] = the next float above the key of
//    rank thr_rank (1-based) when total >= thr_rank, no segment overflowed and
//    total <= kCandMax; otherwise thr_out[q] = thr_fallback[q] (+inf if null);
//  * result mode: the kp smallest (key, index) words form the shortlist, then
//    re-rank / output as launch_select.  A query whose candidates cannot be
//    trusted (overflow, total < need, total > kCandMax) is appended to
//    fail_idx (count in *fail_cnt) and gets no result.
constexpr int kCandMax = 2048;
constexpr int kMaxKpScan = 512;  // longest shortlist the threshold scan's selection keeps
constexpr int kScanMaxSegs = 512;  // candidate segments per query (splits x kScanParts)
struct CandSelect {
    const uint64_t* cand = nullptr;
    const uint32_t* cnt = nullptr;
    int nseg = 0;
    int cap = 0;
    int64_t Q = 0;
    const uint32_t* skip_if = nullptr;       // the kernel does nothing when *skip_if != 0
    const uint32_t* skip_if_zero = nullptr;  // the kernel does nothing when *skip_if_zero == 0
    float* thr_out = nullptr;
    int thr_rank = 0;
    const float* thr_fallback = nullptr;
    int kp = 0;
    int k = 0;
    int need = 0;
    int rerank = 1;
    const float* corpus = nullptr;
    int64_t ldc = 0;
    const float* queries = nullptr;
    int64_t ldq = 0;
    int D = 0;
    const float* qn = nullptr;
    float* out_dist = nullptr;
    int32_t* out_idx = nullptr;
    float* out_idx_f = nullptr;
    int32_t* fail_idx = nullptr;
    uint32_t* fail_cnt = nullptr;
    // exact-key test (optional): keys and distances are exact integers when every corpus and
    // query value is an integer, 2 * D * max|x|^2 < 2^24 and the BF16 copies are exact; the
    // re-rank is then skipped (distance = key + qn[q], the same value it would compute)
    const uint32_t* int_stats = nullptr;  // [0] not-integer flag, [1] max|x| bits (corpus and queries)
    const uint32_t* bf16_inexact = nullptr;
    // per-warp candidate buffer (words): result mode takes it as the caller's bound on one
    // query's stored candidates (0 = kCandMax; a query above it fails over to the fix-up);
    // threshold mode sets it from nseg * cap
    int buf_words = 0;
};
cudaError_t launch_select_cand(const CandSelect& c, cudaStream_t s);

// Running top-k (have entries, row pitch k) merged with a block's top-kb (pitch kb,
// indices + offset) into out (pitch k, min(k, have + kb) entries); out_idx_f optional.
cudaError_t launch_merge_topk(const float* run_d, const int32_t* run_i, int have, const float* blk_d,
                              const int32_t* blk_i, int kb, int32_t offset, int64_t Q, int k, float* out_d,
                              int32_t* out_i, float* out_idx_f, cudaStream_t s);

// out[i] = src[i * stride] for i < n, pad for n <= i < n_pad (+inf: norms of padding rows), the
// norms of a strided corpus sample; nothing when skip_unless is given and *skip_unless == 0.
cudaError_t launch_gather_norms(const float* src, int64_t n, int64_t stride, float* out, int64_t n_pad,
                                cudaStream_t s, float pad = std::numeric_limits<float>::infinity(),
                                const uint32_t* skip_unless = nullptr);

}  // namespace knn
