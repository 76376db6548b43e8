// kernels.h -- launchers of the engine's CUDA kernels (internal interface).
#pragma once

#include <cstdint>
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

// CUDA-core FP32 fused distance + shortlist.  qpb in {32, 128}.
size_t simt_smem_bytes(int qpb, int kp);
// tile_redo (optional): a CTA runs only when tile_redo[blockIdx.x] != 0.
cudaError_t launch_simt(const float* corpus, int64_t N, int64_t ldc, const float* cn,
                        const float* queries, int64_t Q, int64_t ldq, int D, int kp, int qpb,
                        int64_t split_len, int splits, uint64_t* part, uint32_t* thr_g, cudaStream_t s,
                        const uint32_t* tile_redo = nullptr);

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
    float* dump;              // optional: raw dot tile of CTA (0,0), tile 0, [128][128]
    int* err;                 // device error word
    int D;
    int dp;                   // D rounded up to kChunkK
    int dpb;                  // D rounded up to 64 (BF16 boxes)
    int kp;
    int stages;
};
size_t tc_smem_bytes(int kp, int stages);
int tc_max_stages(int kp);
// Launches the BF16 (bf16 = true) or TF32 variant; each returns at once unless
// *a.not_exact selects it (BF16: inputs exact in BF16; TF32: otherwise).
cudaError_t launch_tc(const TcArgs& a, int splits, bool bf16, cudaStream_t s);

// Merge of the per-split shortlists, optional exact re-rank, final top-k.
// Extra modes (all optional):
//  * thr_out: instead of results, write the order-mapped key of the merged
//    shortlist's entry thr_rank (1-based; all ones when missing) per query;
//  * redo_out / need: when the merged shortlist holds fewer than `need` real
//    entries, set redo_out[q / qtile] = 1 and write no result for q;
//  * redo_in: process only queries whose tile has redo_in[q / qtile] != 0.
struct SelectExtra {
    uint32_t* thr_out = nullptr;
    int thr_rank = 0;
    uint32_t* redo_out = nullptr;
    int need = 0;
    const uint32_t* redo_in = nullptr;
    int qtile = 128;
};
size_t select_smem_bytes(int kp, int D, int rerank);
cudaError_t launch_select(const uint64_t* part, int splits, int64_t Q, int kp, int k,
                          const float* corpus, int64_t ldc, const float* queries, int64_t ldq,
                          int D, int rerank, const float* qn, float* out_dist, int32_t* out_idx,
                          float* out_idx_f, cudaStream_t s, const SelectExtra& ex = SelectExtra());

// out[i] = src[i * stride] for i < n, +inf for n <= i < n_pad (norms of a strided corpus sample).
cudaError_t launch_gather_norms(const float* src, int64_t n, int64_t stride, float* out, int64_t n_pad,
                                cudaStream_t s);

}  // namespace knn
