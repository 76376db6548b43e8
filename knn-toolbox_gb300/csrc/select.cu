// select.cu -- merge of the per-split shortlists, exact re-rank, final top-k.
//
// Replaces the reference's cross-chunk host merge (mergeResBitonic,
// src/cuknnBitonic.cu:381-417; mergeResHeap, src/cuknnHeap.cu:26-62) and the
// final +||q||^2 pass (dot3, include/utils.h:485-491).  One warp per query:
// the `splits` sorted shortlists are merged pairwise by rank (ties: earlier
// split first, which is also lower index, so the reference's "earlier chunk
// wins" rule holds), then either
//   rerank = 1: every shortlisted candidate gets its exact distance
//               (direct difference, oracle convention), the shortlist is
//               re-sorted by (distance, index) and the first k are returned;
//   rerank = 0: the first k by GEMM-form key are returned with
//               distance = key + ||q||^2 (the reference's output contract).
#include <cstdint>
#include <cuda_runtime.h>
#include "common.cuh"
#include "kernels.h"

namespace knn {

namespace {
constexpr int kSelWarps = 4;

__host__ __device__ inline int pow2_at_least(int x)
{
    int p = 32;
    while (p < x) p <<= 1;
    return p;
}
}  // namespace

__global__ void __launch_bounds__(kSelWarps * 32)
select_kernel(const uint64_t* __restrict__ part, int splits, int64_t Q, int kp, int k,
              const float* __restrict__ corpus, int64_t ldc, const float* __restrict__ queries,
              int64_t ldq, int D, int rerank, const float* __restrict__ qn,
              float* __restrict__ out_dist, int32_t* __restrict__ out_idx, float* __restrict__ out_idx_f,
              const SelectExtra ex)
{
    extern __shared__ __align__(16) unsigned char smem[];
    const int P = pow2_at_least(kp);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // per warp: cur[P], nxt[P], other[kp], query vector[D]
    size_t per_warp_words = (size_t)3 * P;
    uint64_t* cur = reinterpret_cast<uint64_t*>(smem) + warp * per_warp_words;
    uint64_t* nxt = cur + P;
    uint64_t* oth = nxt + P;
    float* qv = reinterpret_cast<float*>(reinterpret_cast<uint64_t*>(smem) + kSelWarps * per_warp_words) +
                (size_t)warp * ((D + 3) & ~3);

    const int64_t q = (int64_t)blockIdx.x * kSelWarps + warp;
    if (q >= Q) return;
    if (ex.redo_in != nullptr && ex.redo_in[q / ex.qtile] == 0u) return;

    for (int j = lane; j < kp; j += 32) cur[j] = part[(size_t)q * kp + j];
    __syncwarp();
    for (int s = 1; s < splits; ++s) {
        const uint64_t* src = part + ((size_t)s * Q + q) * kp;
        for (int j = lane; j < kp; j += 32) oth[j] = src[j];
        __syncwarp();
        warp_merge_lists(cur, oth, nxt, kp);
        uint64_t* t = cur; cur = nxt; nxt = t;
        __syncwarp();
    }

    if (ex.thr_out != nullptr) {
        // threshold extraction: key of the thr_rank-th entry
        if (lane == 0) {
            const uint64_t w = cur[ex.thr_rank - 1];
            ex.thr_out[q] = w == kSentinel ? 0xFFFFFFFFu : (uint32_t)(w >> 32);
        }
        return;
    }
    if (ex.redo_out != nullptr && ex.need > 0 && cur[ex.need - 1] == kSentinel) {
        // fewer entries than required passed a seeded threshold: this query's tile is redone
        if (lane == 0) ex.redo_out[q / ex.qtile] = 1u;
        return;
    }

    if (rerank) {
        const float* qrow = queries + q * ldq;
        for (int d = lane; d < D; d += 32) qv[d] = __ldg(qrow + d);
        __syncwarp();
        for (int j = lane; j < P; j += 32) {
            uint64_t w = j < kp ? cur[j] : kSentinel;
            if (w != kSentinel) {
                uint32_t n = unpack_idx(w);
                float dist = exact_dist_row(qv, corpus + (int64_t)n * ldc, D);
                w = pack_key(dist, n);
            }
            cur[j] = w;
        }
        __syncwarp();
        warp_sort_smem(cur, P);
        for (int j = lane; j < k; j += 32) {
            uint64_t w = cur[j];
            bool ok = w != kSentinel;
            float dv = ok ? unpack_key(w) : __int_as_float(0x7f800000);
            int32_t iv = ok ? (int32_t)unpack_idx(w) : -1;
            if (out_dist) out_dist[q * k + j] = dv;
            if (out_idx) out_idx[q * k + j] = iv;
            if (out_idx_f) out_idx_f[q * k + j] = (float)iv;
        }
    } else {
        const float qq = qn[q];
        for (int j = lane; j < k; j += 32) {
            uint64_t w = cur[j];
            bool ok = w != kSentinel;
            float dv = ok ? __fadd_rn(unpack_key(w), qq) : __int_as_float(0x7f800000);
            int32_t iv = ok ? (int32_t)unpack_idx(w) : -1;
            if (out_dist) out_dist[q * k + j] = dv;
            if (out_idx) out_idx[q * k + j] = iv;
            if (out_idx_f) out_idx_f[q * k + j] = (float)iv;
        }
    }
}

size_t select_smem_bytes(int kp, int D, int rerank)
{
    int P = pow2_at_least(kp);
    return (size_t)kSelWarps * 3 * P * 8 + (rerank ? (size_t)kSelWarps * ((D + 3) & ~3) * 4 : 0);
}

cudaError_t launch_select(const uint64_t* part, int splits, int64_t Q, int kp, int k,
                          const float* corpus, int64_t ldc, const float* queries, int64_t ldq,
                          int D, int rerank, const float* qn, float* out_dist, int32_t* out_idx,
                          float* out_idx_f, cudaStream_t s, const SelectExtra& ex)
{
    if (Q <= 0) return cudaSuccess;
    size_t smem = select_smem_bytes(kp, D, rerank);
    cudaError_t e = cudaFuncSetAttribute(select_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    unsigned blocks = (unsigned)((Q + kSelWarps - 1) / kSelWarps);
    select_kernel<<<blocks, kSelWarps * 32, smem, s>>>(part, splits, Q, kp, k, corpus, ldc, queries, ldq, D,
                                                       rerank, qn, out_dist, out_idx, out_idx_f, ex);
    return cudaGetLastError();
}

}  // namespace knn
