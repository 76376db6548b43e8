// select.cu -- merge of the per-split shortlists (or of the threshold scan's
// candidate segments), exact re-rank, final top-k.
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
#include <algorithm>
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

// cur[0..kp) holds the query's shortlist sorted by (key, index) (sentinels at
// the end); cur has room for pow2_at_least(kp) words.  Writes the k results of
// query q (re-ranked by exact distance, or key + ||q||^2).
__device__ __forceinline__ void finish_query(uint64_t* cur, int kp, int k, int64_t q, int rerank,
                                             const float* __restrict__ corpus, int64_t ldc,
                                             const float* __restrict__ queries, int64_t ldq, int D,
                                             const float* __restrict__ qn, float* qv, float* out_dist,
                                             int32_t* out_idx, float* out_idx_f)
{
    const int lane = threadIdx.x & 31;
    if (rerank) {
        const int P = pow2_at_least(kp);
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
}  // namespace

__global__ void __launch_bounds__(kSelWarps * 32)
select_kernel(const uint64_t* __restrict__ part, int splits, int64_t Q, int kp, int k,
              const float* __restrict__ corpus, int64_t ldc, const float* __restrict__ queries,
              int64_t ldq, int D, int rerank, const float* __restrict__ qn,
              float* __restrict__ out_dist, int32_t* __restrict__ out_idx, float* __restrict__ out_idx_f,
              const SelectExtra ex)
{
    extern __shared__ __align__(16) unsigned char smem[];
    if (ex.skip_if_zero != nullptr && *ex.skip_if_zero == 0u) return;
    const int P = pow2_at_least(kp);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // per warp: cur[P], nxt[P], other[kp], query vector[D]
    size_t per_warp_words = (size_t)3 * P;
    uint64_t* cur = reinterpret_cast<uint64_t*>(smem) + warp * per_warp_words;
    uint64_t* nxt = cur + P;
    uint64_t* oth = nxt + P;
    float* qv = reinterpret_cast<float*>(reinterpret_cast<uint64_t*>(smem) + kSelWarps * per_warp_words) +
                (size_t)warp * ((D + 3) & ~3);

    const int64_t q = (int64_t)blockIdx.x * kSelWarps + warp;  // row of `part`
    if (q >= Q) return;
    if (ex.redo_in != nullptr && ex.redo_in[q / ex.qtile] == 0u) return;
    int64_t qout = q;  // query whose results this row holds
    if (ex.qcount != nullptr) {
        if (ex.qbase + q >= (int64_t)*ex.qcount) return;
        qout = ex.qmap[ex.qbase + q];
    }

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
    finish_query(cur, kp, k, qout, rerank, corpus, ldc, queries, ldq, D, qn, qv, out_dist, out_idx, out_idx_f);
}

// ---------------------------------------------------------------- threshold-scan selection
namespace {
// rows of candidate vectors staged per re-rank batch: [rows][D + 1] floats (about 8 KB: the
// staging area sets the warp's shared memory, hence how many queries run per SM)
__host__ __device__ inline int cand_stage_rows(int D) { return D <= 128 ? 16 : (D <= 512 ? 8 : 4); }

// candidate words a warp can hold: threshold mode (seeding passes) and result mode
constexpr int kCandThrMax = 1024;

// re-rank: the sorted shortlist cur[0, P) (P = pow2_at_least(kp)) then the staged rows
__host__ __device__ inline size_t cand_warp_bytes(int D, bool thr_mode, bool rerank, int buf_words, int kp)
{
    const size_t sel = (size_t)buf_words * 8;
    const size_t rr =
        rerank && !thr_mode ? (size_t)pow2_at_least(kp) * 8 + (size_t)cand_stage_rows(D) * (D + 1) * 4 : 0;
    const size_t w = sel > rr ? sel : rr;
    return (w + 15) & ~(size_t)15;
}

// scan word (raw float bits of the key << 32 | index) -> ordered word (pack_key)
__device__ __forceinline__ uint64_t raw_to_ordered(uint64_t w)
{
    return pack_key(__uint_as_float((uint32_t)(w >> 32)), (uint32_t)w);
}

// number of words w[0..n) (shared memory) not above x, summed over the warp
// Radix-4 step of the rank search: the counts of values not above y0 < y1 < y2 in one
// pass (n <= 65,535, so two counts share a 32-bit reduction), and the 2-bit digit d of the
// rank-th smallest value: the number of thresholds with fewer than `rank` values not
// above them.  Half the dependent rounds of a bitwise search.
template <typename V, typename F>
__device__ __forceinline__ uint32_t radix4_digit(const uint64_t* w, int n, V y0, V y1, V y2, uint32_t rank, F val)
{
    const int lane = threadIdx.x & 31;
    uint32_t a = 0, b = 0;
    for (int e = lane; e < n; e += 32) {
        const V v = val(w[e]);
        a += (v <= y0 ? 1u : 0u) + (v <= y1 ? 0x10000u : 0u);
        b += v <= y2 ? 1u : 0u;
    }
    a = __reduce_add_sync(0xffffffffu, a);
    b = __reduce_add_sync(0xffffffffu, b);
    return ((a & 0xffffu) < rank ? 1u : 0u) + ((a >> 16) < rank ? 1u : 0u) + (b < rank ? 1u : 0u);
}

// Threshold mode with few keys: at most kThrRegs keys per lane, ranks up to kThrRankRegs.
constexpr int kThrRegs = 8;
constexpr int kThrRankRegs = 64;

// The ordered key of rank `rank` (1-based, ties counted) among the key halves of w[0..n),
// n <= 32 * kThrRegs, n >= rank: lane l holds w[l + 32 i], sorted in registers (Batcher's
// odd-even merge network for 8); each round the warp minimum of the lanes' heads is found, every
// lane whose head equals it drops its head, and the count of dropped keys decides the rank.
__device__ __forceinline__ uint32_t rank_in_registers(const uint64_t* w, int n, uint32_t rank)
{
    const int lane = threadIdx.x & 31;
    uint32_t k[kThrRegs];
#pragma unroll
    for (int i = 0; i < kThrRegs; ++i) k[i] = lane + 32 * i < n ? (uint32_t)(w[lane + 32 * i] >> 32) : 0xFFFFFFFFu;
    auto ce = [&](int a, int b) {
        const uint32_t lo = min(k[a], k[b]), hi = max(k[a], k[b]);
        k[a] = lo;
        k[b] = hi;
    };
    ce(0, 1); ce(2, 3); ce(4, 5); ce(6, 7);
    ce(0, 2); ce(1, 3); ce(4, 6); ce(5, 7);
    ce(1, 2); ce(5, 6);
    ce(0, 4); ce(1, 5); ce(2, 6); ce(3, 7);
    ce(2, 4); ce(3, 5);
    ce(1, 2); ce(3, 4); ce(5, 6);
    uint32_t removed = 0, x = 0xFFFFFFFFu;
    for (uint32_t it = 0; it < rank; ++it) {  // every round drops at least one key
        const uint32_t m = __reduce_min_sync(0xffffffffu, k[0]);
        const bool hit = k[0] == m;
        removed += (uint32_t)__popc(__ballot_sync(0xffffffffu, hit));
        if (removed >= rank) {  // warp-uniform
            x = m;
            break;
        }
        if (hit) {
#pragma unroll
            for (int i = 0; i < kThrRegs - 1; ++i) k[i] = k[i + 1];
            k[kThrRegs - 1] = 0xFFFFFFFFu;
        }
    }
    return x;
}

// Exact distances of cur[0..kp) (direct difference, oracle order: eight partial
// sums over d mod 8, fixed final tree).  Candidate rows are staged in shared
// memory ([rows][D + 1]: conflict-free per-lane walks) four rows at a time with
// coalesced loads; lane j of a batch computes candidate b0 + j.
__device__ __forceinline__ void rerank_staged(uint64_t* cur, int kp, const float* __restrict__ corpus, int64_t ldc,
                                              const float* qv, int D, float* rows)
{
    const int lane = threadIdx.x & 31;
    const int RB = cand_stage_rows(D);
    const int pitch = D + 1;
    for (int b0 = 0; b0 < kp; b0 += RB) {
        const int nb = min(RB, kp - b0);
        for (int r0 = 0; r0 < nb; r0 += 4) {
            const float* src[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const uint64_t w = r0 + u < nb ? cur[b0 + r0 + u] : kSentinel;
                src[u] = w == kSentinel ? nullptr : corpus + (int64_t)unpack_idx(w) * ldc;
            }
            for (int d0 = 0; d0 < D; d0 += 64) {
                float v[8];
#pragma unroll
                for (int u = 0; u < 4; ++u)
#pragma unroll
                    for (int h = 0; h < 2; ++h) {
                        const int d = d0 + 32 * h + lane;
                        v[2 * u + h] = (src[u] != nullptr && d < D) ? __ldg(src[u] + d) : 0.f;
                    }
#pragma unroll
                for (int u = 0; u < 4; ++u)
#pragma unroll
                    for (int h = 0; h < 2; ++h) {
                        const int d = d0 + 32 * h + lane;
                        if (d < D) rows[(r0 + u) * pitch + d] = v[2 * u + h];
                    }
            }
        }
        __syncwarp();
        if (lane < nb) {
            const uint64_t w = cur[b0 + lane];
            if (w != kSentinel) {
                const float* c = rows + lane * pitch;
                float p[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
                int d = 0;
                for (; d + 8 <= D; d += 8) {
#pragma unroll
                    for (int u = 0; u < 8; ++u) {
                        const float t = __fsub_rn(qv[d + u], c[d + u]);
                        p[u] = __fmaf_rn(t, t, p[u]);
                    }
                }
                for (; d < D; ++d) {
                    const float t = __fsub_rn(qv[d], c[d]);
                    p[d & 7] = __fmaf_rn(t, t, p[d & 7]);
                }
                const float dist = __fadd_rn(__fadd_rn(__fadd_rn(p[0], p[1]), __fadd_rn(p[2], p[3])),
                                             __fadd_rn(__fadd_rn(p[4], p[5]), __fadd_rn(p[6], p[7])));
                cur[b0 + lane] = pack_key(dist, unpack_idx(w));
            }
        }
        __syncwarp();
    }
}
}  // namespace

// One warp per query over the threshold scan's segments.
template <bool kThr>
__global__ void __launch_bounds__(kSelWarps * 32) select_cand_kernel(const CandSelect c)
{
    extern __shared__ __align__(16) unsigned char smem[];
    if (c.skip_if != nullptr && *c.skip_if != 0u) return;
    if (c.skip_if_zero != nullptr && *c.skip_if_zero == 0u) return;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const size_t wb = cand_warp_bytes(c.D, kThr, c.rerank != 0, c.buf_words, c.kp);
    const int buf_max = c.buf_words;
    uint64_t* buf = reinterpret_cast<uint64_t*>(smem + (size_t)warp * wb);
    float* qv = reinterpret_cast<float*>(smem + (size_t)kSelWarps * wb) + (size_t)warp * ((c.D + 3) & ~3);
    const int64_t q = (int64_t)blockIdx.x * kSelWarps + warp;
    if (q >= c.Q) return;

    // segments s = lane + 32 r: their counts, all loaded at once
    constexpr int kSegPerLane = kScanMaxSegs / 32;
    uint32_t n4[kSegPerLane];
    uint32_t stored = 0, found = 0;
    bool over = false;
#pragma unroll
    for (int r = 0; r < kSegPerLane; ++r) {
        const int s = lane + 32 * r;
        const uint32_t n = s < c.nseg ? __ldg(c.cnt + (size_t)s * c.Q + q) : 0u;
        found += n;
        over |= n > (uint32_t)c.cap;
        n4[r] = min(n, (uint32_t)c.cap);
        stored += n4[r];
    }
    const uint32_t total = __reduce_add_sync(0xffffffffu, stored);
    const uint32_t found_all = __reduce_add_sync(0xffffffffu, found);
    const bool overflow = __any_sync(0xffffffffu, over);

    const uint32_t need = kThr ? (uint32_t)c.thr_rank : (uint32_t)c.need;
    if (overflow || found_all < need || total > (uint32_t)buf_max) {
        if (lane == 0) {
            if (kThr) {
                c.thr_out[q] = c.thr_fallback ? c.thr_fallback[q] : __int_as_float(0x7f800000);
            } else {
                const uint32_t pos = atomicAdd(c.fail_cnt, 1u);
                c.fail_idx[pos] = (int32_t)q;
            }
        }
        return;
    }

    // gather: each lane copies its own segments (segment-major prefix over r, then lanes)
    uint32_t base = 0;
#pragma unroll
    for (int r = 0; r < kSegPerLane; ++r) {
        if (32 * r >= c.nseg) break;  // warp-uniform: no segments left
        uint32_t pre = n4[r];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t v = __shfl_up_sync(0xffffffffu, pre, o);
            if (lane >= o) pre += v;
        }
        const uint32_t tot_r = __shfl_sync(0xffffffffu, pre, 31);
        const uint32_t my = base + pre - n4[r];
        const uint64_t* src = c.cand + ((size_t)(lane + 32 * r) * c.Q + q) * c.cap;
        for (uint32_t i0 = 0; i0 < n4[r]; i0 += 8) {
            uint64_t v[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) v[u] = i0 + u < n4[r] ? __ldg(src + i0 + u) : 0ull;
#pragma unroll
            for (int u = 0; u < 8; ++u)
                if (i0 + u < n4[r]) buf[my + i0 + u] = raw_to_ordered(v[u]);
        }
        base += tot_r;
    }
    __syncwarp();
    const int n = (int)total;

    if (kThr) {
        // smallest key x with at least thr_rank keys not above it
        uint32_t x = 0;
        if (n <= 32 * kThrRegs && c.thr_rank <= kThrRankRegs) {
            // few keys, small rank: each lane sorts its keys in registers, then the warp takes
            // minima in rank order (each round removes the lanes' heads equal to the minimum)
            x = rank_in_registers(buf, n, (uint32_t)c.thr_rank);
        } else {
            // radix-4 search, two bits per round: x's digit at bits [b0, b0 + 2) is the number
            // of the thresholds x | d 2^b0 | (2^b0 - 1), d = 0, 1, 2, with fewer than thr_rank
            // keys not above them
            for (int b0 = 30; b0 >= 0; b0 -= 2) {
                const uint32_t low = (1u << b0) - 1u;
                const uint32_t d = radix4_digit(buf, n, x | low, x | (1u << b0) | low, x | (2u << b0) | low,
                                                (uint32_t)c.thr_rank, [](uint64_t v) { return (uint32_t)(v >> 32); });
                x |= d << b0;
            }
        }
        if (lane == 0) {
            const float key = ord2f(x);
            // strictly above the key of rank thr_rank: that key itself passes a "< T" test
            c.thr_out[q] = key < __int_as_float(0x7f800000) ? nextafterf(key, __int_as_float(0x7f800000)) : key;
        }
        return;
    }

    // a bound W on the words kept: every word not above W is kept, the kp smallest (key,
    // index) words among them (words are distinct: indices are)
    const int kp = c.kp;
    const int P = pow2_at_least(kp);
    uint64_t W = kSentinel;
    if (n > kp) {
        // the kp-th smallest key K (2-bit digits of the key half); when the words with keys
        // up to K fit the sort, all of them are kept and the sort orders K's ties by index.
        // K lies between the smallest and the largest key, so it shares the bits above the
        // highest one in which they differ: the search starts at that bit's digit.
        uint32_t kmin = 0xFFFFFFFFu, kmax = 0u;
        for (int e = lane; e < n; e += 32) {
            const uint32_t v = (uint32_t)(buf[e] >> 32);
            kmin = min(kmin, v);
            kmax = max(kmax, v);
        }
        kmin = __reduce_min_sync(0xffffffffu, kmin);
        kmax = __reduce_max_sync(0xffffffffu, kmax);
        const uint32_t diff = kmin ^ kmax;
        const int top = diff ? (31 - __clz(diff)) & ~1 : -2;  // first digit to search
        uint32_t xk = top >= 30 ? 0u : top < 0 ? kmin : (kmin >> (top + 2)) << (top + 2);
        for (int b0 = top; b0 >= 0; b0 -= 2) {
            const uint32_t low = (1u << b0) - 1u;
            const uint32_t d = radix4_digit(buf, n, xk | low, xk | (1u << b0) | low, xk | (2u << b0) | low,
                                            (uint32_t)kp, [](uint64_t v) { return (uint32_t)(v >> 32); });
            xk |= d << b0;
        }
        uint32_t le = 0;
        for (int e = lane; e < n; e += 32) le += (uint32_t)(buf[e] >> 32) <= xk ? 1u : 0u;
        le = __reduce_add_sync(0xffffffffu, le);
        if (le <= (uint32_t)P) {
            W = ((uint64_t)xk << 32) | 0xffffffffull;
        } else {
            // many ties at K: the kp-th smallest word itself (its key half is K)
            uint64_t x = (uint64_t)xk << 32;
            for (int b0 = 30; b0 >= 0; b0 -= 2) {
                const uint64_t low = (uint64_t(1) << b0) - 1u;
                const uint64_t d = radix4_digit(buf, n, x | low, x | (uint64_t(1) << b0) | low,
                                                x | (uint64_t(2) << b0) | low, (uint32_t)kp,
                                                [](uint64_t v) { return v; });
                x |= d << b0;
            }
            W = x;
        }
    }
    // compact the words not above W (at most P of them) to the front, then sort them
    uint64_t* cur = buf;  // in place: the compacted prefix never overtakes the read position
    uint32_t m = 0;
    for (int e0 = 0; e0 < n; e0 += 32) {
        const int e = e0 + lane;
        const uint64_t w = e < n ? buf[e] : kSentinel;
        const bool keep = e < n && w <= W;
        const uint32_t bal = __ballot_sync(0xffffffffu, keep);
        __syncwarp();
        if (keep) cur[m + __popc(bal & ((1u << lane) - 1u))] = w;
        m += __popc(bal);
        __syncwarp();
    }
    for (int j = (int)m + lane; j < P; j += 32) cur[j] = kSentinel;
    __syncwarp();
    warp_sort_smem(cur, P);
    // the shortlist is cur[0, kp): words past it (ties kept above) are dropped
    for (int j = kp + lane; j < P; j += 32) cur[j] = kSentinel;
    __syncwarp();

    // exact integer keys: the ranking by key is the ranking by distance, distance = key + ||q||^2
    bool exact = false;
    if (c.int_stats != nullptr && c.qn != nullptr) {
        const float mx = __uint_as_float(__ldg(c.int_stats + 1));
        exact = __ldg(c.int_stats) == 0u && (c.bf16_inexact == nullptr || __ldg(c.bf16_inexact) == 0u) &&
                2.0 * (double)c.D * (double)mx * (double)mx < 16777216.0;
    }
    if (c.rerank && !exact) {
        const float* qrow = c.queries + q * c.ldq;
        for (int d = lane; d < c.D; d += 32) qv[d] = __ldg(qrow + d);
        __syncwarp();
        rerank_staged(cur, kp, c.corpus, c.ldc, qv, c.D, reinterpret_cast<float*>(buf + P));
        warp_sort_smem(cur, P);
        for (int j = lane; j < c.k; j += 32) {
            const uint64_t w = cur[j];
            const bool ok = w != kSentinel;
            const float dv = ok ? unpack_key(w) : __int_as_float(0x7f800000);
            const int32_t iv = ok ? (int32_t)unpack_idx(w) : -1;
            if (c.out_dist) c.out_dist[q * c.k + j] = dv;
            if (c.out_idx) c.out_idx[q * c.k + j] = iv;
            if (c.out_idx_f) c.out_idx_f[q * c.k + j] = (float)iv;
        }
    } else {
        finish_query(cur, kp, c.k, q, 0, c.corpus, c.ldc, c.queries, c.ldq, c.D, c.qn, qv, c.out_dist, c.out_idx,
                     c.out_idx_f);
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

// Merge of a corpus block's top-kb into the running top-k of every query (the
// reference's cross-block merge of its host-streamed corpus blocks,
// src/cuknnBitonic.cu:550-589, done on the device): both lists are sorted by
// (distance, index); block indices are shifted by the block's first row; the
// first min(k, have + kb) entries of the union in (distance, index) order go to
// the output list (and, as floats, to out_idx_f when given).  One thread per query.
__global__ void merge_topk_kernel(const float* __restrict__ run_d, const int32_t* __restrict__ run_i, int have,
                                  const float* __restrict__ blk_d, const int32_t* __restrict__ blk_i, int kb,
                                  int32_t offset, int64_t Q, int k, float* __restrict__ out_d,
                                  int32_t* __restrict__ out_i, float* __restrict__ out_idx_f)
{
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= Q) return;
    const float* rd = run_d + q * k;
    const int32_t* ri = run_i + q * k;
    const float* bd = blk_d + q * kb;
    const int32_t* bi = blk_i + q * kb;
    const int n = min(k, have + kb);
    int a = 0, b = 0;
    for (int j = 0; j < n; ++j) {
        bool take_a;
        if (a >= have) {
            take_a = false;
        } else if (b >= kb) {
            take_a = true;
        } else {
            const float da = rd[a], db = bd[b];
            const int32_t ia = ri[a], ib = bi[b] + offset;
            take_a = da < db || (da == db && ia < ib);
        }
        const float d = take_a ? rd[a] : bd[b];
        const int32_t i = take_a ? ri[a] : bi[b] + offset;
        a += take_a ? 1 : 0;
        b += take_a ? 0 : 1;
        out_d[q * k + j] = d;
        out_i[q * k + j] = i;
        if (out_idx_f) out_idx_f[q * k + j] = (float)i;
    }
}

cudaError_t launch_merge_topk(const float* run_d, const int32_t* run_i, int have, const float* blk_d,
                              const int32_t* blk_i, int kb, int32_t offset, int64_t Q, int k, float* out_d,
                              int32_t* out_i, float* out_idx_f, cudaStream_t s)
{
    if (Q <= 0) return cudaSuccess;
    if (k < 1 || kb < 0 || kb > k || have < 0 || have > k || (have > 0 && (!run_d || !run_i)) || !out_d || !out_i ||
        (kb > 0 && (!blk_d || !blk_i)))
        return cudaErrorInvalidValue;
    merge_topk_kernel<<<(unsigned)((Q + 127) / 128), 128, 0, s>>>(run_d, run_i, have, blk_d, blk_i, kb, offset, Q, k,
                                                                  out_d, out_i, out_idx_f);
    return cudaGetLastError();
}

cudaError_t launch_select_cand(const CandSelect& c_in, cudaStream_t s)
{
    if (c_in.Q <= 0) return cudaSuccess;
    CandSelect c = c_in;
    const bool thr = c.thr_out != nullptr;
    // threshold mode: a query stores at most nseg * cap words, often far fewer than the
    // buffer's limit at the coarse seeding levels; a smaller buffer lets more warps run
    if (thr)
        c.buf_words = (int)std::min<int64_t>(kCandThrMax, ((int64_t)c.nseg * c.cap + 31) / 32 * 32);
    else if (c.kp >= 1 && c.kp <= kMaxKpScan)
        c.buf_words = c.buf_words > 0 ? std::min(kCandMax, std::max((c.buf_words + 31) / 32 * 32, pow2_at_least(c.kp)))
                                      : kCandMax;
    if (c.nseg < 1 || c.nseg > kScanMaxSegs || c.cap < 1 ||
        (!thr && (c.kp < 1 || c.kp > kMaxKpScan || c.k > c.kp || c.fail_idx == nullptr || c.fail_cnt == nullptr ||
                  (!c.rerank && c.qn == nullptr))) ||
        (thr && (c.thr_rank < 1 || c.thr_rank > kCandThrMax)))
        return cudaErrorInvalidValue;
    const size_t smem = (size_t)kSelWarps * cand_warp_bytes(c.D, thr, c.rerank != 0, c.buf_words, c.kp) +
                        (size_t)kSelWarps * ((c.D + 3) & ~3) * 4;
    const unsigned blocks = (unsigned)((c.Q + kSelWarps - 1) / kSelWarps);
    cudaError_t e;
    if (thr) {
        e = cudaFuncSetAttribute(select_cand_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        select_cand_kernel<true><<<blocks, kSelWarps * 32, smem, s>>>(c);
    } else {
        e = cudaFuncSetAttribute(select_cand_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        select_cand_kernel<false><<<blocks, kSelWarps * 32, smem, s>>>(c);
    }
    return cudaGetLastError();
}

}  // namespace knn
