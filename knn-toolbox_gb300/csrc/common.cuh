// common.cuh -- shared device helpers for the GB300 brute-force kNN engine.
//
// Ranking keys are carried as one 64-bit word: the high 32 bits are the float
// key mapped to an order-preserving unsigned integer, the low 32 bits are the
// global corpus index.  Comparing two words as unsigned integers therefore
// orders candidates by (key, index), i.e. ties go to the lower index, the rule
// demo/knn.m:5 gets from MATLAB's stable sort.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace knn {

constexpr uint64_t kSentinel = 0xFFFFFFFFFFFFFFFFull;
constexpr int kWarp = 32;

__device__ __forceinline__ uint32_t f2ord(float f)
{
    uint32_t u = __float_as_uint(f);
    if (u == 0x80000000u) u = 0u;  // -0 sorts with +0
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

__device__ __forceinline__ float ord2f(uint32_t o)
{
    uint32_t u = (o & 0x80000000u) ? (o & 0x7FFFFFFFu) : ~o;
    return __uint_as_float(u);
}

__device__ __forceinline__ uint64_t pack_key(float key, uint32_t idx)
{
    return ((uint64_t)f2ord(key) << 32) | (uint64_t)idx;
}

__device__ __forceinline__ float unpack_key(uint64_t w) { return ord2f((uint32_t)(w >> 32)); }
__device__ __forceinline__ uint32_t unpack_idx(uint64_t w) { return (uint32_t)(w & 0xFFFFFFFFull); }

// Threshold implied by the last kept list entry (+inf while the list is not full).
__device__ __forceinline__ float thr_of(uint64_t last)
{
    return last == kSentinel ? __int_as_float(0x7f800000) : unpack_key(last);
}

// ---------------------------------------------------------------------------
// Exact distance convention for the re-rank (bit-identical to the oracle):
// eight float partial sums over d mod 8 of t*t, t = q_d - c_d, fmaf.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float exact_dist_row(const float* __restrict__ q,
                                                const float* __restrict__ c, int D)
{
    float p[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    int d = 0;
    for (; d + 8 <= D; d += 8) {
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            float t = __fsub_rn(q[d + u], __ldg(c + d + u));
            p[u] = __fmaf_rn(t, t, p[u]);
        }
    }
    for (; d < D; ++d) {
        float t = __fsub_rn(q[d], __ldg(c + d));
        p[d & 7] = __fmaf_rn(t, t, p[d & 7]);
    }
    return __fadd_rn(__fadd_rn(__fadd_rn(p[0], p[1]), __fadd_rn(p[2], p[3])),
                     __fadd_rn(__fadd_rn(p[4], p[5]), __fadd_rn(p[6], p[7])));
}

// ---------------------------------------------------------------------------
// Warp-level primitives
// ---------------------------------------------------------------------------

// Bitonic sort of one 64-bit word per lane, ascending by lane.
__device__ __forceinline__ uint64_t warp_sort32(uint64_t v)
{
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int size = 2; size <= 32; size <<= 1) {
#pragma unroll
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            uint64_t o = __shfl_xor_sync(0xffffffffu, v, stride);
            bool up = (lane & size) == 0;
            bool lower = (lane & stride) == 0;
            bool keep_min = (lower == up);
            uint64_t mn = o < v ? o : v;
            uint64_t mx = o < v ? v : o;
            v = keep_min ? mn : mx;
        }
    }
    return v;
}

// lower_bound: number of a[0..n) strictly below x (a sorted ascending)
__device__ __forceinline__ int count_less(const uint64_t* a, int n, uint64_t x)
{
    int lo = 0;
    while (n > 0) {
        int half = n >> 1;
        if (a[lo + half] < x) { lo += half + 1; n -= half + 1; }
        else n = half;
    }
    return lo;
}

// upper_bound: number of a[0..n) not above x
__device__ __forceinline__ int count_not_above(const uint64_t* a, int n, uint64_t x)
{
    int lo = 0;
    while (n > 0) {
        int half = n >> 1;
        if (a[lo + half] <= x) { lo += half + 1; n -= half + 1; }
        else n = half;
    }
    return lo;
}

// Candidate buffer layout: slot c of query row ql lives at buf[c * pitch + (ql ^ c)]
// (pitch = rows per CTA, >= 32).  Appends of one warp (equal c, consecutive ql)
// and a merge's read of one query's 32 slots are both free of bank conflicts.
__device__ __forceinline__ int buf_index(int pitch, int c, int ql) { return c * pitch + (ql ^ c); }

// upper_bound over the 32 sorted buffer slots of query row qs
__device__ __forceinline__ int count_not_above_slots(const uint64_t* buf, int pitch, int qs, uint64_t x)
{
    int lo = 0, n = 32;
    while (n > 0) {
        int half = n >> 1;
        if (buf[buf_index(pitch, lo + half, qs)] <= x) { lo += half + 1; n -= half + 1; }
        else n = half;
    }
    return lo;
}

// Merge 32 sorted words (one per lane, ascending by lane) into the sorted list
// L[0..kp) in shared memory, keeping the kp smallest.  The same 32 words sit
// sorted in query row qs's buffer slots (read for the ranks of the list
// entries).  kp is a multiple of 16, at most 512.  Stable: on equal words the
// buffered word goes first (only sentinels can be equal).
__device__ __forceinline__ void warp_merge32(uint64_t* L, int kp, uint64_t b, const uint64_t* buf, int pitch, int qs)
{
    const int lane = threadIdx.x & 31;
    const int pb = lane + count_less(L, kp, b);
    const int nt = (kp + 31) >> 5;
    uint64_t lv[16];
    int lp[16];
#pragma unroll
    for (int t = 0; t < 16; ++t) {
        const int j = lane + (t << 5);
        lp[t] = kp;
        if (t < nt && j < kp) {
            lv[t] = L[j];
            lp[t] = j + count_not_above_slots(buf, pitch, qs, lv[t]);
        }
    }
    __syncwarp();
    if (pb < kp) L[pb] = b;
#pragma unroll
    for (int t = 0; t < 16; ++t)
        if (t < nt && lp[t] < kp) L[lp[t]] = lv[t];
    __syncwarp();
}

// Merge two sorted lists A, B of length kp (shared memory) into out[0..kp)
// (kp smallest), one warp.  out must not alias A or B.  Stable: A first on ties.
__device__ __forceinline__ void warp_merge_lists(const uint64_t* A, const uint64_t* B, uint64_t* out, int kp)
{
    const int lane = threadIdx.x & 31;
    for (int j = lane; j < kp; j += 32) {
        uint64_t a = A[j];
        int pa = j + count_less(B, kp, a);
        if (pa < kp) out[pa] = a;
        uint64_t bb = B[j];
        int pbb = j + count_not_above(A, kp, bb);
        if (pbb < kp) out[pbb] = bb;
    }
    __syncwarp();
}

// Bitonic sort of n (power of two, <= 1024) words in shared memory by one warp.
__device__ __forceinline__ void warp_sort_smem(uint64_t* a, int n)
{
    const int lane = threadIdx.x & 31;
    for (int size = 2; size <= n; size <<= 1) {
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            for (int i = lane; i < (n >> 1); i += 32) {
                int lo = 2 * i - (i & (stride - 1));
                int hi = lo + stride;
                bool up = (lo & size) == 0;
                uint64_t x = a[lo], y = a[hi];
                if ((x > y) == up) { a[lo] = y; a[hi] = x; }
            }
            __syncwarp();
        }
    }
}

// ---------------------------------------------------------------------------
// Per-query candidate filter with a shared-memory shortlist.
//
// Each owner thread holds one query: `thr_local` (the key of the kp-th kept
// entry) and `cnt` (entries waiting in its buffer).  A candidate enters the
// buffer when key < thr_local; candidates are visited in increasing corpus
// index, so a key equal to thr_local can never win its tie and strict < is
// the exact rule.  Buffers of lanes that would overflow are merged into the
// lists warp-cooperatively, 32 candidates at a time.
// ---------------------------------------------------------------------------
constexpr int kBufCap = 32;   // buffered candidates per query

struct ShortlistView {
    uint64_t* list;     // [nq][kp_pitch]
    uint64_t* buf;      // [kBufCap][buf_pitch], slots swizzled (buf_index)
    int kp;
    int kp_pitch;
    int buf_pitch;      // nq (>= 32)
};

// Per-lane filter state: entries waiting in the buffer and the key of the kp-th
// kept entry.  Passed by value so that it stays in registers across calls.
struct LaneState {
    int cnt;
    float thr_local;
};

// Merge the buffers of every lane in `mask`; lane `ql` is the query row of this lane.
__device__ __forceinline__ LaneState flush_lanes(const ShortlistView& v, unsigned mask, int ql, LaneState st)
{
    const int lane = threadIdx.x & 31;
    while (mask) {
        const int src = __ffs(mask) - 1;
        mask &= mask - 1;
        const int c = __shfl_sync(0xffffffffu, st.cnt, src);
        const int qs = __shfl_sync(0xffffffffu, ql, src);
        uint64_t* slot = v.buf + buf_index(v.buf_pitch, lane, qs);
        uint64_t b = lane < c ? *slot : kSentinel;
        b = warp_sort32(b);
        *slot = b;  // query qs's slots now hold the sorted words
        __syncwarp();
        uint64_t* L = v.list + (size_t)qs * v.kp_pitch;
        warp_merge32(L, v.kp, b, v.buf, v.buf_pitch, qs);
        if (lane == src) {
            st.cnt = 0;
            st.thr_local = thr_of(L[v.kp - 1]);
        }
    }
    __syncwarp();
    return st;
}

// Merge every non-empty buffer of the warp (end of a split).
static __device__ __noinline__ LaneState flush_all(ShortlistView v, int ql, LaneState st)
{
    unsigned m = __ballot_sync(0xffffffffu, st.cnt > 0);
    if (m) st = flush_lanes(v, m, ql, st);
    return st;
}

// Threshold shared by every CTA working on one query (other corpus splits):
// the order-mapped key of some split's full kp-th entry, kept with atomicMin.
// Any such value bounds the final kp-th key from above, so candidates with a
// larger key can be dropped; equal keys are kept (their index may still win).
__device__ __forceinline__ float shared_thr_of(uint32_t g)
{
    if (g >= 0xFF800000u) return __int_as_float(0x7f800000);  // unset (or +inf)
    return ord2f(g + 1u);                                       // next float above the bound
}

__device__ __forceinline__ void publish_thr(uint32_t* thr_g, int64_t q, float thr_local)
{
    if (thr_g != nullptr && thr_local < __int_as_float(0x7f800000)) atomicMin(thr_g + q, f2ord(thr_local));
}

// Offer 32 consecutive candidates of this lane's query: keys[0..31] (shared
// memory, this lane's own row) with corpus indices nbase + j, visited in
// increasing index.  thr_glob is the decoded shared threshold (+inf when
// unused).  Buffers that would overflow are merged first; lanes that merged
// publish their new kp-th key.  Called by the whole warp once some lane has a
// candidate below its threshold; each lane then appends only its own hits.
static __device__ __noinline__ LaneState offer_staged(ShortlistView v, const float* keys, uint32_t nbase, int ql,
                                                      LaneState st, float thr_glob, uint32_t* thr_g, int64_t q)
{
    float thr = fminf(st.thr_local, thr_glob);
    uint32_t m = 0;
#pragma unroll
    for (int j = 0; j < 32; ++j) m |= (keys[j] < thr ? 1u : 0u) << j;
    const bool need = st.cnt + __popc(m) > kBufCap;
    const unsigned fl = __ballot_sync(0xffffffffu, need);
    if (fl) {
        st = flush_lanes(v, fl, ql, st);
        if (need) {
            publish_thr(thr_g, q, st.thr_local);
            thr = fminf(st.thr_local, thr_glob);
            m = 0;
#pragma unroll
            for (int j = 0; j < 32; ++j) m |= (keys[j] < thr ? 1u : 0u) << j;
        }
    }
    while (m) {
        const int j = __ffs(m) - 1;
        m &= m - 1;
        v.buf[buf_index(v.buf_pitch, st.cnt, ql)] = pack_key(keys[j], nbase + (uint32_t)j);
        ++st.cnt;
    }
    __syncwarp();
    return st;
}

// Minimum of 32 keys (fast rejection: no candidate when min >= threshold).
__device__ __forceinline__ float min32(const float (&key)[32])
{
    float m0 = fminf(key[0], key[1]), m1 = fminf(key[2], key[3]), m2 = fminf(key[4], key[5]),
          m3 = fminf(key[6], key[7]);
#pragma unroll
    for (int j = 8; j < 32; j += 4) {
        m0 = fminf(m0, key[j]);
        m1 = fminf(m1, key[j + 1]);
        m2 = fminf(m2, key[j + 2]);
        m3 = fminf(m3, key[j + 3]);
    }
    return fminf(fminf(m0, m1), fminf(m2, m3));
}

}  // namespace knn
