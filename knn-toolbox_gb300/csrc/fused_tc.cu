// fused_tc.cu -- tensor-core fused distance + per-query shortlist for sm_103a.
//
// Replaces, for one CTA's 128 queries and one corpus split, the reference's
// distance stage (cublasSgemm in pdist_NT, include/utils.h:957-985, then the
// pdot norm-add pass) and its selection stage (bitonic_shared /
// bitonic_shared2 / relloc, src/cuknnBitonic.cu:45-254): the distance matrix
// stays in tensor memory and only shortlist survivors reach shared memory.
//
// Two precisions share the kernel (template parameter kBF16); both are
// launched and the one that does not match the data returns at once (a
// device flag set by the preparation pass decides, so the host never waits):
//  * BF16-exact data (every corpus and query element equals its BF16
//    rounding, e.g. integer descriptors up to 256): q.c runs as
//    tcgen05.mma.kind::f16 with BF16 operands and FP32 accumulation -- exact
//    products, so the keys are the FP32 keys;
//  * otherwise 3xTF32: with x = hi + lo (hi = tf32(x), lo = tf32(x - hi)),
//    q.c ~= qhi.chi + qhi.clo + qlo.chi, accumulated in FP32 by
//    tcgen05.mma.kind::tf32.  A corpus tile (or the query tile) whose low part
// is all zero skips its correction product: it would add exact zeros, so the
// accumulator is bit-identical either way.  For integer data below 2^11 every
// low part is zero and the products and sums are exact, so the keys equal the
// oracle's bit for bit.
//
// Warp roles (192 threads):
//   warp 0      producer: per tile, the corpus norms (1-D bulk copy into a
//               4-slot ring) and the corpus hi/lo K-chunks (2-D TMA, 128 rows x
//               32 fp32, 128-byte swizzle) into a shared-memory ring;
//   warp 1      TMEM owner + MMA issuer: A (this CTA's queries, hi and lo)
//               sits in TMEM columns [0, 2*dp); two 128-column FP32
//               accumulators at columns 256 and 384 alternate between tiles;
//   warps 2..5  epilogue: thread = query (= TMEM lane); loads its query into
//               TMEM, then per tile reads its 128 dot products (tcgen05.ld,
//               double-buffered), forms key = ||c||^2 - 2 q.c and runs the
//               shortlist filter.
// Every mbarrier wait is bounded; on timeout the kernel records an error
// code in the device error word and winds down without hanging the GPU.
#include <cstdint>
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include "common.cuh"
#include "kernels.h"
#include "tc_ptx.cuh"

namespace knn {

namespace {
constexpr int kTcThreads = 192;
constexpr uint32_t kHalfBytes = kTileN * 128u;     // one operand chunk: 128 rows x 32 fp32 (16 KB)
constexpr uint32_t kStageBytes = 2u * kHalfBytes;  // hi + lo
constexpr int kMaxStages = 4;                      // hi+lo stages (8 hi-only slots)
constexpr int kNormSlots = 4;                      // tiles of corpus norms in flight
constexpr uint32_t kNormBytes = kNormSlots * kTileN * 4u;
constexpr uint32_t kCtrlBytes = 320;               // barriers and flags (284 bytes used)
constexpr int kStagePitch = 33;                    // staged keys: [4 warps][32 lanes][33 floats]
constexpr uint32_t kKeyStageBytes = 4u * 32u * kStagePitch * 4u;
constexpr uint32_t kTmemCols = 512;
constexpr uint32_t kAccCol = 256;
constexpr uint64_t kTimeoutNs = 4000000000ull;  // bound of every barrier wait unless TcArgs names another
constexpr uint32_t kIdesc = ptx::idesc_tf32(kTileQ, kTileN);
constexpr uint32_t kIdescBf16 = ptx::idesc_bf16(kTileQ, kTileN);
constexpr int kBoxElemsBf16 = 64;                  // bf16 elements per 128-byte swizzle row

__device__ __forceinline__ float tf32_rne_dev(float x)
{
    uint32_t u = __float_as_uint(x);
    if ((u & 0x7f800000u) == 0x7f800000u) return x;
    u += 0xfffu + ((u >> 13) & 1u);
    u &= 0xffffe000u;
    return __uint_as_float(u);
}

struct TcSmem {
    unsigned char* ring;      // operand slots, 1024-aligned
    float* norms;             // [kNormSlots][128]
    uint64_t* full;           // [2 * kMaxStages]
    uint64_t* empty;          // [2 * kMaxStages]
    uint64_t* accf;           // [2]
    uint64_t* acce;           // [2]
    uint64_t* nfull;          // [kNormSlots]
    uint64_t* nempty;         // [kNormSlots]
    uint64_t* aready;
    uint64_t* drain;
    uint32_t* tmem_holder;
    volatile int* abort;
    volatile uint32_t* alo_flag;  // 1 when any query of this tile has a nonzero TF32 low part
    volatile uint32_t* stage_lo;  // [2 * kMaxStages] 1 when the slot carries the chunk's low part
    uint64_t* list;
    uint64_t* buf;
    float* keystage;
};

__host__ __device__ inline size_t tc_list_offset(int stages)
{
    return (size_t)stages * kStageBytes + kNormBytes + kCtrlBytes;
}
}  // namespace

size_t tc_smem_bytes(int kp, int stages)
{
    return tc_list_offset(stages) + (size_t)kTileQ * kp * 8 + (size_t)kBufCap * kTileQ * 8 + kKeyStageBytes;
}

int tc_max_stages(int kp)
{
    int best = 0;
    for (int s = 1; s <= kMaxStages; ++s)
        if (tc_smem_bytes(kp, s) <= 232448) best = s;
    return best;
}

__device__ __forceinline__ void tc_fail(const TcArgs& a, const TcSmem& s, int code)
{
    atomicCAS(a.err, 0, code);
    *s.abort = 1;
}

__device__ __forceinline__ uint64_t tc_timeout(const TcArgs& a) { return a.timeout_ns ? a.timeout_ns : kTimeoutNs; }

__device__ __forceinline__ bool tc_wait(const TcArgs& a, const TcSmem& s, uint64_t* bar, uint32_t parity, int code)
{
    // a completed barrier returns before the abort flag is read; a wait that would block sees it first
    if (ptx::mbar_try_wait(bar, parity)) return true;
    if (*s.abort) return false;
    if (ptx::mbar_wait(bar, parity, tc_timeout(a))) return true;
    tc_fail(a, s, code);
    return false;
}

// key = ||c||^2 - 2 q.c for 32 columns (norms from shared memory)
__device__ __forceinline__ void tc_keys(const float (&vals)[32], const float* nrm, float (&key)[32])
{
    const float4* n4 = reinterpret_cast<const float4*>(nrm);
#pragma unroll
    for (int u = 0; u < 8; ++u) {
        const float4 c4 = n4[u];
        key[4 * u + 0] = __fmaf_rn(-2.0f, vals[4 * u + 0], c4.x);
        key[4 * u + 1] = __fmaf_rn(-2.0f, vals[4 * u + 1], c4.y);
        key[4 * u + 2] = __fmaf_rn(-2.0f, vals[4 * u + 2], c4.z);
        key[4 * u + 3] = __fmaf_rn(-2.0f, vals[4 * u + 3], c4.w);
    }
}

// One 32-column chunk: keys, their minimum and one vote; when some lane of the
// warp has a candidate below its threshold, the keys are staged in this lane's
// shared-memory row and the full filter runs out of line.  No TMEM load may be
// outstanding when the slow path is entered.
__device__ __forceinline__ bool tc_chunk_hot(const float (&vals)[32], const float* nrm, float thr, float (&key)[32])
{
    tc_keys(vals, nrm, key);
    return __any_sync(0xffffffffu, min32(key) < thr);
}

__device__ __forceinline__ void stage_keys(float* srow, const float (&key)[32])
{
#pragma unroll
    for (int j = 0; j < 32; ++j) srow[j] = key[j];
}

template <bool kBF16>
__global__ void __launch_bounds__(kTcThreads, 1) tc_kernel(const __grid_constant__ TcArgs a)
{
    extern __shared__ __align__(1024) unsigned char sm[];
    // redo pass: only flagged query tiles run
    if (a.tile_redo != nullptr && a.tile_redo[blockIdx.x] == 0u) return;
    // compacted-query mode: rows past the listed queries accept nothing; empty tiles return
    int64_t qvalid = a.Q;
    if (a.qcount != nullptr) {
        qvalid = min(a.Q, (int64_t)*a.qcount - a.qbase);
        if ((int64_t)blockIdx.x * kTileQ >= qvalid) return;
    }
    // only the variant that matches the data runs
    if (a.not_exact != nullptr) {
        if ((*a.not_exact != 0u) == kBF16) return;
    } else if (kBF16) {
        return;
    }
    // The operand ring needs 1024-byte alignment (128-byte swizzle atoms).
    // The dynamic shared-memory window starts 1024-aligned; refuse to run otherwise.
    if ((ptx::smem_u32(sm) & 1023u) != 0u) {
        if (threadIdx.x == 0) atomicCAS(a.err, 0, kDevMisaligned);
        return;
    }

    const int stages = a.stages;
    // Ring layout (TF32): with a low part anywhere in the corpus, `stages`
    // slots of hi+lo; otherwise twice as many hi-only slots (deeper prefetch).
    // Ring layout (BF16): slots of whole tiles (all K boxes, one commit per
    // tile) when two fit, else one box per slot.
    const int nbox_bf = a.dpb / kBoxElemsBf16;
    const int bps = (2 * nbox_bf * (int)kHalfBytes <= stages * (int)kStageBytes) ? nbox_bf : 1;
    const bool ring_lo = !kBF16 && (a.corpus_any_lo == nullptr || *a.corpus_any_lo != 0u);
    const uint32_t slot_bytes = kBF16 ? (uint32_t)bps * kHalfBytes : (ring_lo ? kStageBytes : kHalfBytes);
    const int nslot = (int)min((uint32_t)(2 * kMaxStages), (uint32_t)(stages * kStageBytes) / slot_bytes);

    TcSmem s;
    s.ring = sm;
    s.norms = reinterpret_cast<float*>(sm + (size_t)stages * kStageBytes);
    uint64_t* bars = reinterpret_cast<uint64_t*>(sm + (size_t)stages * kStageBytes + kNormBytes);
    s.full = bars;
    s.empty = bars + 2 * kMaxStages;
    s.accf = bars + 4 * kMaxStages;
    s.acce = s.accf + 2;
    s.nfull = s.acce + 2;
    s.nempty = s.nfull + kNormSlots;
    s.aready = s.nempty + kNormSlots;
    s.drain = s.aready + 1;
    uint32_t* words = reinterpret_cast<uint32_t*>(s.drain + 1);
    s.tmem_holder = words;
    s.abort = reinterpret_cast<volatile int*>(words + 1);
    s.alo_flag = words + 2;
    s.stage_lo = words + 3;
    s.list = reinterpret_cast<uint64_t*>(sm + tc_list_offset(stages));
    s.buf = s.list + (size_t)kTileQ * a.kp;
    s.keystage = reinterpret_cast<float*>(s.buf + (size_t)kBufCap * kTileQ);

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int64_t q0 = (int64_t)blockIdx.x * kTileQ;
    const int64_t n_begin = (int64_t)blockIdx.y * a.split_len;
    const int64_t n_end = min(a.N, n_begin + a.split_len);
    const int ntiles = (int)((n_end - n_begin + kTileN - 1) / kTileN);
    // K steps: TF32 chunks of 32 elements per 128-byte row; BF16 groups of `bps` boxes of 64
    const int nchunks = kBF16 ? nbox_bf / bps : a.dp / kChunkK;

    if (tid == 0) {
        for (int i = 0; i < nslot; ++i) {
            ptx::mbar_init(&s.full[i], 1);
            ptx::mbar_init(&s.empty[i], 1);
        }
        for (int b = 0; b < 2; ++b) {
            ptx::mbar_init(&s.accf[b], 1);
            ptx::mbar_init(&s.acce[b], 4);
        }
        for (int b = 0; b < kNormSlots; ++b) {
            ptx::mbar_init(&s.nfull[b], 1);
            ptx::mbar_init(&s.nempty[b], 4);
        }
        ptx::mbar_init(s.aready, 4 * 32);
        ptx::mbar_init(s.drain, 1);
        *s.abort = 0;
        *s.alo_flag = 0;
        ptx::fence_mbar_init();
        if (kBF16) {
            ptx::tma_prefetch_desc(&a.tm_bf);
        } else {
            ptx::tma_prefetch_desc(&a.tm_hi);
            ptx::tma_prefetch_desc(&a.tm_lo);
        }
    }
    if (warp == 1) {
        ptx::tmem_alloc(s.tmem_holder, kTmemCols);
        ptx::tmem_relinquish();
    }
    for (int i = tid; i < kTileQ * a.kp; i += kTcThreads) s.list[i] = kSentinel;
    ptx::tc_fence_before();
    __syncthreads();
    ptx::tc_fence_after();
    const uint32_t tmem = *s.tmem_holder;

    if (warp == 0) {
        // ------------------------------------------------------------ producer
        // (test_stall: no copy is ever issued, so the first data wait of the MMA issuer and the
        // epilogue's accumulator wait run out: the bounded-wait wind-down is exercised, with
        // nothing in flight)
        if (lane == 0 && !a.test_stall) {
            int it = 0;
            bool ok = true;
            const int64_t tile0 = n_begin / kTileN;
            for (int t = 0; t < ntiles && ok; ++t) {
                const int64_t n0 = n_begin + (int64_t)t * kTileN;
                // corpus norms of this tile (the array is padded with +inf to a multiple of 128)
                const int ns = t % kNormSlots;
                if (!tc_wait(a, s, &s.nempty[ns], ((uint32_t)(t / kNormSlots) & 1u) ^ 1u, kDevTimeoutProducer)) {
                    ok = false;
                    break;
                }
                ptx::mbar_arrive_expect_tx(&s.nfull[ns], kTileN * 4u);
                ptx::bulk_load(s.norms + ns * kTileN, a.cn + n0, kTileN * 4u, &s.nfull[ns]);
                // corpus tiles whose TF32 low part is zero skip the lo copy and its products
                const uint32_t need_lo = ring_lo ? (a.lo_flags ? __ldg(a.lo_flags + tile0 + t) : 1u) : 0u;
                for (int c = 0; c < nchunks; ++c, ++it) {
                    const int st = it % nslot;
                    const uint32_t ph = (uint32_t)(it / nslot) & 1u;
                    if (!tc_wait(a, s, &s.empty[st], ph ^ 1u, kDevTimeoutProducer)) { ok = false; break; }
                    unsigned char* dst = s.ring + (size_t)st * slot_bytes;
                    if (kBF16) {
                        ptx::mbar_arrive_expect_tx(&s.full[st], slot_bytes);
                        for (int bx = 0; bx < bps; ++bx)
                            ptx::tma_load_2d(dst + bx * kHalfBytes, &a.tm_bf, &s.full[st],
                                             (c * bps + bx) * kBoxElemsBf16, (int)n0);
                    } else {
                        s.stage_lo[st] = need_lo;  // published by the arrive below
                        ptx::mbar_arrive_expect_tx(&s.full[st], need_lo ? kStageBytes : kHalfBytes);
                        ptx::tma_load_2d(dst, &a.tm_hi, &s.full[st], c * kChunkK, (int)n0);
                        if (need_lo)
                            ptx::tma_load_2d(dst + kHalfBytes, &a.tm_lo, &s.full[st], c * kChunkK, (int)n0);
                    }
                }
            }
            if (!ok) {
                // let copies already issued land before the CTA winds down
                const int first = it - nslot > 0 ? it - nslot : 0;
                for (int j = first; j < it; ++j)
                    ptx::mbar_wait(&s.full[j % nslot], (uint32_t)(j / nslot) & 1u, tc_timeout(a));
            }
        }
    } else if (warp == 1) {
        // ------------------------------------------------------------ MMA issuer
        if (lane == 0) {
            bool ok = tc_wait(a, s, s.aready, 0, kDevTimeoutAload);
            ptx::tc_fence_after();
            const uint32_t a_lo = *s.alo_flag;
            int it = 0;
            for (int t = 0; t < ntiles && ok; ++t) {
                const int b = t & 1;
                const uint32_t use = (uint32_t)(t >> 1);
                if (!tc_wait(a, s, &s.acce[b], (use & 1u) ^ 1u, kDevTimeoutMma)) { ok = false; break; }
                ptx::tc_fence_after();
                const uint32_t d_tmem = tmem + kAccCol + (uint32_t)b * kTileN;
                for (int c = 0; c < nchunks; ++c, ++it) {
                    const int st = it % nslot;
                    const uint32_t ph = (uint32_t)(it / nslot) & 1u;
                    if (!tc_wait(a, s, &s.full[st], ph, kDevTimeoutMma)) { ok = false; break; }
                    ptx::tc_fence_after();
                    const uint32_t hi_addr = ptx::smem_u32(s.ring + (size_t)st * slot_bytes);
                    if (kBF16) {
                        // bps boxes of 64 bf16 (128-byte rows); K = 16 per instruction
                        for (int bx = 0; bx < bps; ++bx) {
                            const uint32_t box = (uint32_t)(c * bps + bx);
#pragma unroll
                            for (int kk = 0; kk < 4; ++kk) {
                                const uint64_t db = ptx::desc_sw128_kmajor(hi_addr + bx * kHalfBytes + kk * 32);
                                const uint32_t acol = tmem + box * 32u + (uint32_t)(kk * 8);
                                ptx::mma_bf16_ts(d_tmem, acol, db, kIdescBf16, (c | bx | kk) != 0);
                            }
                        }
                    } else {
                        const uint32_t b_lo = s.stage_lo[st];
                        const uint32_t lo_addr = hi_addr + kHalfBytes;
#pragma unroll
                        for (int kk = 0; kk < kChunkK / 8; ++kk) {
                            const uint64_t dh = ptx::desc_sw128_kmajor(hi_addr + kk * 32);
                            const uint32_t ahi = tmem + (uint32_t)(c * kChunkK + kk * 8);
                            const uint32_t alo = ahi + (uint32_t)a.dp;
                            // an all-zero low part contributes exact zeros: skipping it leaves
                            // the FP32 accumulator bit-identical
                            ptx::mma_tf32_ts(d_tmem, ahi, dh, kIdesc, (c | kk) != 0);
                            if (b_lo)
                                ptx::mma_tf32_ts(d_tmem, ahi, ptx::desc_sw128_kmajor(lo_addr + kk * 32), kIdesc, 1u);
                            if (a_lo) ptx::mma_tf32_ts(d_tmem, alo, dh, kIdesc, 1u);
                        }
                    }
                    // after the tile's last MMAs the accumulator-ready commit goes first
                    if (c == nchunks - 1) ptx::mma_commit(&s.accf[b]);
                    ptx::mma_commit(&s.empty[st]);
                }
                if (!ok) break;
            }
            // all MMAs issued by this thread retire before TMEM is released
            ptx::mma_commit(s.drain);
            ptx::mbar_wait(s.drain, 0, tc_timeout(a));
        }
    } else {
        // ------------------------------------------------------------ epilogue
        const int quad = warp & 3;
        const int row = quad * 32 + lane;
        const int64_t q = q0 + row;
        const uint32_t lane_base = (uint32_t)(quad * 32) << 16;
        ShortlistView v;
        v.list = s.list;
        v.buf = s.buf;
        v.kp = a.kp;
        v.kp_pitch = a.kp;
        v.buf_pitch = kTileQ;
        float* srow = s.keystage + ((warp - 2) * 32 + lane) * kStagePitch;

        // A operand: this thread's query row into TMEM (BF16 pairs, or TF32 hi/lo)
        const bool qok = q < qvalid;
        const int64_t qsrc = !qok ? 0 : (a.qmap != nullptr ? (int64_t)a.qmap[a.qbase + q] : q);
        const float* qrow = a.queries + qsrc * a.ldq;
        uint32_t any_lo = 0;
        if (kBF16) {
            for (int bx = 0; bx < nbox_bf; ++bx) {
                float packed[32];
#pragma unroll
                for (int u = 0; u < 32; ++u) {
                    const int d0 = bx * kBoxElemsBf16 + 2 * u;
                    const float x0 = (qok && d0 < a.D) ? __ldg(qrow + d0) : 0.f;
                    const float x1 = (qok && d0 + 1 < a.D) ? __ldg(qrow + d0 + 1) : 0.f;
                    // lower K index in the low half of the 32-bit column
                    const uint32_t lo16 = (uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(x0));
                    const uint32_t hi16 = (uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(x1));
                    packed[u] = __uint_as_float(lo16 | (hi16 << 16));
                }
                __syncwarp();
                ptx::tmem_st32(tmem + lane_base + (uint32_t)(bx * 32), packed);
            }
        }
        for (int c = 0; c < (kBF16 ? 0 : nchunks); ++c) {
            float hi[32], lo[32];
#pragma unroll
            for (int u = 0; u < 32; ++u) {
                const int d = c * kChunkK + u;
                const float x = (qok && d < a.D) ? __ldg(qrow + d) : 0.f;
                hi[u] = tf32_rne_dev(x);
                lo[u] = tf32_rne_dev(__fsub_rn(x, hi[u]));
                any_lo |= (lo[u] != 0.f) ? 1u : 0u;
            }
            __syncwarp();
            ptx::tmem_st32(tmem + lane_base + (uint32_t)(c * kChunkK), hi);
            ptx::tmem_st32(tmem + lane_base + (uint32_t)(a.dp + c * kChunkK), lo);
        }
        ptx::tmem_wait_st();
        if (any_lo) atomicOr(const_cast<uint32_t*>(s.alo_flag), 1u);
        ptx::tc_fence_before();
        ptx::mbar_arrive(s.aready);

        // padding rows of the last query tile accept nothing
        LaneState st{0, qok ? __int_as_float(0x7f800000) : -__int_as_float(0x7f800000)};
        uint32_t* thr_g = qok ? a.thr_g : nullptr;
        uint32_t g_pending = thr_g ? __ldcg(thr_g + q) : 0xFFFFFFFFu;
        const bool dump = a.dump != nullptr && blockIdx.x == 0 && blockIdx.y == 0;
        for (int t = 0; t < ntiles; ++t) {
            const int b = t & 1;
            const uint32_t use = (uint32_t)(t >> 1);
            const int ns = t % kNormSlots;
            // warp-uniform outcome: tcgen05.ld below is warp-collective
            const bool ok = tc_wait(a, s, &s.accf[b], use & 1u, kDevTimeoutEpilogue) &&
                            tc_wait(a, s, &s.nfull[ns], (uint32_t)(t / kNormSlots) & 1u, kDevTimeoutEpilogue);
            if (!__all_sync(0xffffffffu, ok)) break;
            ptx::tc_fence_after();
            // shared threshold loaded one tile ago; fetch the next one now
            const float thr_glob = shared_thr_of(g_pending);
            if (thr_g) g_pending = __ldcg(thr_g + q);
            float thr = fminf(st.thr_local, thr_glob);
            const uint32_t nb = (uint32_t)(n_begin + (int64_t)t * kTileN);
            const float* nrm = s.norms + ns * kTileN;
            const uint32_t tb = tmem + kAccCol + (uint32_t)b * kTileN + lane_base;
            // four 32-column chunks; the next chunk's TMEM load overlaps this chunk's test
            float va[32], vb[32];
            __syncwarp();
            ptx::tmem_ld32(tb, va);
            ptx::tmem_wait_ld_regs(va);
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int c0 = 2 * h, c1 = 2 * h + 1;
                float key[32];
                __syncwarp();
                ptx::tmem_ld32(tb + (uint32_t)(32 * c1), vb);
                if (dump && t == 0) {
#pragma unroll
                    for (int u = 0; u < 32; ++u) a.dump[row * kTileN + 32 * c0 + u] = va[u];
                }
                if (tc_chunk_hot(va, nrm + 32 * c0, thr, key)) {
                    ptx::tmem_wait_ld_regs(vb);
                    stage_keys(srow, key);
                    st = offer_staged(v, srow, nb + 32 * c0, row, st, thr_glob, thr_g, q);
                    thr = fminf(st.thr_local, thr_glob);
                }
                ptx::tmem_wait_ld_regs(vb);
                if (h == 0) {
                    __syncwarp();
                    ptx::tmem_ld32(tb + (uint32_t)(32 * (c1 + 1)), va);
                }
                if (dump && t == 0) {
#pragma unroll
                    for (int u = 0; u < 32; ++u) a.dump[row * kTileN + 32 * c1 + u] = vb[u];
                }
                if (tc_chunk_hot(vb, nrm + 32 * c1, thr, key)) {
                    if (h == 0) ptx::tmem_wait_ld_regs(va);
                    stage_keys(srow, key);
                    st = offer_staged(v, srow, nb + 32 * c1, row, st, thr_glob, thr_g, q);
                    thr = fminf(st.thr_local, thr_glob);
                }
                if (h == 0) ptx::tmem_wait_ld_regs(va);
            }
            // accumulator b and norms slot ns fully consumed
            ptx::tc_fence_before();
            __syncwarp();
            if (lane == 0) {
                ptx::mbar_arrive(&s.acce[b]);
                ptx::mbar_arrive(&s.nempty[ns]);
            }
        }
        st = flush_all(v, row, st);
    }

    ptx::tc_fence_before();
    __syncthreads();
    ptx::tc_fence_after();
    if (warp == 1) {
        __syncwarp();
        ptx::tmem_dealloc(tmem, kTmemCols);
    }

    const int64_t nq = min((int64_t)kTileQ, qvalid - q0);
    uint64_t* out = a.part + ((size_t)blockIdx.y * a.Q + q0) * a.kp;
    for (int64_t i = tid; i < nq * a.kp; i += kTcThreads) out[i] = s.list[i];
}

cudaError_t launch_tc(const TcArgs& a, int splits, bool bf16, cudaStream_t st)
{
    if (a.stages < 1 || a.stages > kMaxStages || a.dp % kChunkK != 0 || a.kp % 16 != 0 ||
        a.dpb % kBoxElemsBf16 != 0 || a.dpb / 2 > kMaxDpTC || (!bf16 && a.dp > kMaxDpTC))
        return cudaErrorInvalidValue;
    const size_t smem = tc_smem_bytes(a.kp, a.stages);
    dim3 grid((unsigned)((a.Q + kTileQ - 1) / kTileQ), (unsigned)splits);
    cudaError_t e;
    if (bf16) {
        e = cudaFuncSetAttribute(tc_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        tc_kernel<true><<<grid, kTcThreads, smem, st>>>(a);
    } else {
        e = cudaFuncSetAttribute(tc_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        tc_kernel<false><<<grid, kTcThreads, smem, st>>>(a);
    }
    return cudaGetLastError();
}

}  // namespace knn
