// scan_tf32.cu -- tensor-core 3xTF32 threshold scan for FP32 data of any width and
// shortlists of up to 512 entries.
//
// The exact form's distance stage for the shapes the shortlist kernel
// (fused_tc.cu: queries in tensor memory, D <= 128; shortlists in shared
// memory, <= 128 entries) cannot take: the reference's pdist_NT SGEMM
// (include/utils.h:957-985) followed by its selections (bitonic_shared,
// src/cuknnBitonic.cu:45-254, up to k = 512; the heap of src/cuknnHeap.cu:146-291
// for large k), restructured as the BF16 threshold scan is (scan_bf16.cu): every
// key ||c||^2 - 2 q.c strictly below the query's seeded threshold is appended to
// the query's candidate segment, and select_cand_kernel takes the shortlist from
// the segments and re-ranks it by exact distance.
//
// Keys: with x = hi + lo (hi = tf32(x), lo = tf32(x - hi)), q.c is accumulated in
// FP32 as qhi.chi + qhi.clo + qlo.chi by tcgen05.mma.kind::tf32; a correction
// product whose low part is zero for the whole corpus tile (or query tile) is
// skipped -- it would add exact zeros.
//
// Tile: 128 queries (MMA M, TMEM lanes) x 128 corpus rows (MMA N), K in chunks of
// 32 FP32 columns (one 128-byte swizzle row).  Both operands come from shared
// memory, so any D works and tensor memory holds only accumulators: four of 128
// columns.  A ring slot carries one K chunk of the query tile and of the corpus
// tile, high and low parts (4 x 16 KB).
// Warp roles (608 threads):
//   warp 0      producer: per tile and K chunk the query and corpus boxes (2-D TMA,
//               32 fp32 x 128 rows, 128-byte swizzle), low parts only where present;
//               per tile the corpus norms (1-D bulk copy);
//   warps 1, 18 MMA issuers, into accumulator t mod 4: of the even / odd tiles when a
//               tile takes at most half the ring, else warp 1 alone (see below);
//   warps 2..17 epilogue: thread = query (TMEM lane); warp 2 + 4p + j reads
//               columns [32p, 32p + 32) of lane quarter j, releases the
//               accumulator, forms the keys, appends those below the threshold.
// Every mbarrier wait is bounded; on timeout the kernel records an error code in
// the device error word and winds down without hanging the GPU.
#include <algorithm>
#include <cstdint>
#include <cuda.h>
#include <cuda_runtime.h>
#include "common.cuh"
#include "kernels.h"
#include "scan_common.cuh"
#include "tc_ptx.cuh"

namespace knn {

namespace {
constexpr int kTN = 128;                     // corpus rows per tile
constexpr int kParts = kScanParts;           // epilogue column parts (32 columns each)
constexpr int kEpi = 4 * kParts;             // epilogue warps
constexpr int kIss = 2;                      // MMA issuing threads
constexpr int kThreads = 32 * (1 + kIss + kEpi);
constexpr int kAcc = 4;                      // TMEM accumulators of 128 columns
constexpr int kNorm = 8;                     // tiles of corpus norms in flight
constexpr uint32_t kBox = 128u * 128u;       // one operand box: 128 rows x 32 fp32
constexpr uint32_t kSlot = 4u * kBox;        // query hi, query lo, corpus hi, corpus lo
constexpr int kMaxRing = 3;
constexpr uint32_t kCtrl = 512;
constexpr uint64_t kTimeout = 4000000000ull;
constexpr uint32_t kIdesc = ptx::idesc_tf32(kTileQ, kTN);

struct TSmem {
    unsigned char* ring;
    float* norms;       // [kNorm][kTN]
    uint64_t* full;     // [kMaxRing]
    uint64_t* empty;    // [kMaxRing]
    uint64_t* accf;     // [kAcc]
    uint64_t* acce;     // [kAcc]
    uint64_t* nfull;    // [kNorm]
    uint64_t* nempty;   // [kNorm]
    uint64_t* drain;
    uint32_t* tmem_holder;
    volatile int* abort;
    volatile uint32_t* slot_lo;  // [kMaxRing]: bit 0 query low part loaded, bit 1 corpus low part
};

__device__ __forceinline__ bool t_wait(const TscanArgs& a, const TSmem& s, uint64_t* bar, uint32_t parity, int code)
{
    if (ptx::mbar_try_wait(bar, parity)) return true;
    if (*s.abort) return false;
    if (ptx::mbar_wait(bar, parity, kTimeout)) return true;
    atomicCAS(a.err, 0, code);
    *s.abort = 1;
    return false;
}

__global__ void __launch_bounds__(kThreads, 1) tscan_kernel(const __grid_constant__ TscanArgs a)
{
    extern __shared__ __align__(1024) unsigned char sm[];
    // device-side path choice: the kernel runs only when *run_if != 0
    if (a.run_if != nullptr && *a.run_if == 0u) return;
    if ((ptx::smem_u32(sm) & 1023u) != 0u) {
        if (threadIdx.x == 0) atomicCAS(a.err, 0, kDevMisaligned);
        return;
    }
    const int R = a.ring;
    TSmem s;
    s.ring = sm;
    s.norms = reinterpret_cast<float*>(sm + (size_t)R * kSlot);
    uint64_t* bars = reinterpret_cast<uint64_t*>(s.norms + kNorm * kTN);
    s.full = bars;
    s.empty = bars + kMaxRing;
    s.accf = bars + 2 * kMaxRing;
    s.acce = s.accf + kAcc;
    s.nfull = s.acce + kAcc;
    s.nempty = s.nfull + kNorm;
    s.drain = s.nempty + kNorm;
    uint32_t* words = reinterpret_cast<uint32_t*>(s.drain + 1);
    s.tmem_holder = words;
    s.abort = reinterpret_cast<volatile int*>(words + 1);
    s.slot_lo = words + 2;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int64_t q0 = (int64_t)blockIdx.x * kTileQ;
    const int split = a.split0 + (int)blockIdx.y;
    const int64_t n_begin = (int64_t)split * a.split_len;
    const int64_t n_end = min(a.N, n_begin + a.split_len);
    const int ntiles = n_end > n_begin ? (int)((n_end - n_begin + kTN - 1) / kTN) : 0;
    const int nch = a.dp / 32;

    if (tid == 0) {
        for (int i = 0; i < R; ++i) {
            ptx::mbar_init(&s.full[i], 1);
            ptx::mbar_init(&s.empty[i], 1);
        }
        for (int b = 0; b < kAcc; ++b) {
            ptx::mbar_init(&s.accf[b], 1);
            ptx::mbar_init(&s.acce[b], kEpi);
        }
        for (int b = 0; b < kNorm; ++b) {
            ptx::mbar_init(&s.nfull[b], 1);
            ptx::mbar_init(&s.nempty[b], kEpi);
        }
        ptx::mbar_init(s.drain, kIss);
        *s.abort = 0;
        ptx::fence_mbar_init();
        ptx::tma_prefetch_desc(&a.tm_qhi);
        ptx::tma_prefetch_desc(&a.tm_qlo);
        ptx::tma_prefetch_desc(&a.tm_chi);
        ptx::tma_prefetch_desc(&a.tm_clo);
    }
    if (warp == 1) {
        ptx::tmem_alloc(s.tmem_holder, 512);
        ptx::tmem_relinquish();
    }
    ptx::tc_fence_before();
    __syncthreads();
    ptx::tc_fence_after();
    const uint32_t tmem = *s.tmem_holder;

    if (warp == 0) {
        // ------------------------------------------------------------ producer
        if (lane == 0) {
            const uint32_t qlo = a.qlo_flags ? __ldg(a.qlo_flags + blockIdx.x) : 1u;
            int it = 0;
            bool ok = true;
            for (int t = 0; t < ntiles && ok; ++t) {
                const int64_t n0 = n_begin + (int64_t)t * kTN;
                // view rows are whole 128-row tiles of the flags' corpus (main pass: split_len % 128 == 0)
                const uint32_t clo = a.clo_flags ? __ldg(a.clo_flags + n0 / kTN) : 1u;
                for (int c = 0; c < nch; ++c, ++it) {
                    const int st = it % R;
                    const uint32_t ph = (uint32_t)(it / R) & 1u;
                    if (!t_wait(a, s, &s.empty[st], ph ^ 1u, kDevTimeoutProducer)) { ok = false; break; }
                    unsigned char* dst = s.ring + (size_t)st * kSlot;
                    s.slot_lo[st] = (qlo ? 1u : 0u) | (clo ? 2u : 0u);  // published by the arrive below
                    ptx::mbar_arrive_expect_tx(&s.full[st], kBox * (2u + (qlo ? 1u : 0u) + (clo ? 1u : 0u)));
                    ptx::tma_load_2d(dst, &a.tm_qhi, &s.full[st], c * 32, (int)q0);
                    if (qlo) ptx::tma_load_2d(dst + kBox, &a.tm_qlo, &s.full[st], c * 32, (int)q0);
                    ptx::tma_load_2d(dst + 2 * kBox, &a.tm_chi, &s.full[st], c * 32, (int)n0);
                    if (clo) ptx::tma_load_2d(dst + 3 * kBox, &a.tm_clo, &s.full[st], c * 32, (int)n0);
                }
                if (!ok) break;
                const int ns = t % kNorm;
                if (!t_wait(a, s, &s.nempty[ns], ((uint32_t)(t / kNorm) & 1u) ^ 1u, kDevTimeoutProducer)) {
                    ok = false;
                    break;
                }
                // the norms are padded with +inf at least one tile past the view
                ptx::mbar_arrive_expect_tx(&s.nfull[ns], kTN * 4u);
                ptx::bulk_load(s.norms + ns * kTN, a.cn + n0, kTN * 4u, &s.nfull[ns]);
            }
            if (!ok) {
                // let copies already issued land before the CTA winds down
                const int first = it - R > 0 ? it - R : 0;
                for (int j = first; j < it; ++j) ptx::mbar_wait(&s.full[j % R], (uint32_t)(j / R) & 1u, kTimeout);
            }
        }
    } else if (warp == 1 || warp == 2 + kEpi) {
        // ------------------------------------------------------------ MMA issuers
        // Two issuers alternate tiles only when a tile's chunks fill at most half the ring: an
        // issuer's wait on a slot must never run two phases ahead of the slot's barrier, which
        // is guaranteed when the slot's previous use (R chunks back) is one of its own chunks
        // (or none).  With longer tiles a second issuer could wait on a slot whose previous
        // use, in the other issuer's tile, has not landed yet -- its parity would then read
        // as complete -- so warp 1 issues every tile in order and warp 18 only drains.
        const int nissue = 2 * nch <= R ? kIss : 1;
        if (lane == 0) {
            const int iss = warp == 1 ? 0 : 1;
            bool ok = true;
            for (int t = iss; t < ntiles && ok && iss < nissue; t += nissue) {
                const int b = t % kAcc;
                const uint32_t use = (uint32_t)(t / kAcc);
                if (!t_wait(a, s, &s.acce[b], (use & 1u) ^ 1u, kDevTimeoutMma)) { ok = false; break; }
                ptx::tc_fence_after();
                const uint32_t d_tmem = tmem + (uint32_t)b * kTN;
                int it = t * nch;
                for (int c = 0; c < nch; ++c, ++it) {
                    const int st = it % R;
                    const uint32_t ph = (uint32_t)(it / R) & 1u;
                    if (!t_wait(a, s, &s.full[st], ph, kDevTimeoutMma)) { ok = false; break; }
                    ptx::tc_fence_after();
                    const uint32_t lo = s.slot_lo[st];
                    const uint32_t base = ptx::smem_u32(s.ring + (size_t)st * kSlot);
#pragma unroll
                    for (int kk = 0; kk < 4; ++kk) {
                        // K steps of 8 fp32 (32 bytes) within the 128-byte swizzle rows
                        const uint64_t qh = ptx::desc_sw128_kmajor(base + kk * 32);
                        const uint64_t ch = ptx::desc_sw128_kmajor(base + 2 * kBox + kk * 32);
                        ptx::mma_tf32_ss(d_tmem, qh, ch, kIdesc, (c | kk) != 0);
                        if (lo & 2u) ptx::mma_tf32_ss(d_tmem, qh, ptx::desc_sw128_kmajor(base + 3 * kBox + kk * 32), kIdesc, 1u);
                        if (lo & 1u) ptx::mma_tf32_ss(d_tmem, ptx::desc_sw128_kmajor(base + kBox + kk * 32), ch, kIdesc, 1u);
                    }
                    // the tile's last chunk: accumulator-ready first (the epilogue waits on it)
                    if (c == nch - 1) ptx::mma_commit(&s.accf[b]);
                    ptx::mma_commit(&s.empty[st]);
                }
                if (!ok) break;
            }
            // all MMAs issued by this thread retire before TMEM is released
            ptx::mma_commit(s.drain);
            ptx::mbar_wait(s.drain, 0, kTimeout);
        }
    } else {
        // ------------------------------------------------------------ epilogue
        const int ew = warp - 2;
        const int quad = warp & 3;  // TMEM lane quarter this warp may access
        const int part = ew >> 2;   // columns [32 part, 32 part + 32) of every tile
        const int row = quad * 32 + lane;
        const int64_t q = q0 + row;
        const bool valid = q < a.Q;
        const uint32_t lane_base = (uint32_t)(quad * 32) << 16;
        const float T = valid ? (a.thr ? __ldg(a.thr + q) : __int_as_float(0x7f800000)) : -__int_as_float(0x7f800000);
        const size_t seg = (size_t)split * kParts + part;
        uint64_t* out = a.cand + (seg * (size_t)a.Q + (size_t)(valid ? q : 0)) * (size_t)a.cap;
        uint32_t cnt = 0;
        const uint32_t cap = (uint32_t)a.cap;
        for (int t = 0; t < ntiles; ++t) {
            const int b = t % kAcc;
            const uint32_t use = (uint32_t)(t / kAcc);
            const int ns = t % kNorm;
            // warp-uniform outcome: tcgen05.ld below is warp-collective
            const bool ok = t_wait(a, s, &s.accf[b], use & 1u, kDevTimeoutEpilogue) &&
                            t_wait(a, s, &s.nfull[ns], (uint32_t)(t / kNorm) & 1u, kDevTimeoutEpilogue);
            if (!__all_sync(0xffffffffu, ok)) break;
            ptx::tc_fence_after();
            float v[32];
            __syncwarp();
            ptx::tmem_ld32(tmem + (uint32_t)b * kTN + lane_base + (uint32_t)(32 * part), v);
            ptx::tmem_wait_ld_regs(v);
            ptx::tc_fence_before();
            __syncwarp();
            if (lane == 0) ptx::mbar_arrive(&s.acce[b]);
            const float* nrm = s.norms + ns * kTN + 32 * part;
            const uint32_t g = chunk_keys<32, false>(v, nrm, nrm, -2.0f, T, v);
            if (__any_sync(0xffffffffu, g != 0u))
                chunk_append<32>(v, g, T, (uint32_t)(n_begin + (int64_t)t * kTN) + (uint32_t)(32 * part), out, cap, cnt);
            __syncwarp();
            if (lane == 0) ptx::mbar_arrive(&s.nempty[ns]);
        }
        if (valid) a.cnt[seg * (size_t)a.Q + (size_t)q] = cnt;
    }

    ptx::tc_fence_before();
    __syncthreads();
    ptx::tc_fence_after();
    if (warp == 1) {
        __syncwarp();
        ptx::tmem_dealloc(tmem, 512);
    }
}

// ---------------------------------------------------------------- queries in tensor memory
// Rows of at most 128 columns: the query tile's TF32 hi and lo parts sit in tensor memory (A
// from TMEM, tcgen05.mma kind::tf32 [d], [a], b-desc), so the ring carries only corpus chunks
// (high and low parts, 2 x 16 KB per slot) and each MMA reads one operand from shared memory:
// with both operands there, the MMA reads and the TMA fills together exceed the shared-memory
// bandwidth.  Tensor memory: A hi [0, dp), A lo [dp, 2 dp), two 128-column accumulators at
// 256 and 384.  Two MMA issuers, warps 1 and 18, take the even and the odd tiles, one
// accumulator each: the tensor pipe queues little work beyond the MMA being issued, so one
// thread's barrier waits and commits idle it.  A slot wait must not read an older phase of
// the slot's barrier as complete.  An issuer waits for tile t's accumulator before its slots,
// after which the epilogue has consumed tile t - 2: every use of the ring up to tile t - 2
// has landed and been released.  With at most as many chunks per tile as ring slots (4 and
// 6), a slot's use two rounds back lies in tile t - 2 or earlier, so it is released.  If the
// slot's previous use was one of this issuer's own, it waited for that fill; if it was the
// other issuer's, the issuer first waits for that use's release (which follows its fill) and
// only then for the slot's next fill.  The release wait costs nothing: the producer waits for
// it before refilling the slot.  Keys, epilogue and segments are those of tscan_kernel, so
// the candidates are the same.
constexpr int kAccTA = 2;
constexpr uint32_t kAccColTA = 256;
constexpr uint32_t kSlotTA = 2u * kBox;  // corpus hi, corpus lo
constexpr int kMaxRingTA = 6;

struct TaSmem {
    unsigned char* ring;
    float* norms;       // [kNorm][kTN]
    uint64_t* full;     // [kMaxRingTA]
    uint64_t* empty;    // [kMaxRingTA]
    uint64_t* accf;     // [kAccTA]
    uint64_t* acce;     // [kAccTA]
    uint64_t* nfull;    // [kNorm]
    uint64_t* nempty;   // [kNorm]
    uint64_t* aready;
    uint64_t* drain;
    uint32_t* tmem_holder;
    volatile int* abort;
    volatile uint32_t* slot_lo;  // [kMaxRingTA]: 1 when the slot's corpus low part was loaded
    uint32_t* alo;               // 1 when some query of the tile has a low part
};

__device__ __forceinline__ bool ta_wait(const TscanArgs& a, const TaSmem& s, uint64_t* bar, uint32_t parity, int code)
{
    if (ptx::mbar_try_wait(bar, parity)) return true;
    if (*s.abort) return false;
    if (ptx::mbar_wait(bar, parity, kTimeout)) return true;
    atomicCAS(a.err, 0, code);
    *s.abort = 1;
    return false;
}

__device__ __forceinline__ float tf32_round(float x)
{
    uint32_t u = __float_as_uint(x);
    if ((u & 0x7f800000u) == 0x7f800000u) return x;
    u += 0xfffu + ((u >> 13) & 1u);
    u &= 0xffffe000u;
    return __uint_as_float(u);
}

__global__ void __launch_bounds__(kThreads, 1) tscan_ta_kernel(const __grid_constant__ TscanArgs a)
{
    extern __shared__ __align__(1024) unsigned char sm[];
    // device-side path choice: the kernel runs only when *run_if != 0
    if (a.run_if != nullptr && *a.run_if == 0u) return;
    if ((ptx::smem_u32(sm) & 1023u) != 0u) {
        if (threadIdx.x == 0) atomicCAS(a.err, 0, kDevMisaligned);
        return;
    }
    const int R = a.ring;
    TaSmem s;
    s.ring = sm;
    s.norms = reinterpret_cast<float*>(sm + (size_t)R * kSlotTA);
    uint64_t* bars = reinterpret_cast<uint64_t*>(s.norms + kNorm * kTN);
    s.full = bars;
    s.empty = bars + kMaxRingTA;
    s.accf = bars + 2 * kMaxRingTA;
    s.acce = s.accf + kAccTA;
    s.nfull = s.acce + kAccTA;
    s.nempty = s.nfull + kNorm;
    s.aready = s.nempty + kNorm;
    s.drain = s.aready + 1;
    uint32_t* words = reinterpret_cast<uint32_t*>(s.drain + 1);
    s.tmem_holder = words;
    s.abort = reinterpret_cast<volatile int*>(words + 1);
    s.alo = words + 2;
    s.slot_lo = words + 3;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int64_t q0 = (int64_t)blockIdx.x * kTileQ;
    const int split = a.split0 + (int)blockIdx.y;
    const int64_t n_begin = (int64_t)split * a.split_len;
    const int64_t n_end = min(a.N, n_begin + a.split_len);
    const int ntiles = n_end > n_begin ? (int)((n_end - n_begin + kTN - 1) / kTN) : 0;
    const int nch = a.dp / 32;
    const int niss = nch <= R ? 2 : 1;  // MMA issuers (see above; the launcher keeps nch <= R)

    if (tid == 0) {
        for (int i = 0; i < R; ++i) {
            ptx::mbar_init(&s.full[i], 1);
            ptx::mbar_init(&s.empty[i], 1);
        }
        for (int b = 0; b < kAccTA; ++b) {
            ptx::mbar_init(&s.accf[b], 1);
            ptx::mbar_init(&s.acce[b], kEpi);
        }
        for (int b = 0; b < kNorm; ++b) {
            ptx::mbar_init(&s.nfull[b], 1);
            ptx::mbar_init(&s.nempty[b], kEpi);
        }
        ptx::mbar_init(s.aready, 4);
        ptx::mbar_init(s.drain, niss);
        *s.abort = 0;
        *s.alo = 0;
        ptx::fence_mbar_init();
        ptx::tma_prefetch_desc(&a.tm_chi);
        ptx::tma_prefetch_desc(&a.tm_clo);
    }
    if (warp == 1) {
        ptx::tmem_alloc(s.tmem_holder, 512);
        ptx::tmem_relinquish();
    }
    ptx::tc_fence_before();
    __syncthreads();
    ptx::tc_fence_after();
    const uint32_t tmem = *s.tmem_holder;

    if (warp == 0) {
        // ------------------------------------------------------------ producer
        if (lane == 0) {
            int it = 0;
            bool ok = true;
            for (int t = 0; t < ntiles && ok; ++t) {
                const int64_t n0 = n_begin + (int64_t)t * kTN;
                const uint32_t clo = a.clo_flags ? __ldg(a.clo_flags + n0 / kTN) : 1u;
                for (int c = 0; c < nch; ++c, ++it) {
                    const int st = it % R;
                    const uint32_t ph = (uint32_t)(it / R) & 1u;
                    if (!ta_wait(a, s, &s.empty[st], ph ^ 1u, kDevTimeoutProducer)) { ok = false; break; }
                    unsigned char* dst = s.ring + (size_t)st * kSlotTA;
                    s.slot_lo[st] = clo;  // published by the arrive below
                    ptx::mbar_arrive_expect_tx(&s.full[st], kBox * (clo ? 2u : 1u));
                    ptx::tma_load_2d(dst, &a.tm_chi, &s.full[st], c * 32, (int)n0);
                    if (clo) ptx::tma_load_2d(dst + kBox, &a.tm_clo, &s.full[st], c * 32, (int)n0);
                }
                if (!ok) break;
                const int ns = t % kNorm;
                if (!ta_wait(a, s, &s.nempty[ns], ((uint32_t)(t / kNorm) & 1u) ^ 1u, kDevTimeoutProducer)) {
                    ok = false;
                    break;
                }
                // the norms are padded with +inf at least one tile past the view
                ptx::mbar_arrive_expect_tx(&s.nfull[ns], kTN * 4u);
                ptx::bulk_load(s.norms + ns * kTN, a.cn + n0, kTN * 4u, &s.nfull[ns]);
            }
            if (!ok) {
                // let copies already issued land before the CTA winds down
                const int first = it - R > 0 ? it - R : 0;
                for (int j = first; j < it; ++j) ptx::mbar_wait(&s.full[j % R], (uint32_t)(j / R) & 1u, kTimeout);
            }
        }
    } else if (warp == 1 || (warp == 2 + kEpi && niss == 2)) {
        // ------------------------------------------------------------ MMA issuers
        // issuer i takes the tiles t = i (mod niss); each commit tracks only its own MMAs
        if (lane == 0) {
            const int iss = warp == 1 ? 0 : 1;
            bool ok = ta_wait(a, s, s.aready, 0, kDevTimeoutAload);
            ptx::tc_fence_after();
            const uint32_t alo = *s.alo;
            for (int t = iss; t < ntiles && ok; t += niss) {
                const int b = t % kAccTA;
                const uint32_t use = (uint32_t)(t / kAccTA);
                if (!ta_wait(a, s, &s.acce[b], (use & 1u) ^ 1u, kDevTimeoutMma)) { ok = false; break; }
                ptx::tc_fence_after();
                const uint32_t d_tmem = tmem + kAccColTA + (uint32_t)b * kTN;
                int it = t * nch;
                for (int c = 0; c < nch; ++c, ++it) {
                    const int st = it % R;
                    const uint32_t ph = (uint32_t)(it / R) & 1u;
                    // the slot's previous use in the other issuer's tile: its release first
                    const int prev = it - R;
                    if (niss == 2 && prev >= 0 && (prev / nch) % 2 != iss &&
                        !ta_wait(a, s, &s.empty[st], ph ^ 1u, kDevTimeoutMma)) {
                        ok = false;
                        break;
                    }
                    if (!ta_wait(a, s, &s.full[st], ph, kDevTimeoutMma)) { ok = false; break; }
                    ptx::tc_fence_after();
                    const uint32_t clo = s.slot_lo[st];
                    const uint32_t base = ptx::smem_u32(s.ring + (size_t)st * kSlotTA);
#pragma unroll
                    for (int kk = 0; kk < 4; ++kk) {
                        // K steps of 8 fp32 (32 bytes) within the 128-byte swizzle rows
                        const uint64_t ch = ptx::desc_sw128_kmajor(base + kk * 32);
                        const uint32_t ahi = tmem + (uint32_t)(c * 32 + kk * 8);
                        ptx::mma_tf32_ts(d_tmem, ahi, ch, kIdesc, (c | kk) != 0);
                        if (clo) ptx::mma_tf32_ts(d_tmem, ahi, ptx::desc_sw128_kmajor(base + kBox + kk * 32), kIdesc, 1u);
                        if (alo) ptx::mma_tf32_ts(d_tmem, ahi + (uint32_t)a.dp, ch, kIdesc, 1u);
                    }
                    // the tile's last chunk: accumulator-ready first (the epilogue waits on it)
                    if (c == nch - 1) ptx::mma_commit(&s.accf[b]);
                    ptx::mma_commit(&s.empty[st]);
                }
                if (!ok) break;
            }
            // all MMAs issued by this thread retire before TMEM is released
            ptx::mma_commit(s.drain);
            ptx::mbar_wait(s.drain, 0, kTimeout);
        }
    } else if (warp < 2 + kEpi) {
        // ------------------------------------------------------------ epilogue
        const int ew = warp - 2;
        const int quad = warp & 3;  // TMEM lane quarter this warp may access
        const int part = ew >> 2;   // columns [32 part, 32 part + 32) of every tile
        const int row = quad * 32 + lane;
        const int64_t q = q0 + row;
        const bool valid = q < a.Q;
        const uint32_t lane_base = (uint32_t)(quad * 32) << 16;
        if (part == 0) {
            // A operand: this lane's query as TF32 hi / lo parts into TMEM
            const float* qrow = a.queries + (valid ? q : 0) * a.ldq;
            uint32_t any_lo = 0;
            for (int c = 0; c < nch; ++c) {
                float hi[32], lo[32];
#pragma unroll
                for (int u = 0; u < 32; ++u) {
                    const int d = c * 32 + u;
                    const float x = (valid && d < a.D) ? __ldg(qrow + d) : 0.f;
                    hi[u] = tf32_round(x);
                    lo[u] = tf32_round(__fsub_rn(x, hi[u]));
                    any_lo |= (lo[u] != 0.f) ? 1u : 0u;
                }
                __syncwarp();
                ptx::tmem_st32(tmem + lane_base + (uint32_t)(c * 32), hi);
                ptx::tmem_st32(tmem + lane_base + (uint32_t)(a.dp + c * 32), lo);
            }
            ptx::tmem_wait_st();
            if (__any_sync(0xffffffffu, any_lo != 0u) && lane == 0) atomicOr(s.alo, 1u);
            ptx::tc_fence_before();
            __syncwarp();
            if (lane == 0) ptx::mbar_arrive(s.aready);
        }
        const float T = valid ? (a.thr ? __ldg(a.thr + q) : __int_as_float(0x7f800000)) : -__int_as_float(0x7f800000);
        const size_t seg = (size_t)split * kParts + part;
        uint64_t* out = a.cand + (seg * (size_t)a.Q + (size_t)(valid ? q : 0)) * (size_t)a.cap;
        uint32_t cnt = 0;
        const uint32_t cap = (uint32_t)a.cap;
        for (int t = 0; t < ntiles; ++t) {
            const int b = t % kAccTA;
            const uint32_t use = (uint32_t)(t / kAccTA);
            const int ns = t % kNorm;
            // warp-uniform outcome: tcgen05.ld below is warp-collective
            const bool ok = ta_wait(a, s, &s.accf[b], use & 1u, kDevTimeoutEpilogue) &&
                            ta_wait(a, s, &s.nfull[ns], (uint32_t)(t / kNorm) & 1u, kDevTimeoutEpilogue);
            if (!__all_sync(0xffffffffu, ok)) break;
            ptx::tc_fence_after();
            float v[32];
            __syncwarp();
            ptx::tmem_ld32(tmem + kAccColTA + (uint32_t)b * kTN + lane_base + (uint32_t)(32 * part), v);
            ptx::tmem_wait_ld_regs(v);
            ptx::tc_fence_before();
            __syncwarp();
            if (lane == 0) ptx::mbar_arrive(&s.acce[b]);
            const float* nrm = s.norms + ns * kTN + 32 * part;
            const uint32_t g = chunk_keys<32, false>(v, nrm, nrm, -2.0f, T, v);
            if (__any_sync(0xffffffffu, g != 0u))
                chunk_append<32>(v, g, T, (uint32_t)(n_begin + (int64_t)t * kTN) + (uint32_t)(32 * part), out, cap, cnt);
            __syncwarp();
            if (lane == 0) ptx::mbar_arrive(&s.nempty[ns]);
        }
        if (valid) a.cnt[seg * (size_t)a.Q + (size_t)q] = cnt;
    }

    ptx::tc_fence_before();
    __syncthreads();
    ptx::tc_fence_after();
    if (warp == 1) {
        __syncwarp();
        ptx::tmem_dealloc(tmem, 512);
    }
}
}  // namespace

size_t tscan_smem_bytes(int ring, bool tmem_a)
{
    return (size_t)ring * (tmem_a ? kSlotTA : kSlot) + (size_t)kNorm * kTN * 4 + kCtrl;
}

int tscan_ring(bool tmem_a)
{
    int r = tmem_a ? kMaxRingTA : kMaxRing;
    while (r > 2 && tscan_smem_bytes(r, tmem_a) > kScanSmemLimit) --r;
    return r;
}

cudaError_t launch_tscan(const TscanArgs& a, int splits, cudaStream_t st)
{
    const bool ta = a.tmem_a != 0;
    if (a.dp < 32 || a.dp % 32 != 0 || a.split_len % kTN != 0 || a.cap < 1 || splits < 1 || a.split0 < 0 ||
        a.ring < 2 || a.ring > (ta ? kMaxRingTA : kMaxRing) || (ta && (a.dp > 128 || !a.queries || a.D > a.dp)))
        return cudaErrorInvalidValue;
    const size_t smem = tscan_smem_bytes(a.ring, ta);
    if (smem > kScanSmemLimit) return cudaErrorInvalidValue;
    if (a.Q <= 0) return cudaSuccess;
    cudaError_t e = cudaFuncSetAttribute(ta ? tscan_ta_kernel : tscan_kernel,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    dim3 grid((unsigned)((a.Q + kTileQ - 1) / kTileQ), (unsigned)splits);
    if (ta)
        tscan_ta_kernel<<<grid, kThreads, smem, st>>>(a);
    else
        tscan_kernel<<<grid, kThreads, smem, st>>>(a);
    return cudaGetLastError();
}

}  // namespace knn
