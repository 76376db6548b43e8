// scan_bf16.cu -- tensor-core BF16 distance scan that collects, per query, every
// corpus row whose key falls below a per-query threshold.
//
// This is the bulk stage of the reference's distance + selection path
// (cublasSgemm in pdist_NT, include/utils.h:957-985, followed by
// bitonic_shared / relloc, src/cuknnBitonic.cu:45-254), restructured for
// large corpora: instead of keeping a sorted shortlist per query in shared
// memory, each query carries a threshold T (seeded from samples of the
// corpus by the engine) and every key strictly below T is appended to the
// query's candidate segment in global memory.  The final top-kp is chosen
// from the segments by select_cand_kernel.  Keys are the reference's ranking
// key ||c||^2 - 2 q.c (demo/knn.m:5), formed whole by the tensor core: A = -2 q
// (exact in BF16) against the corpus rows, then an all-ones A block against the
// rows' norms split into three BF16 parts (n1 + n2 + n3 = ||c||^2 exactly), one
// more K step of 16; products are exact and accumulate in FP32, so on integer
// data every key is exact.  The epilogue only compares.
// The E4M3 variant (kF8) takes both operands as FP8 E4M3 codes with per-row
// absmax scales (x = s_x * codes): kind::f8f6f4 MMAs accumulate the code
// products in FP32 and the epilogue forms ||c||^2 + (-2 s_q) * (s_c * acc),
// with the corpus scales streamed beside the norms.  A 128-byte K box holds
// 64 BF16 or 128 E4M3 values; everything else is shared.
//
// Tile: 128 queries (MMA M, TMEM lanes) x TN corpus rows (MMA N), TN = 224
// for up to 128 BF16 columns, 192 for up to 256.  Tensor memory holds two
// TN-column FP32 accumulators and the A operand (this CTA's queries) in the
// remaining dpb/2 columns, so shared memory carries only the corpus tiles
// (a ring of whole tiles where three fit) with their norm parts (32 bytes per
// row, 32-byte swizzle) and the 4 KB ones block (E4M3 keys: a ring of norms
// and scales instead).  Every CTA loads
// its own corpus tiles (CTAs of neighbouring query tiles read the same tiles
// from L2 at about the same time).
// Warp roles (608 threads):
//   warp 0      producer: per tile the corpus K-boxes (2-D TMA, 64 bf16 x TN
//               rows, 128-byte swizzle) and the norm parts with the tile's last
//               slot (E4M3 keys: norms and scales by 1-D bulk copies);
//   warp 1      TMEM owner (512 columns) and MMA issuer of the even tiles
//               (tcgen05.mma kind::f16 / kind::f8f6f4, A from TMEM, B from
//               shared memory) into accumulator 0;
//   warp 18     MMA issuer of the odd tiles into accumulator 1.  The tensor
//               pipe queues little work ahead of the instruction being issued,
//               so with one issuer every barrier wait and commit of that thread
//               idled it; two issuers overlap one's waits with the other's MMAs;
//   warps 2..17 epilogue: thread = query (TMEM lane); warps 2..5 first write
//               the queries into TMEM; warps 2+4p..5+4p (p = 0..3) read a
//               quarter of each tile's columns as a 32-column chunk and a
//               tail (16 + 8 columns for TN = 224, 16 for 192): all three
//               tcgen05.ld in flight at once, one wait, the accumulator released
//               (its round trip to the issuers is what the pipeline waits on),
//               then per chunk the minima of its 8-column groups (E4M3 keys:
//               formed first by packed multiply and fma), one vote; only groups
//               holding a key below some lane's threshold are appended.  The
//               view's last tile masks its columns past the view (+inf).
// Every mbarrier wait is bounded; on timeout the kernel records an error code
// in the device error word and winds down without hanging the GPU.
#include <algorithm>
#include <cstdint>
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include "common.cuh"
#include "kernels.h"
#include "scan_common.cuh"
#include "tc_ptx.cuh"

namespace knn {

namespace {
constexpr int kEpiWarps = 4 * kScanParts;  // 4 TMEM lane quarters x kScanParts column ranges
constexpr int kIssuers = 2;                 // MMA issuing threads (warps 1 and 2 + kEpiWarps)
constexpr int kScanThreads = 32 * (1 + kIssuers + kEpiWarps);
constexpr int kNormSlots = 8;
constexpr int kMaxAcc = 4;  // TMEM accumulators (barrier slots reserved for the largest variant)
constexpr uint32_t kCtrlBytes = 512;
constexpr uint32_t kTmemCols = 512;
constexpr uint64_t kTimeoutNs = 4000000000ull;

__host__ __device__ constexpr uint32_t box_bytes(int tn) { return (uint32_t)tn * 128u; }  // 64 bf16 x tn rows
// E4M3 keys: norm ring of kNormSlots tiles of norms, then as many tiles of corpus scales
__host__ __device__ constexpr uint32_t norm_bytes(int tn) { return (uint32_t)kNormSlots * tn * 8u; }
// BF16 keys: per ring slot the tile's norm parts (32 bytes per corpus row), and one block of
// 128 x 16 BF16 ones, the A operand that adds them to the keys
__host__ __device__ constexpr uint32_t np_bytes(int tn) { return (uint32_t)tn * 32u; }
constexpr uint32_t kOnesBytes = 128u * 32u;
// shared memory beside the ring
__host__ __device__ constexpr uint32_t side_bytes(int tn, bool f8, int ring)
{
    return f8 ? norm_bytes(tn) : (uint32_t)ring * np_bytes(tn) + kOnesBytes;
}

struct ScanSmem {
    unsigned char* ring;
    float* norms;
    uint64_t* full;    // [kScanMaxRing]
    uint64_t* empty;   // [kScanMaxRing]
    uint64_t* accf;    // [2]
    uint64_t* acce;    // [2]
    uint64_t* nfull;   // [kNormSlots]
    uint64_t* nempty;  // [kNormSlots]
    uint64_t* aready;
    uint64_t* drain;
    uint32_t* tmem_holder;
    volatile int* abort;
};

__device__ __forceinline__ bool scan_wait(const ScanArgs& a, const ScanSmem& s, uint64_t* bar, uint32_t parity,
                                          int code)
{
    // a completed barrier returns before the abort flag is read (the flag costs a shared
    // load on every hand-off otherwise); a wait that would block sees it first
    if (ptx::mbar_try_wait(bar, parity)) return true;
    if (*s.abort) return false;
    if (ptx::mbar_wait(bar, parity, kTimeoutNs)) return true;
    atomicCAS(a.err, 0, code);
    *s.abort = 1;
    return false;
}

template <int TN, int kNacc, bool kF8>
__global__ void __launch_bounds__(kScanThreads, 1)
    scan_kernel(const __grid_constant__ ScanArgs a)
{
    // Each epilogue part reads TN / 4 columns of a tile as up to three chunks, every
    // TMEM load at a multiple of its own width: [W1 p, W1 p + W1), [B2 + W2 p, ...) and
    // [B3 + W3 p, ...): 32 + 16 + 8 (TN = 224), 32 + 16 (192), 16 + 8 (96)
    constexpr int PC = TN / kScanParts;
    constexpr int W1 = PC >= 32 ? 32 : 16;
    constexpr int W2 = W1 / 2;
    constexpr int W3 = PC - W1 - W2;
    constexpr int B2 = kScanParts * W1;
    constexpr int B3 = B2 + kScanParts * W2;
    static_assert(W3 == 0 || W3 == W2 / 2, "chunks of halving widths");
    static_assert(kNacc * TN % 32 == 0 && TN % 32 == 0, "accumulators at 32-column boundaries");
    constexpr uint32_t kBoxB = box_bytes(TN);
    constexpr uint32_t kIdesc = kF8 ? ptx::idesc_e4m3(kTileQ, TN) : ptx::idesc_bf16(kTileQ, TN);
    constexpr uint32_t kACol = (uint32_t)kNacc * TN;  // A operand columns [kACol, kACol + dpb/2)
    // BF16 keys come out of the MMA whole: A = -2 q in TMEM against the corpus rows, then the
    // ones block against the rows' norm parts, key = ||c||^2 - 2 q.c (E4M3 keys: the epilogue
    // scales the accumulator and adds the norms)
    constexpr bool kNM = !kF8;

    extern __shared__ __align__(1024) unsigned char sm[];
    // device-side path choice: the kernel runs only when *skip_if == 0
    if (a.skip_if != nullptr && *a.skip_if != 0u) return;
    // 128-byte swizzle atoms need a 1024-aligned window; refuse to run otherwise
    if ((ptx::smem_u32(sm) & 1023u) != 0u) {
        if (threadIdx.x == 0) atomicCAS(a.err, 0, kDevMisaligned);
        return;
    }

    const int nbox = a.dpb / 64;
    const int bps = a.bps, R = a.ring;
    const uint32_t slot_bytes = (uint32_t)bps * kBoxB;
    const int slots_per_tile = nbox / bps;

    ScanSmem s;
    s.ring = sm;
    unsigned char* side = s.ring + (size_t)R * slot_bytes;
    s.norms = reinterpret_cast<float*>(side);   // E4M3 keys: the norm ring
    float* scales = s.norms + kNormSlots * TN;  // E4M3 keys: corpus scales, same slots as the norms
    unsigned char* np_ring = side;              // BF16 keys: norm parts of ring slot i at i * np_bytes
    unsigned char* ones = side + (size_t)R * np_bytes(TN);
    uint64_t* bars = reinterpret_cast<uint64_t*>(side + side_bytes(TN, kF8, R));
    s.full = bars;
    s.empty = bars + kScanMaxRing;
    s.accf = bars + 2 * kScanMaxRing;
    s.acce = s.accf + kMaxAcc;
    s.nfull = s.acce + kMaxAcc;
    s.nempty = s.nfull + kNormSlots;
    s.aready = s.nempty + kNormSlots;
    s.drain = s.aready + 1;
    uint32_t* words = reinterpret_cast<uint32_t*>(s.drain + 1);
    s.tmem_holder = words;
    s.abort = reinterpret_cast<volatile int*>(words + 1);

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int64_t q0 = (int64_t)blockIdx.x * kTileQ;
    const int split = a.split0 + (int)blockIdx.y;
    const int64_t n_begin = (int64_t)split * a.split_len;
    const int64_t n_end = min(a.N, n_begin + a.split_len);
    const int ntiles = n_end > n_begin ? (int)((n_end - n_begin + TN - 1) / TN) : 0;

    if (tid == 0) {
        for (int i = 0; i < R; ++i) {
            ptx::mbar_init(&s.full[i], 1);
            ptx::mbar_init(&s.empty[i], 1);
        }
        for (int b = 0; b < kNacc; ++b) {
            ptx::mbar_init(&s.accf[b], 1);
            ptx::mbar_init(&s.acce[b], kEpiWarps);
        }
        for (int b = 0; b < kNormSlots; ++b) {
            ptx::mbar_init(&s.nfull[b], 1);
            ptx::mbar_init(&s.nempty[b], kEpiWarps);
        }
        ptx::mbar_init(s.aready, 4);
        ptx::mbar_init(s.drain, kIssuers);
        *s.abort = 0;
        ptx::fence_mbar_init();
        ptx::tma_prefetch_desc(&a.tm_c);
        if (kNM) ptx::tma_prefetch_desc(&a.tm_np);
    }
    if constexpr (kNM) {
        // the ones block (any layout: every element is 1), visible to the tensor core
        uint32_t* o = reinterpret_cast<uint32_t*>(ones);
        for (int i = tid; i < (int)(kOnesBytes / 4); i += blockDim.x) o[i] = 0x3F803F80u;
        ptx::fence_proxy_async_smem();
    }
    if (warp == 1) {
        ptx::tmem_alloc(s.tmem_holder, kTmemCols);
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
                const int64_t n0 = n_begin + (int64_t)t * TN;
                for (int c = 0; c < slots_per_tile; ++c, ++it) {
                    const int st = it % R;
                    const uint32_t ph = (uint32_t)(it / R) & 1u;
                    if (!scan_wait(a, s, &s.empty[st], ph ^ 1u, kDevTimeoutProducer)) { ok = false; break; }
                    unsigned char* dst = s.ring + (size_t)st * slot_bytes;
                    // BF16 keys: the tile's norm parts travel with its last slot
                    const bool np_here = kNM && c == slots_per_tile - 1;
                    ptx::mbar_arrive_expect_tx(&s.full[st], slot_bytes + (np_here ? np_bytes(TN) : 0u));
                    for (int bx = 0; bx < bps; ++bx)
                        ptx::tma_load_2d(dst + (size_t)bx * kBoxB, &a.tm_c, &s.full[st], (c * bps + bx) * 64, (int)n0);
                    if (np_here) ptx::tma_load_2d(np_ring + (size_t)st * np_bytes(TN), &a.tm_np, &s.full[st], 0, (int)n0);
                }
                if (!ok) break;
                if constexpr (kF8) {
                    // norms and scales (needed by the epilogue only, after the MMAs); the arrays
                    // are padded (+inf norms) at least one tile past the view
                    const int ns = t % kNormSlots;
                    if (!scan_wait(a, s, &s.nempty[ns], ((uint32_t)(t / kNormSlots) & 1u) ^ 1u,
                                   kDevTimeoutProducer)) {
                        ok = false;
                        break;
                    }
                    ptx::mbar_arrive_expect_tx(&s.nfull[ns], TN * 8u);
                    ptx::bulk_load(s.norms + ns * TN, a.cn + n0, TN * 4u, &s.nfull[ns]);
                    ptx::bulk_load(scales + ns * TN, a.cs + n0, TN * 4u, &s.nfull[ns]);
                }
            }
            // let copies already issued land before the CTA winds down
            if (!ok) {
                const int first = it - R > 0 ? it - R : 0;
                for (int j = first; j < it; ++j) ptx::mbar_wait(&s.full[j % R], (uint32_t)(j / R) & 1u, kTimeoutNs);
            }
        }
    } else if (warp == 1 || warp == 2 + kEpiWarps) {
        // ------------------------------------------------------------ MMA issuers
        // issuer i takes the tiles t = i (mod 2), into accumulator t mod kNacc; each
        // commit tracks only its own thread's MMAs
        if (lane == 0) {
            const int iss = warp == 1 ? 0 : 1;
            bool ok = scan_wait(a, s, s.aready, 0, kDevTimeoutAload);
            ptx::tc_fence_after();
            const uint32_t a_tmem = tmem + kACol;
            for (int t = iss; t < ntiles && ok; t += kIssuers) {
                const int b = t % kNacc;
                const uint32_t use = (uint32_t)(t / kNacc);
                if (!scan_wait(a, s, &s.acce[b], (use & 1u) ^ 1u, kDevTimeoutMma)) { ok = false; break; }
                ptx::tc_fence_after();
                const uint32_t d_tmem = tmem + (uint32_t)b * TN;
                int it = t * slots_per_tile;
                for (int c = 0; c < slots_per_tile; ++c, ++it) {
                    const int st = it % R;
                    const uint32_t ph = (uint32_t)(it / R) & 1u;
                    if (!scan_wait(a, s, &s.full[st], ph, kDevTimeoutMma)) { ok = false; break; }
                    ptx::tc_fence_after();
                    const uint32_t b_base = ptx::smem_u32(s.ring + (size_t)st * slot_bytes);
                    for (int bx = 0; bx < bps; ++bx) {
                        const int box = c * bps + bx;
                        // K steps (32 bytes) past the last data column hold zeros on both sides: skipped
                        const int kn = min(4, a.ksteps - 4 * box);
                        for (int kk = 0; kk < kn; ++kk) {
                            const uint64_t db = ptx::desc_sw128_kmajor(b_base + bx * kBoxB + kk * 32);
                            if (kF8)
                                ptx::mma_f8_ts(d_tmem, a_tmem + (uint32_t)(box * 32 + kk * 8), db, kIdesc,
                                               (box | kk) != 0);
                            else
                                ptx::mma_bf16_ts(d_tmem, a_tmem + (uint32_t)(box * 32 + kk * 8), db, kIdesc,
                                                 (box | kk) != 0);
                        }
                    }
                    // BF16 keys: + ones x norm parts, the norms added inside the tensor core
                    if (kNM && c == slots_per_tile - 1)
                        ptx::mma_bf16_ss(d_tmem, ptx::desc_sw32_kmajor(ptx::smem_u32(ones)),
                                         ptx::desc_sw32_kmajor(ptx::smem_u32(np_ring + (size_t)st * np_bytes(TN))),
                                         kIdesc, 1u);
                    // after the tile's last MMAs the accumulator-ready commit goes first: the
                    // epilogue is on the critical path, the producer has the ring's slack
                    if (c == slots_per_tile - 1) ptx::mma_commit(&s.accf[b]);
                    ptx::mma_commit(&s.empty[st]);
                }
                if (!ok) break;
            }
            // all MMAs issued by this thread retire before TMEM is released
            ptx::mma_commit(s.drain);
            ptx::mbar_wait(s.drain, 0, kTimeoutNs);
        }
    } else {
        // ------------------------------------------------------------ epilogue
        const int ew = warp - 2;
        const int quad = warp & 3;  // TMEM lane quarter this warp may access
        const int part = ew >> 2;   // one quarter of each tile's columns (see below)
        const int row = quad * 32 + lane;
        const int64_t q = q0 + row;
        const bool valid = q < a.Q;
        const uint32_t lane_base = (uint32_t)(quad * 32) << 16;
        if (part == 0) {
            // A operand: this lane's query into TMEM (BF16 pairs or E4M3 quads per 32-bit column,
            // lower K index in the low bits); BF16 keys take -2 q (exact: a power of two)
            const uint32_t* qrow = reinterpret_cast<const uint32_t*>(a.qbf) + (valid ? q : 0) * (a.dpb / 2);
            for (int bx = 0; bx < nbox; ++bx) {
                float w[32];
#pragma unroll
                for (int u = 0; u < 32; ++u) {
                    uint32_t x = valid ? __ldg(qrow + bx * 32 + u) : 0u;
                    if (kNM) {
                        __nv_bfloat162 h = *reinterpret_cast<const __nv_bfloat162*>(&x);
                        h = __hmul2(h, __float2bfloat162_rn(-2.f));
                        x = *reinterpret_cast<const uint32_t*>(&h);
                    }
                    w[u] = __uint_as_float(x);
                }
                __syncwarp();
                ptx::tmem_st32(tmem + lane_base + kACol + (uint32_t)(bx * 32), w);
            }
            ptx::tmem_wait_st();
            ptx::tc_fence_before();
            __syncwarp();
            if (lane == 0) ptx::mbar_arrive(s.aready);
        }
        // padding lanes of the last query tile collect nothing
        const float T = valid ? (a.thr ? __ldg(a.thr + q) : __int_as_float(0x7f800000)) : -__int_as_float(0x7f800000);
        const float m = kF8 ? -2.0f * (valid ? __ldg(a.qs + q) : 0.f) : -2.0f;
        const size_t seg = (size_t)split * kScanParts + part;
        uint64_t* out = a.cand + (seg * (size_t)a.Q + (size_t)(valid ? q : 0)) * (size_t)a.cap;
        uint32_t cnt = 0;
        const uint32_t cap = (uint32_t)a.cap;
        for (int t = 0; t < ntiles; ++t) {
            const int b = t % kNacc;
            const uint32_t use = (uint32_t)(t / kNacc);
            const int ns = t % kNormSlots;
            // warp-uniform outcome: tcgen05.ld below is warp-collective
            bool ok = scan_wait(a, s, &s.accf[b], use & 1u, kDevTimeoutEpilogue);
            if (kF8) ok = ok && scan_wait(a, s, &s.nfull[ns], (uint32_t)(t / kNormSlots) & 1u, kDevTimeoutEpilogue);
            if (!__all_sync(0xffffffffu, ok)) break;
            ptx::tc_fence_after();
            // this part's columns (see the chunk layout above)
            const float* nrm = s.norms + ns * TN;
            const float* scl = scales + ns * TN;
            const uint32_t tb = tmem + (uint32_t)b * TN + lane_base;
            const uint32_t nb = (uint32_t)(n_begin + (int64_t)t * TN);
            const int c1 = W1 * part, c2 = B2 + W2 * part, c3 = B3 + W3 * part;
            // all loads in flight together, one wait, then the accumulator is released:
            // the MMA may overwrite it while the keys are formed (in place) and tested
            float va[W1], vb[W2], vc[W3 > 0 ? W3 : 4];
            __syncwarp();
            ptx::tmem_ld<W1>(tb + (uint32_t)c1, va);
            ptx::tmem_ld<W2>(tb + (uint32_t)c2, vb);
            if constexpr (W3 > 0) ptx::tmem_ld<W3>(tb + (uint32_t)c3, vc);
            ptx::tmem_wait_ld();
            ptx::tie_regs(va);
            ptx::tie_regs(vb);
            if constexpr (W3 > 0) ptx::tie_regs(vc);
            ptx::tc_fence_before();
            __syncwarp();
            if (lane == 0) ptx::mbar_arrive(&s.acce[b]);
            uint32_t ga, gb, gc = 0u;
            if constexpr (kNM) {
                // the accumulator holds the keys; the view's last tile masks its rows past the view
                const int64_t rem = a.N - (n_begin + (int64_t)t * TN);
                if (rem < TN) {
                    chunk_mask<W1>(va, c1, (int)rem);
                    chunk_mask<W2>(vb, c2, (int)rem);
                    if constexpr (W3 > 0) chunk_mask<W3>(vc, c3, (int)rem);
                }
                ga = chunk_test<W1>(va, T);
                gb = chunk_test<W2>(vb, T);
                if constexpr (W3 > 0) gc = chunk_test<W3>(vc, T);
            } else {
                ga = chunk_keys<W1, kF8>(va, nrm + c1, scl + c1, m, T, va);
                gb = chunk_keys<W2, kF8>(vb, nrm + c2, scl + c2, m, T, vb);
                if constexpr (W3 > 0) gc = chunk_keys<W3, kF8>(vc, nrm + c3, scl + c3, m, T, vc);
            }
            if (__any_sync(0xffffffffu, ga != 0u)) chunk_append<W1>(va, ga, T, nb + (uint32_t)c1, out, cap, cnt);
            if (__any_sync(0xffffffffu, (gb | gc) != 0u)) {
                chunk_append<W2>(vb, gb, T, nb + (uint32_t)c2, out, cap, cnt);
                if constexpr (W3 > 0) chunk_append<W3>(vc, gc, T, nb + (uint32_t)c3, out, cap, cnt);
            }
            if constexpr (kF8) {
                // norm slot ns fully read
                __syncwarp();
                if (lane == 0) ptx::mbar_arrive(&s.nempty[ns]);
            }
        }
        if (valid) a.cnt[seg * (size_t)a.Q + (size_t)q] = cnt;
    }

    ptx::tc_fence_before();
    __syncthreads();
    ptx::tc_fence_after();
    if (warp == 1) {
        __syncwarp();
        ptx::tmem_dealloc(tmem, kTmemCols);
    }
}
}  // namespace

// two accumulators of 224 columns (192 above 128 BF16 columns), or four of 96 (any width up to
// 256): tensor memory holds the accumulators at 32-column boundaries and the A operand after them
int scan_tile_rows(int dpb, int accs)
{
    if (accs == 4) return 96;
    return dpb <= 128 ? 224 : 192;
}

int scan_box_rows(int dpb, int accs) { return scan_tile_rows(dpb, accs); }

// every epilogue part collects the same share of a tile's columns
int scan_part_cols(int dpb, int accs) { return scan_tile_rows(dpb, accs) / kScanParts; }

size_t scan_smem_bytes(int dpb, int bps, int ring, bool fp8, int accs)
{
    const int tn = scan_tile_rows(dpb, accs);
    return (size_t)ring * bps * box_bytes(tn) + side_bytes(tn, fp8, ring) + kCtrlBytes;
}

int scan_plan(int dpb, int want_bps, int* bps, int* ring, bool fp8, int accs)
{
    const int nbox = dpb / 64;
    if (dpb % 64 != 0 || nbox < 1 || nbox > 4 || (accs != 2 && accs != 4)) return -1;
    const int tn = scan_tile_rows(dpb, accs);
    // E4M3 keys: the norm ring beside the slots; BF16 keys: norm parts in every slot, the ones block
    const size_t fixed = (fp8 ? norm_bytes(tn) : kOnesBytes) + kCtrlBytes;
    const size_t per_slot_side = fp8 ? 0 : np_bytes(tn);
    auto slots = [&](int b) {
        return (int)std::min<size_t>(kScanMaxRing,
                                     (kScanSmemLimit - fixed) / ((size_t)b * box_bytes(tn) + per_slot_side));
    };
    int b = 0;
    if (want_bps > 0) {
        if (nbox % want_bps != 0 || slots(want_bps) < 2) return -1;
        b = want_bps;
    } else {
        // whole-tile slots (one commit per tile) when three fit, else the largest divisor with two
        for (int cand : {nbox, 2, 1})
            if (cand <= nbox && nbox % cand == 0 && slots(cand) >= 3) { b = cand; break; }
        if (b == 0)
            for (int cand : {nbox, 2, 1})
                if (cand <= nbox && nbox % cand == 0 && slots(cand) >= 2) { b = cand; break; }
    }
    if (b == 0) return -1;
    *bps = b;
    *ring = slots(b);
    return 0;
}

template <int TN, int kNacc, bool kF8>
static cudaError_t launch_scan_t(const ScanArgs& a, dim3 grid, size_t smem, cudaStream_t st)
{
    cudaError_t e = cudaFuncSetAttribute(scan_kernel<TN, kNacc, kF8>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    scan_kernel<TN, kNacc, kF8><<<grid, kScanThreads, smem, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_scan(const ScanArgs& a, int splits, cudaStream_t st)
{
    const int nbox = a.dpb / 64;
    if (a.accs != 2 && a.accs != 4) return cudaErrorInvalidValue;
    const int tn = scan_tile_rows(a.dpb, a.accs);
    const bool f8 = a.fp8 != 0;
    if (a.dpb % 64 != 0 || nbox < 1 || nbox > 4 || a.bps < 1 || nbox % a.bps != 0 || a.ring < 2 ||
        a.ring > kScanMaxRing || a.split_len % tn != 0 || a.cap < 1 || splits < 1 || a.split0 < 0 || a.qbf == nullptr ||
        a.ksteps < 1 || a.ksteps > 4 * nbox || (f8 && (a.cs == nullptr || a.qs == nullptr)))
        return cudaErrorInvalidValue;
    const size_t smem = scan_smem_bytes(a.dpb, a.bps, a.ring, f8, a.accs);
    if (smem > kScanSmemLimit) return cudaErrorInvalidValue;
    // the two issuers alternate tiles: a slot's previous use must be the waiting issuer's own
    // (a tile's slots at most half the ring), else a wait could run two phases ahead of its barrier
    if (2 * (nbox / a.bps) > a.ring) return cudaErrorInvalidValue;
    if (a.Q <= 0) return cudaSuccess;
    const int64_t qt = (a.Q + kTileQ - 1) / kTileQ;
    dim3 grid((unsigned)qt, (unsigned)splits);
    if (tn == 96) return f8 ? launch_scan_t<96, 4, true>(a, grid, smem, st) : launch_scan_t<96, 4, false>(a, grid, smem, st);
    if (tn == 224)
        return f8 ? launch_scan_t<224, 2, true>(a, grid, smem, st) : launch_scan_t<224, 2, false>(a, grid, smem, st);
    return f8 ? launch_scan_t<192, 2, true>(a, grid, smem, st) : launch_scan_t<192, 2, false>(a, grid, smem, st);
}

}  // namespace knn
