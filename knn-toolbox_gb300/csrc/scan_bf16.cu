// scan_bf16.cu -- tensor-core BF16 distance scan that collects, per query, every
// corpus row whose key falls below a per-query threshold.
//
// This is the bulk stage of the reference's distance + selection path
// (cublasSgemm in pdist_NT, include/utils.h:957-985, followed by
// bitonic_shared / relloc, src/cuknnBitonic.cu:45-254), restructured for
// large corpora: instead of keeping a sorted shortlist per query in shared
// memory, each query carries a threshold T (seeded from a sample of the
// corpus, see engine.cu) and every key strictly below T is appended to the
// query's candidate segment in global memory.  The final top-kp is chosen
// from the segments by select_cand_kernel.  Keys are the reference's ranking
// key ||c||^2 - 2 q.c (demo/knn.m:5), q.c from BF16 operands with FP32
// accumulation (exact products), the norm added with one FP32 fma.
//
// Tile: 128 queries (MMA M, TMEM lanes) x 256 corpus rows (MMA N).
// Warp roles (320 threads):
//   warp 0      producer: the CTA's queries (A, BF16, K-major, 128-byte
//               swizzle) once, then per tile the corpus norms (1-D bulk copy)
//               and the corpus K-boxes (2-D TMA, 64 bf16 x 256 rows) into a
//               ring of slots;
//   warp 1      TMEM owner (512 columns = two 256-column FP32 accumulators)
//               and single-thread MMA issuer (tcgen05.mma kind::f16, A and B
//               from shared memory);
//   warps 2..9  epilogue: thread = query (TMEM lane); warps 2..5 read the
//               tile's columns 0..127, warps 6..9 columns 128..255; per
//               32-column chunk: one tcgen05.ld, 16 packed fma, the minima of
//               four 8-column groups, one vote; only the groups holding a key
//               below the lane's threshold are appended, out of line.
// Every mbarrier wait is bounded; on timeout the kernel records an error code
// in the device error word and winds down without hanging the GPU.
#include <algorithm>
#include <cstdint>
#include <cuda.h>
#include <cuda_runtime.h>
#include "common.cuh"
#include "kernels.h"
#include "tc_ptx.cuh"

namespace knn {

namespace {
constexpr int kScanThreads = 320;
constexpr uint32_t kBoxA = kTileQ * 128u;      // 64 bf16 x 128 query rows (16 KB)
constexpr uint32_t kBoxB = kScanTileN * 128u;  // 64 bf16 x 256 corpus rows (32 KB)
constexpr int kNormSlots = 4;
constexpr uint32_t kNormBytes = kNormSlots * kScanTileN * 4u;
constexpr uint32_t kCtrlBytes = 512;
constexpr int kRowPitch = 36;  // staged keys: [8 warps][32 lanes][36 floats] (conflict-free 16-byte stores)
constexpr uint32_t kStageBytes = 8u * 32u * kRowPitch * 4u;
constexpr uint32_t kTmemCols = 512;
constexpr uint64_t kTimeoutNs = 4000000000ull;
constexpr uint32_t kIdesc = ptx::idesc_bf16(kTileQ, kScanTileN);

struct ScanSmem {
    unsigned char* a;
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
    float* stage;      // [8][32][kRowPitch]
};

__device__ __forceinline__ bool scan_wait(const ScanArgs& a, const ScanSmem& s, uint64_t* bar, uint32_t parity,
                                          int code)
{
    if (*s.abort) return false;
    if (ptx::mbar_wait(bar, parity, kTimeoutNs)) return true;
    atomicCAS(a.err, 0, code);
    *s.abort = 1;
    return false;
}

// Out of line (one copy of the code): append the keys below T of the flagged
// 8-column groups of one lane's staged 32-key row, in increasing corpus index.
static __device__ __noinline__ uint32_t offer_groups(const float* row, uint32_t gm, float T, uint32_t base,
                                                     uint64_t* out, uint32_t cap, uint32_t cnt)
{
    while (gm) {
        const int g = __ffs(gm) - 1;
        gm &= gm - 1;
        const float4 lo = *reinterpret_cast<const float4*>(row + 8 * g);
        const float4 hi = *reinterpret_cast<const float4*>(row + 8 * g + 4);
        const float k8[8] = {lo.x, lo.y, lo.z, lo.w, hi.x, hi.y, hi.z, hi.w};
        const uint32_t b = base + 8u * (uint32_t)g;
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const bool h = k8[j] < T;
            if (h && cnt < cap) out[cnt] = pack_key(k8[j], b + (uint32_t)j);
            cnt += h ? 1u : 0u;
        }
    }
    return cnt;
}

// Minimum of 8 keys (four min instructions).
__device__ __forceinline__ float min8(const float* k)
{
    return fminf(ptx::fmin3(ptx::fmin3(k[0], k[1], k[2]), ptx::fmin3(k[3], k[4], k[5]), k[6]), k[7]);
}

// One 32-column chunk of one lane: keys = ||c||^2 - 2 q.c, the minimum of each
// 8-column group, one warp vote; when some lane has a group with a key below
// its threshold, the keys are staged in the lane's shared-memory row and the
// flagged groups are appended out of line.
__device__ __forceinline__ void scan_chunk(const float (&v)[32], const float* nrm, float T, uint32_t base,
                                           uint64_t* out, uint32_t cap, uint32_t& cnt, float* srow)
{
    float key[32];
    const float4* n4 = reinterpret_cast<const float4*>(nrm);
#pragma unroll
    for (int u = 0; u < 8; ++u) {
        const float4 c = n4[u];
        ptx::fma2(key[4 * u], key[4 * u + 1], v[4 * u], v[4 * u + 1], -2.0f, c.x, c.y);
        ptx::fma2(key[4 * u + 2], key[4 * u + 3], v[4 * u + 2], v[4 * u + 3], -2.0f, c.z, c.w);
    }
    const uint32_t gm = (min8(key) < T ? 1u : 0u) | (min8(key + 8) < T ? 2u : 0u) |
                        (min8(key + 16) < T ? 4u : 0u) | (min8(key + 24) < T ? 8u : 0u);
    if (__any_sync(0xffffffffu, gm != 0u)) {
        if (gm != 0u) {
            float4* s4 = reinterpret_cast<float4*>(srow);
#pragma unroll
            for (int u = 0; u < 8; ++u) s4[u] = make_float4(key[4 * u], key[4 * u + 1], key[4 * u + 2], key[4 * u + 3]);
            cnt = offer_groups(srow, gm, T, base, out, cap, cnt);
        }
    }
}
}  // namespace

size_t scan_smem_bytes(int dpb, int bps, int ring)
{
    return (size_t)(dpb / 64) * kBoxA + (size_t)ring * bps * kBoxB + kNormBytes + kCtrlBytes + kStageBytes;
}

int scan_plan(int dpb, int want_bps, int* bps, int* ring)
{
    const int nbox = dpb / 64;
    if (dpb % 64 != 0 || nbox < 1 || nbox > 4) return -1;
    const size_t fixed = (size_t)nbox * kBoxA + kNormBytes + kCtrlBytes + kStageBytes;
    auto slots = [&](int b) { return (int)std::min<size_t>(kScanMaxRing, (kScanSmemLimit - fixed) / ((size_t)b * kBoxB)); };
    int b = 0;
    if (want_bps > 0) {
        if (nbox % want_bps != 0 || slots(want_bps) < 2) return -1;
        b = want_bps;
    } else {
        // whole-tile slots (one commit per tile) when two fit, else pairs of boxes, else single boxes
        for (int cand : {nbox, 2, 1})
            if (cand <= nbox && nbox % cand == 0 && slots(cand) >= 2) { b = cand; break; }
    }
    if (b == 0) return -1;
    *bps = b;
    *ring = slots(b);
    return 0;
}

__global__ void __launch_bounds__(kScanThreads, 1) scan_kernel(const __grid_constant__ ScanArgs a)
{
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
    s.a = sm;
    s.ring = sm + (size_t)nbox * kBoxA;
    s.norms = reinterpret_cast<float*>(s.ring + (size_t)R * slot_bytes);
    uint64_t* bars = reinterpret_cast<uint64_t*>(reinterpret_cast<unsigned char*>(s.norms) + kNormBytes);
    s.full = bars;
    s.empty = bars + kScanMaxRing;
    s.accf = bars + 2 * kScanMaxRing;
    s.acce = s.accf + 2;
    s.nfull = s.acce + 2;
    s.nempty = s.nfull + kNormSlots;
    s.aready = s.nempty + kNormSlots;
    s.drain = s.aready + 1;
    uint32_t* words = reinterpret_cast<uint32_t*>(s.drain + 1);
    s.tmem_holder = words;
    s.abort = reinterpret_cast<volatile int*>(words + 1);
    s.stage = reinterpret_cast<float*>(reinterpret_cast<unsigned char*>(bars) + kCtrlBytes);

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int64_t q0 = (int64_t)blockIdx.x * kTileQ;
    const int64_t n_begin = (int64_t)blockIdx.y * a.split_len;
    const int64_t n_end = min(a.N, n_begin + a.split_len);
    const int ntiles = n_end > n_begin ? (int)((n_end - n_begin + kScanTileN - 1) / kScanTileN) : 0;

    if (tid == 0) {
        for (int i = 0; i < R; ++i) {
            ptx::mbar_init(&s.full[i], 1);
            ptx::mbar_init(&s.empty[i], 1);
        }
        for (int b = 0; b < 2; ++b) {
            ptx::mbar_init(&s.accf[b], 1);
            ptx::mbar_init(&s.acce[b], 8);
        }
        for (int b = 0; b < kNormSlots; ++b) {
            ptx::mbar_init(&s.nfull[b], 1);
            ptx::mbar_init(&s.nempty[b], 8);
        }
        ptx::mbar_init(s.aready, 1);
        ptx::mbar_init(s.drain, 1);
        *s.abort = 0;
        ptx::fence_mbar_init();
        ptx::tma_prefetch_desc(&a.tm_c);
        ptx::tma_prefetch_desc(&a.tm_q);
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
            // this CTA's queries: rows q0.. of the BF16 query copy (rows past Q read as zeros)
            ptx::mbar_arrive_expect_tx(s.aready, (uint32_t)nbox * kBoxA);
            for (int bx = 0; bx < nbox; ++bx)
                ptx::tma_load_2d(s.a + (size_t)bx * kBoxA, &a.tm_q, s.aready, bx * 64, (int)q0);
            int it = 0;
            bool ok = true;
            for (int t = 0; t < ntiles && ok; ++t) {
                const int64_t n0 = n_begin + (int64_t)t * kScanTileN;
                const int ns = t % kNormSlots;
                if (!scan_wait(a, s, &s.nempty[ns], ((uint32_t)(t / kNormSlots) & 1u) ^ 1u, kDevTimeoutProducer)) {
                    ok = false;
                    break;
                }
                // norms array padded with +inf to a multiple of 256 rows
                ptx::mbar_arrive_expect_tx(&s.nfull[ns], kScanTileN * 4u);
                ptx::bulk_load(s.norms + ns * kScanTileN, a.cn + n0, kScanTileN * 4u, &s.nfull[ns]);
                for (int c = 0; c < slots_per_tile; ++c, ++it) {
                    const int st = it % R;
                    const uint32_t ph = (uint32_t)(it / R) & 1u;
                    if (!scan_wait(a, s, &s.empty[st], ph ^ 1u, kDevTimeoutProducer)) { ok = false; break; }
                    unsigned char* dst = s.ring + (size_t)st * slot_bytes;
                    ptx::mbar_arrive_expect_tx(&s.full[st], slot_bytes);
                    for (int bx = 0; bx < bps; ++bx)
                        ptx::tma_load_2d(dst + (size_t)bx * kBoxB, &a.tm_c, &s.full[st], (c * bps + bx) * 64, (int)n0);
                }
            }
            // let copies already issued land before the CTA winds down
            ptx::mbar_wait(s.aready, 0, kTimeoutNs);
            if (!ok) {
                const int first = it - R > 0 ? it - R : 0;
                for (int j = first; j < it; ++j) ptx::mbar_wait(&s.full[j % R], (uint32_t)(j / R) & 1u, kTimeoutNs);
            }
        }
    } else if (warp == 1) {
        // ------------------------------------------------------------ MMA issuer
        if (lane == 0) {
            bool ok = scan_wait(a, s, s.aready, 0, kDevTimeoutAload);
            ptx::tc_fence_after();
            const uint32_t a_base = ptx::smem_u32(s.a);
            int it = 0;
            for (int t = 0; t < ntiles && ok; ++t) {
                const int b = t & 1;
                const uint32_t use = (uint32_t)(t >> 1);
                if (!scan_wait(a, s, &s.acce[b], (use & 1u) ^ 1u, kDevTimeoutMma)) { ok = false; break; }
                ptx::tc_fence_after();
                const uint32_t d_tmem = tmem + (uint32_t)b * kScanTileN;
                for (int c = 0; c < slots_per_tile; ++c, ++it) {
                    const int st = it % R;
                    const uint32_t ph = (uint32_t)(it / R) & 1u;
                    if (!scan_wait(a, s, &s.full[st], ph, kDevTimeoutMma)) { ok = false; break; }
                    ptx::tc_fence_after();
                    const uint32_t b_base = ptx::smem_u32(s.ring + (size_t)st * slot_bytes);
                    for (int bx = 0; bx < bps; ++bx) {
                        const uint32_t box = (uint32_t)(c * bps + bx);
#pragma unroll
                        for (int kk = 0; kk < 4; ++kk) {
                            const uint64_t da = ptx::desc_sw128_kmajor(a_base + box * kBoxA + kk * 32);
                            const uint64_t db = ptx::desc_sw128_kmajor(b_base + bx * kBoxB + kk * 32);
                            ptx::mma_bf16_ss(d_tmem, da, db, kIdesc, (box | (uint32_t)kk) != 0u);
                        }
                    }
                    ptx::mma_commit(&s.empty[st]);
                }
                if (!ok) break;
                ptx::mma_commit(&s.accf[b]);
            }
            // all MMAs issued by this thread retire before TMEM is released
            ptx::mma_commit(s.drain);
            ptx::mbar_wait(s.drain, 0, kTimeoutNs);
        }
    } else {
        // ------------------------------------------------------------ epilogue
        const int ew = warp - 2;
        const int quad = warp & 3;  // TMEM lane quarter this warp may access
        const int half = ew >> 2;   // columns [128*half, 128*half + 128) of each tile
        const int row = quad * 32 + lane;
        const int64_t q = q0 + row;
        const bool valid = q < a.Q;
        const uint32_t lane_base = (uint32_t)(quad * 32) << 16;
        // padding lanes of the last query tile collect nothing
        const float T = valid ? (a.thr ? __ldg(a.thr + q) : __int_as_float(0x7f800000)) : -__int_as_float(0x7f800000);
        const size_t seg = (size_t)blockIdx.y * 2 + half;
        uint64_t* out = a.cand + (seg * (size_t)a.Q + (size_t)(valid ? q : 0)) * (size_t)a.cap;
        uint32_t cnt = 0;
        const uint32_t cap = (uint32_t)a.cap;
        float* srow = s.stage + (size_t)(ew * 32 + lane) * kRowPitch;
        for (int t = 0; t < ntiles; ++t) {
            const int b = t & 1;
            const uint32_t use = (uint32_t)(t >> 1);
            const int ns = t % kNormSlots;
            // warp-uniform outcome: tcgen05.ld below is warp-collective
            const bool ok = scan_wait(a, s, &s.accf[b], use & 1u, kDevTimeoutEpilogue) &&
                            scan_wait(a, s, &s.nfull[ns], (uint32_t)(t / kNormSlots) & 1u, kDevTimeoutEpilogue);
            if (!__all_sync(0xffffffffu, ok)) break;
            ptx::tc_fence_after();
            const float* nrm = s.norms + ns * kScanTileN + half * 128;
            const uint32_t tb = tmem + (uint32_t)b * kScanTileN + (uint32_t)(half * 128) + lane_base;
            const uint32_t nb = (uint32_t)(n_begin + (int64_t)t * kScanTileN + half * 128);
            // four 32-column chunks; the next chunk's TMEM load overlaps this chunk's work
            float va[32], vb[32];
            __syncwarp();
            ptx::tmem_ld32(tb, va);
            ptx::tmem_wait_ld_regs(va);
            __syncwarp();
            ptx::tmem_ld32(tb + 32u, vb);
            scan_chunk(va, nrm, T, nb, out, cap, cnt, srow);
            ptx::tmem_wait_ld_regs(vb);
            __syncwarp();
            ptx::tmem_ld32(tb + 64u, va);
            scan_chunk(vb, nrm + 32, T, nb + 32u, out, cap, cnt, srow);
            ptx::tmem_wait_ld_regs(va);
            __syncwarp();
            ptx::tmem_ld32(tb + 96u, vb);
            scan_chunk(va, nrm + 64, T, nb + 64u, out, cap, cnt, srow);
            ptx::tmem_wait_ld_regs(vb);
            // accumulator b fully read: the MMA may overwrite it while the last chunk is tested
            ptx::tc_fence_before();
            __syncwarp();
            if (lane == 0) ptx::mbar_arrive(&s.acce[b]);
            scan_chunk(vb, nrm + 96, T, nb + 96u, out, cap, cnt, srow);
            // norm slot ns fully read
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
        ptx::tmem_dealloc(tmem, kTmemCols);
    }
}

cudaError_t launch_scan(const ScanArgs& a, int splits, cudaStream_t st)
{
    const int nbox = a.dpb / 64;
    if (a.dpb % 64 != 0 || nbox < 1 || nbox > 4 || a.bps < 1 || nbox % a.bps != 0 || a.ring < 2 ||
        a.ring > kScanMaxRing || a.split_len % kScanTileN != 0 || a.cap < 1 || splits < 1)
        return cudaErrorInvalidValue;
    const size_t smem = scan_smem_bytes(a.dpb, a.bps, a.ring);
    if (smem > kScanSmemLimit) return cudaErrorInvalidValue;
    if (a.Q <= 0) return cudaSuccess;
    cudaError_t e = cudaFuncSetAttribute(scan_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    dim3 grid((unsigned)((a.Q + kTileQ - 1) / kTileQ), (unsigned)splits);
    scan_kernel<<<grid, kScanThreads, smem, st>>>(a);
    return cudaGetLastError();
}

}  // namespace knn
