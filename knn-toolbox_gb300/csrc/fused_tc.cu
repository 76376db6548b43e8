// fused_tc.cu -- tensor-core fused distance + per-query shortlist for sm_103a.
//
// Replaces, for one CTA's 128 queries and one corpus split, the reference's
// distance stage (cublasSgemm in pdist_NT, include/utils.h:957-985, then the
// pdot norm-add pass) and its selection stage (bitonic_shared /
// bitonic_shared2 / relloc, src/cuknnBitonic.cu:45-254): the distance matrix
// stays in tensor memory and only shortlist survivors reach shared memory.
//
// q.c runs as 3xTF32: with x = hi + lo (hi = tf32(x), lo = tf32(x - hi)),
// q.c ~= qhi.chi + qhi.clo + qlo.chi, accumulated in FP32 by
// tcgen05.mma.kind::tf32.  For integer data below 2^11 lo is zero and the
// products and sums are exact, so the keys equal the oracle's bit for bit.
//
// Warp roles (192 threads):
//   warp 0      TMA producer: corpus hi/lo K-chunks (128 rows x 32 fp32,
//               128-byte swizzle) into a `stages`-deep shared-memory ring;
//   warp 1      TMEM owner + MMA issuer: A (this CTA's queries, hi and lo)
//               sits in TMEM columns [0, 2*dp); two 128-column FP32
//               accumulators at columns 256 and 384 alternate between tiles;
//   warps 2..5  epilogue: thread = query (= TMEM lane); loads its query into
//               TMEM, then per tile reads its 128 dot products (tcgen05.ld),
//               forms key = ||c||^2 - 2 q.c and runs the shortlist filter.
// Every mbarrier wait is bounded; on timeout the kernel records an error
// code in the device error word and winds down without hanging the GPU.
#include <cstdint>
#include <cuda.h>
#include <cuda_runtime.h>
#include "common.cuh"
#include "kernels.h"
#include "tc_ptx.cuh"

namespace knn {

namespace {
constexpr int kTcThreads = 192;
constexpr uint32_t kStageBytes = 2u * kTileN * 128u;   // hi + lo, 128 rows x 128 B each
constexpr uint32_t kTmemCols = 512;
constexpr uint32_t kAccCol = 256;
constexpr uint64_t kTimeoutNs = 4000000000ull;
constexpr uint32_t kIdesc = ptx::idesc_tf32(kTileQ, kTileN);

__device__ __forceinline__ float tf32_rne_dev(float x)
{
    uint32_t u = __float_as_uint(x);
    if ((u & 0x7f800000u) == 0x7f800000u) return x;
    u += 0xfffu + ((u >> 13) & 1u);
    u &= 0xffffe000u;
    return __uint_as_float(u);
}

struct TcSmem {
    unsigned char* stages;   // [stages][hi 16K | lo 16K], 1024-aligned
    uint64_t* full;
    uint64_t* empty;
    uint64_t* accf;
    uint64_t* acce;
    uint64_t* aready;
    uint64_t* drain;
    uint32_t* tmem_holder;
    volatile int* abort;
    uint64_t* list;
    uint64_t* buf;
    uint64_t* scratch;
};

__host__ __device__ inline size_t tc_list_offset(int stages)
{
    // stages, then 256 bytes of barriers / holders
    return (size_t)stages * kStageBytes + 256;
}
}  // namespace

size_t tc_smem_bytes(int kp, int stages)
{
    return 1024 + tc_list_offset(stages) + (size_t)kTileQ * kp * 8 + (size_t)kBufCap * (kTileQ + 1) * 8 +
           (size_t)4 * 32 * 8;
}

int tc_max_stages(int kp)
{
    int best = 0;
    for (int s = 1; s <= 6; ++s)
        if (tc_smem_bytes(kp, s) <= 232448) best = s;
    return best;
}

__device__ __forceinline__ void tc_fail(const TcArgs& a, const TcSmem& s, int code)
{
    atomicCAS(a.err, 0, code);
    *s.abort = 1;
}

__device__ __forceinline__ bool tc_wait(const TcArgs& a, const TcSmem& s, uint64_t* bar, uint32_t parity, int code)
{
    if (*s.abort) return false;
    if (ptx::mbar_wait(bar, parity, kTimeoutNs)) return true;
    tc_fail(a, s, code);
    return false;
}

__global__ void __launch_bounds__(kTcThreads, 1) tc_kernel(const __grid_constant__ TcArgs a)
{
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    const uint32_t raw_addr = ptx::smem_u32(smem_raw);
    unsigned char* sm = smem_raw + ((1024u - (raw_addr & 1023u)) & 1023u);

    const int stages = a.stages;
    TcSmem s;
    s.stages = sm;
    uint64_t* bars = reinterpret_cast<uint64_t*>(sm + (size_t)stages * kStageBytes);
    s.full = bars;
    s.empty = bars + stages;
    s.accf = bars + 2 * stages;
    s.acce = s.accf + 2;
    s.aready = s.acce + 2;
    s.drain = s.aready + 1;
    s.tmem_holder = reinterpret_cast<uint32_t*>(s.drain + 1);
    s.abort = reinterpret_cast<volatile int*>(s.tmem_holder + 1);
    s.list = reinterpret_cast<uint64_t*>(sm + tc_list_offset(stages));
    s.buf = s.list + (size_t)kTileQ * a.kp;
    s.scratch = s.buf + (size_t)kBufCap * (kTileQ + 1);

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int64_t q0 = (int64_t)blockIdx.x * kTileQ;
    const int64_t n_begin = (int64_t)blockIdx.y * a.split_len;
    const int64_t n_end = min(a.N, n_begin + a.split_len);
    const int ntiles = (int)((n_end - n_begin + kTileN - 1) / kTileN);
    const int nchunks = a.dp / kChunkK;

    if (tid == 0) {
        for (int i = 0; i < stages; ++i) {
            ptx::mbar_init(&s.full[i], 1);
            ptx::mbar_init(&s.empty[i], 1);
        }
        for (int b = 0; b < 2; ++b) {
            ptx::mbar_init(&s.accf[b], 1);
            ptx::mbar_init(&s.acce[b], 4);
        }
        ptx::mbar_init(s.aready, 4 * 32);
        ptx::mbar_init(s.drain, 1);
        *s.abort = 0;
        ptx::fence_mbar_init();
        ptx::tma_prefetch_desc(&a.tm_hi);
        ptx::tma_prefetch_desc(&a.tm_lo);
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
        if (lane == 0) {
            int it = 0;
            bool ok = true;
            for (int t = 0; t < ntiles && ok; ++t) {
                const int y = (int)(n_begin + (int64_t)t * kTileN);
                for (int c = 0; c < nchunks; ++c, ++it) {
                    const int st = it % stages;
                    const uint32_t ph = (uint32_t)(it / stages) & 1u;
                    if (!tc_wait(a, s, &s.empty[st], ph ^ 1u, kDevTimeoutProducer)) { ok = false; break; }
                    unsigned char* dst = s.stages + (size_t)st * kStageBytes;
                    ptx::mbar_arrive_expect_tx(&s.full[st], kStageBytes);
                    ptx::tma_load_2d(dst, &a.tm_hi, &s.full[st], c * kChunkK, y);
                    ptx::tma_load_2d(dst + kStageBytes / 2, &a.tm_lo, &s.full[st], c * kChunkK, y);
                }
            }
            if (!ok) {
                // let copies already issued land before the CTA winds down
                const int first = it - stages > 0 ? it - stages : 0;
                for (int j = first; j < it; ++j)
                    ptx::mbar_wait(&s.full[j % stages], (uint32_t)(j / stages) & 1u, kTimeoutNs);
            }
        }
    } else if (warp == 1) {
        // ------------------------------------------------------------ MMA issuer
        if (lane == 0) {
            bool ok = tc_wait(a, s, s.aready, 0, kDevTimeoutAload);
            ptx::tc_fence_after();
            int it = 0;
            for (int t = 0; t < ntiles && ok; ++t) {
                const int b = t & 1;
                const uint32_t use = (uint32_t)(t >> 1);
                if (!tc_wait(a, s, &s.acce[b], (use & 1u) ^ 1u, kDevTimeoutMma)) { ok = false; break; }
                ptx::tc_fence_after();
                const uint32_t d_tmem = tmem + kAccCol + (uint32_t)b * kTileN;
                for (int c = 0; c < nchunks; ++c, ++it) {
                    const int st = it % stages;
                    const uint32_t ph = (uint32_t)(it / stages) & 1u;
                    if (!tc_wait(a, s, &s.full[st], ph, kDevTimeoutMma)) { ok = false; break; }
                    ptx::tc_fence_after();
                    const uint32_t hi_addr = ptx::smem_u32(s.stages + (size_t)st * kStageBytes);
                    const uint32_t lo_addr = hi_addr + kStageBytes / 2;
#pragma unroll
                    for (int kk = 0; kk < kChunkK / 8; ++kk) {
                        const uint64_t dh = ptx::desc_sw128_kmajor(hi_addr + kk * 32);
                        const uint64_t dl = ptx::desc_sw128_kmajor(lo_addr + kk * 32);
                        const uint32_t ahi = tmem + (uint32_t)(c * kChunkK + kk * 8);
                        const uint32_t alo = ahi + (uint32_t)a.dp;
                        ptx::mma_tf32_ts(d_tmem, ahi, dh, kIdesc, (c | kk) != 0);
                        ptx::mma_tf32_ts(d_tmem, ahi, dl, kIdesc, 1u);
                        ptx::mma_tf32_ts(d_tmem, alo, dh, kIdesc, 1u);
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
        const int quad = warp & 3;
        const int row = quad * 32 + lane;
        const int64_t q = q0 + row;
        const uint32_t lane_base = (uint32_t)(quad * 32) << 16;
        ShortlistView v;
        v.list = s.list;
        v.buf = s.buf;
        v.scratch = s.scratch;
        v.kp = a.kp;
        v.kp_pitch = a.kp;
        v.buf_pitch = kTileQ + 1;
        uint64_t* scr = s.scratch + (warp - 2) * 32;

        // A operand: this thread's query row, split into TF32 hi/lo, into TMEM
        const float* qrow = a.queries + (q < a.Q ? q : 0) * a.ldq;
        for (int c = 0; c < nchunks; ++c) {
            float hi[32], lo[32];
#pragma unroll
            for (int u = 0; u < 32; ++u) {
                const int d = c * kChunkK + u;
                const float x = (q < a.Q && d < a.D) ? __ldg(qrow + d) : 0.f;
                hi[u] = tf32_rne_dev(x);
                lo[u] = tf32_rne_dev(__fsub_rn(x, hi[u]));
            }
            __syncwarp();
            ptx::tmem_st32(tmem + lane_base + (uint32_t)(c * kChunkK), hi);
            ptx::tmem_st32(tmem + lane_base + (uint32_t)(a.dp + c * kChunkK), lo);
        }
        ptx::tmem_wait_st();
        ptx::tc_fence_before();
        ptx::mbar_arrive(s.aready);

        int cnt = 0;
        float thr = __int_as_float(0x7f800000);
        for (int t = 0; t < ntiles; ++t) {
            const int b = t & 1;
            const uint32_t use = (uint32_t)(t >> 1);
            // warp-uniform outcome: tcgen05.ld below is warp-collective
            const bool ok = __all_sync(0xffffffffu, tc_wait(a, s, &s.accf[b], use & 1u, kDevTimeoutEpilogue));
            if (!ok) break;
            ptx::tc_fence_after();
            const int64_t n0 = n_begin + (int64_t)t * kTileN;
            const uint32_t tb = tmem + kAccCol + (uint32_t)b * kTileN + lane_base;
#pragma unroll 1
            for (int cc = 0; cc < kTileN / 32; ++cc) {
                float vals[32];
                __syncwarp();
                ptx::tmem_ld32(tb + (uint32_t)(cc * 32), vals);
                ptx::tmem_wait_ld();
                if (cc == kTileN / 32 - 1) {
                    ptx::tc_fence_before();
                    __syncwarp();
                    if (lane == 0) ptx::mbar_arrive(&s.acce[b]);
                }
                if (a.dump != nullptr && blockIdx.x == 0 && blockIdx.y == 0 && t == 0) {
#pragma unroll
                    for (int u = 0; u < 32; ++u) a.dump[row * kTileN + cc * 32 + u] = vals[u];
                }
                const float* cnp = a.cn + n0 + cc * 32;
                const uint32_t nb = (uint32_t)(n0 + cc * 32);
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    maybe_flush(v, row, cnt, thr, scr);
#pragma unroll
                    for (int u = 0; u < 16; ++u) {
                        const int j = h * 16 + u;
                        const float key = __fmaf_rn(-2.0f, vals[j], __ldg(cnp + j));
                        offer(v, row, cnt, thr, key, nb + (uint32_t)j);
                    }
                }
            }
        }
        flush_all(v, row, cnt, thr, scr);
    }

    ptx::tc_fence_before();
    __syncthreads();
    ptx::tc_fence_after();
    if (warp == 1) {
        __syncwarp();
        ptx::tmem_dealloc(tmem, kTmemCols);
    }

    const int64_t nq = min((int64_t)kTileQ, a.Q - q0);
    uint64_t* out = a.part + ((size_t)blockIdx.y * a.Q + q0) * a.kp;
    for (int64_t i = tid; i < nq * a.kp; i += kTcThreads) out[i] = s.list[i];
}

cudaError_t launch_tc(const TcArgs& a, int splits, cudaStream_t st)
{
    const size_t smem = tc_smem_bytes(a.kp, a.stages);
    cudaError_t e = cudaFuncSetAttribute(tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    dim3 grid((unsigned)((a.Q + kTileQ - 1) / kTileQ), (unsigned)splits);
    tc_kernel<<<grid, kTcThreads, smem, st>>>(a);
    return cudaGetLastError();
}

}  // namespace knn
