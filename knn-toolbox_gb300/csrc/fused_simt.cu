// fused_simt.cu -- CUDA-core FP32 fused distance + per-query shortlist.
//
// The general path: any dimension, shortlists up to 512 entries.  It computes
// the GEMM-form key ||c||^2 - 2 q.c of the reference's pdist_NT + pdot
// (include/utils.h:957-985, 383-397) with a sequential fmaf dot product (the
// oracle's convention, so its keys are bit-identical to the oracle's) and
// feeds the keys straight into the shortlist filter: the Q x N distance
// matrix of the reference (written by cuBLAS, re-read by pdot and by
// bitonic_shared, src/cuknnBitonic.cu:45-121) never exists.
//
// Grid: (query tiles, corpus splits).  Block: 256 threads.  Each CTA owns
// `QPB` queries and one contiguous corpus split; the first QPB threads are the
// query owners that run the filter.
#include <cstdint>
#include <cuda_runtime.h>
#include "common.cuh"
#include "kernels.h"

namespace knn {

namespace {
constexpr int kThreads = 256;
constexpr int kKC = 32;
constexpr int kNT = kSimtTileN;

__host__ __device__ constexpr size_t simt_gemm_bytes(int qpb)
{
    return (size_t)kKC * (qpb + 4) * 4 + (size_t)kKC * (kNT + 4) * 4 + (size_t)qpb * (kNT + 1) * 4;
}
}  // namespace

template <int QPB>
__global__ void __launch_bounds__(kThreads)
simt_kernel(const float* __restrict__ corpus, int64_t N, int64_t ldc, const float* __restrict__ cn,
            const float* __restrict__ queries, int64_t Q, int64_t ldq, int D, int kp,
            int64_t split_len, uint64_t* __restrict__ part, uint32_t* __restrict__ thr_g_all,
            const uint32_t* __restrict__ tile_redo, const int32_t* __restrict__ qmap,
            const uint32_t* __restrict__ qcount, int64_t qbase)
{
    if (tile_redo != nullptr && tile_redo[blockIdx.x] == 0u) return;
    // compacted rows: row r is query qmap[qbase + r], present while qbase + r < *qcount
    int64_t qvalid = Q;
    if (qcount != nullptr) {
        qvalid = min(Q, (int64_t)*qcount - qbase);
        if ((int64_t)blockIdx.x * QPB >= qvalid) return;
    }
    constexpr int RQ = QPB / 16;
    extern __shared__ __align__(16) unsigned char smem[];
    float* qs = reinterpret_cast<float*>(smem);
    float* cs = qs + kKC * (QPB + 4);
    float* tile = cs + kKC * (kNT + 4);
    uint64_t* sl = reinterpret_cast<uint64_t*>(smem + ((simt_gemm_bytes(QPB) + 15) & ~size_t(15)));
    ShortlistView v;
    v.list = sl;
    v.kp = kp;
    v.kp_pitch = kp;
    v.buf_pitch = QPB;
    v.buf = sl + (size_t)QPB * kp;

    const int tid = threadIdx.x;
    const int64_t q0 = (int64_t)blockIdx.x * QPB;
    const int64_t n_begin = (int64_t)blockIdx.y * split_len;
    const int64_t n_end = min(N, n_begin + split_len);

    for (int i = tid; i < QPB * kp; i += kThreads) v.list[i] = kSentinel;
    __syncthreads();

    const bool owner = tid < QPB;
    const int64_t q = q0 + tid;
    LaneState st{0, q < qvalid ? __int_as_float(0x7f800000) : -__int_as_float(0x7f800000)};
    uint32_t* thr_g = (owner && q < qvalid) ? thr_g_all : nullptr;
    const int tx = tid & 15, ty = tid >> 4;

    for (int64_t n0 = n_begin; n0 < n_end; n0 += kNT) {
        float acc[RQ][4];
#pragma unroll
        for (int r = 0; r < RQ; ++r)
#pragma unroll
            for (int c = 0; c < 4; ++c) acc[r][c] = 0.f;

        for (int d0 = 0; d0 < D; d0 += kKC) {
            for (int i = tid; i < QPB * kKC; i += kThreads) {
                int q = i / kKC, d = i - q * kKC;
                float val = 0.f;
                if (q0 + q < qvalid && d0 + d < D) {
                    const int64_t src = qmap != nullptr ? (int64_t)__ldg(qmap + qbase + q0 + q) : q0 + q;
                    val = __ldg(queries + src * ldq + d0 + d);
                }
                qs[d * (QPB + 4) + q] = val;
            }
            for (int i = tid; i < kNT * kKC; i += kThreads) {
                int j = i / kKC, d = i - j * kKC;
                float val = 0.f;
                if (n0 + j < n_end && d0 + d < D) val = __ldg(corpus + (n0 + j) * ldc + d0 + d);
                cs[d * (kNT + 4) + j] = val;
            }
            __syncthreads();
            const int dlim = min(kKC, D - d0);
            for (int d = 0; d < dlim; ++d) {
                float a[RQ];
#pragma unroll
                for (int r = 0; r < RQ; ++r) a[r] = qs[d * (QPB + 4) + ty * RQ + r];
                float4 b = *reinterpret_cast<const float4*>(cs + d * (kNT + 4) + tx * 4);
#pragma unroll
                for (int r = 0; r < RQ; ++r) {
                    acc[r][0] = __fmaf_rn(a[r], b.x, acc[r][0]);
                    acc[r][1] = __fmaf_rn(a[r], b.y, acc[r][1]);
                    acc[r][2] = __fmaf_rn(a[r], b.z, acc[r][2]);
                    acc[r][3] = __fmaf_rn(a[r], b.w, acc[r][3]);
                }
            }
            __syncthreads();
        }
#pragma unroll
        for (int r = 0; r < RQ; ++r)
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                int j = tx * 4 + c;
                int64_t n = n0 + j;
                // cn is padded with +inf to a multiple of 128 rows
                float key = n < n_end ? __fmaf_rn(-2.0f, acc[r][c], __ldg(cn + n))
                                      : __int_as_float(0x7f800000);
                tile[(ty * RQ + r) * (kNT + 1) + j] = key;
            }
        __syncthreads();
        if (owner) {
            const float thr_glob = thr_g ? shared_thr_of(__ldcg(thr_g + q)) : __int_as_float(0x7f800000);
#pragma unroll 1
            for (int j0 = 0; j0 < kNT; j0 += 32) {
                const float* row = tile + tid * (kNT + 1) + j0;
                float key[32];
#pragma unroll
                for (int j = 0; j < 32; ++j) key[j] = row[j];
                const float thr = fminf(st.thr_local, thr_glob);
                if (__any_sync(0xffffffffu, min32(key) < thr))
                    st = offer_staged(v, row, (uint32_t)(n0 + j0), tid, st, thr_glob, thr_g, q);
            }
        }
        __syncthreads();
    }
    if (owner) st = flush_all(v, tid, st);
    __syncthreads();
    uint64_t* out = part + ((size_t)blockIdx.y * Q + q0) * kp;
    const int64_t nq = min((int64_t)QPB, qvalid - q0);
    for (int64_t i = tid; i < nq * kp; i += kThreads) out[i] = v.list[i];
}

size_t simt_smem_bytes(int qpb, int kp)
{
    return ((simt_gemm_bytes(qpb) + 15) & ~size_t(15)) + (size_t)qpb * kp * 8 + (size_t)kBufCap * qpb * 8;
}

cudaError_t launch_simt(const float* corpus, int64_t N, int64_t ldc, const float* cn,
                        const float* queries, int64_t Q, int64_t ldq, int D, int kp, int qpb,
                        int64_t split_len, int splits, uint64_t* part, uint32_t* thr_g, cudaStream_t s,
                        const uint32_t* tile_redo, const int32_t* qmap, const uint32_t* qcount, int64_t qbase)
{
    if ((qmap == nullptr) != (qcount == nullptr) || qbase < 0) return cudaErrorInvalidValue;
    size_t smem = simt_smem_bytes(qpb, kp);
    dim3 grid((unsigned)((Q + qpb - 1) / qpb), (unsigned)splits);
    if (qpb == 128) {
        cudaError_t e = cudaFuncSetAttribute(simt_kernel<128>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
        if (e != cudaSuccess) return e;
        simt_kernel<128><<<grid, kThreads, smem, s>>>(corpus, N, ldc, cn, queries, Q, ldq, D, kp,
                                                      split_len, part, thr_g, tile_redo, qmap, qcount, qbase);
    } else {
        cudaError_t e = cudaFuncSetAttribute(simt_kernel<32>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
        if (e != cudaSuccess) return e;
        simt_kernel<32><<<grid, kThreads, smem, s>>>(corpus, N, ldc, cn, queries, Q, ldq, D, kp,
                                                     split_len, part, thr_g, tile_redo, qmap, qcount, qbase);
    }
    return cudaGetLastError();
}

}  // namespace knn
