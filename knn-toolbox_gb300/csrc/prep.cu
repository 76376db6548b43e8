// prep.cu -- corpus/query preparation: row norms and the TF32 hi/lo split.
//
// Replaces the reference's norm kernels crpdot2_* / dot4_* (include/utils.h:72-357,
// 516-766), which reduce x_d^2 in float with a warp-synchronous tree.  Here a
// row norm is the float rounding of a double sum taken in d order (exact for
// the integer-valued data of the 1M x 128 workload and within one rounding of
// exact otherwise); the same convention is used by the CPU oracle.
#include <algorithm>
#include <cstdint>
#include <cuda_bf16.h>
#include <cuda_fp8.h>
#include <cuda_runtime.h>
#include "common.cuh"
#include "kernels.h"

namespace knn {

__global__ void norms_kernel(const float* __restrict__ x, int64_t n, int64_t ld, int D,
                             float* __restrict__ out, int64_t n_pad)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_pad) return;
    if (i >= n) {  // padding rows never enter a shortlist
        out[i] = __int_as_float(0x7f800000);
        return;
    }
    const float* r = x + i * ld;
    double acc = 0.0;
    int d = 0;
    for (; d + 4 <= D; d += 4) {
        float a = __ldg(r + d), b = __ldg(r + d + 1), c = __ldg(r + d + 2), e = __ldg(r + d + 3);
        acc = __fma_rn((double)a, (double)a, acc);
        acc = __fma_rn((double)b, (double)b, acc);
        acc = __fma_rn((double)c, (double)c, acc);
        acc = __fma_rn((double)e, (double)e, acc);
    }
    for (; d < D; ++d) {
        float a = __ldg(r + d);
        acc = __fma_rn((double)a, (double)a, acc);
    }
    out[i] = __double2float_rn(acc);
}

// Round a float to the nearest TF32 value (10 explicit mantissa bits, ties to
// even), returned as a float whose low 13 bits are zero.
__device__ __forceinline__ float tf32_rne(float x)
{
    uint32_t u = __float_as_uint(x);
    if ((u & 0x7f800000u) == 0x7f800000u) return x;  // inf / nan unchanged
    u += 0xfffu + ((u >> 13) & 1u);
    u &= 0xffffe000u;
    return __uint_as_float(u);
}

// BF16 copy of a row-major matrix, rows padded with zeros to dpb columns, and
// a global "not exactly representable" flag: *not_exact becomes 1 when some
// element differs from its BF16 rounding (inf/nan count as not exact).  One
// block per 128-row tile.
__global__ void bf16_tiles_kernel(const float* __restrict__ x, int64_t n, int64_t ld, int D, int dpb,
                                  __nv_bfloat16* __restrict__ out, uint32_t* __restrict__ not_exact)
{
    const int64_t r0 = (int64_t)blockIdx.x * 128;
    const int64_t rows = min((int64_t)128, n - r0);
    const int64_t total = rows * dpb;
    int bad = 0;
    for (int64_t i = threadIdx.x; i < total; i += blockDim.x) {
        const int64_t r = r0 + i / dpb;
        const int c = (int)(i % dpb);
        const float v = c < D ? __ldg(x + r * ld + c) : 0.f;
        const __nv_bfloat16 b = __float2bfloat16_rn(v);
        if (out) out[r * dpb + c] = b;
        bad |= !(__bfloat162float(b) == v);
    }
    bad = __syncthreads_or(bad);
    if (threadIdx.x == 0 && bad) atomicOr(not_exact, 1u);
}

// hi = tf32(x), lo = tf32(x - hi); rows padded with zeros to dp columns.
// One block per 128-row tile; lo_flags[tile] = 1 when any lo in the tile is
// nonzero (the tensor-core kernel skips the correction products otherwise).
__global__ void split_tiles_kernel(const float* __restrict__ x, int64_t n, int64_t ld, int D, int dp,
                                   float* __restrict__ hi, float* __restrict__ lo, uint32_t* __restrict__ lo_flags,
                                   uint32_t* __restrict__ any_lo, const uint32_t* __restrict__ skip_unless)
{
    // BF16-exact inputs are searched by the BF16 kernel: nothing to prepare
    if (skip_unless && *skip_unless == 0u) return;
    const int64_t r0 = (int64_t)blockIdx.x * 128;
    const int64_t rows = min((int64_t)128, n - r0);
    const int64_t total = rows * dp;
    int any = 0;
    for (int64_t i = threadIdx.x; i < total; i += blockDim.x) {
        const int64_t r = r0 + i / dp;
        const int c = (int)(i % dp);
        const float v = c < D ? __ldg(x + r * ld + c) : 0.f;
        const float h = tf32_rne(v);
        const float l = tf32_rne(__fsub_rn(v, h));
        hi[r * dp + c] = h;
        lo[r * dp + c] = l;
        any |= (l != 0.f);
    }
    any = __syncthreads_or(any);
    if (threadIdx.x == 0) {
        if (lo_flags) lo_flags[blockIdx.x] = any ? 1u : 0u;
        if (any && any_lo) atomicOr(any_lo, 1u);
    }
}

__global__ void gather_norms_kernel(const float* __restrict__ src, int64_t n, int64_t stride, float* __restrict__ out,
                                    int64_t n_pad, float pad)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_pad) return;
    out[i] = i < n ? src[i * stride] : pad;
}

// Fused preparation of a row-major matrix in one coalesced read: rows staged in
// shared memory ([rows][pitch], pitch odd: conflict-free per-row walks), then
//  * BF16 copy into out[n][dpb] (zero padded) and the "not exactly
//    representable" flag (*not_exact |= 1), when out / not_exact are given;
//  * E4M3 copy into f8[n][f8_bytes] (zero padded) with per-row absmax scales
//    (scale = max|x| / 448, codes = satfinite(x * 448 / max|x|)), when given;
//  * row norms into norms[0..n_pad) (+inf for n <= i < n_pad), when given:
//    the float rounding of the double sum of x_d^2 in d order.  A row of
//    integers whose float sum stays below 2^24 is summed in float: every
//    partial sum is then an exact integer, so the result is the same value.
template <int kRows>
__global__ void __launch_bounds__(256) prep_rows_kernel(const float* __restrict__ x, int64_t n, int64_t ld, int D,
                                                        int dpb, __nv_bfloat16* __restrict__ out,
                                                        float* __restrict__ norms, int64_t n_pad,
                                                        uint32_t* __restrict__ not_exact,
                                                        uint32_t* __restrict__ int_stats,
                                                        uint8_t* __restrict__ f8, int f8_bytes,
                                                        float* __restrict__ scales)
{
    extern __shared__ float tile[];
    const int pitch = D | 1;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t r0 = (int64_t)blockIdx.x * kRows;
    const int rows = (int)max((int64_t)0, min((int64_t)kRows, n - r0));
    for (int r = warp; r < rows; r += 8) {
        const float* src = x + (r0 + r) * ld;
        for (int c = lane; c < D; c += 32) tile[r * pitch + c] = __ldg(src + c);
    }
    __syncthreads();
    if (int_stats != nullptr) {
        // integrality and magnitude of the data: int_stats[0] |= 1 when some value is not an
        // integer, int_stats[1] = max(|x|) as float bits (non-negative floats order as integers)
        int frac = 0;
        float mx = 0.f;
        for (int r = warp; r < rows; r += 8)
            for (int c = lane; c < D; c += 32) {
                const float v = tile[r * pitch + c];
                frac |= !(v == rintf(v));
                mx = fmaxf(mx, fabsf(v));
            }
        frac = __syncthreads_or(frac);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        if (lane == 0) atomicMax(int_stats + 1, __float_as_uint(mx));
        if (threadIdx.x == 0 && frac) atomicOr(int_stats, 1u);
    }
    if (out != nullptr || not_exact != nullptr) {
        int bad = 0;
        for (int r = warp; r < rows; r += 8) {
            for (int c = 2 * lane; c < dpb; c += 64) {
                const float v0 = c < D ? tile[r * pitch + c] : 0.f;
                const float v1 = c + 1 < D ? tile[r * pitch + c + 1] : 0.f;
                const __nv_bfloat162 b = __floats2bfloat162_rn(v0, v1);
                if (out) *reinterpret_cast<__nv_bfloat162*>(out + (r0 + r) * dpb + c) = b;
                bad |= !(__low2float(b) == v0) | !(__high2float(b) == v1);
            }
        }
        bad = __syncthreads_or(bad);
        if (threadIdx.x == 0 && bad && not_exact) atomicOr(not_exact, 1u);
    }
    if (f8 != nullptr) {
        for (int r = warp; r < rows; r += 8) {
            const float* row = tile + r * pitch;
            float mx = 0.f;
            for (int c = lane; c < D; c += 32) mx = fmaxf(mx, fabsf(row[c]));
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
            const float inv = mx > 0.f ? 448.f / mx : 0.f;
            uint32_t* dst = reinterpret_cast<uint32_t*>(f8 + (r0 + r) * (int64_t)f8_bytes);
            for (int c = 4 * lane; c < f8_bytes; c += 128) {
                float v[4];
#pragma unroll
                for (int j = 0; j < 4; ++j) v[j] = c + j < D ? row[c + j] * inv : 0.f;
                const uint32_t lo = __nv_cvt_float2_to_fp8x2(make_float2(v[0], v[1]), __NV_SATFINITE, __NV_E4M3);
                const uint32_t hi = __nv_cvt_float2_to_fp8x2(make_float2(v[2], v[3]), __NV_SATFINITE, __NV_E4M3);
                dst[c >> 2] = lo | (hi << 16);
            }
            if (lane == 0) scales[r0 + r] = mx / 448.f;
        }
        for (int r = rows + (int)threadIdx.x; r < kRows && r0 + r < n_pad; r += blockDim.x) scales[r0 + r] = 0.f;
    }
    if (norms != nullptr && threadIdx.x < kRows) {
        const int64_t i = r0 + threadIdx.x;
        if (i < n) {
            const float* row = tile + threadIdx.x * pitch;
            float s32 = 0.f;
            bool ints = true;
            for (int d = 0; d < D; ++d) {
                const float v = row[d];
                ints &= v == rintf(v);
                s32 = __fmaf_rn(v, v, s32);
            }
            if (!(ints && s32 < 16777216.f)) {
                double acc = 0.0;
                for (int d = 0; d < D; ++d) {
                    const double v = (double)row[d];
                    acc = __fma_rn(v, v, acc);
                }
                s32 = __double2float_rn(acc);
            }
            norms[i] = s32;
        } else if (i < n_pad) {
            norms[i] = __int_as_float(0x7f800000);
        }
    }
}

cudaError_t launch_prep_rows(const float* x, int64_t n, int64_t ld, int D, int dpb, void* out, float* norms,
                             int64_t n_pad, uint32_t* not_exact, cudaStream_t s, uint32_t* int_stats, void* f8,
                             int f8_bytes, float* scales)
{
    const int64_t rows = std::max(n, (norms || scales) ? n_pad : n);
    if (rows <= 0) return cudaSuccess;
    const int pitch = D | 1;
    if (f8 != nullptr && (D > kPrepMaxD || scales == nullptr || f8_bytes % 128 != 0 || f8_bytes < D))
        return cudaErrorInvalidValue;
    uint8_t* f8b = static_cast<uint8_t*>(f8);
    if (D > kPrepMaxD) {
        // wide rows: separate passes
        cudaError_t e = cudaSuccess;
        if (norms) e = launch_norms(x, n, ld, D, norms, n_pad, s);
        if (e == cudaSuccess && (out || not_exact)) e = launch_bf16(x, n, ld, D, dpb, out, not_exact, s);
        if (e == cudaSuccess && int_stats) e = cudaMemsetAsync(int_stats, 0xFF, sizeof(uint32_t), s);  // unknown
        return e;
    }
    if (D <= 128) {
        const size_t smem = (size_t)128 * pitch * 4;
        cudaError_t e = cudaFuncSetAttribute(prep_rows_kernel<128>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
        if (e != cudaSuccess) return e;
        prep_rows_kernel<128><<<(unsigned)((rows + 127) / 128), 256, smem, s>>>(
            x, n, ld, D, dpb, static_cast<__nv_bfloat16*>(out), norms, n_pad, not_exact, int_stats, f8b, f8_bytes,
            scales);
    } else {
        const size_t smem = (size_t)64 * pitch * 4;
        cudaError_t e = cudaFuncSetAttribute(prep_rows_kernel<64>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
        if (e != cudaSuccess) return e;
        prep_rows_kernel<64><<<(unsigned)((rows + 63) / 64), 256, smem, s>>>(
            x, n, ld, D, dpb, static_cast<__nv_bfloat16*>(out), norms, n_pad, not_exact, int_stats, f8b, f8_bytes,
            scales);
    }
    return cudaGetLastError();
}

cudaError_t launch_gather_norms(const float* src, int64_t n, int64_t stride, float* out, int64_t n_pad,
                                cudaStream_t s, float pad)
{
    if (n_pad <= 0) return cudaSuccess;
    gather_norms_kernel<<<(unsigned)((n_pad + 255) / 256), 256, 0, s>>>(src, n, stride, out, n_pad, pad);
    return cudaGetLastError();
}

cudaError_t launch_norms(const float* x, int64_t n, int64_t ld, int D, float* out, int64_t n_pad,
                         cudaStream_t s)
{
    if (n_pad <= 0) return cudaSuccess;
    int threads = 256;
    int64_t blocks = (n_pad + threads - 1) / threads;
    norms_kernel<<<(unsigned)blocks, threads, 0, s>>>(x, n, ld, D, out, n_pad);
    return cudaGetLastError();
}

cudaError_t launch_split(const float* x, int64_t n, int64_t ld, int D, int dp, float* hi, float* lo,
                         uint32_t* lo_flags, uint32_t* any_lo, const uint32_t* skip_unless, cudaStream_t s)
{
    if (n <= 0) return cudaSuccess;
    const int64_t tiles = (n + 127) / 128;
    split_tiles_kernel<<<(unsigned)tiles, 256, 0, s>>>(x, n, ld, D, dp, hi, lo, lo_flags, any_lo, skip_unless);
    return cudaGetLastError();
}

cudaError_t launch_bf16(const float* x, int64_t n, int64_t ld, int D, int dpb, void* out, uint32_t* not_exact,
                        cudaStream_t s)
{
    if (n <= 0) return cudaSuccess;
    const int64_t tiles = (n + 127) / 128;
    bf16_tiles_kernel<<<(unsigned)tiles, 256, 0, s>>>(x, n, ld, D, dpb, static_cast<__nv_bfloat16*>(out), not_exact);
    return cudaGetLastError();
}

}  // namespace knn
