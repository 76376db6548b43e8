// scan_common.cuh -- epilogue helpers shared by the threshold scans (scan_bf16.cu,
// scan_tf32.cu): keys of a chunk of accumulator columns, the test against the
// query's threshold, and the append of the keys below it to the query's segment.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>
#include "tc_ptx.cuh"

namespace knn {
namespace {

// Minimum of 8 keys (four min instructions).
__device__ __forceinline__ float min8(const float* k)
{
    return fminf(ptx::fmin3(ptx::fmin3(k[0], k[1], k[2]), ptx::fmin3(k[3], k[4], k[5]), k[6]), k[7]);
}

// Keys ||c||^2 - 2 q.c of a W-column chunk and the mask of its 8-column groups
// that hold a key below the lane's threshold.  BF16: q.c = acc, m = -2;
// E4M3: q.c = s_q s_c acc with m = -2 s_q and the corpus scales s_c at scl.
template <int W, bool kF8>
__device__ __forceinline__ uint32_t chunk_keys(const float (&v)[W], const float* nrm, const float* scl, float m,
                                               float T, float (&key)[W])
{
    const float4* n4 = reinterpret_cast<const float4*>(nrm);
    const float4* s4 = reinterpret_cast<const float4*>(scl);
#pragma unroll
    for (int u = 0; u < W / 4; ++u) {
        const float4 c = n4[u];
        if (kF8) {
            const float4 sc = s4[u];
            float t0, t1, t2, t3;
            ptx::mul2(t0, t1, v[4 * u], v[4 * u + 1], sc.x, sc.y);
            ptx::mul2(t2, t3, v[4 * u + 2], v[4 * u + 3], sc.z, sc.w);
            ptx::fma2(key[4 * u], key[4 * u + 1], t0, t1, m, c.x, c.y);
            ptx::fma2(key[4 * u + 2], key[4 * u + 3], t2, t3, m, c.z, c.w);
        } else {
            ptx::fma2(key[4 * u], key[4 * u + 1], v[4 * u], v[4 * u + 1], m, c.x, c.y);
            ptx::fma2(key[4 * u + 2], key[4 * u + 3], v[4 * u + 2], v[4 * u + 3], m, c.z, c.w);
        }
    }
    // groups of 8 columns (4 for the 4-column chunk)
    constexpr int G = W < 8 ? W : 8;
    uint32_t gm = 0;
#pragma unroll
    for (int g = 0; g < W / G; ++g) {
        const float* kg = key + G * g;
        const float mn = G == 8 ? min8(kg) : fminf(ptx::fmin3(kg[0], kg[1], kg[2]), kg[G - 1]);
        gm |= (mn < T ? 1u : 0u) << g;
    }
    return gm;
}

// Mask of the 8-column groups of a W-column chunk of keys that hold a key below T.
template <int W>
__device__ __forceinline__ uint32_t chunk_test(const float (&key)[W], float T)
{
    constexpr int G = W < 8 ? W : 8;
    uint32_t gm = 0;
#pragma unroll
    for (int g = 0; g < W / G; ++g) {
        const float* kg = key + G * g;
        const float mn = G == 8 ? min8(kg) : fminf(ptx::fmin3(kg[0], kg[1], kg[2]), kg[G - 1]);
        gm |= (mn < T ? 1u : 0u) << g;
    }
    return gm;
}

// Keys of the columns at or past `rem` (rows past the corpus view in its last tile) set to +inf.
template <int W>
__device__ __forceinline__ void chunk_mask(float (&key)[W], int c0, int rem)
{
#pragma unroll
    for (int j = 0; j < W; ++j)
        if (c0 + j >= rem) key[j] = __int_as_float(0x7f800000);
}

// Append the keys below T of the flagged groups, in increasing corpus index.
// Words hold the raw key bits above the index; the selection maps them to
// ordered keys.  A lane whose group holds a single key below T (the usual case
// where a warp appends at all) stores the group's minimum at the key's position
// found from the mask of hits; more hits take the column walk.
template <int W>
__device__ __forceinline__ void chunk_append(const float (&key)[W], uint32_t gm, float T, uint32_t base,
                                             uint64_t* out, uint32_t cap, uint32_t& cnt)
{
    constexpr int G = W < 8 ? W : 8;
#pragma unroll
    for (int g = 0; g < W / G; ++g) {
        if ((gm >> g) & 1u) {
            const float* kg = key + G * g;
            uint32_t hm = 0;
#pragma unroll
            for (int j = 0; j < G; ++j) hm |= (kg[j] < T ? 1u : 0u) << j;
            if ((hm & (hm - 1u)) == 0u) {
                const float k = G == 8 ? min8(kg) : fminf(ptx::fmin3(kg[0], kg[1], kg[2]), kg[G - 1]);
                if (cnt < cap)
                    out[cnt] = ((uint64_t)__float_as_uint(k) << 32) |
                               (uint64_t)(base + (uint32_t)(G * g + __ffs((int)hm) - 1));
                ++cnt;
            } else {
#pragma unroll
                for (int j = 0; j < G; ++j) {
                    const float k = kg[j];
                    const bool h = k < T;
                    if (h && cnt < cap)
                        out[cnt] = ((uint64_t)__float_as_uint(k) << 32) | (uint64_t)(base + (uint32_t)(G * g + j));
                    cnt += h ? 1u : 0u;
                }
            }
        }
    }
}

}  // namespace
}  // namespace knn
