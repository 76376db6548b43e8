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
// One block per 128-row tile, one warp per row at a time (eight rows in flight per block), each
// lane a float4 of columns: coalesced 16-byte loads and stores.  lo_flags[tile] = 1 when any lo
// in the tile is nonzero (the tensor-core kernels skip the correction products otherwise).
__global__ void __launch_bounds__(256) split_tiles_kernel(const float* __restrict__ x, int64_t n, int64_t ld, int D,
                                                          int dp, float* __restrict__ hi, float* __restrict__ lo,
                                                          uint32_t* __restrict__ lo_flags,
                                                          uint32_t* __restrict__ any_lo,
                                                          const uint32_t* __restrict__ skip_unless)
{
    // BF16-exact inputs are searched by the BF16 kernels: nothing to prepare
    if (skip_unless && *skip_unless == 0u) return;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t r0 = (int64_t)blockIdx.x * 128;
    // 16-byte loads when every row starts 16-byte aligned and holds whole float4s
    const bool vec = (ld % 4 == 0) && (D % 4 == 0) && ((reinterpret_cast<uintptr_t>(x) & 15u) == 0);
    int any = 0;
    for (int rr = warp; rr < 128; rr += 8) {
        const int64_t r = r0 + rr;
        if (r >= n) break;  // warp-uniform
        const float* row = x + r * ld;
        float4* H = reinterpret_cast<float4*>(hi + r * dp);
        float4* L = reinterpret_cast<float4*>(lo + r * dp);
        for (int c = 4 * lane; c < dp; c += 128) {
            float v[4];
            if (vec) {
                float4 t = make_float4(0.f, 0.f, 0.f, 0.f);
                if (c < D) t = __ldg(reinterpret_cast<const float4*>(row + c));
                v[0] = t.x;
                v[1] = t.y;
                v[2] = t.z;
                v[3] = t.w;
            } else {
#pragma unroll
                for (int i = 0; i < 4; ++i) v[i] = c + i < D ? __ldg(row + c + i) : 0.f;
            }
            float h[4], l[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                h[i] = tf32_rne(v[i]);
                l[i] = tf32_rne(__fsub_rn(v[i], h[i]));
                any |= (l[i] != 0.f);
            }
            H[c >> 2] = make_float4(h[0], h[1], h[2], h[3]);
            L[c >> 2] = make_float4(l[0], l[1], l[2], l[3]);
        }
    }
    any = __syncthreads_or(any);
    if (threadIdx.x == 0) {
        if (lo_flags) lo_flags[blockIdx.x] = any ? 1u : 0u;
        if (any && any_lo) atomicOr(any_lo, 1u);
    }
}

__global__ void gather_norms_kernel(const float* __restrict__ src, int64_t n, int64_t stride, float* __restrict__ out,
                                    int64_t n_pad, float pad, const uint32_t* __restrict__ skip_unless)
{
    if (skip_unless && *skip_unless == 0u) return;
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_pad) return;
    out[i] = i < n ? src[i * stride] : pad;
}

// Fused preparation of a row-major matrix in one coalesced read, one warp per
// row: lane l holds columns 128 j + 4 l .. 128 j + 4 l + 3 of every 128-column
// chunk j < kChunks (float4 loads when rows are 16-byte aligned), kU rows per
// warp in flight.  Per row, as requested:
//  * BF16 copy into out[n][dpb] (zero padded) and the "not exactly
//    representable" flag (*not_exact |= 1);
//  * integrality and magnitude: int_stats[0] |= 1 when some value is not an
//    integer, int_stats[1] = max |x| as float bits;
//  * E4M3 copy into f8[n][f8_bytes] (zero padded) with per-row absmax scales
//    (scale = max|x| / 448, codes = satfinite(x * 448 / max|x|));
//  * row norms into norms[0..n_pad) (+inf for n <= i < n_pad): the float
//    rounding of the double sum of x_d^2 taken in d order (the convention of
//    norms_kernel and the CPU oracle), certified from a float-float sum -- see
//    certified_norm -- with the serial double loop for the rare rows the
//    certificate does not settle.
struct PrepArgs {
    const float* x;
    int64_t n, ld, n_pad;
    int D, dpb, f8_bytes, vec;
    __nv_bfloat16* out;
    float* norms;
    uint32_t* not_exact;
    uint32_t* int_stats;
    uint8_t* f8;
    float* scales;
    __nv_bfloat16* np;  // optional: norm parts, kNormParts BF16 per row
};

// s + t = a + b exactly (Knuth's TwoSum; no contraction: explicit roundings)
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& t)
{
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    t = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// Norm of a row from the lanes' float-float partial sums (hi, lo).  The TwoSums
// are exact, so S_ff = hi + lo differs from the exact sum S only by the roundings
// of the lo additions and by residuals of squares below the float range
// (< 2^-149 each).  Every term folded into lo is at most 2^-24 of a partial sum:
// a lane's TwoSum residuals total at most m 2^-24 of its share of S (m <= 12
// elements), its square residuals 2^-24 of it, and the 31 butterfly TwoSums 2^-24 S
// each, so the terms total E <= 44 2^-24 S.  A lane's 2m lo roundings err by at
// most 2^-24 of its share of E each and the 5 butterfly levels by 2 2^-24 E, so
// |S_ff - S| <= 34 2^-24 E + D 2^-149 < 2^-36 S + D 2^-149.  The double d-order sum
// differs from S by at most D 2^-52 S.  When [S_ff - B, S_ff + B] (B the sum of
// both bounds, S bounded by 1.01 (hi + |lo|)) lies strictly inside the rounding
// interval of f = fl(S_ff) -- half the spacing below f on one side, half the
// spacing above on the other (they differ at powers of two) -- the double sum
// rounds to f as well; otherwise the caller recomputes the row in double.
__device__ __forceinline__ bool certified_norm(float hi, float lo, int D, float& f)
{
    f = __fadd_rn(hi, lo);
    if (!(f >= 0x1p-100f && f <= 0x1p126f)) return false;  // also rejects nan
    const float r = __fadd_rn(__fsub_rn(hi, f), lo);        // S_ff - f: hi - f exact (Sterbenz)
    const float S = 1.01f * (hi + fabsf(lo));
    const float B = (0x1p-36f + (float)D * 0x1p-52f) * S + 0x1p-139f;
    const float rr = fabsf(r) * 0.0001f;                      // rounding of r itself
    const float h_dn = 0.5f * (f - nextafterf(f, 0.f));
    const float h_up = 0.5f * (nextafterf(f, 0x1p127f) - f);
    return r + rr + B < h_up && r - rr - B > -h_dn;
}

// (h, l) += (oh, ol) as float-float: exact TwoSum of the high parts, the low parts and
// the residual added.  Symmetric: both partners of a butterfly step get the same values
// (the TwoSum residual is the exact error whatever the operand order).
__device__ __forceinline__ void ff_add(float& h, float& l, float oh, float ol)
{
    float s, t;
    two_sum(h, oh, s, t);
    h = s;
    l = __fadd_rn(__fadd_rn(l, ol), t);
}

// Sums of kU rows' float-float partials over the warp, transposed: the first log2(kU)
// levels halve the rows a lane holds (it keeps the rows of its half of the warp and
// receives its partner's partials of them), the remaining levels are a butterfly within
// groups of 32 / kU lanes.  Each row is still summed by a complete pairwise tree of depth
// 5 over the 32 lanes' partials (31 exact TwoSums, low parts added along paths of 5
// levels), so certified_norm's bound holds as for a plain 32-lane butterfly, at a quarter
// of the shuffles for four rows.  Lane l ends with row l / (32 / kU), identical across
// its group.
template <int kU>
__device__ __forceinline__ void ff_reduce_rows(const float (&hi)[kU], const float (&lo)[kU], int lane, float& h,
                                               float& l)
{
    static_assert(kU == 1 || kU == 2 || kU == 4, "1, 2 or 4 rows per warp");
    constexpr unsigned kAll = 0xffffffffu;
    if constexpr (kU == 4) {
        const bool up = (lane & 16) != 0;  // keeps rows 2, 3 (else 0, 1)
        float h0 = up ? hi[2] : hi[0], l0 = up ? lo[2] : lo[0];
        float h1 = up ? hi[3] : hi[1], l1 = up ? lo[3] : lo[1];
        const float s0h = up ? hi[0] : hi[2], s0l = up ? lo[0] : lo[2];
        const float s1h = up ? hi[1] : hi[3], s1l = up ? lo[1] : lo[3];
        ff_add(h0, l0, __shfl_xor_sync(kAll, s0h, 16), __shfl_xor_sync(kAll, s0l, 16));
        ff_add(h1, l1, __shfl_xor_sync(kAll, s1h, 16), __shfl_xor_sync(kAll, s1l, 16));
        const bool up3 = (lane & 8) != 0;  // keeps the second of the two
        h = up3 ? h1 : h0;
        l = up3 ? l1 : l0;
        const float sh = up3 ? h0 : h1, sl = up3 ? l0 : l1;
        ff_add(h, l, __shfl_xor_sync(kAll, sh, 8), __shfl_xor_sync(kAll, sl, 8));
    } else if constexpr (kU == 2) {
        const bool up = (lane & 16) != 0;  // keeps row 1 (else 0)
        h = up ? hi[1] : hi[0];
        l = up ? lo[1] : lo[0];
        const float sh = up ? hi[0] : hi[1], sl = up ? lo[0] : lo[1];
        ff_add(h, l, __shfl_xor_sync(kAll, sh, 16), __shfl_xor_sync(kAll, sl, 16));
    } else {
        h = hi[0];
        l = lo[0];
    }
    constexpr int kFirst = kU == 4 ? 4 : kU == 2 ? 8 : 16;
#pragma unroll
    for (int o = kFirst; o > 0; o >>= 1) ff_add(h, l, __shfl_xor_sync(kAll, h, o), __shfl_xor_sync(kAll, l, o));
}

// v[g] for a lane-dependent g < kU without indexing a register array
template <int kU>
__device__ __forceinline__ float pick_row(const float (&v)[kU], int g)
{
    float x = v[0];
#pragma unroll
    for (int u = 1; u < kU; ++u) x = g == u ? v[u] : x;
    return x;
}

// The norm f as three BF16 parts, then zeros: one 32-byte row of the operand that adds ||c||^2
// inside the BF16 scan's MMA.  n1 + n2 + n3 == f exactly for f = 0 and f >= 2^-100 (each
// remainder is exact by Sterbenz's lemma, a multiple of f's FP32 ulp, and the last one holds at
// most 8 significant bits, all within BF16's normal range); smaller norms are kept to within
// 2^-133, BF16's subnormal spacing.  Norms that are not finite in BF16 (past 3.39e38) keep n1
// alone (+inf).
__device__ __forceinline__ void store_norm_parts(__nv_bfloat16* dst, float f)
{
    const __nv_bfloat16 n1 = __float2bfloat16_rn(f);
    __nv_bfloat16 n2 = __float2bfloat16_rn(0.f), n3 = n2;
    if (isfinite(__bfloat162float(n1))) {
        const float r1 = __fsub_rn(f, __bfloat162float(n1));
        n2 = __float2bfloat16_rn(r1);
        n3 = __float2bfloat16_rn(__fsub_rn(r1, __bfloat162float(n2)));
    }
    uint4 w0;
    w0.x = (uint32_t)__bfloat16_as_ushort(n1) | ((uint32_t)__bfloat16_as_ushort(n2) << 16);
    w0.y = (uint32_t)__bfloat16_as_ushort(n3);
    w0.z = 0u;
    w0.w = 0u;
    static_assert(kNormParts * 2 == 2 * sizeof(uint4), "one row of norm parts is two 16-byte words");
    uint4* d = reinterpret_cast<uint4*>(dst);
    d[0] = w0;
    d[1] = make_uint4(0u, 0u, 0u, 0u);
}

template <int kChunks, int kU>
__global__ void __launch_bounds__(256) prep_rows_kernel(const PrepArgs p)
{
    const int lane = threadIdx.x & 31;
    const int64_t gw = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int D = p.D;
    int frac = 0, bad = 0;
    float mx_all = 0.f;
    for (int64_t base = gw * kU; base < p.n; base += nw * kU) {
        float v[kU][kChunks][4];
#pragma unroll
        for (int u = 0; u < kU; ++u) {
            const int64_t r = base + u;
            const float* row = p.x + (r < p.n ? r : 0) * p.ld;
#pragma unroll
            for (int j = 0; j < kChunks; ++j) {
                const int c = 128 * j + 4 * lane;
                if (p.vec) {
                    float4 t = make_float4(0.f, 0.f, 0.f, 0.f);
                    if (r < p.n && c < D) t = __ldg(reinterpret_cast<const float4*>(row + c));
                    v[u][j][0] = t.x;
                    v[u][j][1] = t.y;
                    v[u][j][2] = t.z;
                    v[u][j][3] = t.w;
                } else {
#pragma unroll
                    for (int i = 0; i < 4; ++i) v[u][j][i] = (r < p.n && c + i < D) ? __ldg(row + c + i) : 0.f;
                }
            }
        }
        // per row: integrality and max |x| (in every lane); rows past n hold zeros and change
        // nothing
        float rmx[kU];
        bool rinteger[kU];
#pragma unroll
        for (int u = 0; u < kU; ++u) {
            float mx = 0.f;
            int rfrac = 0;
#pragma unroll
            for (int j = 0; j < kChunks; ++j)
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    const float x = v[u][j][i];  // zero past D
                    rfrac |= !(x == rintf(x));
                    mx = fmaxf(mx, fabsf(x));
                }
            frac |= rfrac;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
            rmx[u] = mx;
            rinteger[u] = !__any_sync(0xffffffffu, rfrac);
        }
#pragma unroll
        for (int u = 0; u < kU; ++u) {
            const int64_t r = base + u;
            if (r >= p.n) break;  // warp-uniform
            if (p.out != nullptr || p.not_exact != nullptr) {
#pragma unroll
                for (int j = 0; j < kChunks; ++j) {
                    const int c = 128 * j + 4 * lane;
                    const __nv_bfloat162 b0 = __floats2bfloat162_rn(v[u][j][0], v[u][j][1]);
                    const __nv_bfloat162 b1 = __floats2bfloat162_rn(v[u][j][2], v[u][j][3]);
                    bad |= !(__low2float(b0) == v[u][j][0]) | !(__high2float(b0) == v[u][j][1]) |
                           !(__low2float(b1) == v[u][j][2]) | !(__high2float(b1) == v[u][j][3]);
                    if (p.out != nullptr && c < p.dpb) {
                        uint2 w;
                        w.x = *reinterpret_cast<const uint32_t*>(&b0);
                        w.y = *reinterpret_cast<const uint32_t*>(&b1);
                        *reinterpret_cast<uint2*>(p.out + r * p.dpb + c) = w;
                    }
                }
            }
            // the row's max |x| (E4M3 scale, int_stats, the integer test of the norm)
            const float mx = rmx[u];
            mx_all = fmaxf(mx_all, mx);
            if (p.f8 != nullptr) {
                const float inv = mx > 0.f ? 448.f / mx : 0.f;
                uint32_t* dst = reinterpret_cast<uint32_t*>(p.f8 + r * (int64_t)p.f8_bytes);
#pragma unroll
                for (int j = 0; j < kChunks; ++j) {
                    const int c = 128 * j + 4 * lane;
                    if (c < p.f8_bytes) {
                        const uint32_t a = __nv_cvt_float2_to_fp8x2(make_float2(v[u][j][0] * inv, v[u][j][1] * inv),
                                                                    __NV_SATFINITE, __NV_E4M3);
                        const uint32_t b = __nv_cvt_float2_to_fp8x2(make_float2(v[u][j][2] * inv, v[u][j][3] * inv),
                                                                    __NV_SATFINITE, __NV_E4M3);
                        dst[c >> 2] = a | (b << 16);
                    }
                }
                if (lane == 0) p.scales[r] = mx / 448.f;
            }
        }
        if (p.norms != nullptr || p.np != nullptr) {
            // the kU rows' norms together: lane l settles row g = l / (32 / kU) of the batch
            constexpr int kGroup = 32 / kU;
            const int g = lane / kGroup;
            bool all_int = true;
#pragma unroll
            for (int u = 0; u < kU; ++u) all_int = all_int && rinteger[u] && (float)D * rmx[u] * rmx[u] < 16777216.f;
            float f;
            bool ok = true;
            if (all_int) {
                // integers whose squares sum below 2^24: every partial sum is an exact integer,
                // so any order gives the double sum's value
                float fr[kU];
#pragma unroll
                for (int u = 0; u < kU; ++u) {
                    float s32 = 0.f;
#pragma unroll
                    for (int j = 0; j < kChunks; ++j)
#pragma unroll
                        for (int i = 0; i < 4; ++i) s32 = __fmaf_rn(v[u][j][i], v[u][j][i], s32);
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1) s32 = __fadd_rn(s32, __shfl_xor_sync(0xffffffffu, s32, o));
                    fr[u] = s32;
                }
                f = pick_row(fr, g);
            } else {
                // float-float partials per lane (exact products split by fma, TwoSum additions)
                float hi[kU], lo[kU];
#pragma unroll
                for (int u = 0; u < kU; ++u) {
                    hi[u] = 0.f;
                    lo[u] = 0.f;
#pragma unroll
                    for (int j = 0; j < kChunks; ++j)
#pragma unroll
                        for (int i = 0; i < 4; ++i) {
                            const float x = v[u][j][i];
                            const float q = __fmul_rn(x, x);
                            const float qe = __fmaf_rn(x, x, -q);
                            float sum, t;
                            two_sum(hi[u], q, sum, t);
                            hi[u] = sum;
                            lo[u] = __fadd_rn(lo[u], __fadd_rn(t, qe));
                        }
                }
                float h, l;
                ff_reduce_rows<kU>(hi, lo, lane, h, l);
                ok = certified_norm(h, l, D, f);
                if (!ok && pick_row(rmx, g) == 0.f) {  // an all-zero row
                    ok = true;
                    f = 0.f;
                }
            }
            const int64_t r = base + g;
            if (lane % kGroup == 0 && r < p.n) {
                if (!ok) {
                    const float* row = p.x + r * p.ld;
                    double acc = 0.0;
                    for (int d = 0; d < D; ++d) {
                        const double a = (double)__ldg(row + d);
                        acc = __fma_rn(a, a, acc);
                    }
                    f = __double2float_rn(acc);
                }
                if (p.norms) p.norms[r] = f;
                if (p.np) store_norm_parts(p.np + r * kNormParts, f);
            }
        }
    }
    // padding rows past n
    for (int64_t i = p.n + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < p.n_pad;
         i += (int64_t)gridDim.x * blockDim.x) {
        if (p.norms) p.norms[i] = __int_as_float(0x7f800000);
        if (p.scales) p.scales[i] = 0.f;
    }
    // flags: one atomic per warp
    if (p.not_exact != nullptr && __any_sync(0xffffffffu, bad) && lane == 0) atomicOr(p.not_exact, 1u);
    if (p.int_stats != nullptr) {
        if (__any_sync(0xffffffffu, frac) && lane == 0) atomicOr(p.int_stats, 1u);
        if (lane == 0 && mx_all > 0.f) atomicMax(p.int_stats + 1, __float_as_uint(mx_all));
    }
}

cudaError_t launch_prep_rows(const float* x, int64_t n, int64_t ld, int D, int dpb, void* out, float* norms,
                             int64_t n_pad, uint32_t* not_exact, cudaStream_t s, uint32_t* int_stats, void* f8,
                             int f8_bytes, float* scales, void* np)
{
    const int64_t rows = std::max(n, (norms || scales) ? n_pad : n);
    if (rows <= 0) return cudaSuccess;
    if (f8 != nullptr && (D > kPrepMaxD || scales == nullptr || f8_bytes % 128 != 0 || f8_bytes < D))
        return cudaErrorInvalidValue;
    // the kernel covers ceil(D / 128) chunks of 128 columns (or bytes)
    const int span = (D + 127) / 128 * 128;
    if (out != nullptr && (dpb % 64 != 0 || dpb < D || (D <= kPrepMaxD && dpb > span))) return cudaErrorInvalidValue;
    if (f8 != nullptr && f8_bytes > span) return cudaErrorInvalidValue;
    if (np != nullptr && D > kPrepMaxD) return cudaErrorInvalidValue;
    if (D > kPrepMaxD) {
        // wide rows: separate passes
        cudaError_t e = cudaSuccess;
        if (norms) e = launch_norms(x, n, ld, D, norms, n_pad, s);
        if (e == cudaSuccess && (out || not_exact)) e = launch_bf16(x, n, ld, D, dpb, out, not_exact, s);
        if (e == cudaSuccess && int_stats) e = cudaMemsetAsync(int_stats, 0xFF, sizeof(uint32_t), s);  // unknown
        return e;
    }
    PrepArgs a;
    a.x = x;
    a.n = n;
    a.ld = ld;
    a.n_pad = std::max(n, n_pad);
    a.D = D;
    a.dpb = dpb;
    a.f8_bytes = f8_bytes;
    a.vec = (ld % 4 == 0 && D % 4 == 0 && (reinterpret_cast<uintptr_t>(x) & 15u) == 0) ? 1 : 0;
    a.out = static_cast<__nv_bfloat16*>(out);
    a.norms = norms;
    a.not_exact = not_exact;
    a.int_stats = int_stats;
    a.f8 = static_cast<uint8_t*>(f8);
    a.scales = scales;
    a.np = static_cast<__nv_bfloat16*>(np);
    auto blocks = [&](int ku) {
        const int64_t b = (rows + 8 * ku - 1) / (8 * ku);
        return (unsigned)std::max<int64_t>(1, std::min<int64_t>(b, 16384));
    };
    if (D <= 128)
        prep_rows_kernel<1, 4><<<blocks(4), 256, 0, s>>>(a);
    else if (D <= 256)
        prep_rows_kernel<2, 2><<<blocks(2), 256, 0, s>>>(a);
    else
        prep_rows_kernel<3, 1><<<blocks(1), 256, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_gather_norms(const float* src, int64_t n, int64_t stride, float* out, int64_t n_pad,
                                cudaStream_t s, float pad, const uint32_t* skip_unless)
{
    if (n_pad <= 0) return cudaSuccess;
    gather_norms_kernel<<<(unsigned)((n_pad + 255) / 256), 256, 0, s>>>(src, n, stride, out, n_pad, pad,
                                                                         skip_unless);
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
    if (dp % 4 != 0 || dp < D) return cudaErrorInvalidValue;  // rows of whole float4s
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
