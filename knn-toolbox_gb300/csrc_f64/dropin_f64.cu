// dropin_f64.cu -- the double-precision library (libknngb300_double.so), the
// counterpart of the reference's libcuknn_double.a (Makefile:60-64: the same
// sources built with -D__DOUBLE__, knntype = double).  It exports the same C
// names with double arguments (include/cuknns.h with __DOUBLE__ defined) plus a
// status-returning device API (include/knn_gb300_f64.h).
//
// GB300's FP64 rate is a small fraction of its FP32 / tensor rate, so the
// double path does not scan the corpus in FP64.  Instead:
//   1. corpus and queries are rounded to FP32 and the float engine returns,
//      per query, the kp nearest rows by FP32 distance (kp > k);
//   2. those kp candidates are re-ranked by FP64 direct-difference distance
//      (sum over d, in d order, of (q_d - c_d)^2 with separate multiply and add)
//      and the first k kept;
//   3. a query is accepted only if no row outside its shortlist can belong to
//      its FP64 top-k: every outside row has an FP32 distance >= the shortlist's
//      largest, D32, and an FP64 distance >= D32 - E, where E bounds the error
//      of an FP32 distance of rounded data, E = (D/8 + 10) * 2^-24 *
//      (|q| + max|c|)^2 + 1e-5 * D32 (the last term covers the float engine's
//      own ranking tolerance); accepted when the k-th FP64 distance < D32 - E;
//   4. any other query is searched again by an FP64 brute-force kernel.
// Results: the exact FP64 top-k ordered by (distance, index).
#include <cfloat>
#include <cmath>
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>

#include <cuda_runtime.h>

#include "cuknns.h"
#include "knn_gb300.h"
#include "knn_gb300_f64.h"

namespace knn64 {

namespace {
thread_local std::string g_err;

int fail(int code, const char* fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_err = buf;
    return code;
}

#define F64_CUDA(call)                                                                                            \
    do {                                                                                                          \
        cudaError_t e_ = (call);                                                                                  \
        if (e_ != cudaSuccess) return fail(KNNS_ERR_CUDA, "%s failed: %s", #call, cudaGetErrorString(e_));       \
    } while (0)

struct Buf {
    void* p = nullptr;
    size_t cap = 0;
    int ensure(size_t bytes)
    {
        if (bytes <= cap) return KNNS_OK;
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
        if (cudaMalloc(&p, bytes) != cudaSuccess) {
            (void)cudaGetLastError();
            return fail(KNNS_ERR_NOMEM, "cudaMalloc(%zu) failed", bytes);
        }
        cap = bytes;
        return KNNS_OK;
    }
};

struct Work {
    std::mutex mu;
    Buf c32, q32, cand_d, cand_i, qn, cmax, fails, hc, hq, hd, hi;
};

std::mutex g_mu;
std::map<int, std::unique_ptr<Work>> g_work;

Work* work_for_device()
{
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lk(g_mu);
    auto& w = g_work[dev];
    if (!w) w.reset(new Work());
    return w.get();
}

constexpr int kSortMax = 512;    // shortlist entries one warp re-ranks
constexpr int kBruteBuf = 2048;  // candidate buffer of the brute-force kernel

__global__ void to_f32_kernel(const double* __restrict__ x, int64_t rows, int64_t ld, int D, float* __restrict__ out)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= rows * D) return;
    const int64_t r = i / D, c = i % D;
    out[i] = (float)x[r * ld + c];
}

// row norms |x| (FP64) and their maximum (as ordered bits in *mx)
__global__ void norms64_kernel(const double* __restrict__ x, int64_t rows, int64_t ld, int D, double* __restrict__ out,
                               unsigned long long* __restrict__ mx)
{
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= rows) return;
    double acc = 0.0;
    for (int d = 0; d < D; ++d) acc = __dadd_rn(acc, __dmul_rn(x[r * ld + d], x[r * ld + d]));
    const double n = sqrt(acc);
    if (out) out[r] = n;
    if (mx) atomicMax(mx, (unsigned long long)__double_as_longlong(n));
}

__device__ __forceinline__ double dist64(const double* __restrict__ q, const double* __restrict__ c, int D)
{
    double acc = 0.0;
    for (int d = 0; d < D; ++d) {
        const double t = __dsub_rn(q[d], c[d]);
        acc = __dadd_rn(acc, __dmul_rn(t, t));
    }
    return acc;
}

__device__ __forceinline__ bool pair_less(double a, int ia, double b, int ib) { return a < b || (a == b && ia < ib); }

// Bitonic sort of n (power of two) (distance, index) pairs in shared memory by one warp.
__device__ void warp_sort_pairs(double* d, int* ix, int n)
{
    const int lane = threadIdx.x & 31;
    for (int size = 2; size <= n; size <<= 1)
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            for (int i = lane; i < (n >> 1); i += 32) {
                const int lo = 2 * i - (i & (stride - 1)), hi = lo + stride;
                const bool up = (lo & size) == 0;
                if (pair_less(d[hi], ix[hi], d[lo], ix[lo]) == up) {
                    const double td = d[lo];
                    d[lo] = d[hi];
                    d[hi] = td;
                    const int ti = ix[lo];
                    ix[lo] = ix[hi];
                    ix[hi] = ti;
                }
            }
            __syncwarp();
        }
}

// One warp per query: FP64 re-rank of the kp FP32 candidates, the acceptance
// test, the k results or an entry in the failure list.
__global__ void rerank64_kernel(const double* __restrict__ data, int64_t ldc, const double* __restrict__ queries,
                                int64_t ldq, int D, int64_t N, const float* __restrict__ cd32,
                                const int32_t* __restrict__ ci, int kp, int k, int64_t Q,
                                const unsigned long long* __restrict__ cmax_bits, double* __restrict__ out_d,
                                int32_t* __restrict__ out_i, uint32_t* __restrict__ fails)
{
    extern __shared__ unsigned char sm[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t q = (int64_t)blockIdx.x * (blockDim.x >> 5) + warp;
    if (q >= Q) return;
    int P = 32;
    while (P < kp) P <<= 1;
    double* dd = reinterpret_cast<double*>(sm) + (size_t)warp * kSortMax;
    int* ii = reinterpret_cast<int*>(reinterpret_cast<double*>(sm) + (size_t)(blockDim.x >> 5) * kSortMax) +
              (size_t)warp * kSortMax;
    const double* qv = queries + q * ldq;
    for (int j = lane; j < P; j += 32) {
        const int32_t n = j < kp ? ci[q * kp + j] : -1;
        dd[j] = n >= 0 ? dist64(qv, data + (int64_t)n * ldc, D) : __longlong_as_double(0x7ff0000000000000ll);
        ii[j] = n >= 0 ? n : 0x7fffffff;
    }
    __syncwarp();
    warp_sort_pairs(dd, ii, P);
    // acceptance: the shortlist covers the corpus, or its k-th FP64 distance stays below
    // the smallest FP64 distance any row outside it can have
    bool ok = kp >= N;
    if (!ok) {
        double qq = 0.0;
        for (int d = lane; d < D; d += 32) qq = __dadd_rn(qq, __dmul_rn(qv[d], qv[d]));
        for (int o = 16; o > 0; o >>= 1) qq += __shfl_xor_sync(0xffffffffu, qq, o);
        const double s = sqrt(qq) + __longlong_as_double((long long)*cmax_bits);
        const double d32 = (double)cd32[q * kp + kp - 1];
        const double E = ((double)D / 8.0 + 10.0) * 5.9604644775390625e-08 * s * s + 1e-5 * d32;
        ok = dd[k - 1] < d32 - E;
    }
    if (!ok) {
        if (lane == 0) fails[1 + atomicAdd(fails, 1u)] = (uint32_t)q;
        return;
    }
    for (int j = lane; j < k; j += 32) {
        out_d[q * k + j] = dd[j];
        out_i[q * k + j] = ii[j];
    }
}

// One CTA per listed query: FP64 distances to every row, kept in a shared
// buffer below a shrinking threshold, sorted and trimmed to k when it fills.
__global__ void __launch_bounds__(256) brute64_kernel(const double* __restrict__ data, int64_t ldc, int64_t N,
                                                      const double* __restrict__ queries, int64_t ldq, int D, int k,
                                                      const uint32_t* __restrict__ fails, double* __restrict__ out_d,
                                                      int32_t* __restrict__ out_i)
{
    __shared__ double bd[kBruteBuf];
    __shared__ int bi[kBruteBuf];
    __shared__ int cnt;
    __shared__ double T;
    if (blockIdx.x >= fails[0]) return;
    const int64_t q = fails[1 + blockIdx.x];
    const double* qv = queries + q * ldq;
    if (threadIdx.x == 0) {
        cnt = 0;
        T = __longlong_as_double(0x7ff0000000000000ll);
    }
    __syncthreads();
    auto trim = [&]() {
        // sort the buffer (padded to kBruteBuf), keep the first k, threshold = k-th (if full)
        for (int j = cnt + threadIdx.x; j < kBruteBuf; j += blockDim.x) {
            bd[j] = __longlong_as_double(0x7ff0000000000000ll);
            bi[j] = 0x7fffffff;
        }
        __syncthreads();
        for (int size = 2; size <= kBruteBuf; size <<= 1)
            for (int stride = size >> 1; stride > 0; stride >>= 1) {
                for (int i = threadIdx.x; i < kBruteBuf / 2; i += blockDim.x) {
                    const int lo = 2 * i - (i & (stride - 1)), hi = lo + stride;
                    const bool up = (lo & size) == 0;
                    if (pair_less(bd[hi], bi[hi], bd[lo], bi[lo]) == up) {
                        const double td = bd[lo];
                        bd[lo] = bd[hi];
                        bd[hi] = td;
                        const int ti = bi[lo];
                        bi[lo] = bi[hi];
                        bi[hi] = ti;
                    }
                }
                __syncthreads();
            }
        if (threadIdx.x == 0) {
            cnt = min(cnt, k);
            if (cnt == k) T = bd[k - 1];
        }
        __syncthreads();
    };
    for (int64_t base = 0; base < N; base += blockDim.x) {
        if (cnt + (int)blockDim.x > kBruteBuf) trim();
        const int64_t n = base + threadIdx.x;
        if (n < N) {
            const double v = dist64(qv, data + n * ldc, D);
            // rows arrive in increasing index order: a later row never wins a tie
            if (v < T) {
                const int slot = atomicAdd(&cnt, 1);
                bd[slot] = v;
                bi[slot] = (int)n;
            }
        }
        __syncthreads();
    }
    trim();
    for (int j = threadIdx.x; j < k; j += blockDim.x) {
        out_d[q * k + j] = bd[j];
        out_i[q * k + j] = bi[j];
    }
}

int shortlist_len(int k, int64_t N) { return (int)std::min<int64_t>(N, std::min(kSortMax, std::max(k + 32, 2 * k))); }

int search_device(const double* corpus, int64_t N, int64_t ldc, const double* queries, int64_t Q, int64_t ldq, int D,
                  int k, double* dist, int32_t* idx, cudaStream_t s)
{
    if (N <= 0 || D <= 0 || k <= 0 || Q < 0 || ldc < D || ldq < D || !corpus || (Q > 0 && !queries))
        return fail(KNNS_ERR_INVALID, "invalid arguments");
    if (k > N) return fail(KNNS_ERR_INVALID, "k=%d exceeds the corpus size N=%lld", k, (long long)N);
    if (k > kSortMax) return fail(KNNS_ERR_UNSUPPORTED, "the double path returns at most %d neighbours", kSortMax);
    if (N > 0x7fffffffLL) return fail(KNNS_ERR_UNSUPPORTED, "corpus larger than 2^31-1 rows");
    if (Q == 0) return KNNS_OK;
    Work* W = work_for_device();
    std::lock_guard<std::mutex> lk(W->mu);
    const int kp = shortlist_len(k, N);
    int rc = W->c32.ensure((size_t)N * D * 4);
    if (!rc) rc = W->q32.ensure((size_t)Q * D * 4);
    if (!rc) rc = W->cand_d.ensure((size_t)Q * kp * 4);
    if (!rc) rc = W->cand_i.ensure((size_t)Q * kp * 4);
    if (!rc) rc = W->cmax.ensure(8);
    if (!rc) rc = W->fails.ensure((size_t)(Q + 1) * 4);
    if (rc) return rc;
    const int T = 256;
    to_f32_kernel<<<(unsigned)((N * D + T - 1) / T), T, 0, s>>>(corpus, N, ldc, D, (float*)W->c32.p);
    to_f32_kernel<<<(unsigned)((Q * D + T - 1) / T), T, 0, s>>>(queries, Q, ldq, D, (float*)W->q32.p);
    F64_CUDA(cudaMemsetAsync(W->cmax.p, 0, 8, s));
    F64_CUDA(cudaMemsetAsync(W->fails.p, 0, 4, s));
    norms64_kernel<<<(unsigned)((N + T - 1) / T), T, 0, s>>>(corpus, N, ldc, D, nullptr,
                                                              (unsigned long long*)W->cmax.p);
    F64_CUDA(cudaGetLastError());
    // FP32 shortlist of kp rows per query, ordered by exact FP32 distance
    rc = knns_search_device((const float*)W->c32.p, N, D, (const float*)W->q32.p, Q, D, D, kp, (float*)W->cand_d.p,
                            (int32_t*)W->cand_i.p, nullptr, s);
    if (rc) return fail(rc, "float shortlist: %s", knns_last_error());
    const int warps = 4;
    const size_t smem = (size_t)warps * kSortMax * (8 + 4);
    F64_CUDA(cudaFuncSetAttribute(rerank64_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    rerank64_kernel<<<(unsigned)((Q + warps - 1) / warps), warps * 32, smem, s>>>(
        corpus, ldc, queries, ldq, D, N, (const float*)W->cand_d.p, (const int32_t*)W->cand_i.p, kp, k, Q,
        (const unsigned long long*)W->cmax.p, dist, idx, (uint32_t*)W->fails.p);
    // queries whose shortlist could not be proven complete (the grid covers every query; the
    // CTAs past the failure count return at once)
    brute64_kernel<<<(unsigned)Q, 256, 0, s>>>(corpus, ldc, N, queries, ldq, D, k, (const uint32_t*)W->fails.p,
                                                dist, idx);
    F64_CUDA(cudaGetLastError());
    rc = knns_check_device(s);
    if (rc) return fail(rc, "%s", knns_last_error());
    return KNNS_OK;
}

int search_host(const double* query, const double* data, double* values, double* indices, int N, int Q, int D,
                int k, double* seconds)
{
    if (!query || !data || N <= 0 || Q < 0 || D <= 0 || k <= 0) return fail(KNNS_ERR_INVALID, "invalid arguments");
    Work* W = work_for_device();
    cudaStream_t s = nullptr;
    F64_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    int rc;
    {
        std::lock_guard<std::mutex> lk(W->mu);
        rc = W->hc.ensure((size_t)N * D * 8);
        if (!rc) rc = W->hq.ensure((size_t)Q * D * 8 + 8);
        if (!rc) rc = W->hd.ensure((size_t)Q * k * 8 + 8);
        if (!rc) rc = W->hi.ensure((size_t)Q * k * 4 + 8);
    }
    std::unique_ptr<int32_t[]> ih(new int32_t[(size_t)Q * k + 1]);
    if (!rc) {
        cudaEventRecord(e0, s);
        cudaMemcpyAsync(W->hc.p, data, (size_t)N * D * 8, cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(W->hq.p, query, (size_t)Q * D * 8, cudaMemcpyHostToDevice, s);
        rc = search_device((const double*)W->hc.p, N, D, (const double*)W->hq.p, Q, D, D, k, (double*)W->hd.p,
                           (int32_t*)W->hi.p, s);
        if (!rc) {
            cudaMemcpyAsync(values, W->hd.p, (size_t)Q * k * 8, cudaMemcpyDeviceToHost, s);
            cudaMemcpyAsync(ih.get(), W->hi.p, (size_t)Q * k * 4, cudaMemcpyDeviceToHost, s);
            cudaEventRecord(e1, s);
            if (cudaStreamSynchronize(s) != cudaSuccess) rc = fail(KNNS_ERR_CUDA, "copy back failed");
        }
    }
    if (!rc) {
        for (int64_t i = 0; i < (int64_t)Q * k; ++i) indices[i] = (double)ih[i];
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (seconds) *seconds = ms / 1000.0;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaStreamDestroy(s);
    return rc;
}

}  // namespace
}  // namespace knn64

using namespace knn64;

extern "C" {

int knns_search_device_f64(const double* corpus, int64_t N, int64_t ldc, const double* queries, int64_t Q,
                           int64_t ldq, int D, int k, double* dist, int32_t* idx, void* stream)
{
    g_err.clear();
    return search_device(corpus, N, ldc, queries, Q, ldq, D, k, dist, idx, (cudaStream_t)stream);
}

int knns_search_host_f64(const double* corpus, int64_t N, const double* queries, int64_t Q, int D, int k,
                         double* dist, int32_t* idx)
{
    g_err.clear();
    if (N > 0x7fffffffLL || Q > 0x7fffffffLL) return fail(KNNS_ERR_UNSUPPORTED, "sizes beyond int");
    std::unique_ptr<double[]> fi(new double[(size_t)Q * k + 1]);
    double secs = 0;
    int rc = search_host(queries, corpus, dist, fi.get(), (int)N, (int)Q, D, k, &secs);
    if (!rc && idx)
        for (int64_t i = 0; i < Q * k; ++i) idx[i] = (int32_t)fi[i];
    return rc;
}

const char* knns_f64_last_error(void) { return g_err.c_str(); }

// include/cuknns.h:75 (src/cuknnBitonic.cu:422), knntype = double
double gpuknnsBitonic(double* query, double* data, double* values, double* indices, int objects, int numQueries,
                      int attributes, int k, int numStreams)
{
    (void)numStreams;
    g_err.clear();
    double secs = 0;
    if (search_host(query, data, values, indices, objects, numQueries, attributes, k, &secs)) return DBL_MAX;
    return secs;
}

// include/cuknns.h:83 (src/cuknnHeap.cu:394): same engine, same contract
double gpuknnsHeap(double* query, double* data, double* values, double* indices, int objects, int numQueries,
                   int attributes, int k, int numStreams)
{
    return gpuknnsBitonic(query, data, values, indices, objects, numQueries, attributes, k, numStreams);
}

// include/cuknns.h:85 (src/knnsplan.cu:25): the double engine has one configuration
void knnsplan(knnplan* plan, long int N, long int Q, long int D, long int k)
{
    if (!plan) return;
    plan->pt2Function = gpuknnsBitonic;
    plan->objects = (int)N;
    plan->numQueries = (int)Q;
    plan->dimentions = (int)D;
    plan->k = (int)k;
    plan->numStreams = 1;
}

// include/cuknns.h:87 (src/knnsexecute.cu:6)
void knnsexecute(knnplan plan, double* data, double* queries, double* KNNdist, double* KNNidx)
{
    const double t = plan.pt2Function(queries, data, KNNdist, KNNidx, plan.objects, plan.numQueries, plan.dimentions,
                                      plan.k, plan.numStreams);
    printf("Time Elapsed: %f\n", t);
}

}  // extern "C"
