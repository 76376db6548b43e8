// noalloc.cu -- a search entry point that allocates no device memory.
//
// Some callers cannot let a library call cudaMalloc during a search:
//   * processes whose device memory is already handed out by another
//     allocator (a framework's caching allocator that reserved the HBM), where
//     a fresh cudaMalloc fails or fragments;
//   * latency-critical callers, for which cudaMalloc / cudaFree may
//     synchronise the device and stall unrelated streams;
//   * plug-in hosts that own all allocation themselves (for example an
//     application embedding the reference's MEX-style gateway).
// knns_search_device_noalloc serves them.  Its scratch (corpus norms,
// per-query shared thresholds and the per-split shortlists) lives in a
// file-scope __device__ array of fixed size, which every GPU that loads this
// library keeps until the process exits.  It runs the CUDA-core fused kernel
// (the tensor-core kernel needs TF32 copies of the corpus, too large for a
// fixed array) followed by the shortlist merge / re-rank kernel.
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <mutex>

#include <cuda_runtime.h>

#include "engine.h"
#include "kernels.h"
#include "knn_gb300.h"

namespace knn {

namespace {
// Scratch: norms (rows rounded up to 128) + thresholds (Q words) + shortlists
// (splits x Q x kp words of 8 bytes).  8 MiB.
constexpr size_t kNoAllocScratchBytes = size_t(8) << 20;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mu;
void* g_scratch_addr[kMaxDevices] = {};

inline int64_t cdiv64(int64_t a, int64_t b) { return (a + b - 1) / b; }
inline size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

// Device address of the scratch array on the current device.  In host code
// the array's name is only a host-side stand-in, so the address is looked up
// once per device (with that device current) and cached.  Under lazy module
// loading (the CUDA default) this first lookup is also what loads the module
// and reserves the array's device memory.  The cached address belongs to the
// device's primary context: after a cudaDeviceReset it is stale (as is every
// buffer the engine keeps), so the entry point is not to be used across one.
int scratch_address(void** out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return set_error(KNNS_ERR_CUDA, "cudaGetDevice failed: %s", cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return set_error(KNNS_ERR_UNSUPPORTED, "device index %d out of range", dev);
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p)
            return set_error(KNNS_ERR_CUDA, "cudaGetSymbolAddress(scratch) failed: %s", cudaGetErrorString(e));
        g_scratch_addr[dev] = p;
    }
    *out = g_scratch_addr[dev];
    return KNNS_OK;
}
}  // namespace

}  // namespace knn

using namespace knn;

extern "C" {

int knns_noalloc_prepare(void)
{
    clear_error();
    void* p = nullptr;
    return scratch_address(&p);
}

int knns_search_device_noalloc(const float* corpus, int64_t N, int64_t ldc, const float* queries, int64_t Q,
                               int64_t ldq, int D, int k, float* dist, int32_t* idx, void* stream)
{
    clear_error();
    if (N <= 0 || D <= 0 || k <= 0 || Q < 0)
        return set_error(KNNS_ERR_INVALID, "invalid sizes N=%lld Q=%lld D=%d k=%d", (long long)N, (long long)Q, D, k);
    if (k > N) return set_error(KNNS_ERR_INVALID, "k=%d exceeds the corpus size N=%lld", k, (long long)N);
    if (N > 0x7fffffffLL) return set_error(KNNS_ERR_UNSUPPORTED, "corpus larger than 2^31-1 rows");
    if (ldc < D || ldq < D) return set_error(KNNS_ERR_INVALID, "row pitch smaller than D");
    if (!corpus || (Q > 0 && !queries)) return set_error(KNNS_ERR_INVALID, "null input pointer");
    if (Q == 0) return KNNS_OK;

    // the shortlist of the regular entry point's CUDA-core path: k plus the re-rank margin,
    // without the margin where that would pass the kernel's 512 entries
    int kp = auto_kp(k, 1);
    if (kp > 512 && k <= 512) kp = std::max((k + 15) & ~15, 32);
    if (kp > 512) return set_error(KNNS_ERR_UNSUPPORTED, "k=%d needs a shortlist above 512 entries", k);
    const int qtile = kp <= 128 ? 128 : 32;
    const int64_t n_pad = cdiv64(N, 128) * 128;
    const size_t norms_bytes = align256((size_t)n_pad * sizeof(float));
    const size_t thr_bytes = align256((size_t)Q * sizeof(uint32_t));
    const size_t per_split = (size_t)Q * kp * sizeof(uint64_t);
    if (norms_bytes + thr_bytes + per_split > kNoAllocScratchBytes)
        return set_error(KNNS_ERR_UNSUPPORTED,
                         "N=%lld, Q=%lld, k=%d need %zu bytes of scratch; the allocation-free entry point has %zu",
                         (long long)N, (long long)Q, k, norms_bytes + thr_bytes + per_split, kNoAllocScratchBytes);

    // corpus splits: as many as the scratch holds, up to the automatic choice
    int sms = 0;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return set_error(KNNS_ERR_CUDA, "device query failed: %s", cudaGetErrorString(e));
    const int64_t tiles = cdiv64(N, kSimtTileN);
    int splits = auto_splits(cdiv64(Q, qtile), tiles, sms, 64);
    const int64_t fit = (int64_t)((kNoAllocScratchBytes - norms_bytes - thr_bytes) / per_split);
    if (splits > fit) splits = (int)fit;
    if (splits < 1) splits = 1;
    const int64_t split_len = cdiv64(tiles, splits) * kSimtTileN;
    splits = (int)cdiv64(N, split_len);

    void* base = nullptr;
    int rc = scratch_address(&base);
    if (rc) return rc;
    unsigned char* sb = static_cast<unsigned char*>(base);
    float* cn = reinterpret_cast<float*>(sb);
    uint32_t* thr = reinterpret_cast<uint32_t*>(sb + norms_bytes);
    uint64_t* part = reinterpret_cast<uint64_t*>(sb + norms_bytes + thr_bytes);
    cudaStream_t s = (cudaStream_t)stream;

    // The scratch keeps the previous call's contents: the thresholds must
    // start at "unset" (all ones); norms and shortlists are fully rewritten.
    e = cudaMemsetAsync(thr, 0xFF, (size_t)Q * sizeof(uint32_t), s);
    if (e == cudaSuccess) e = launch_norms(corpus, N, ldc, D, cn, n_pad, s);
    if (e == cudaSuccess)
        e = launch_simt(corpus, N, ldc, cn, queries, Q, ldq, D, kp, qtile, split_len, splits, part, thr, s);
    if (e == cudaSuccess)
        e = launch_select(part, splits, Q, kp, k, corpus, ldc, queries, ldq, D, 1, nullptr, dist, idx, nullptr, s);
    if (e != cudaSuccess) return set_error(KNNS_ERR_CUDA, "launch failed: %s", cudaGetErrorString(e));
    return KNNS_OK;
}

}  // extern "C"
