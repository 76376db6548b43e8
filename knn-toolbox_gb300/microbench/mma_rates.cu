// mma_rates.cu -- issue rate of tcgen05.mma on this GPU for the shapes the
// fused kernel can use (TF32 / BF16, A from TMEM or shared memory, N = 128 or
// 256), and the cost of committing every 4 MMAs and of alternating
// accumulators.  One CTA per SM; one thread issues `iters` groups of 4 MMAs
// (the 4 K-steps of one 128-byte swizzle row) on constant operands, then
// commits and waits; clock64 around the loop.  Build and run:
//   nvcc -O3 -std=c++17 -gencode arch=compute_103a,code=sm_103a \
//        -I knn-toolbox_gb300/csrc knn-toolbox_gb300/microbench/mma_rates.cu -o mma_rates && ./mma_rates
#include <cstdio>
#include <cstdint>
#include <cuda_runtime.h>
#include "tc_ptx.cuh"
using namespace knn::ptx;

__device__ __forceinline__ void mma_ss(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc, int f16) {
    if (f16)
        asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\ttcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
                     ::"r"(d), "l"(a), "l"(b), "r"(idesc), "r"(acc) : "memory");
    else
        asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\ttcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}"
                     ::"r"(d), "l"(a), "l"(b), "r"(idesc), "r"(acc) : "memory");
}
__device__ __forceinline__ void mma_ts(uint32_t d, uint32_t a, uint64_t b, uint32_t idesc, uint32_t acc, int f16) {
    if (f16)
        asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\ttcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p;\n\t}"
                     ::"r"(d), "r"(a), "l"(b), "r"(idesc), "r"(acc) : "memory");
    else
        asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\ttcgen05.mma.cta_group::1.kind::tf32 [%0], [%1], %2, %3, p;\n\t}"
                     ::"r"(d), "r"(a), "l"(b), "r"(idesc), "r"(acc) : "memory");
}

__global__ void __launch_bounds__(128, 1) bench(int iters, int f16, int a_tmem, int N, int commit_every, int alt, long long* out) {
    extern __shared__ __align__(1024) unsigned char sm[];
    // A tile: 128 rows x 128 B (16 KB) at 0; B tile: N rows x 128 B at 16 KB (N <= 256 -> 32 KB)
    __shared__ uint64_t bar, cbar;
    __shared__ uint32_t holder;
    const int warp = threadIdx.x >> 5;
    for (int i = threadIdx.x; i < (16384 + 32768) / 4; i += blockDim.x) ((uint32_t*)sm)[i] = 0x3f800000u;  // 1.0f / bf16 pair
    if (threadIdx.x == 0) { mbar_init(&bar, 1); mbar_init(&cbar, 1); fence_mbar_init(); }
    if (warp == 0) { tmem_alloc(&holder, 512); tmem_relinquish(); }
    tc_fence_before(); __syncthreads(); tc_fence_after();
    const uint32_t tmem = holder;
    if (threadIdx.x == 0) {
        const uint32_t idesc = (1u << 4) | ((f16 ? 1u : 2u) << 7) | ((f16 ? 1u : 2u) << 10) | ((uint32_t)(N >> 3) << 17) | (8u << 24);
        const uint32_t a_addr = smem_u32(sm), b_addr = smem_u32(sm + 16384);
        long long t0 = clock64();
        for (int it = 0; it < iters; ++it) {
            // alternate between two 128-column accumulators every `alt` groups (alt=0: one accumulator)
            const uint32_t d_tmem = tmem + 256 + ((alt && N == 128) ? (uint32_t)(((it / alt) & 1) * 128) : 0u);
#pragma unroll
            for (int kk = 0; kk < 4; ++kk) {
                const uint64_t bd = desc_sw128_kmajor(b_addr + kk * 32);
                if (a_tmem) mma_ts(d_tmem, tmem + kk * 8, bd, idesc, (it | kk) != 0, f16);
                else mma_ss(d_tmem, desc_sw128_kmajor(a_addr + kk * 32), bd, idesc, (it | kk) != 0, f16);
            }
            if (commit_every && (it % commit_every) == commit_every - 1) mma_commit(&cbar);
        }
        mma_commit(&bar);
        mbar_wait(&bar, 0, 4000000000ull);
        long long t1 = clock64();
        out[blockIdx.x] = t1 - t0;
    }
    tc_fence_before(); __syncthreads(); tc_fence_after();
    if (warp == 0) { __syncwarp(); tmem_dealloc(tmem, 512); }
}

int main() {
    int sms = 0; cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
    long long* d; cudaMalloc(&d, sizeof(long long) * sms);
    long long* h = new long long[sms];
    cudaFuncSetAttribute(bench, cudaFuncAttributeMaxDynamicSharedMemorySize, 16384 + 32768 + 1024);
    struct V { const char* name; int f16, a_tmem, N, commit_every, alt, iters; } vs[] = {
        // instruction shapes, back to back
        {"tf32 A=TMEM N=128", 0, 1, 128, 0, 0, 4096}, {"tf32 A=SMEM N=128", 0, 0, 128, 0, 0, 4096},
        {"tf32 A=SMEM N=256", 0, 0, 256, 0, 0, 4096}, {"tf32 A=TMEM N=256", 0, 1, 256, 0, 0, 4096},
        {"bf16 A=SMEM N=128", 1, 0, 128, 0, 0, 4096}, {"bf16 A=SMEM N=256", 1, 0, 256, 0, 0, 4096},
        {"bf16 A=TMEM N=128", 1, 1, 128, 0, 0, 4096}, {"bf16 A=TMEM N=256", 1, 1, 256, 0, 0, 4096},
        // pipeline effects: commit every 4 MMAs, alternate accumulators every 16
        {"tf32 TMEM N128 commit/4", 0, 1, 128, 1, 0, 4096}, {"tf32 TMEM N128 commit/4 alt16", 0, 1, 128, 1, 4, 4096},
        {"tf32 TMEM N128 alt16", 0, 1, 128, 0, 4, 4096}, {"bf16 TMEM N128 commit/4 alt16", 1, 1, 128, 1, 4, 4096},
        {"bf16 TMEM N256 commit/4", 1, 1, 256, 1, 0, 4096},
        {"tf32 TMEM N128 latency(1 group)", 0, 1, 128, 0, 0, 1}, {"tf32 TMEM N128 (4 groups)", 0, 1, 128, 0, 0, 4}};
    for (auto& v : vs) {
        const int iters = v.iters;
        bench<<<sms, 128, 16384 + 32768 + 1024>>>(iters, v.f16, v.a_tmem, v.N, v.commit_every, v.alt, d);
        cudaError_t e = cudaDeviceSynchronize();
        if (e != cudaSuccess) { printf("%s: error %s\n", v.name, cudaGetErrorString(e)); return 1; }
        cudaMemcpy(h, d, sizeof(long long) * sms, cudaMemcpyDeviceToHost);
        double cyc = 0; for (int i = 0; i < sms; ++i) cyc += h[i]; cyc /= sms;
        const int K = v.f16 ? 16 : 8;
        double flop = 2.0 * 128 * v.N * K * 4.0 * iters;
        printf("%-34s cycles/MMA %7.1f  flop/clk/SM %7.0f  GPU TFLOP/s at 2.07 GHz %7.1f\n", v.name, cyc / (4.0 * iters),
               flop / cyc, flop / cyc * sms * 2.07e9 / 1e12);
    }
    return 0;
}
