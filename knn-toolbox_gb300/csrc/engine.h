// engine.h -- host engine internals shared by the C ABI translation units.
#pragma once

#include <cstddef>
#include <cstdint>
#include <mutex>
#include <vector>
#include <cuda_runtime.h>

#include "knn_gb300.h"

namespace knn {

struct DevBuf {
    void* p = nullptr;
    size_t cap = 0;
    int ensure(size_t bytes);
    void release();
};

struct Config {
    int algo = 0;
    int kp = 0;
    int rerank = 1;
    bool pilot = true;
    int precision = 0;
    int splits = 1;
    int64_t split_len = 0;
    int qtile = 128;
    int dp = 0;
    int dpb = 0;
    int stages = 0;
};

struct Engine {
    int device = 0;
    int sms = 1;
    int cc = 0;
    std::mutex mu;
    cudaEvent_t last_done = nullptr;
    DevBuf cn, qn, part, hi, lo, bf, err, thr, loflags, cn_s, thr2, redo;
    // threshold-scan path: BF16 queries, candidate segments and counts, seeded
    // thresholds, sample norms, failed-query list
    DevBuf qbf, cand, cnt, tq, cnv, fail;
    DevBuf in_corpus, in_queries, out_dist, out_idx;
    // stage timing: kTimingEvents events per timed search (start, after prep,
    // after threshold seeding, after the main fused kernel, after the main
    // selection, end)
    static constexpr int kTimingEvents = 6;
    std::vector<cudaEvent_t> tev;
    int tcount = 0;
    int timing_slot(cudaEvent_t out[kTimingEvents]);
    cudaStream_t host_stream();
    cudaEvent_t t0();
    cudaEvent_t t1();

  private:
    cudaStream_t stream_ = nullptr;
    cudaEvent_t ev0_ = nullptr, ev1_ = nullptr;
};

int set_error(int code, const char* fmt, ...);
void clear_error();
int get_engine(Engine** out);
int auto_kp(int k, int rerank);
int auto_splits(int64_t qtiles, int64_t tiles, int sms, int max_splits);
int resolve_config(const Engine& E, int64_t N, int64_t Q, int D, int k, const knns_options& o, Config* c);
int run_search(Engine& E, const float* corpus, int64_t N, int64_t ldc, const float* queries, int64_t Q, int64_t ldq,
               int D, int k, float* dist, int32_t* idx, float* idx_f, const knns_options& o, cudaStream_t s,
               knns_stats* st);
int check_device_error(Engine& E, cudaStream_t s);
int search_host(const float* corpus, int64_t N, const float* queries, int64_t Q, int D, int k, float* dist,
                int32_t* idx, float* idx_f_host, const knns_options& o, double* seconds, knns_stats* st);
void remember_stats(const knns_stats& st);

}  // namespace knn
