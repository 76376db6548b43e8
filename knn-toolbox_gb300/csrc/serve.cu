// serve.cu -- serving form: continuous batching of kNN requests over a resident index.
//
// The reference has no server; its nearest caller pattern is the MEX gateways'
// query blocking (src/mexknnsGen.cu:196), which splits one large query set into
// fixed blocks and runs them one after another.  Here requests of uneven size
// and k arrive at any time (knns_server_submit) and one worker thread packs
// them into launches:
//   * admission: a request is admitted into a batch when it fits the batch's
//     workspace (at most max_batch queries per launch).  In the exact form
//     requests of different k share a launch: it runs with the largest k of its
//     requests and each request keeps the first k of its rows -- the results
//     are sorted by (distance, index), so that prefix is the request's own
//     top-k, the one it gets alone.  In the BF16 / FP8 forms the shortlist
//     length is c*k, so a launch takes one k (a request's recall is then the
//     one it gets alone);
//   * slots: `slots` batches are in flight at once, each on its own stream with
//     its own workspace, so a batch formed while another runs overlaps it on the
//     device; as a slot completes, its requests are answered and the slot takes
//     the next batch;
//   * graphs: every (size bucket, k) is captured once per slot into a CUDA graph
//     (bucket = the next power of two >= the packed query count, from 32 up to
//     max_batch); a batch is one host->device copy, one graph launch and one
//     device->host copy;
//   * autotuning: before a (bucket, k) graph is captured, candidate corpus split
//     counts are timed on the slot's stream and the fastest is captured.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "engine.h"
#include "kernels.h"
#include "knn_gb300.h"

#define KNN_CUDA_RET(call)                                                                          \
    do {                                                                                            \
        cudaError_t e_ = (call);                                                                    \
        if (e_ != cudaSuccess)                                                                      \
            return set_error(KNNS_ERR_CUDA, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), \
                             __FILE__, __LINE__);                                                   \
    } while (0)

namespace knn {
namespace {

double now_ms()
{
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

struct Request {
    int64_t id = 0;
    int k = 0;
    int64_t Q = 0;
    std::vector<float> q;  // Q x D
    std::vector<float> dist;
    std::vector<int32_t> idx;
    double t_submit = 0, t_done = 0;
    bool done = false;
    int status = KNNS_OK;
    std::string error;
};

struct Slot {
    Engine E;
    cudaStream_t stream = nullptr;
    cudaEvent_t done_ev = nullptr;
    float* d_q = nullptr;
    float* d_dist = nullptr;
    int32_t* d_idx = nullptr;
    float* h_q = nullptr;
    float* h_dist = nullptr;
    int32_t* h_idx = nullptr;
    std::map<std::pair<int, int>, cudaGraphExec_t> graphs;
    std::map<std::pair<int, int>, int> tuned;  // split count chosen per (bucket, k)
    std::vector<void*> snapshot;  // workspace pointers the graphs were captured with
    std::vector<std::shared_ptr<Request>> batch;
    std::vector<int64_t> offs;
    int k = 0, bucket = 0;
    bool busy = false;      // holds a batch (or is being warmed up)
    bool launched = false;  // its batch is on the GPU: the slot's completion thread waits for it
    int status = KNNS_OK;   // launch failure to report
    uint64_t seq = 0;
    std::thread completer;
};

std::vector<void*> workspace_pointers(const Engine& E)
{
    return {E.cn.p,   E.qn.p,  E.part.p, E.hi.p,  E.lo.p,  E.bf.p,   E.err.p,  E.thr.p,  E.loflags.p, E.cn_s.p,
            E.thr2.p, E.redo.p, E.qbf.p, E.cand.p, E.cnt.p, E.tq.p,   E.cnv.p,  E.fail.p, E.words.p};
}

}  // namespace
}  // namespace knn

using namespace knn;

struct knns_server {
    knns_index* ix = nullptr;
    const PreparedCorpus* pc = nullptr;
    knns_server_config cfg{};
    int device = 0;
    std::vector<std::unique_ptr<Slot>> slots;
    std::mutex mu;
    std::condition_variable cv, done_cv;
    std::deque<std::shared_ptr<Request>> pending;
    std::map<int64_t, std::shared_ptr<Request>> reqs;
    int64_t next_id = 1;
    uint64_t next_seq = 1;
    bool stop = false;
    std::thread worker;
    int64_t n_batches = 0, n_queries = 0, n_graphs = 0, n_requests = 0;

    int setup();
    void run();
    void run_completer(Slot* sl);
    int launch(Slot& sl, std::vector<std::shared_ptr<Request>>& take, int k, int64_t total);
    int get_graph(Slot& sl, int bucket, int k, cudaGraphExec_t* out);
    int tune(Slot& sl, int bucket, int k, int* splits);
    void complete(Slot& sl, int status, const char* err);
    knns_options opts(int splits) const;
    Slot* free_slot();
    Slot* oldest_busy();
};

knns_options knns_server::opts(int splits) const
{
    knns_options o;
    knns_default_options(&o);
    o.precision = cfg.precision;
    o.shortlist = cfg.shortlist;
    o.splits = splits;
    return o;
}

int knns_server::setup()
{
    Engine* G = nullptr;
    int rc = get_engine(&G);
    if (rc) return rc;
    device = G->device;
    const int D = pc->D;
    const int kmax = kMaxKpTC;
    for (int i = 0; i < cfg.slots; ++i) {
        std::unique_ptr<Slot> sl(new Slot());
        sl->E.device = G->device;
        sl->E.sms = G->sms;
        sl->E.cc = G->cc;
        if (cudaEventCreateWithFlags(&sl->E.last_done, cudaEventDisableTiming) != cudaSuccess ||
            cudaStreamCreateWithFlags(&sl->stream, cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&sl->done_ev, cudaEventDisableTiming) != cudaSuccess)
            return set_error(KNNS_ERR_CUDA, "server slot: stream / event creation failed");
        if ((rc = sl->E.err.ensure(sizeof(int)))) return rc;
        if (cudaMemset(sl->E.err.p, 0, sizeof(int)) != cudaSuccess) return set_error(KNNS_ERR_CUDA, "memset");
        const size_t qb = (size_t)cfg.max_batch * D * sizeof(float), ob = (size_t)cfg.max_batch * kmax * 4;
        if (cudaMalloc(&sl->d_q, qb) != cudaSuccess || cudaMalloc(&sl->d_dist, ob) != cudaSuccess ||
            cudaMalloc(&sl->d_idx, ob) != cudaSuccess || cudaMallocHost(&sl->h_q, qb) != cudaSuccess ||
            cudaMallocHost(&sl->h_dist, ob) != cudaSuccess || cudaMallocHost(&sl->h_idx, ob) != cudaSuccess)
            return set_error(KNNS_ERR_NOMEM, "server slot buffers (%d queries) could not be allocated", cfg.max_batch);
        // rows past a batch's queries are computed and discarded: keep them finite
        memset(sl->h_q, 0, qb);
        if (cudaMemset(sl->d_q, 0, qb) != cudaSuccess) return set_error(KNNS_ERR_CUDA, "memset");
        slots.push_back(std::move(sl));
    }
    worker = std::thread([this] { run(); });
    for (auto& sl : slots) {
        Slot* p = sl.get();
        sl->completer = std::thread([this, p] { run_completer(p); });
    }
    return KNNS_OK;
}

Slot* knns_server::free_slot()
{
    for (auto& s : slots)
        if (!s->busy) return s.get();
    return nullptr;
}

Slot* knns_server::oldest_busy()
{
    Slot* best = nullptr;
    for (auto& s : slots)
        if (s->busy && s->seq != ~0ull && (!best || s->seq < best->seq)) best = s.get();
    return best;
}

// Choose (once per slot and (bucket, k)) the corpus split count: candidates
// timed over three runs each on the slot's stream; every candidate is also run
// once, so the workspace reaches the size that configuration needs.
int knns_server::tune(Slot& sl, int bucket, int k, int* splits)
{
    auto key = std::make_pair(bucket, k);
    auto it = sl.tuned.find(key);
    if (it != sl.tuned.end()) {
        *splits = it->second;
        return KNNS_OK;
    }
    const PreparedCorpus& P = *pc;
    auto search = [&](int sp) {
        knns_options o = opts(sp);
        return run_search(sl.E, P.corpus, P.N, P.ldc, sl.d_q, bucket, P.D, P.D, k, sl.d_dist, sl.d_idx, nullptr, o,
                          sl.stream, nullptr, &P, false);
    };
    int best_splits = 0;
    if (cfg.autotune) {
        cudaEvent_t e0, e1;
        if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess)
            return set_error(KNNS_ERR_CUDA, "autotune events");
        float best = 1e30f;
        for (int sp : {0, 4, 8, 16, 32, 76}) {
            int rc = search(sp);  // warm (allocates)
            if (rc) continue;
            cudaEventRecord(e0, sl.stream);
            for (int r = 0; r < 3 && !rc; ++r) rc = search(sp);
            cudaEventRecord(e1, sl.stream);
            if (rc || cudaEventSynchronize(e1) != cudaSuccess) continue;
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            if (ms < best) {
                best = ms;
                best_splits = sp;
            }
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
    }
    int rc = search(best_splits);
    if (rc) return rc;
    KNN_CUDA_RET(cudaStreamSynchronize(sl.stream));
    rc = check_device_error(sl.E, sl.stream);
    if (rc) return rc;
    sl.tuned[key] = best_splits;
    *splits = best_splits;
    return KNNS_OK;
}

// Capture (once per slot) the search of `bucket` packed queries with this k.
int knns_server::get_graph(Slot& sl, int bucket, int k, cudaGraphExec_t* out)
{
    auto key = std::make_pair(bucket, k);
    auto it = sl.graphs.find(key);
    if (it != sl.graphs.end()) {
        *out = it->second;
        return KNNS_OK;
    }
    const PreparedCorpus& P = *pc;
    int splits = 0;
    int rc = tune(sl, bucket, k, &splits);
    if (rc) return rc;
    // a grown workspace buffer moved: graphs captured before hold stale pointers
    auto ptrs = workspace_pointers(sl.E);
    if (ptrs != sl.snapshot) {
        for (auto& g : sl.graphs) cudaGraphExecDestroy(g.second);
        sl.graphs.clear();
        sl.snapshot = ptrs;
    }
    cudaGraph_t g = nullptr;
    KNN_CUDA_RET(cudaStreamBeginCapture(sl.stream, cudaStreamCaptureModeThreadLocal));
    knns_options o = opts(splits);
    rc = run_search(sl.E, P.corpus, P.N, P.ldc, sl.d_q, bucket, P.D, P.D, k, sl.d_dist, sl.d_idx, nullptr, o,
                    sl.stream, nullptr, &P, true);
    cudaError_t ce = cudaStreamEndCapture(sl.stream, &g);
    if (rc) {
        if (g) cudaGraphDestroy(g);
        return rc;
    }
    if (ce != cudaSuccess) return set_error(KNNS_ERR_CUDA, "graph capture failed: %s", cudaGetErrorString(ce));
    cudaGraphExec_t ge = nullptr;
    ce = cudaGraphInstantiate(&ge, g, 0);
    cudaGraphDestroy(g);
    if (ce != cudaSuccess) return set_error(KNNS_ERR_CUDA, "graph instantiation failed: %s", cudaGetErrorString(ce));
    sl.graphs[key] = ge;
    ++n_graphs;
    *out = ge;
    return KNNS_OK;
}

int knns_server::launch(Slot& sl, std::vector<std::shared_ptr<Request>>& take, int k, int64_t total)
{
    const int D = pc->D;
    int bucket = 32;
    while (bucket < total) bucket *= 2;
    bucket = std::min(bucket, cfg.max_batch);
    sl.batch = take;
    sl.offs.clear();
    int64_t off = 0;
    for (auto& r : take) {
        memcpy(sl.h_q + off * D, r->q.data(), (size_t)r->Q * D * sizeof(float));
        sl.offs.push_back(off);
        off += r->Q;
    }
    sl.k = k;
    sl.bucket = bucket;
    cudaGraphExec_t ge = nullptr;
    int rc = get_graph(sl, bucket, k, &ge);
    if (rc) return rc;
    KNN_CUDA_RET(cudaMemcpyAsync(sl.d_q, sl.h_q, (size_t)bucket * D * sizeof(float), cudaMemcpyHostToDevice, sl.stream));
    KNN_CUDA_RET(cudaGraphLaunch(ge, sl.stream));
    KNN_CUDA_RET(cudaMemcpyAsync(sl.h_dist, sl.d_dist, (size_t)total * k * 4, cudaMemcpyDeviceToHost, sl.stream));
    KNN_CUDA_RET(cudaMemcpyAsync(sl.h_idx, sl.d_idx, (size_t)total * k * 4, cudaMemcpyDeviceToHost, sl.stream));
    KNN_CUDA_RET(cudaEventRecord(sl.done_ev, sl.stream));
    return KNNS_OK;
}

void knns_server::complete(Slot& sl, int status, const char* err)
{
    const double t = now_ms();
    {
        std::lock_guard<std::mutex> lk(mu);
        for (size_t i = 0; i < sl.batch.size(); ++i) {
            Request& r = *sl.batch[i];
            if (status == KNNS_OK) {
                // rows of the launch's k; the request keeps the first r.k of each
                const int64_t o = sl.offs[i];
                r.dist.resize((size_t)r.Q * r.k);
                r.idx.resize((size_t)r.Q * r.k);
                for (int64_t q = 0; q < r.Q; ++q) {
                    memcpy(r.dist.data() + q * r.k, sl.h_dist + (o + q) * sl.k, (size_t)r.k * sizeof(float));
                    memcpy(r.idx.data() + q * r.k, sl.h_idx + (o + q) * sl.k, (size_t)r.k * sizeof(int32_t));
                }
            } else if (r.error.empty()) {
                r.error = err ? err : "";
            }
            r.status = status;
            r.t_done = t;
            r.done = true;
        }
        sl.batch.clear();
        sl.busy = false;
    }
    done_cv.notify_all();
    cv.notify_all();
}

// Dispatcher: forms a batch whenever requests are pending and a slot is free.
void knns_server::run()
{
    cudaSetDevice(device);
    for (;;) {
        std::unique_lock<std::mutex> lk(mu);
        cv.wait(lk, [&] { return stop || (!pending.empty() && free_slot() != nullptr); });
        if (stop) {
            // requests never launched are answered with an error
            for (auto& r : pending) {
                r->status = KNNS_ERR_INVALID;
                r->error = "the server stopped before the request was launched";
                r->done = true;
            }
            pending.clear();
            lk.unlock();
            done_cv.notify_all();
            return;
        }
        Slot* fs = free_slot();
        // admit, oldest first, the pending requests that fit one launch: any k in the exact
        // form (the launch runs the largest), the oldest request's k in the precision forms
        const bool mix_k = cfg.precision == KNNS_PREC_EXACT;
        const int k0 = pending.front()->k;
        int k = k0;
        std::vector<std::shared_ptr<Request>> take;
        int64_t total = 0;
        for (auto it = pending.begin(); it != pending.end();) {
            if ((mix_k || (*it)->k == k0) && total + (*it)->Q <= cfg.max_batch) {
                total += (*it)->Q;
                k = std::max(k, (*it)->k);
                take.push_back(*it);
                it = pending.erase(it);
            } else {
                ++it;
            }
        }
        fs->busy = true;
        fs->seq = next_seq++;
        ++n_batches;
        n_queries += total;
        lk.unlock();
        const int rc = launch(*fs, take, k, total);
        if (rc) {
            for (auto& r : take) r->error = knns_last_error();
        }
        lk.lock();
        fs->batch = take;
        fs->status = rc;
        fs->launched = true;
        lk.unlock();
        cv.notify_all();
    }
}

// Completion: one thread per slot waits for its batch and answers the requests.
void knns_server::run_completer(Slot* sl)
{
    cudaSetDevice(device);
    for (;;) {
        std::unique_lock<std::mutex> lk(mu);
        cv.wait(lk, [&] { return sl->launched || (stop && !sl->busy); });
        if (!sl->launched) return;
        int rc = sl->status;
        lk.unlock();
        std::string msg = rc ? knns_last_error() : "";
        if (rc == KNNS_OK) {
            cudaError_t e = cudaEventSynchronize(sl->done_ev);
            rc = e == cudaSuccess ? KNNS_OK : set_error(KNNS_ERR_CUDA, "batch failed: %s", cudaGetErrorString(e));
            if (rc == KNNS_OK) rc = check_device_error(sl->E, sl->stream);
            if (rc) msg = knns_last_error();
        }
        {
            std::lock_guard<std::mutex> g(mu);
            sl->launched = false;
        }
        complete(*sl, rc, rc ? msg.c_str() : nullptr);
    }
}

extern "C" {

void knns_server_default_config(knns_server_config* cfg)
{
    if (!cfg) return;
    memset(cfg, 0, sizeof(*cfg));
    cfg->slots = 2;
    cfg->max_batch = 1024;
    cfg->precision = KNNS_PREC_EXACT;
    cfg->shortlist = 0;
    cfg->autotune = 1;
}

int knns_server_create(knns_index* ix, const knns_server_config* cfg, knns_server** out)
{
    clear_error();
    if (!ix || !out) return set_error(KNNS_ERR_INVALID, "null index or output");
    *out = nullptr;
    std::unique_ptr<knns_server> sv(new knns_server());
    sv->ix = ix;
    sv->pc = &ix->pc;
    if (cfg) sv->cfg = *cfg;
    else knns_server_default_config(&sv->cfg);
    const knns_server_config& c = sv->cfg;
    if (c.slots < 1 || c.slots > 8) return set_error(KNNS_ERR_INVALID, "slots must be 1..8");
    if (c.max_batch < 32 || c.max_batch > 65536 || (c.max_batch & (c.max_batch - 1)))
        return set_error(KNNS_ERR_INVALID, "max_batch must be a power of two in [32, 65536]");
    if (c.precision != KNNS_PREC_EXACT && c.precision != KNNS_PREC_BF16 && c.precision != KNNS_PREC_FP8)
        return set_error(KNNS_ERR_INVALID, "unknown precision %d", c.precision);
    int rc = sv->setup();
    if (rc) {
        knns_server_destroy(sv.release());
        return rc;
    }
    *out = sv.release();
    return KNNS_OK;
}

int64_t knns_server_submit(knns_server* sv, const float* queries, int64_t Q, int k)
{
    clear_error();
    if (!sv || !queries) return -set_error(KNNS_ERR_INVALID, "null server or queries");
    if (Q < 1 || Q > sv->cfg.max_batch)
        return -set_error(KNNS_ERR_INVALID, "a request holds 1..%d queries (got %lld)", sv->cfg.max_batch,
                          (long long)Q);
    if (k < 1 || k > kMaxKpTC || k > sv->pc->N)
        return -set_error(KNNS_ERR_INVALID, "k=%d outside 1..min(%d, N)", k, kMaxKpTC);
    std::shared_ptr<Request> r(new Request());
    r->k = k;
    r->Q = Q;
    r->q.assign(queries, queries + Q * sv->pc->D);
    {
        std::lock_guard<std::mutex> lk(sv->mu);
        if (sv->stop) return -set_error(KNNS_ERR_INVALID, "server is stopping");
        r->id = sv->next_id++;
        r->t_submit = now_ms();
        sv->pending.push_back(r);
        sv->reqs[r->id] = r;
        ++sv->n_requests;
    }
    sv->cv.notify_all();
    return r->id;
}

int knns_server_wait(knns_server* sv, int64_t id, float* dist, int32_t* idx, double* latency_ms)
{
    clear_error();
    if (!sv) return set_error(KNNS_ERR_INVALID, "null server");
    std::shared_ptr<Request> r;
    {
        std::unique_lock<std::mutex> lk(sv->mu);
        auto it = sv->reqs.find(id);
        if (it == sv->reqs.end()) return set_error(KNNS_ERR_INVALID, "unknown request %lld", (long long)id);
        r = it->second;
        sv->done_cv.wait(lk, [&] { return r->done; });
        sv->reqs.erase(it);
    }
    if (r->status != KNNS_OK) return set_error(r->status, "%s", r->error.c_str());
    if (dist) memcpy(dist, r->dist.data(), r->dist.size() * sizeof(float));
    if (idx) memcpy(idx, r->idx.data(), r->idx.size() * sizeof(int32_t));
    if (latency_ms) *latency_ms = r->t_done - r->t_submit;
    return KNNS_OK;
}

int knns_server_warmup(knns_server* sv, const int* buckets, int nb, const int* ks, int nk)
{
    clear_error();
    if (!sv || (nb > 0 && !buckets) || (nk > 0 && !ks)) return set_error(KNNS_ERR_INVALID, "bad warm-up arguments");
    // take every slot out of service while its graphs are captured
    std::vector<Slot*> mine;
    {
        std::unique_lock<std::mutex> lk(sv->mu);
        sv->cv.wait(lk, [&] {
            for (auto& sl : sv->slots)
                if (sl->busy) return false;
            return true;
        });
        for (auto& sl : sv->slots) {
            sl->busy = true;
            sl->seq = ~0ull;  // never "oldest": the worker does not wait on a warming slot
            mine.push_back(sl.get());
        }
    }
    // two passes: tune (and so size the workspace for) every configuration, then capture
    // them all -- no capture is invalidated by a later buffer growth
    int rc = KNNS_OK;
    for (int pass = 0; pass < 2 && !rc; ++pass)
        for (Slot* sl : mine)
            for (int b = 0; b < nb && !rc; ++b)
                for (int j = 0; j < nk && !rc; ++j) {
                    int bucket = 32;
                    while (bucket < buckets[b]) bucket *= 2;
                    if (bucket > sv->cfg.max_batch || ks[j] < 1 || ks[j] > kMaxKpTC || ks[j] > sv->pc->N) {
                        rc = set_error(KNNS_ERR_INVALID, "warm-up bucket %d / k %d outside the server's range",
                                       buckets[b], ks[j]);
                        break;
                    }
                    if (pass == 0) {
                        int sp;
                        rc = sv->tune(*sl, bucket, ks[j], &sp);
                    } else {
                        cudaGraphExec_t ge;
                        rc = sv->get_graph(*sl, bucket, ks[j], &ge);
                    }
                }
    {
        std::lock_guard<std::mutex> lk(sv->mu);
        for (Slot* sl : mine) sl->busy = false;
    }
    sv->cv.notify_all();
    return rc;
}

int knns_server_stats(knns_server* sv, int64_t out[4])
{
    if (!sv || !out) return set_error(KNNS_ERR_INVALID, "null server or output");
    std::lock_guard<std::mutex> lk(sv->mu);
    out[0] = sv->n_requests;
    out[1] = sv->n_batches;
    out[2] = sv->n_queries;
    out[3] = sv->n_graphs;
    return KNNS_OK;
}

void knns_server_destroy(knns_server* sv)
{
    if (!sv) return;
    {
        std::lock_guard<std::mutex> lk(sv->mu);
        sv->stop = true;
    }
    sv->cv.notify_all();
    if (sv->worker.joinable()) sv->worker.join();
    // completion threads finish the batches in flight, then leave
    for (auto& sl : sv->slots)
        if (sl->completer.joinable()) sl->completer.join();
    for (auto& sl : sv->slots) {
        if (sl->stream) cudaStreamSynchronize(sl->stream);
        for (auto& g : sl->graphs) cudaGraphExecDestroy(g.second);
        if (sl->stream) cudaStreamDestroy(sl->stream);
        if (sl->done_ev) cudaEventDestroy(sl->done_ev);
        if (sl->E.last_done) cudaEventDestroy(sl->E.last_done);
        cudaFree(sl->d_q);
        cudaFree(sl->d_dist);
        cudaFree(sl->d_idx);
        cudaFreeHost(sl->h_q);
        cudaFreeHost(sl->h_dist);
        cudaFreeHost(sl->h_idx);
        for (DevBuf* b : {&sl->E.cn, &sl->E.qn, &sl->E.part, &sl->E.hi, &sl->E.lo, &sl->E.bf, &sl->E.err, &sl->E.thr,
                          &sl->E.loflags, &sl->E.cn_s, &sl->E.thr2, &sl->E.redo, &sl->E.qbf, &sl->E.cand, &sl->E.cnt,
                          &sl->E.tq, &sl->E.cnv, &sl->E.fail, &sl->E.words, &sl->E.in_corpus, &sl->E.in_queries,
                          &sl->E.out_dist, &sl->E.out_idx})
            b->release();
    }
    delete sv;
}

}  // extern "C"
