// engine_serve.cpp -- a request server with continuous batching.
//
// Requests (one series each, any measure mix) are submitted from any thread
// and queued with their arrival time.  K worker threads, each owning a private
// engine context (stream, side streams, device arena, pinned staging), loop:
// take queued requests in arrival order while they fit the worker's
// device-memory budget and one work quantum (at least one request), run them
// as one batch (engine_batch.cpp) -- or, when only one was taken, through the
// per-series path -- and complete them.  A request that arrives while batches are
// on the GPU is picked up by the next free worker, so batches overlap on the
// device and nobody waits for a fixed batching window.  Results are written
// straight into the caller's output buffers, which must stay valid until the
// request is waited for; inputs are copied at submission.
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "engine.hpp"

namespace accrqa {
namespace {

typedef std::chrono::steady_clock Clock;

struct Request {
    int64_t id = 0;
    accrqa_gb300_series_job job;
    std::vector<char> x, thr;   // owned copies of the inputs
    size_t bytes = 0;
    double work = 0;   // cells x thresholds x measures, float64 weighted
    Clock::time_point t_submit, t_done;
    bool done = false;
    Accrqa_Error err = SUCCESS;
};

}  // namespace

}  // namespace accrqa

// The opaque server handle of the C ABI.
struct accrqa_gb300_server {
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<accrqa::Request *> pending;
    std::unordered_map<int64_t, std::unique_ptr<accrqa::Request>> live;
    int64_t next_id = 0;
    bool stop = false;
    int device = 0;
    size_t budget = 0;   // device bytes per worker batch
    double quantum = 0;  // estimated work (cell-thresholds) per worker batch
    std::vector<std::thread> workers;
    std::vector<accrqa::Context *> ctxs;
    uint64_t batches = 0, served = 0;
    // At most one request larger than a quantum runs at a time: two of them
    // side by side only stretch each other, while small batches still fill
    // the GPU around one.
    std::mutex big_mu;

    void work(int w) {
        using namespace accrqa;
        cudaSetDevice(device);
        Context *c = ctxs[(size_t)w];
        for (;;) {
            std::vector<Request *> take;
            {
                std::unique_lock<std::mutex> lk(mu);
                cv_work.wait(lk, [&] { return stop || !pending.empty(); });
                if (pending.empty()) return;   // stop requested and nothing left
                // Admission: device bytes within the worker's share of free
                // HBM, and estimated work within one batch quantum, so a
                // large request runs on its own while small ones batch up.
                size_t used = 0;
                double work = 0.0;
                while (!pending.empty()) {
                    Request *r = pending.front();
                    if (!take.empty() &&
                        (used + r->bytes > budget || work + r->work > quantum))
                        break;
                    used += r->bytes;
                    work += r->work;
                    take.push_back(r);
                    pending.pop_front();
                }
            }
            // A request taken alone goes through the per-series path (no
            // batch planning, graph or job tables to build for one series).
            Accrqa_Error e;
            if (take.size() == 1 && take[0]->work > quantum) {
                std::lock_guard<std::mutex> big(big_mu);
                e = run_job_plain(*c, take[0]->job);
            } else if (take.size() == 1) {
                e = run_job_plain(*c, take[0]->job);
            } else {
                std::vector<accrqa_gb300_series_job> jobs;
                jobs.reserve(take.size());
                for (Request *r : take) jobs.push_back(r->job);
                e = run_batch_in(*c, jobs.data(), (int)jobs.size(), budget);
            }
            const auto now = Clock::now();
            {
                std::lock_guard<std::mutex> lk(mu);
                for (Request *r : take) {
                    r->err = e;
                    r->done = true;
                    r->t_done = now;
                }
                batches++;
                served += take.size();
            }
            cv_done.notify_all();
        }
    }
};

typedef accrqa_gb300_server Server;

extern "C" {

Server *accrqa_gb300_server_create(int32_t workers, double hbm_fraction) {
    using namespace accrqa;
    if (workers < 1) workers = 1;
    if (!(hbm_fraction > 0.0) || hbm_fraction > 0.9) hbm_fraction = 0.5;
    Accrqa_Error err = SUCCESS;
    if (!current_context(&err)) return nullptr;   // checks that a device exists
    std::unique_ptr<Server> s(new Server());
    cudaGetDevice(&s->device);
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
        cudaGetLastError();
        free_b = (size_t)8 << 30;
    }
    s->budget = (size_t)((double)free_b * hbm_fraction / workers);
    // about 1 ms of float32 work on a GB300 (~1.7e13 cell-thresholds per
    // second): a request in a batch completes when the whole batch does, and
    // one series already fills the GPU, so batches stay short
    s->quantum = 2.0e10;
    for (int w = 0; w < workers; w++) {
        Context *c = context_create(&err);
        if (!c) return nullptr;
        s->ctxs.push_back(c);
    }
    Server *raw = s.get();
    for (int w = 0; w < workers; w++) raw->workers.emplace_back([raw, w] { raw->work(w); });
    return s.release();
}

int64_t accrqa_gb300_server_submit(Server *s, const accrqa_gb300_series_job *job) {
    using namespace accrqa;
    if (!s || !job) return -(int64_t)ERR_MEM_ALLOC_FAILURE;
    const Accrqa_Error e = check_batch_job(*job);
    if (e) return -(int64_t)e;
    std::unique_ptr<Request> r(new Request());
    r->job = *job;
    const size_t es = job->dtype == ACCRQA_GB300_F32 ? 4 : 8;
    r->x.assign((const char *)job->x, (const char *)job->x + (size_t)job->n * es);
    r->thr.assign((const char *)job->thresholds,
                  (const char *)job->thresholds + (size_t)job->nthr * es);
    r->job.x = r->x.data();
    r->job.thresholds = r->thr.data();
    r->bytes = batch_job_bytes(r->job);
    {
        const double nc = (double)(job->n - (int64_t)(job->emb - 1) * job->tau);
        const int measures = (job->rr_out ? 1 : 0) + (job->det_out ? 1 : 0) + (job->lam_out ? 2 : 0);
        // float64 runs through the float filter at about half the float32 speed
        r->work = nc * nc * (double)job->nthr * measures * (job->dtype == ACCRQA_GB300_F64 ? 2.0 : 1.0);
    }
    r->t_submit = std::chrono::steady_clock::now();
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->stop) return -(int64_t)ERR_RUNTIME;
    r->id = s->next_id++;
    const int64_t id = r->id;
    s->pending.push_back(r.get());
    s->live[id] = std::move(r);
    s->cv_work.notify_one();
    return id;
}

Accrqa_Error accrqa_gb300_server_wait(Server *s, int64_t ticket, double *latency_ms) {
    using namespace accrqa;
    if (!s) return ERR_MEM_ALLOC_FAILURE;
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->live.find(ticket);
    if (it == s->live.end()) return ERR_INVALID_ARGUMENT;
    Request *r = it->second.get();
    s->cv_done.wait(lk, [&] { return r->done; });
    if (latency_ms)
        *latency_ms = std::chrono::duration<double, std::milli>(r->t_done - r->t_submit).count();
    const Accrqa_Error e = r->err;
    s->live.erase(it);
    return e;
}

void accrqa_gb300_server_stats(Server *s, uint64_t *batches, uint64_t *served) {
    if (!s) return;
    std::lock_guard<std::mutex> lk(s->mu);
    if (batches) *batches = s->batches;
    if (served) *served = s->served;
}

void accrqa_gb300_server_destroy(Server *s) {
    if (!s) return;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->cv_work.notify_all();
    for (std::thread &t : s->workers) t.join();
    for (accrqa::Context *c : s->ctxs) {
        cudaStreamSynchronize(c->stream);
        // device buffers and streams of a worker context are released here
        c->series.release();
        c->series_hi.release();
        c->series_lo.release();
        c->counts.release();
        c->hist.release();
        c->maxlen.release();
        c->arena.release();
        if (c->pinned) cudaFreeHost(c->pinned);
        for (cudaStream_t st : c->side) cudaStreamDestroy(st);
        cudaStreamDestroy(c->stream);
        delete c;
    }
    delete s;
}

}  // extern "C"
