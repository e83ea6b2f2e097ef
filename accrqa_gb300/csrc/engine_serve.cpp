// engine_serve.cpp -- a request server with continuous batching.
//
// Requests (one series each, any measure mix) are submitted from any thread.
// Their life:
//   waiting  -> submitted; the inputs are copied, nothing is on the device.
//   resident -> admitted: one admission thread takes waiting requests in
//               arrival order and admits each when its device bytes fit the
//               server's fraction of the device memory free at that moment
//               (cudaMemGetInfo at every decision, so memory other work frees
//               or takes counts at once); the series (and the float filter's
//               split of a float64 series) is uploaded once, on an upload
//               stream that overlaps the passes already on the GPU, and stays
//               on the device until the request completes.
//   running  -> K worker threads, each with a private engine context
//               (stream, side streams, arena, pinned staging), take resident
//               requests in arrival order up to one work quantum, run them
//               as one batch -- or, taken alone, through the per-series path
//               -- on the resident series, write the results to the caller's
//               buffers, complete the requests and free their device memory,
//               which lets the admission thread admit more.
// Requests that arrive while batches are on the GPU are admitted and picked
// up by the next free worker, so their work overlaps on the device and
// nobody waits for a fixed batching window.  A request whose device bytes do
// not fit even on an otherwise empty server completes with
// ERR_CUDA_NOT_ENOUGH_MEMORY.  Results are written straight into the
// caller's output buffers, which must stay valid until the request is
// waited for.
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
    size_t bytes = 0;           // device bytes admission reserves for it
    size_t series_bytes = 0;    // of which the resident series (and split)
    double work = 0;            // cells x thresholds x measures, float64 weighted
    Clock::time_point t_submit, t_done;
    bool done = false;
    Accrqa_Error err = SUCCESS;
    // resident state
    bool admitted = false;      // counted in the server's admitted bytes
    void *d_block = nullptr;
    ResidentSeries rs;
    cudaEvent_t uploaded = nullptr;
};

}  // namespace

}  // namespace accrqa

// The opaque server handle of the C ABI.
struct accrqa_gb300_server {
    std::mutex mu;
    std::condition_variable cv_admit, cv_work, cv_done;
    std::deque<accrqa::Request *> waiting, resident;
    std::unordered_map<int64_t, std::unique_ptr<accrqa::Request>> live;
    int64_t next_id = 0;
    bool stop = false;        // no more submissions; drain and end
    bool admit_done = false;  // the admission thread has ended
    int device = 0;
    double fraction = 0.5;    // of the device memory free at each admission
    size_t admitted_bytes = 0;
    int admitted = 0;         // resident or running requests
    size_t peak_admitted_bytes = 0;
    double quantum = 0;       // estimated work (cell-thresholds) per worker batch
    cudaStream_t upload = nullptr;
    std::thread admitter;
    std::vector<std::thread> workers;
    std::vector<accrqa::Context *> ctxs;
    uint64_t batches = 0, served = 0;
    // At most one request larger than a quantum runs at a time: two of them
    // side by side only stretch each other, while small batches still fill
    // the GPU around one.
    std::mutex big_mu;

    void complete(std::vector<accrqa::Request *> &rs, Accrqa_Error e) {
        const auto now = accrqa::Clock::now();
        {
            std::lock_guard<std::mutex> lk(mu);
            for (accrqa::Request *r : rs) {
                r->err = e;
                r->done = true;
                r->t_done = now;
                if (r->admitted) {
                    admitted_bytes -= r->bytes;
                    admitted--;
                    r->admitted = false;
                }
            }
            served += rs.size();
        }
        cv_done.notify_all();
        cv_admit.notify_all();
    }

    // Upload one admitted request's series (and float filter split) into its
    // device block, on the upload stream.
    Accrqa_Error upload_series(accrqa::Request &r) {
        using namespace accrqa;
        const accrqa_gb300_series_job &J = r.job;
        const size_t es = J.dtype == ACCRQA_GB300_F32 ? 4 : 8;
        const size_t xb = (size_t)(J.n + ACCRQA_SERIES_PAD) * es;
        char *base = (char *)r.d_block;
        cudaError_t e = cudaMemcpyAsync(base, J.x, (size_t)J.n * es, cudaMemcpyHostToDevice, upload);
        if (e == cudaSuccess)
            e = cudaMemsetAsync(base + (size_t)J.n * es, 0, ACCRQA_SERIES_PAD * es, upload);
        transfer_stats_add((size_t)J.n * es, 0);
        r.rs.x = base;
        if (e == cudaSuccess && J.dtype == ACCRQA_GB300_F64 && r.series_bytes > xb) {
            const size_t fb = (size_t)(J.n + ACCRQA_SERIES_PAD) * 4;
            std::vector<float> hi((size_t)J.n + ACCRQA_SERIES_PAD, 0.0f),
                lo((size_t)J.n + ACCRQA_SERIES_PAD, 0.0f);
            double m = 0.0;
            f64_split((const double *)J.x, J.n, hi.data(), lo.data(), &m);
            e = cudaMemcpyAsync(base + xb, hi.data(), fb, cudaMemcpyHostToDevice, upload);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(base + xb + fb, lo.data(), fb, cudaMemcpyHostToDevice, upload);
            // the host vectors must outlive the (pageable) copies
            if (e == cudaSuccess) e = cudaStreamSynchronize(upload);
            transfer_stats_add(2 * fb, 0);
            r.rs.hi = (const float *)(base + xb);
            r.rs.lo = (const float *)(base + xb + fb);
            r.rs.maxabs = m;
        }
        if (e == cudaSuccess) e = cudaEventRecord(r.uploaded, upload);
        return e == cudaSuccess ? SUCCESS : cuda_error(e, "request upload");
    }

    void admit_loop() {
        using namespace accrqa;
        cudaSetDevice(device);
        for (;;) {
            Request *r = nullptr;
            {
                std::unique_lock<std::mutex> lk(mu);
                cv_admit.wait(lk, [&] { return stop || !waiting.empty(); });
                if (waiting.empty()) break;   // stop requested and nothing left
                r = waiting.front();
            }
            // Admission by the device memory free now: the admitted requests'
            // bytes plus this one's within `fraction` of (free + admitted).
            bool fits = false, alone = false;
            for (;;) {
                size_t free_b = 0, total_b = 0;
                if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
                    cudaGetLastError();
                    free_b = 0;
                }
                std::unique_lock<std::mutex> lk(mu);
                const double cap = fraction * (double)(free_b + admitted_bytes);
                fits = (double)(admitted_bytes + r->bytes) <= cap;
                alone = admitted == 0;
                if (fits || alone) break;
                // wait for a completion to free memory
                const int before = admitted;
                cv_admit.wait_for(lk, std::chrono::milliseconds(20),
                                  [&] { return admitted < before; });
            }
            Accrqa_Error err = SUCCESS;
            if (!fits) {
                set_last_error("request needs %zu device bytes, more than the server may use",
                               r->bytes);
                err = ERR_CUDA_NOT_ENOUGH_MEMORY;
            } else {
                // stream-ordered: no device-wide synchronisation, and the
                // memory returns to the pool when the worker frees it
                cudaError_t e = alloc_fault() ? cudaErrorMemoryAllocation
                                              : cudaMallocAsync(&r->d_block, r->series_bytes, upload);
                if (e != cudaSuccess) {
                    cudaGetLastError();
                    r->d_block = nullptr;
                    err = cuda_error(e, "cudaMalloc(request)");
                } else if ((e = cudaEventCreateWithFlags(&r->uploaded,
                                                         cudaEventDisableTiming)) != cudaSuccess) {
                    err = cuda_error(e, "cudaEventCreate");
                } else {
                    err = upload_series(*r);
                }
            }
            {
                std::lock_guard<std::mutex> lk(mu);
                waiting.pop_front();
                if (r->d_block && err == SUCCESS) {
                    r->admitted = true;
                    admitted_bytes += r->bytes;
                    admitted++;
                    if (admitted_bytes > peak_admitted_bytes) peak_admitted_bytes = admitted_bytes;
                    resident.push_back(r);
                }
            }
            if (err != SUCCESS) {
                if (r->d_block) cudaFreeAsync(r->d_block, upload);
                r->d_block = nullptr;
                if (r->uploaded) cudaEventDestroy(r->uploaded);
                r->uploaded = nullptr;
                std::vector<Request *> one{r};
                complete(one, err);
            } else {
                cv_work.notify_one();
            }
        }
        std::lock_guard<std::mutex> lk(mu);
        admit_done = true;
        cv_work.notify_all();
    }

    void work(int w) {
        using namespace accrqa;
        cudaSetDevice(device);
        Context *c = ctxs[(size_t)w];
        for (;;) {
            std::vector<Request *> take;
            {
                std::unique_lock<std::mutex> lk(mu);
                cv_work.wait(lk, [&] { return !resident.empty() || admit_done; });
                if (resident.empty()) return;   // admission ended and nothing left
                // Work within one batch quantum, so a large request runs on
                // its own while small ones batch up.
                double work = 0.0;
                while (!resident.empty()) {
                    Request *r = resident.front();
                    if (!take.empty() && work + r->work > quantum) break;
                    work += r->work;
                    take.push_back(r);
                    resident.pop_front();
                }
            }
            for (Request *r : take) cudaStreamWaitEvent(c->stream, r->uploaded, 0);
            // A request taken alone goes through the per-series path (no
            // batch planning, graph or job tables to build for one series).
            Accrqa_Error e;
            if (take.size() == 1 && take[0]->work > quantum) {
                std::lock_guard<std::mutex> big(big_mu);
                e = run_job_resident(*c, take[0]->job, take[0]->rs);
            } else if (take.size() == 1) {
                e = run_job_resident(*c, take[0]->job, take[0]->rs);
            } else {
                std::vector<accrqa_gb300_series_job> jobs;
                std::vector<ResidentSeries> rs;
                jobs.reserve(take.size());
                for (Request *r : take) {
                    jobs.push_back(r->job);
                    rs.push_back(r->rs);
                }
                size_t need = 0;
                for (const auto &j : jobs) need += batch_job_bytes(j) + batch_job_level_bytes(j);
                e = run_batch_in(*c, jobs.data(), (int)jobs.size(), need + (need >> 2) + 4096,
                                 rs.data());
            }
            // the results are on the host: free the requests' device memory
            // (stream-ordered, after the passes that read it)
            for (Request *r : take) {
                if (r->d_block) cudaFreeAsync(r->d_block, c->stream);
                r->d_block = nullptr;
                if (r->uploaded) cudaEventDestroy(r->uploaded);
                r->uploaded = nullptr;
            }
            cudaStreamSynchronize(c->stream);
            {
                std::lock_guard<std::mutex> lk(mu);
                batches++;
            }
            complete(take, e);
        }
    }
};

typedef accrqa_gb300_server Server;

namespace {

void release_context(accrqa::Context *c) {
    cudaStreamSynchronize(c->stream);
    // device buffers and streams of a worker context are released here
    c->series.release();
    c->series_hi.release();
    c->series_lo.release();
    c->counts.release();
    c->hist.release();
    c->maxlen.release();
    c->pairs.release();
    c->pair_count.release();
    c->arena.release();
    if (c->pinned) cudaFreeHost(c->pinned);
    for (cudaStream_t st : c->side) cudaStreamDestroy(st);
    cudaStreamDestroy(c->stream);
    delete c;
}

}  // namespace

extern "C" {

Server *accrqa_gb300_server_create(int32_t workers, double hbm_fraction) {
    using namespace accrqa;
    if (workers < 1) workers = 1;
    if (!(hbm_fraction > 0.0) || hbm_fraction > 0.9) hbm_fraction = 0.5;
    Accrqa_Error err = SUCCESS;
    if (!current_context(&err)) return nullptr;   // checks that a device exists
    std::unique_ptr<Server> s(new Server());
    cudaGetDevice(&s->device);
    s->fraction = hbm_fraction;
    // about 1 ms of float32 work on a GB300 (~1.7e13 cell-thresholds per
    // second): a request in a batch completes when the whole batch does, and
    // one series already fills the GPU, so batches stay short
    s->quantum = 2.0e10;
    cudaError_t e = cudaStreamCreateWithFlags(&s->upload, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        cuda_error(e, "cudaStreamCreate(upload)");
        return nullptr;
    }
    for (int w = 0; w < workers; w++) {
        Context *c = context_create(&err);
        if (!c) {
            // release what was made so far
            for (Context *made : s->ctxs) release_context(made);
            cudaStreamDestroy(s->upload);
            return nullptr;
        }
        s->ctxs.push_back(c);
    }
    Server *raw = s.get();
    raw->admitter = std::thread([raw] { raw->admit_loop(); });
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
    // resident: the padded series, and the float filter's split when a
    // float64 series takes it; admitted: that plus what its passes allocate
    r->series_bytes = (size_t)(job->n + ACCRQA_SERIES_PAD) * es;
    double m = 0.0;
    if (job->dtype == ACCRQA_GB300_F64 && f64_filterable((const double *)r->job.x, job->n, &m))
        r->series_bytes += 2 * (size_t)(job->n + ACCRQA_SERIES_PAD) * 4;
    r->bytes = batch_job_bytes(r->job) + batch_job_level_bytes(r->job) + r->series_bytes;
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
    s->waiting.push_back(r.get());
    s->live[id] = std::move(r);
    s->cv_admit.notify_one();
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

uint64_t accrqa_gb300_server_peak_bytes(Server *s) {
    if (!s) return 0;
    std::lock_guard<std::mutex> lk(s->mu);
    return s->peak_admitted_bytes;
}

void accrqa_gb300_server_destroy(Server *s) {
    if (!s) return;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->cv_admit.notify_all();
    s->admitter.join();
    s->cv_work.notify_all();
    for (std::thread &t : s->workers) t.join();
    for (accrqa::Context *c : s->ctxs) release_context(c);
    cudaStreamDestroy(s->upload);
    delete s;
}

}  // extern "C"
