// Request server with continuous batching (imex_server_* of the C ABI).
//
// Callers submit Taylor-Green solves from any thread; a server thread owns
// the GPU work.  Each tick it
//   1. launches one batched tick (imex_batch_step, a CUDA graph of K steps)
//      advancing every active request by up to K steps,
//   2. while that runs, admits queued requests in arrival order as long as
//      a slot is free and the request's device memory fits the budget
//      (creating its lattice and initialising it on its own stream, so the
//      initialisation overlaps the tick), and
//   3. waits for the tick and retires the requests that reached their step
//      count: reads their diagnostics, saves their state if asked (a later
//      request can resume from it), publishes the result, frees their
//      memory and slot.
// Requests therefore join and leave between ticks while the others keep
// running: the batch is the set of requests in flight, not a queue drained
// one job at a time.  Every request's result is bit-identical to running it
// alone (the batched kernel's arithmetic is the single-lattice one).
//
// Admission is first-come first-served by default: a request that does not
// fit waits at the head of the queue (no overtaking), so time-to-result
// includes the queueing time under overload.  IMEX_POLICY_LEAST_WORK admits
// the queued request with the least work (cells x steps) first instead:
// shorter median time-to-result under overload, at the price of large
// requests waiting until the queue drains.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "imexlbm.h"
#include "imexlbm_internal.hpp"
#include "lattice_internal.hpp"

namespace {

using Clock = std::chrono::steady_clock;

struct Pending {
    int64_t id;
    imex_request req;
    double t_submit;
};

struct Active {
    int64_t id;
    imex_request req;
    imex_lattice* h;
    size_t bytes;
    double t_submit, t_admit;
};

double request_work(const imex_request& r) { return (double)r.nx * r.ny * r.nz * (double)r.steps; }

size_t request_bytes(const imex_request& r)
{
    const size_t cells = (size_t)r.nx * r.ny * r.nz;
    return 2 * (size_t)27 * cells * imex::lattice_elem_size(r.precision) + (1u << 20);
}

}  // namespace

struct imex_server {
    size_t budget = 0;
    int max_active = 0;
    int steps_per_tick = 0;
    int policy = IMEX_POLICY_ARRIVAL;
    int device = 0;
    Clock::time_point t0;
    imex_batch* batch = nullptr;

    std::mutex mu;  // guards queue, results, counters below, stop
    std::condition_variable cv;
    std::deque<Pending> queue;
    std::vector<imex_result> results;
    int64_t next_id = 1;
    bool stop = false;
    size_t bytes_in_use = 0;
    int n_active = 0;
    int64_t cell_updates = 0;
    int64_t ticks = 0;
    int64_t completed = 0;
    double busy_seconds = 0;
    std::string fatal;  // first server-thread error (the thread then stops)

    std::vector<Active> active;  // server thread only
    int64_t tuned_cells = 0;     // batch cells when the launch shapes were last tuned
    std::thread worker;

    double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }
};

namespace {

void publish(imex_server* s, const Active& a, int status, const double* cons)
{
    imex_result r{};
    r.id = a.id;
    r.tag = a.req.tag;
    r.status = status;
    if (cons)
        for (int q = 0; q < 5; ++q) r.conserved[q] = cons[q];
    r.steps = a.h ? imex_steps_done(a.h) : 0;
    r.cells = (int64_t)a.req.nx * a.req.ny * a.req.nz;
    r.t_submit = a.t_submit;
    r.t_admit = a.t_admit;
    r.t_done = s->now();
    std::lock_guard<std::mutex> g(s->mu);
    s->results.push_back(r);
    ++s->completed;
}

// Create, initialise and batch the admitted requests.
void admit(imex_server* s, std::vector<Pending>& incoming)
{
    for (Pending& p : incoming) {
        Active a{p.id, p.req, nullptr, request_bytes(p.req), p.t_submit, s->now()};
        const imex_request& q = p.req;
        int rc = imex_create(q.nx, q.ny, q.nz, q.tau, q.rho0, q.u0, q.precision, &a.h);
        if (!rc && q.precision == IMEX_F16DEV) rc = imex_set_rounding(a.h, q.rounding);
        if (!rc)
            rc = q.resume_path[0] ? imex_checkpoint_load(a.h, q.resume_path)
                                  : imex_initialize_phase(a.h, q.phase[0], q.phase[1], q.phase[2]);
        if (!rc) rc = imex_batch_add(s->batch, a.h, q.steps);
        if (rc) {
            publish(s, a, rc, nullptr);
            imex_destroy(a.h);
            std::lock_guard<std::mutex> g(s->mu);
            s->bytes_in_use -= a.bytes;
            --s->n_active;
            continue;
        }
        s->active.push_back(a);
    }
    incoming.clear();
}

// Requests at their step count: diagnostics, result, release.
int retire(imex_server* s)
{
    for (size_t i = 0; i < s->active.size();) {
        Active& a = s->active[i];
        if (imex_steps_done(a.h) < a.req.steps) {
            ++i;
            continue;
        }
        double cons[5];
        int rc2 = imex_batch_remove(s->batch, a.h);
        int rc = imex_conserved(a.h, cons);
        if (a.req.save_path[0]) {
            const int rs = imex_checkpoint_save(a.h, a.req.save_path);
            if (rs && (!rc || rc == IMEX_ERR_NONFINITE)) rc = rs;
        }
        publish(s, a, rc, cons);
        imex_destroy(a.h);
        {
            std::lock_guard<std::mutex> g(s->mu);
            s->bytes_in_use -= a.bytes;
            --s->n_active;
        }
        s->active.erase(s->active.begin() + i);
        if (rc2) return rc2;
    }
    return IMEX_OK;
}

void serve(imex_server* s)
{
    cudaSetDevice(s->device);
    std::vector<Pending> incoming;
    for (;;) {
        // take what fits, in arrival order
        {
            std::unique_lock<std::mutex> lk(s->mu);
            if (s->active.empty() && s->queue.empty() && incoming.empty())
                s->cv.wait_for(lk, std::chrono::milliseconds(20));
            if (s->stop) break;
            while (!s->queue.empty() && s->n_active < s->max_active) {
                // next in line: the head (arrival order), or the queued
                // request with the least work (cells x steps)
                auto pick = s->queue.begin();
                if (s->policy == IMEX_POLICY_LEAST_WORK)
                    for (auto it = s->queue.begin(); it != s->queue.end(); ++it)
                        if (request_work(it->req) < request_work(pick->req)) pick = it;
                const size_t b = request_bytes(pick->req);
                if (s->bytes_in_use + b > s->budget && s->n_active > 0) break;  // it waits for memory
                incoming.push_back(*pick);
                s->queue.erase(pick);
                s->bytes_in_use += b;
                ++s->n_active;
            }
        }
        if (s->active.empty()) {
            admit(s, incoming);
            continue;
        }
        // one tick of the batch; admissions overlap it
        const auto t_tick = Clock::now();
        int64_t before = 0, cells = 0;
        for (const Active& a : s->active) {
            const int64_t c = (int64_t)a.req.nx * a.req.ny * a.req.nz;
            before += imex_steps_done(a.h) * c;
            cells += c;
        }
        // The launch shapes were tuned for the batch as it was; when its
        // size has changed by more than 2x, let the batch tune them again.
        if (cells > 2 * s->tuned_cells || 2 * cells < s->tuned_cells) {
            imex_batch_set_launch(s->batch, 0, 0, 0);
            imex_batch_set_row_launch(s->batch, 0, 0, 0, 1);
            s->tuned_cells = cells;
        }
        int rc = imex_batch_step(s->batch, s->steps_per_tick);
        if (!rc) admit(s, incoming);
        if (!rc) rc = imex_batch_synchronize(s->batch);
        int64_t after = 0;
        for (const Active& a : s->active) after += imex_steps_done(a.h) * (int64_t)a.req.nx * a.req.ny * a.req.nz;
        if (!rc) rc = retire(s);
        {
            std::lock_guard<std::mutex> g(s->mu);
            ++s->ticks;
            s->cell_updates += after - before;
            s->busy_seconds += std::chrono::duration<double>(Clock::now() - t_tick).count();
            if (rc && s->fatal.empty()) s->fatal = imex_batch_last_error(s->batch);
        }
        if (rc) break;
    }
    // stopping: release everything still active or admitted
    admit(s, incoming);
    for (Active& a : s->active) {
        imex_batch_remove(s->batch, a.h);
        publish(s, a, IMEX_ERR_STATE, nullptr);
        imex_destroy(a.h);
    }
    s->active.clear();
}

}  // namespace

extern "C" {

int imex_server_create(size_t budget_bytes, int max_active, int steps_per_tick, imex_server** out)
{
    if (!out) return imex::set_thread_error(IMEX_ERR_ARG, "imex_server_create: null output");
    *out = nullptr;
    if (budget_bytes == 0 || max_active < 1 || max_active > 2048 || steps_per_tick < 1)
        return imex::set_thread_error(IMEX_ERR_ARG, "imex_server_create: need budget > 0, 1 <= max_active <= 2048, "
                                                    "steps_per_tick >= 1");
    imex_server* s = new imex_server();
    s->budget = budget_bytes;
    s->max_active = max_active;
    s->steps_per_tick = steps_per_tick;
    s->t0 = Clock::now();
    cudaError_t e = cudaGetDevice(&s->device);
    if (e != cudaSuccess) {
        delete s;
        cudaGetLastError();
        return imex::set_thread_error(IMEX_ERR_CUDA, std::string("imex_server_create: ") + cudaGetErrorString(e));
    }
    // Keep memory freed by retired requests in the device pool for the next
    // admissions instead of returning it to the driver at every sync.
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, s->device) == cudaSuccess) {
        unsigned long long keep = ~0ull;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    int rc = imex_batch_create(max_active, &s->batch);
    if (rc) {
        delete s;
        return rc;
    }
    imex_batch_set_graph(s->batch, steps_per_tick);
    s->worker = std::thread(serve, s);
    *out = s;
    return IMEX_OK;
}

int imex_server_submit(imex_server* s, const imex_request* req, int64_t* id)
{
    if (!s || !req) return imex::set_thread_error(IMEX_ERR_ARG, "imex_server_submit: null argument");
    if (std::memchr(req->resume_path, 0, sizeof req->resume_path) == nullptr ||
        std::memchr(req->save_path, 0, sizeof req->save_path) == nullptr)
        return imex::set_thread_error(IMEX_ERR_ARG, "imex_server_submit: resume_path and save_path must be "
                                                    "NUL-terminated within 256 bytes");
    if (req->nx < 1 || req->ny < 1 || req->nz < 1 || req->steps < 0 ||
        (req->precision != IMEX_F32 && req->precision != IMEX_F16DEV) ||
        (req->rounding != IMEX_ROUND_NEAREST && req->rounding != IMEX_ROUND_STOCHASTIC))
        return imex::set_thread_error(IMEX_ERR_ARG, "imex_server_submit: bad request (sizes >= 1, steps >= 0, "
                                                    "precision IMEX_F32 or IMEX_F16DEV, a valid rounding)");
    if (request_bytes(*req) > s->budget)
        return imex::set_thread_error(IMEX_ERR_MEMORY, "imex_server_submit: request larger than the memory budget");
    std::lock_guard<std::mutex> g(s->mu);
    if (!s->fatal.empty()) return imex::set_thread_error(IMEX_ERR_STATE, "imex_server_submit: server stopped: " + s->fatal);
    Pending p{s->next_id++, *req, s->now()};
    if (id) *id = p.id;
    s->queue.push_back(p);
    s->cv.notify_one();
    return IMEX_OK;
}

int imex_server_poll(imex_server* s, imex_result* out, int max, int* n)
{
    if (!s || !n || (max > 0 && !out)) return imex::set_thread_error(IMEX_ERR_ARG, "imex_server_poll: null argument");
    std::lock_guard<std::mutex> g(s->mu);
    const int k = (int)std::min<size_t>((size_t)std::max(max, 0), s->results.size());
    for (int i = 0; i < k; ++i) out[i] = s->results[i];
    s->results.erase(s->results.begin(), s->results.begin() + k);
    *n = k;
    return IMEX_OK;
}

int imex_server_get_stats(imex_server* s, imex_server_stats* out)
{
    if (!s || !out) return imex::set_thread_error(IMEX_ERR_ARG, "imex_server_get_stats: null argument");
    std::lock_guard<std::mutex> g(s->mu);
    out->queued = (int64_t)s->queue.size();
    out->active = s->n_active;
    out->completed = s->completed;
    out->bytes_in_use = (int64_t)s->bytes_in_use;
    out->cell_updates = s->cell_updates;
    out->ticks = s->ticks;
    out->busy_seconds = s->busy_seconds;
    out->now = s->now();
    out->failed = s->fatal.empty() ? 0 : 1;
    return IMEX_OK;
}

double imex_server_now(const imex_server* s) { return s ? s->now() : -1.0; }

int imex_server_set_policy(imex_server* s, int policy)
{
    if (!s || (policy != IMEX_POLICY_ARRIVAL && policy != IMEX_POLICY_LEAST_WORK))
        return imex::set_thread_error(IMEX_ERR_ARG, "imex_server_set_policy: null server or unknown policy");
    std::lock_guard<std::mutex> g(s->mu);
    s->policy = policy;
    return IMEX_OK;
}

void imex_server_destroy(imex_server* s)
{
    if (!s) return;
    {
        std::lock_guard<std::mutex> g(s->mu);
        s->stop = true;
    }
    s->cv.notify_all();
    if (s->worker.joinable()) s->worker.join();
    imex_batch_destroy(s->batch);
    delete s;
}

}  // extern "C"
