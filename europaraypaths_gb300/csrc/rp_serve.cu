// rp_serve.cu -- the resident request loop (rp_server_*, rp_submit, rp_poll).
//
// Worker threads, each with its own CUDA stream and rp_workspace, serve
// requests from one FIFO queue under a device-memory budget.  A request is
// cut into steps of at most step_traces traces (the whole request when the
// step is 0).  Each worker call takes the next step of up to max_batch
// requests that are already running (round robin), then admits queued
// requests in FIFO order while they fit the budget and the active-request
// limit, and runs all the fast-form steps it took as one rp_simulate_batch
// call: continuous batching at step granularity.  A request that arrives
// while others run joins at the next call of any worker; short requests
// finish without waiting for long ones; several workers' calls overlap on
// the device.  Queued requests older than max_wait_ms are shed
// (RP_ERR_TIMEOUT).  Host side only; the kernels are those of the two forms.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "rp_internal.h"

namespace {

double now_s() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

enum { Q_QUEUED = 0, Q_ACTIVE = 1, Q_DONE = 2 };

struct SrvReq {
    int64_t id = 0;
    rp_scene* sc = nullptr;
    std::vector<double> tr;
    int64_t ns = 0;
    int form = 0;
    void* out = nullptr;
    int64_t* user_counts = nullptr;
    std::vector<int64_t> counts;
    int64_t fp = 0;
    double t_submit = 0, t_start = 0, t_end = 0;
    int state = Q_QUEUED;
    int rc = RP_OK;
    std::string err;
    // step scheduling (guarded by the server mutex)
    int64_t step = 0;       // traces per step
    int64_t next = 0;       // first trace not yet handed to a worker
    int64_t finished = 0;   // traces whose step completed (or was dropped after a failure)
    int running = 0;        // steps of this request in worker calls now
};

using ReqP = std::shared_ptr<SrvReq>;

bool batchable(const SrvReq& r) { return (r.form & 0xff) == RP_FORM_FAST_F32 && !(r.form & RP_OUT_COMPLEX128); }

size_t out_elem_bytes(const SrvReq& r) { return (r.form & RP_OUT_COMPLEX128) ? 16 : 8; }

// One step of a request in a worker call: traces [c0, c0 + len).
struct Step {
    ReqP r;
    int64_t c0 = 0, len = 0;
    int rc = RP_OK;
    std::string err;
};

}  // namespace

struct rp_server {
    int device = 0;
    int64_t budget = 0;
    int max_batch = 1;
    int64_t step_traces = 0;   // 0: whole requests
    int max_active = 0;        // 0: no limit but the budget
    int max_wait_ms = 0;       // 0: no bound on the queue wait
    bool fake = false;
    rp_executor ex{};
    std::mutex mu;
    std::condition_variable cv;
    std::deque<ReqP> q;
    std::vector<ReqP> active;
    size_t rr = 0;             // round-robin cursor over active
    std::unordered_map<int64_t, ReqP> reqs;
    int64_t next_id = 1;
    int64_t in_flight = 0;
    int running = 0;           // worker calls in progress
    bool stop = false;
    std::vector<std::thread> threads;
    // statistics
    std::vector<double> lat_ms, wait_ms;
    int64_t completed = 0, failed = 0, rejected = 0, cancelled = 0, shed = 0, calls = 0, steps = 0;
    int64_t max_in_call = 0, max_active_seen = 0, max_calls_running = 0;
    double pairs = 0, t_first = -1, t_last = 0;
};

namespace {

// Run the steps of one worker call on the GPU: per-step device buffers, one
// rp_simulate_batch over the steps when they are all fast-form (and more
// than one), else rp_simulate_ws per step; on a batch failure every step
// runs again alone, so an error stays with its own request.  Each step's
// radargram rows and counts land in its request's host output at the step's
// trace offset.
void gpu_call(std::vector<Step>& steps, rp_workspace* ws, cudaStream_t st) {
    const size_t n = steps.size();
    std::vector<double*> d_tr(n, nullptr);
    std::vector<void*> d_out(n, nullptr);
    std::vector<size_t> out_bytes(n, 0);
    bool all_batch = n > 1;
    auto fail_all = [&](int rc) {
        char buf[1024];
        rp_last_error(buf, sizeof(buf));
        for (auto& s : steps) { s.rc = rc; s.err = buf; }
    };
    for (size_t i = 0; i < n; ++i) {
        Step& s = steps[i];
        all_batch = all_batch && batchable(*s.r);
        out_bytes[i] = (size_t)s.len * s.r->sc->nr * out_elem_bytes(*s.r);
        cudaError_t e = cudaMallocAsync((void**)&d_tr[i], sizeof(double) * 9 * s.len, st);
        if (e == cudaSuccess) e = cudaMallocAsync(&d_out[i], out_bytes[i], st);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(d_tr[i], s.r->tr.data() + 9 * s.c0, sizeof(double) * 9 * s.len,
                                cudaMemcpyHostToDevice, st);
        if (e != cudaSuccess) {
            fail_all(rp_cuda_fail(e, "server buffers"));
            goto cleanup;
        }
    }
    {
        int rc = RP_OK;
        if (all_batch) {
            std::vector<rp_job> jobs(n);
            for (size_t i = 0; i < n; ++i)
                jobs[i] = rp_job{steps[i].r->sc, d_tr[i], steps[i].len, d_out[i],
                                 steps[i].r->counts.data() + 2 * steps[i].c0};
            rc = rp_simulate_batch(jobs.data(), (int)n, ws, st);
        }
        for (size_t i = 0; i < n; ++i) {
            Step& s = steps[i];
            int rci = rc;
            if (!all_batch || rc != RP_OK)
                rci = rp_simulate_ws(s.r->sc, ws, d_tr[i], s.len, s.r->form, d_out[i],
                                     s.r->counts.data() + 2 * s.c0, st);
            if (rci == RP_OK) {
                char* dst = static_cast<char*>(s.r->out) + (size_t)s.c0 * s.r->sc->nr * out_elem_bytes(*s.r);
                cudaError_t e = cudaMemcpyAsync(dst, d_out[i], out_bytes[i], cudaMemcpyDeviceToHost, st);
                if (e == cudaSuccess) e = cudaStreamSynchronize(st);
                if (e != cudaSuccess) rci = rp_cuda_fail(e, "server output copy");
            }
            s.rc = rci;
            if (rci != RP_OK) {
                char buf[1024];
                rp_last_error(buf, sizeof(buf));
                s.err = buf;
            }
        }
    }
cleanup:
    for (size_t i = 0; i < n; ++i) {
        if (d_tr[i]) cudaFreeAsync(d_tr[i], st);
        if (d_out[i]) cudaFreeAsync(d_out[i], st);
    }
    cudaStreamSynchronize(st);
}

// Bytes of one output row of a request: nr x (8 or 16), from the scene, or
// from the executor's bins() when an executor stands in for the GPU.
size_t row_bytes(const rp_server* S, const SrvReq& r);

void fake_call(rp_server* S, std::vector<Step>& steps) {
    for (auto& s : steps) {
        SrvReq& r = *s.r;
        char* dst = static_cast<char*>(r.out) + (size_t)s.c0 * row_bytes(S, r);
        s.rc = S->ex.run(S->ex.user, r.sc, r.tr.data() + 9 * s.c0, s.len, r.form, dst, r.counts.data() + 2 * s.c0);
        if (s.rc != RP_OK) s.err = "executor failed";
    }
}

size_t row_bytes(const rp_server* S, const SrvReq& r) {
    const int64_t nr = S->fake ? (S->ex.bins ? S->ex.bins(S->ex.user, r.sc) : 0) : r.sc->nr;
    return (size_t)nr * out_elem_bytes(r);
}

// Finish a request whose traces are all done (caller holds the lock).
void finish(rp_server* S, const ReqP& r, double t) {
    r->t_end = t;
    r->state = Q_DONE;
    S->in_flight -= r->fp;
    if (r->rc == RP_OK) {
        ++S->completed;
        S->lat_ms.push_back(1e3 * (r->t_end - r->t_submit));
        S->wait_ms.push_back(1e3 * (r->t_start - r->t_submit));
        for (int64_t k = 0; k < r->ns; ++k)
            S->pairs += (double)r->counts[2 * k] * (1.0 + 2.0 * (double)r->counts[2 * k + 1]);
        S->t_last = std::max(S->t_last, t);
        if (r->user_counts) std::copy(r->counts.begin(), r->counts.end(), r->user_counts);
    } else {
        ++S->failed;
    }
    S->active.erase(std::find(S->active.begin(), S->active.end(), r));
}

// Take the steps of one worker call (caller holds the lock): shed queued
// requests past the wait bound, then the next step of up to max_batch
// running requests (round robin), then queued requests in FIFO order while
// they fit the budget and the active limit.  A plain-form or complex128
// step runs alone; fast-form steps are grouped.
std::vector<Step> take_steps(rp_server* S, double t) {
    std::vector<Step> out;
    if (S->max_wait_ms > 0) {
        while (!S->q.empty() && 1e3 * (t - S->q.front()->t_submit) > (double)S->max_wait_ms) {
            ReqP r = S->q.front();
            S->q.pop_front();
            r->state = Q_DONE;
            r->rc = RP_ERR_TIMEOUT;
            r->err = "request waited in the queue longer than the server's bound";
            r->t_end = t;
            ++S->shed;
        }
    }
    const int maxa = S->max_active > 0 ? S->max_active : INT32_MAX;
    auto take = [&](const ReqP& r) -> bool {     // false: the call is full
        if (!out.empty() && (!batchable(*out[0].r) || !batchable(*r))) return false;
        Step s;
        s.r = r;
        s.c0 = r->next;
        s.len = std::min(r->step, r->ns - r->next);
        r->next += s.len;
        ++r->running;
        out.push_back(s);
        return (int)out.size() < S->max_batch && batchable(*r);
    };
    bool room = true;
    const size_t na = S->active.size();
    const size_t start = na ? S->rr % na : 0;
    for (size_t k = 0; k < na && room; ++k) {
        const size_t idx = (start + k) % na;
        const ReqP& r = S->active[idx];
        if (r->next >= r->ns || r->rc != RP_OK) continue;
        if (!out.empty() && (!batchable(*out[0].r) || !batchable(*r))) continue;
        room = take(r);
        S->rr = idx + 1;     // the next call starts after the last request served
    }
    while (room && !S->q.empty() && (int)S->active.size() < maxa &&
           S->in_flight + S->q.front()->fp <= S->budget) {
        ReqP r = S->q.front();
        if (!out.empty() && (!batchable(*out[0].r) || !batchable(*r))) break;
        S->q.pop_front();
        S->in_flight += r->fp;
        r->state = Q_ACTIVE;
        r->t_start = t;
        S->active.push_back(r);
        room = take(r);
    }
    S->max_active_seen = std::max<int64_t>(S->max_active_seen, (int64_t)S->active.size());
    return out;
}

void worker_main(rp_server* S) {
    cudaStream_t st = nullptr;
    rp_workspace* ws = nullptr;
    int setup_rc = RP_OK;
    char setup_err[1024] = "";
    if (!S->fake) {
        cudaSetDevice(S->device);
        cudaError_t e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
        if (e != cudaSuccess) setup_rc = rp_cuda_fail(e, "server stream");
        else setup_rc = rp_workspace_create(S->device, &ws);
        if (setup_rc != RP_OK) rp_last_error(setup_err, sizeof(setup_err));
    }
    for (;;) {
        std::vector<Step> steps;
        {
            std::unique_lock<std::mutex> lk(S->mu);
            bool quit = false;
            for (;;) {
                if (S->stop && S->q.empty() && S->active.empty()) { quit = true; break; }
                const int64_t shed0 = S->shed;
                steps = take_steps(S, now_s());
                if (S->shed != shed0) S->cv.notify_all();      // shed requests are finished
                if (!steps.empty()) break;
                // with a queue-wait bound, wake up now and then to shed
                if (S->max_wait_ms > 0) S->cv.wait_for(lk, std::chrono::milliseconds(std::max(1, S->max_wait_ms / 4)));
                else S->cv.wait(lk);
            }
            if (quit) break;
            ++S->running;
            ++S->calls;
            S->steps += (int64_t)steps.size();
            S->max_in_call = std::max<int64_t>(S->max_in_call, (int64_t)steps.size());
            S->max_calls_running = std::max<int64_t>(S->max_calls_running, (int64_t)S->running);
        }
        if (setup_rc != RP_OK) {
            for (auto& s : steps) { s.rc = setup_rc; s.err = setup_err; }
        } else if (S->fake) {
            fake_call(S, steps);
        } else {
            gpu_call(steps, ws, st);
        }
        {
            std::lock_guard<std::mutex> lk(S->mu);
            const double t = now_s();
            for (auto& s : steps) {
                const ReqP& r = s.r;
                --r->running;
                r->finished += s.len;
                if (s.rc != RP_OK && r->rc == RP_OK) {
                    r->rc = s.rc;
                    r->err = s.err;
                    r->finished += r->ns - r->next;    // the rest of the request is dropped
                    r->next = r->ns;
                }
                if (r->finished >= r->ns && r->running == 0 && r->state == Q_ACTIVE) finish(S, r, t);
            }
            --S->running;
        }
        S->cv.notify_all();
    }
    if (ws) rp_workspace_destroy(ws);
    if (st) cudaStreamDestroy(st);
}

double percentile(std::vector<double> v, double p) {
    if (v.empty()) return 0.0;
    std::sort(v.begin(), v.end());
    const double x = p / 100.0 * (double)(v.size() - 1);
    const size_t i = (size_t)x;
    const double f = x - (double)i;
    return (i + 1 < v.size()) ? v[i] * (1 - f) + v[i + 1] * f : v[i];
}

}  // namespace

extern "C" int rp_server_create(int device, int workers, int64_t mem_budget, int max_batch, const rp_executor* ex,
                                rp_server** out) {
    if (!out || workers < 1 || max_batch < 1 || (ex && (!ex->run || !ex->footprint))) {
        rp_set_error("rp_server_create: bad argument");
        return RP_ERR_ARG;
    }
    auto* S = new rp_server();
    S->device = device;
    S->max_batch = max_batch;
    if (ex) { S->fake = true; S->ex = *ex; }
    if (mem_budget > 0) {
        S->budget = mem_budget;
    } else if (S->fake) {
        S->budget = INT64_MAX;
    } else {
        size_t fr = 0, tot = 0;
        cudaSetDevice(device);
        cudaError_t e = cudaMemGetInfo(&fr, &tot);
        if (e != cudaSuccess) { delete S; return rp_cuda_fail(e, "cudaMemGetInfo"); }
        S->budget = (int64_t)(0.6 * (double)fr);
    }
    for (int i = 0; i < workers; ++i) S->threads.emplace_back(worker_main, S);
    *out = S;
    return RP_OK;
}

extern "C" int rp_server_configure(rp_server* S, int64_t step_traces, int max_active, int max_wait_ms) {
    if (!S || step_traces < 0 || max_active < 0 || max_wait_ms < 0) {
        rp_set_error("rp_server_configure: bad argument");
        return RP_ERR_ARG;
    }
    std::lock_guard<std::mutex> lk(S->mu);
    if (!S->reqs.empty() || !S->q.empty() || !S->active.empty()) {
        rp_set_error("rp_server_configure: requests were already submitted");
        return RP_ERR_ARG;
    }
    if (S->fake && step_traces > 0 && !S->ex.bins) {
        rp_set_error("rp_server_configure: steps need the executor's bins()");
        return RP_ERR_ARG;
    }
    S->step_traces = step_traces;
    S->max_active = max_active;
    S->max_wait_ms = max_wait_ms;
    S->cv.notify_all();
    return RP_OK;
}

extern "C" int rp_server_drain(rp_server* S, int timeout_ms) {
    if (!S) { rp_set_error("rp_server_drain: null server"); return RP_ERR_ARG; }
    std::unique_lock<std::mutex> lk(S->mu);
    auto idle = [&] { return S->q.empty() && S->active.empty() && S->running == 0; };
    if (timeout_ms < 0) {
        S->cv.wait(lk, idle);
    } else if (!S->cv.wait_for(lk, std::chrono::milliseconds(timeout_ms), idle)) {
        rp_set_error("rp_server_drain: still busy after %d ms", timeout_ms);
        return RP_ERR_TIMEOUT;
    }
    return RP_OK;
}

extern "C" int rp_server_destroy(rp_server* S) {
    if (!S) return RP_OK;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        S->stop = true;
    }
    S->cv.notify_all();
    for (auto& t : S->threads) t.join();
    delete S;
    return RP_OK;
}

extern "C" int rp_submit(rp_server* S, rp_scene* sc, const double* traces, int64_t ns, int form, void* out,
                         int64_t* counts, int64_t* ticket) {
    if (!S || !sc || ns < 1 || !traces || !out || !ticket) {
        rp_set_error("rp_submit: bad argument");
        return RP_ERR_ARG;
    }
    const int f = form & 0xff;
    if (f != RP_FORM_FAST_F32 && f != RP_FORM_PLAIN_F64) {
        rp_set_error("rp_submit: unknown form %d", form);
        return RP_ERR_ARG;
    }
    auto r = std::make_shared<SrvReq>();
    r->sc = sc;
    r->tr.assign(traces, traces + 9 * ns);
    r->ns = ns;
    r->form = form;
    r->out = out;
    r->user_counts = counts;
    r->counts.assign(2 * (size_t)ns, 0);
    int64_t step;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        step = S->step_traces > 0 ? std::min<int64_t>(S->step_traces, ns) : ns;
    }
    r->step = step;
    // footprint: the largest step's scratch plus its trace table and output
    if (S->fake) {
        r->fp = S->ex.footprint(S->ex.user, sc, step, form);
    } else {
        int64_t scratch = 0;
        for (int64_t c0 = 0; c0 < ns; c0 += step) {
            int64_t b = 0;
            int rc = rp_query_footprint_traces(sc, traces + 9 * c0, std::min(step, ns - c0), form, &b);
            if (rc) return rc;
            scratch = std::max(scratch, b);
        }
        r->fp = scratch + step * (72 + (int64_t)sc->nr * ((form & RP_OUT_COMPLEX128) ? 16 : 8));
    }
    std::lock_guard<std::mutex> lk(S->mu);
    if (r->fp > S->budget) {
        ++S->rejected;
        rp_set_error("rp_submit: request needs %lld bytes, the budget is %lld", (long long)r->fp,
                     (long long)S->budget);
        return RP_ERR_BUDGET;
    }
    r->id = S->next_id++;
    r->t_submit = now_s();
    if (S->t_first < 0) S->t_first = r->t_submit;
    S->reqs[r->id] = r;
    S->q.push_back(r);
    *ticket = r->id;
    S->cv.notify_all();
    return RP_OK;
}

extern "C" int rp_poll(rp_server* S, int64_t ticket, int timeout_ms) {
    if (!S) { rp_set_error("rp_poll: null server"); return RP_ERR_ARG; }
    std::unique_lock<std::mutex> lk(S->mu);
    auto it = S->reqs.find(ticket);
    if (it == S->reqs.end()) {
        rp_set_error("rp_poll: unknown ticket %lld", (long long)ticket);
        return RP_ERR_ARG;
    }
    ReqP r = it->second;
    auto done = [&] { return r->state == Q_DONE; };
    if (timeout_ms < 0) S->cv.wait(lk, done);
    else if (timeout_ms > 0) S->cv.wait_for(lk, std::chrono::milliseconds(timeout_ms), done);
    if (!done()) return RP_PENDING;
    S->reqs.erase(ticket);
    if (r->rc != RP_OK) rp_set_error("%s", r->err.c_str());
    return r->rc;
}

extern "C" int rp_cancel(rp_server* S, int64_t ticket) {
    if (!S) { rp_set_error("rp_cancel: null server"); return RP_ERR_ARG; }
    {
        std::lock_guard<std::mutex> lk(S->mu);
        auto it = S->reqs.find(ticket);
        if (it == S->reqs.end() || it->second->state != Q_QUEUED) {
            rp_set_error("rp_cancel: ticket %lld is not queued", (long long)ticket);
            return RP_ERR_ARG;
        }
        ReqP r = it->second;
        S->q.erase(std::find(S->q.begin(), S->q.end(), r));
        r->state = Q_DONE;
        r->rc = RP_ERR_CANCELLED;
        r->err = "request cancelled before it started";
        r->t_end = now_s();
        ++S->cancelled;
    }
    S->cv.notify_all();
    return RP_OK;
}

extern "C" int rp_server_stats(rp_server* S, double* stats, int n) {
    if (!S || !stats || n < 0) { rp_set_error("rp_server_stats: bad argument"); return RP_ERR_ARG; }
    std::lock_guard<std::mutex> lk(S->mu);
    double mean = 0, wait = 0;
    for (double v : S->lat_ms) mean += v;
    for (double v : S->wait_ms) wait += v;
    if (!S->lat_ms.empty()) { mean /= (double)S->lat_ms.size(); wait /= (double)S->wait_ms.size(); }
    const double wall = (S->t_first >= 0 && S->t_last > S->t_first) ? S->t_last - S->t_first : 0.0;
    const double v[18] = {(double)S->completed, (double)S->failed, (double)S->rejected, (double)S->cancelled,
                          percentile(S->lat_ms, 50), percentile(S->lat_ms, 99), mean, wait, S->pairs,
                          wall > 0 ? S->pairs / wall : 0.0, (double)S->calls, (double)S->max_in_call,
                          (double)S->in_flight, (double)S->shed, (double)S->steps, (double)S->max_active_seen,
                          (double)S->max_calls_running, percentile(S->lat_ms, 90)};
    for (int i = 0; i < n; ++i) stats[i] = i < 18 ? v[i] : 0.0;
    return RP_OK;
}
