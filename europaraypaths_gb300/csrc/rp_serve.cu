// rp_serve.cu -- the resident request loop (rp_server_*, rp_submit, rp_poll).
//
// Worker threads, each with its own CUDA stream and rp_workspace, take
// requests from one FIFO queue under a device-memory budget.  A free worker
// takes the queue head and, while they fit, the following fast-form requests
// (up to max_batch) and runs them as one rp_simulate_batch call: continuous
// batching over the resident scenes.  Host side only; the kernels are those
// of the two forms.
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

enum { Q_QUEUED = 0, Q_RUNNING = 1, Q_DONE = 2 };

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
};

using ReqP = std::shared_ptr<SrvReq>;

bool batchable(const SrvReq& r) { return (r.form & 0xff) == RP_FORM_FAST_F32 && !(r.form & RP_OUT_COMPLEX128); }

}  // namespace

struct rp_server {
    int device = 0;
    int64_t budget = 0;
    int max_batch = 1;
    bool fake = false;
    rp_executor ex{};
    std::mutex mu;
    std::condition_variable cv;
    std::deque<ReqP> q;
    std::unordered_map<int64_t, ReqP> reqs;
    int64_t next_id = 1;
    int64_t in_flight = 0;
    int running = 0;
    bool stop = false;
    std::vector<std::thread> threads;
    // statistics
    std::vector<double> lat_ms, wait_ms;
    int64_t completed = 0, failed = 0, rejected = 0, cancelled = 0, calls = 0, max_in_call = 0;
    double pairs = 0, t_first = -1, t_last = 0;
};

namespace {

// Run one worker call on the GPU: per-request device buffers, one
// rp_simulate_batch for batchable requests (rp_simulate_ws otherwise), and
// on a batch failure each request again alone so that errors stay with their
// own request.
void gpu_call(std::vector<ReqP>& batch, rp_workspace* ws, cudaStream_t st) {
    const size_t n = batch.size();
    std::vector<double*> d_tr(n, nullptr);
    std::vector<void*> d_out(n, nullptr);
    std::vector<size_t> out_bytes(n, 0);
    auto fail_all = [&](int rc) {
        char buf[1024];
        rp_last_error(buf, sizeof(buf));
        for (auto& r : batch) { r->rc = rc; r->err = buf; }
    };
    for (size_t i = 0; i < n; ++i) {
        SrvReq& r = *batch[i];
        r.counts.assign(2 * (size_t)r.ns, 0);
        out_bytes[i] = (size_t)r.ns * r.sc->nr * ((r.form & RP_OUT_COMPLEX128) ? 16 : 8);
        cudaError_t e = cudaMallocAsync((void**)&d_tr[i], sizeof(double) * 9 * r.ns, st);
        if (e == cudaSuccess) e = cudaMallocAsync(&d_out[i], out_bytes[i], st);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(d_tr[i], r.tr.data(), sizeof(double) * 9 * r.ns, cudaMemcpyHostToDevice, st);
        if (e != cudaSuccess) {
            fail_all(rp_cuda_fail(e, "server buffers"));
            goto cleanup;
        }
    }
    {
        int rc = RP_OK;
        if (n > 1) {
            std::vector<rp_job> jobs(n);
            for (size_t i = 0; i < n; ++i)
                jobs[i] = rp_job{batch[i]->sc, d_tr[i], batch[i]->ns, d_out[i], batch[i]->counts.data()};
            rc = rp_simulate_batch(jobs.data(), (int)n, ws, st);
        }
        for (size_t i = 0; i < n; ++i) {
            SrvReq& r = *batch[i];
            int rci = rc;
            if (n == 1 || rc != RP_OK)
                rci = rp_simulate_ws(r.sc, ws, d_tr[i], r.ns, r.form, d_out[i], r.counts.data(), st);
            if (rci == RP_OK) {
                cudaError_t e = cudaMemcpyAsync(r.out, d_out[i], out_bytes[i], cudaMemcpyDeviceToHost, st);
                if (e == cudaSuccess) e = cudaStreamSynchronize(st);
                if (e != cudaSuccess) rci = rp_cuda_fail(e, "server output copy");
            }
            r.rc = rci;
            if (rci != RP_OK) {
                char buf[1024];
                rp_last_error(buf, sizeof(buf));
                r.err = buf;
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

void fake_call(rp_server* S, std::vector<ReqP>& batch) {
    for (auto& r : batch) {
        r->counts.assign(2 * (size_t)r->ns, 0);
        r->rc = S->ex.run(S->ex.user, r->sc, r->tr.data(), r->ns, r->form, r->out, r->counts.data());
        if (r->rc != RP_OK) r->err = "executor failed";
    }
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
        std::vector<ReqP> batch;
        {
            std::unique_lock<std::mutex> lk(S->mu);
            S->cv.wait(lk, [&] {
                return (S->stop && S->q.empty()) ||
                       (!S->q.empty() && S->in_flight + S->q.front()->fp <= S->budget);
            });
            if (S->q.empty()) break;
            const double t = now_s();
            auto take = [&](const ReqP& r) {
                S->q.pop_front();
                S->in_flight += r->fp;
                r->state = Q_RUNNING;
                r->t_start = t;
                batch.push_back(r);
            };
            ReqP h = S->q.front();
            take(h);
            if (batchable(*h))
                while (!S->q.empty() && (int)batch.size() < S->max_batch) {
                    ReqP nx = S->q.front();
                    if (!batchable(*nx) || S->in_flight + nx->fp > S->budget) break;
                    take(nx);
                }
            ++S->running;
            ++S->calls;
            S->max_in_call = std::max<int64_t>(S->max_in_call, (int64_t)batch.size());
        }
        if (setup_rc != RP_OK) {
            for (auto& r : batch) { r->rc = setup_rc; r->err = setup_err; }
        } else if (S->fake) {
            fake_call(S, batch);
        } else {
            gpu_call(batch, ws, st);
        }
        {
            std::lock_guard<std::mutex> lk(S->mu);
            const double t = now_s();
            for (auto& r : batch) {
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

extern "C" int rp_server_drain(rp_server* S, int timeout_ms) {
    if (!S) { rp_set_error("rp_server_drain: null server"); return RP_ERR_ARG; }
    std::unique_lock<std::mutex> lk(S->mu);
    auto idle = [&] { return S->q.empty() && S->running == 0; };
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
    if (S->fake) {
        r->fp = S->ex.footprint(S->ex.user, sc, ns, form);
    } else {
        int64_t scratch = 0;
        int rc = rp_query_footprint_traces(sc, traces, ns, form, &scratch);
        if (rc) return rc;
        r->fp = scratch + ns * (72 + (int64_t)sc->nr * ((form & RP_OUT_COMPLEX128) ? 16 : 8));
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
    const double v[13] = {(double)S->completed, (double)S->failed, (double)S->rejected, (double)S->cancelled,
                          percentile(S->lat_ms, 50), percentile(S->lat_ms, 99), mean, wait, S->pairs,
                          wall > 0 ? S->pairs / wall : 0.0, (double)S->calls, (double)S->max_in_call,
                          (double)S->in_flight};
    for (int i = 0; i < n; ++i) stats[i] = i < 13 ? v[i] : 0.0;
    return RP_OK;
}
