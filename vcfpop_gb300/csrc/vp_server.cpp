// Serving loop: many independent STRUCTURE runs on one device.
//
// The reference runs each (K, replicate) on its own host thread that claims a
// device slot for the run's whole length (BayesianThread and ManageCUDA,
// src/structure.cpp:2467-2501 and 710-756). Here one scheduler thread keeps
// every admitted run's sweeps queued on that run's own stream, in chunks, so
// small runs (launch- and latency-bound on their own) overlap each other and
// large ones, and a run's results are ready the moment its last chunk lands.
//
// Admission is in arrival order, bounded by a device-memory budget (dataset
// upload plus chain state, sized exactly as vp_open / vp_chain_create
// allocate) and by a cap on active runs. Completion is observed with CUDA
// events, never by blocking on a stream.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "vp_internal.h"

namespace {

using Clock = std::chrono::steady_clock;

struct Req {
    int64_t id = 0;
    const vp_dataset* ds = nullptr;
    vp_params P{};
    int64_t bytes = 0;
    int state = VP_REQ_QUEUED;
    int rc = 0;
    bool holds_memory = false;
    std::string err;
    double t_submit = 0, t_start = 0, t_done = 0;
    vp_ctx* ctx = nullptr;
    vp_chain* chain = nullptr;
    cudaEvent_t ev[2] = {nullptr, nullptr};
    int inflight = 0;        // chunks queued whose completion has not been seen (0..2)
    int head = 0;            // event slot of the oldest of them
    bool finishing = false;  // the last chunk (with Arrange) is queued
    int64_t issued = 0, total = 0;
    // the request holds its own reference to the dataset until it is deleted
    ~Req() { if (ds) vp_dataset_free(const_cast<vp_dataset*>(ds)); }
};

}  // namespace

struct vp_server {
    int device = 0, nsm = 0;
    int prio_least = 0, prio_greatest = 0;   // cudaDeviceGetStreamPriorityRange
    int64_t budget = 0, used = 0;
    int max_active = 64, chunk = 16;
    Clock::time_point t0;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Req*> queue;
    std::vector<Req*> active;       // touched by the scheduler thread only
    std::map<int64_t, Req*> reqs;
    int64_t next_id = 1;
    bool stop = false;
    std::thread th;

    double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }
};

namespace {

void free_run(Req* r) {
    if (r->chain) vp_chain_destroy(r->chain);
    if (r->ctx) vp_close(r->ctx);
    for (cudaEvent_t& e : r->ev)
        if (e) { cudaEventDestroy(e); e = nullptr; }
    r->chain = nullptr;
    r->ctx = nullptr;
}

// a run failed on the scheduler thread: record why, give its memory back
void fail(vp_server* s, Req* r, int rc, const char* what) {
    std::string msg = what;
    const char* le = vp_last_error();
    if (le && *le) msg += std::string(": ") + le;
    free_run(r);
    std::lock_guard<std::mutex> lk(s->mu);
    r->rc = rc;
    r->err = msg;
    r->state = VP_REQ_FAILED;
    r->t_done = s->now();
    if (r->holds_memory) { s->used -= r->bytes; r->holds_memory = false; }
    s->cv_done.notify_all();
}

// stream priority of a run: the device's priority levels spread over the
// decades of its expected work (updates x sweeps, admixture sweeps counted
// 4x), smaller runs first, so that a short run is not held behind the blocks
// of long ones. Priorities change only the order in which the device takes
// up queued blocks; results do not depend on them.
int run_priority(const vp_server* s, const Req* r) {
    if (s->prio_least == s->prio_greatest) return s->prio_least;
    vp_dataset_info di{};
    vp_dataset_info_get(r->ds, &di);
    const double sweeps = (double)r->P.nburnin + r->P.nreps + r->P.nadmburnin;
    const double work = (double)di.n_ind * (double)di.n_loc * r->P.K * std::max(1.0, sweeps) * (r->P.admix ? 4.0 : 1.0);
    const int levels = s->prio_least - s->prio_greatest + 1;
    // decades from 1e7 (a few milliseconds of device time) upwards
    int idx = (int)std::floor(std::log10(std::max(work, 1.0)) - 7.0);
    idx = std::min(std::max(idx, 0), levels - 1);
    return s->prio_greatest + idx;
}

// upload the dataset, create the chain and the two completion events
int start_run(vp_server* s, Req* r) {
    int rc = vp_open_ex(r->ds, s->device, run_priority(s, r), &r->ctx);
    if (rc) return rc;
    rc = vp_chain_create(r->ctx, &r->P, &r->chain);
    if (rc) return rc;
    for (cudaEvent_t& e : r->ev)
        if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return VP_E_CUDA;
    int64_t issued = 0, total = 0;
    vp_chain_progress(r->chain, &issued, &total);
    r->issued = issued;
    r->total = total;
    return VP_OK;
}

// retire finished chunks of one run and queue more; true if anything moved
bool advance(vp_server* s, Req* r, bool* finished) {
    bool moved = false;
    *finished = false;
    while (r->inflight > 0) {
        cudaError_t q = cudaEventQuery(r->ev[r->head]);
        if (q == cudaErrorNotReady) break;
        if (q != cudaSuccess) {
            char buf[160];
            snprintf(buf, sizeof buf, "run failed on the device: %s", cudaGetErrorString(q));
            fail(s, r, VP_E_CUDA, buf);
            *finished = true;
            return true;
        }
        r->head ^= 1;
        r->inflight--;
        moved = true;
    }
    if (r->finishing) {
        if (r->inflight == 0) {
            std::lock_guard<std::mutex> lk(s->mu);
            r->state = VP_REQ_DONE;
            r->t_done = s->now();
            s->cv_done.notify_all();
            *finished = true;
        }
        return moved;
    }
    cudaStream_t st = (cudaStream_t)vp_stream(r->ctx);
    while (r->inflight < 2 && !r->finishing) {
        const int64_t left = r->total - r->issued;
        int rc;
        if (left > s->chunk) {
            rc = vp_run(&r->chain, 1, s->chunk);
            if (!rc) {
                std::lock_guard<std::mutex> lk(s->mu);
                r->issued += s->chunk;
            }
        } else {
            rc = vp_finish_issue(&r->chain, 1);
            if (!rc) {
                std::lock_guard<std::mutex> lk(s->mu);
                r->issued = r->total;
                r->finishing = true;
            }
        }
        if (!rc && cudaEventRecord(r->ev[(r->head + r->inflight) & 1], st) != cudaSuccess) rc = VP_E_CUDA;
        if (rc) {
            fail(s, r, rc, "queueing sweeps failed");
            *finished = true;
            return true;
        }
        r->inflight++;
        moved = true;
    }
    return moved;
}

void scheduler(vp_server* s) {
    cudaSetDevice(s->device);
    for (;;) {
        std::vector<Req*> admit;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            if (s->stop) return;
            if (s->active.empty() && s->queue.empty()) {
                s->cv_work.wait_for(lk, std::chrono::milliseconds(20));
                continue;
            }
            // arrival order: the head of the queue waits for room
            while (!s->queue.empty() && (int)(s->active.size() + admit.size()) < s->max_active) {
                Req* r = s->queue.front();
                if (s->used + r->bytes > s->budget) break;
                s->queue.pop_front();
                s->used += r->bytes;
                r->holds_memory = true;
                r->state = VP_REQ_RUNNING;
                r->t_start = s->now();
                admit.push_back(r);
            }
        }
        for (Req* r : admit) {
            int rc = start_run(s, r);
            if (rc) fail(s, r, rc, "starting the run failed");
            else s->active.push_back(r);
        }
        bool moved = !admit.empty();
        for (size_t i = 0; i < s->active.size();) {
            bool finished = false;
            moved |= advance(s, s->active[i], &finished);
            if (finished) {
                s->active.erase(s->active.begin() + i);
                moved = true;
            } else {
                ++i;
            }
        }
        if (!moved) {
            std::unique_lock<std::mutex> lk(s->mu);
            if (s->stop) return;
            // nothing completed: wait a little (or for a new submission)
            s->cv_work.wait_for(lk, std::chrono::microseconds(50));
        }
    }
}

void fill_info(const vp_server* s, const Req* r, vp_request_info* info) {
    memset(info, 0, sizeof *info);
    info->state = r->state;
    info->rc = r->rc;
    info->sweeps_issued = r->issued;
    info->sweeps_total = r->total;
    info->device_bytes = r->bytes;
    info->t_submit = r->t_submit;
    info->t_start = r->t_start;
    info->t_done = r->t_done;
    snprintf(info->error, sizeof info->error, "%s", r->err.c_str());
    (void)s;
}

}  // namespace

extern "C" int vp_server_open(int device, int64_t mem_budget, int32_t max_active, int32_t chunk, vp_server** out) {
    if (!out || mem_budget < 0 || max_active < 0 || chunk < 0) { vp_set_error("bad arguments"); return VP_E_ARG; }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) { vp_set_error("no CUDA device"); return VP_E_NODEV; }
    if (device < 0 || device >= ndev) { vp_set_error("device %d out of range", device); return VP_E_ARG; }
    if (cudaSetDevice(device) != cudaSuccess) { vp_set_error("cudaSetDevice(%d) failed", device); return VP_E_CUDA; }
    auto* s = new vp_server();
    s->device = device;
    cudaDeviceGetAttribute(&s->nsm, cudaDevAttrMultiProcessorCount, device);
    if (cudaDeviceGetStreamPriorityRange(&s->prio_least, &s->prio_greatest) != cudaSuccess)
        s->prio_least = s->prio_greatest = 0;
    if (mem_budget == 0) {
        size_t fr = 0, tot = 0;
        if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) { delete s; vp_set_error("cudaMemGetInfo failed"); return VP_E_CUDA; }
        mem_budget = (int64_t)(fr * 0.9);
    }
    s->budget = mem_budget;
    s->max_active = max_active ? max_active : 64;
    s->chunk = chunk ? chunk : 16;
    s->t0 = Clock::now();
    s->th = std::thread(scheduler, s);
    *out = s;
    return VP_OK;
}

extern "C" int vp_submit(vp_server* s, const vp_dataset* ds, const vp_params* p, int64_t* id) {
    if (!s || !ds || !p || !id) { vp_set_error("null argument"); return VP_E_ARG; }
    if (p->form == VP_FORM_TC) { vp_set_error("the server runs plain-form chains (the tensor-core form batches chains of one dataset)"); return VP_E_ARG; }
    int64_t bytes = vp_request_bytes(ds, p, s->nsm);
    if (bytes < 0) return VP_E_ARG;
    if (bytes > s->budget) {
        vp_set_error("the run needs %lld device bytes, more than the server's budget of %lld", (long long)bytes,
                     (long long)s->budget);
        return VP_E_MEM;
    }
    auto* r = new Req();
    vp_dataset_retain(ds);
    r->ds = ds;
    r->P = *p;
    r->bytes = bytes;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        if (s->stop) { delete r; vp_set_error("server is closing"); return VP_E_STATE; }
        r->id = s->next_id++;
        r->t_submit = s->now();
        s->reqs[r->id] = r;
        s->queue.push_back(r);
    }
    s->cv_work.notify_all();
    *id = r->id;
    return VP_OK;
}

extern "C" int vp_poll(vp_server* s, int64_t id, vp_request_info* info) {
    if (!s || !info) { vp_set_error("null argument"); return VP_E_ARG; }
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) { vp_set_error("unknown run id %lld", (long long)id); return VP_E_ARG; }
    fill_info(s, it->second, info);
    return VP_OK;
}

extern "C" int vp_wait(vp_server* s, int64_t id, double timeout_s, vp_request_info* info) {
    if (!s) { vp_set_error("null argument"); return VP_E_ARG; }
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) { vp_set_error("unknown run id %lld", (long long)id); return VP_E_ARG; }
    Req* r = it->second;
    auto fin = [&] { return r->state == VP_REQ_DONE || r->state == VP_REQ_FAILED; };
    if (timeout_s < 0) s->cv_done.wait(lk, fin);
    else if (!s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), fin)) {
        if (info) fill_info(s, r, info);
        vp_set_error("run %lld not finished after %.3f s", (long long)id, timeout_s);
        return VP_E_STATE;
    }
    if (info) fill_info(s, r, info);
    return VP_OK;
}

extern "C" int vp_request_chain(vp_server* s, int64_t id, vp_chain** chain) {
    if (!s || !chain) { vp_set_error("null argument"); return VP_E_ARG; }
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) { vp_set_error("unknown run id %lld", (long long)id); return VP_E_ARG; }
    if (it->second->state != VP_REQ_DONE) { vp_set_error("run %lld is not done", (long long)id); return VP_E_STATE; }
    *chain = it->second->chain;
    return VP_OK;
}

extern "C" int vp_release(vp_server* s, int64_t id) {
    if (!s) { vp_set_error("null argument"); return VP_E_ARG; }
    Req* r = nullptr;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        auto it = s->reqs.find(id);
        if (it == s->reqs.end()) { vp_set_error("unknown run id %lld", (long long)id); return VP_E_ARG; }
        r = it->second;
        if (r->state != VP_REQ_DONE && r->state != VP_REQ_FAILED) {
            vp_set_error("run %lld is still queued or running", (long long)id);
            return VP_E_STATE;
        }
        s->reqs.erase(it);
    }
    cudaSetDevice(s->device);
    free_run(r);
    {
        std::lock_guard<std::mutex> lk(s->mu);
        if (r->holds_memory) s->used -= r->bytes;
    }
    delete r;
    s->cv_work.notify_all();
    return VP_OK;
}

extern "C" int vp_server_close(vp_server* s) {
    if (!s) return VP_OK;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->cv_work.notify_all();
    if (s->th.joinable()) s->th.join();
    cudaSetDevice(s->device);
    for (auto& kv : s->reqs) {
        free_run(kv.second);
        delete kv.second;
    }
    delete s;
    return VP_OK;
}
