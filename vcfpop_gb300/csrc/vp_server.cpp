// Serving loop: many independent STRUCTURE runs on one device.
//
// The reference runs each (K, replicate) on its own host thread that claims a
// device slot for the run's whole length (BayesianThread and ManageCUDA,
// src/structure.cpp:2467-2501 and 710-756). Here one scheduler thread keeps
// the admitted runs' sweeps queued in chunks. Runs whose sweeps are small
// (launch- and latency-bound on their own) are batched: the runs of one size
// class form a cohort whose every sweep is one launch per kernel for all of
// them (vp_cohort_*), and runs join and leave it as they are admitted and
// finish. Larger runs fill the device alone and keep their own streams. A
// run's results are ready the moment its last chunk lands.
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
    int cls = -1;            // the cohort class it runs in, -1: its own stream
    // the request holds its own reference to the dataset until it is deleted
    ~Req() { if (ds) vp_dataset_free(const_cast<vp_dataset*>(ds)); }
};

// the runs of one size class and one sweep signature (the same kernels,
// launch shapes and scalar arguments) swept together in one cohort: one
// launch per kernel of the sweep for all of them (vp_cohort_*), chunks of
// sweeps queued on the cohort's stream
struct CohortSlot {
    vp_cohort* h = nullptr;
    std::vector<Req*> members;
    std::vector<Req*> joining;     // started, waiting for the next membership change
    cudaEvent_t ev[2] = {nullptr, nullptr};
    int inflight = 0, head = 0;
};

// Cohort classes by the expected device time of one sweep (updates per sweep,
// admixture sweeps weighted 10x, at about 3e12 updates/s): below 3 us, 30 us
// and 300 us. Runs in one cohort have one sweep signature and differ at most
// tenfold in sweep cost, so a cohort sweep costs about one run's sweep and
// its lockstep holds none back for long; larger runs fill the device alone
// and keep their own stream.
constexpr int N_CLASSES = 3;

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
    bool batching = true;           // small runs in cohorts (else every run on its own stream)
    // cohorts by (size class, sweep signature): the runs of one cohort merge
    // every launch of a sweep; touched by the scheduler thread only
    std::map<std::pair<int, uint64_t>, CohortSlot> cohorts;
    int in_cohorts = 0;             // runs in cohorts (members and joining), under mu
    // kernel launches queued and run-sweeps they carry (a cohort sweep of n
    // members carries n run-sweeps)
    int64_t launches = 0, run_sweeps = 0;
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

int run_class(const Req* r) {
    vp_dataset_info di{};
    vp_dataset_info_get(r->ds, &di);
    const double w = (double)di.n_ind * (double)di.n_loc * r->P.K * (r->P.admix ? 10.0 : 1.0);
    const double us = w / 3e6;
    for (int c = 0; c < N_CLASSES; ++c)
        if (us < 3.0 * std::pow(10.0, c)) return c;
    return -1;
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
        const int64_t l0 = vp_launch_count(r->ctx);
        int rc;
        if (left > s->chunk) {
            rc = vp_run(&r->chain, 1, s->chunk);
            if (!rc) {
                std::lock_guard<std::mutex> lk(s->mu);
                r->issued += s->chunk;
                s->launches += vp_launch_count(r->ctx) - l0;
                s->run_sweeps += s->chunk;
            }
        } else {
            rc = vp_finish_issue(&r->chain, 1);
            if (!rc) {
                std::lock_guard<std::mutex> lk(s->mu);
                r->issued = r->total;
                r->finishing = true;
                s->launches += vp_launch_count(r->ctx) - l0;
                s->run_sweeps += left;
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

// every member of slot k fails with the cohort
void fail_cohort(vp_server* s, CohortSlot& k, int rc, const char* what) {
    std::vector<Req*> all = k.members;
    all.insert(all.end(), k.joining.begin(), k.joining.end());
    if (k.h) vp_cohort_set(k.h, nullptr, 0);
    k.members.clear();
    k.joining.clear();
    k.inflight = 0;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->in_cohorts -= (int)all.size();
    }
    for (Req* r : all) fail(s, r, rc, what);
}

// runs that have had every sweep queued leave the cohort (its graph is
// captured again without them, with the runs waiting to join) and queue
// their Arrange on their own stream, which is ordered after the cohort's
// sweeps; their completion is then watched like a run of its own stream
bool cohort_membership(vp_server* s, CohortSlot& k, std::vector<Req*>& finishing) {
    std::vector<Req*> stay;
    bool changed = !k.joining.empty();
    for (Req* r : k.members) {
        int64_t issued = 0, total = 0;
        vp_chain_progress(r->chain, &issued, &total);
        {
            std::lock_guard<std::mutex> lk(s->mu);
            r->issued = issued;
        }
        if (issued >= total) { finishing.push_back(r); changed = true; }
        else stay.push_back(r);
    }
    if (!changed) return false;
    stay.insert(stay.end(), k.joining.begin(), k.joining.end());
    std::vector<vp_chain*> cs;
    for (Req* r : stay) cs.push_back(r->chain);
    int rc = vp_cohort_set(k.h, cs.data(), (int32_t)cs.size());
    k.members = stay;
    k.joining.clear();
    if (rc) {
        fail_cohort(s, k, rc, "forming the cohort failed");
        return true;
    }
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->in_cohorts -= (int)finishing.size();
    }
    for (Req* r : finishing) {
        cudaStream_t st = (cudaStream_t)vp_stream(r->ctx);
        int rc2 = vp_finish_issue(&r->chain, 1);
        if (!rc2 && cudaEventRecord(r->ev[0], st) != cudaSuccess) rc2 = VP_E_CUDA;
        if (rc2) { fail(s, r, rc2, "finishing the run failed"); continue; }
        r->finishing = true;
        r->inflight = 1;
        r->head = 0;
        r->cls = -1;
        std::lock_guard<std::mutex> lk(s->mu);
        r->issued = r->total;
    }
    return true;
}

// retire the cohort's finished chunks, change its members, queue more chunks
bool advance_cohort(vp_server* s, CohortSlot& k, std::vector<Req*>& finishing) {
    bool moved = false;
    while (k.inflight > 0) {
        cudaError_t q = cudaEventQuery(k.ev[k.head]);
        if (q == cudaErrorNotReady) break;
        if (q != cudaSuccess) {
            char buf[160];
            snprintf(buf, sizeof buf, "cohort failed on the device: %s", cudaGetErrorString(q));
            fail_cohort(s, k, VP_E_CUDA, buf);
            return true;
        }
        k.head ^= 1;
        k.inflight--;
        moved = true;
    }
    if (cohort_membership(s, k, finishing)) moved = true;
    cudaStream_t st = (cudaStream_t)vp_cohort_stream(k.h);
    while (k.inflight < 2 && !k.members.empty()) {
        int rc = vp_cohort_run(k.h, s->chunk);
        if (!rc && cudaEventRecord(k.ev[(k.head + k.inflight) & 1], st) != cudaSuccess) rc = VP_E_CUDA;
        if (rc) { fail_cohort(s, k, rc, "queueing the cohort's sweeps failed"); return true; }
        k.inflight++;
        int32_t per = 0;
        vp_cohort_launches(k.h, &per);
        {
            std::lock_guard<std::mutex> lk(s->mu);
            s->launches += (int64_t)per * s->chunk;
            for (Req* r : k.members) s->run_sweeps += std::min<int64_t>(s->chunk, r->total - r->issued);
        }
        moved = true;
        // members whose last sweep is now queued leave at once
        if (cohort_membership(s, k, finishing)) moved = true;
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
            if (s->active.empty() && s->queue.empty() && s->in_cohorts == 0) {
                s->cv_work.wait_for(lk, std::chrono::milliseconds(20));
                continue;
            }
            // arrival order: the head of the queue waits for room
            while (!s->queue.empty() && (int)(s->active.size() + s->in_cohorts + admit.size()) < s->max_active) {
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
            if (rc) { fail(s, r, rc, "starting the run failed"); continue; }
            r->cls = s->batching ? run_class(r) : -1;
            std::pair<int, uint64_t> key(r->cls, 0);
            if (r->cls >= 0) {
                key.second = vp_chain_sweep_signature(r->chain);
                CohortSlot& k = s->cohorts[key];
                if (!k.h) {
                    // smaller classes at higher stream priority (lower numbers run first)
                    const int prio = std::min(s->prio_least, s->prio_greatest + r->cls);
                    if (vp_cohort_open_ex(s->device, prio, &k.h) ||
                        cudaEventCreateWithFlags(&k.ev[0], cudaEventDisableTiming) != cudaSuccess ||
                        cudaEventCreateWithFlags(&k.ev[1], cudaEventDisableTiming) != cudaSuccess) {
                        if (k.h) vp_cohort_close(k.h);
                        for (cudaEvent_t& e : k.ev)
                            if (e) cudaEventDestroy(e);
                        s->cohorts.erase(key);
                        r->cls = -1;
                    }
                }
            }
            if (r->cls >= 0) {
                s->cohorts[key].joining.push_back(r);
                std::lock_guard<std::mutex> lk(s->mu);
                s->in_cohorts++;
            } else {
                s->active.push_back(r);
            }
        }
        bool moved = !admit.empty();
        for (auto it = s->cohorts.begin(); it != s->cohorts.end();) {
            CohortSlot& k = it->second;
            std::vector<Req*> finishing;
            moved |= advance_cohort(s, k, finishing);
            for (Req* r : finishing) s->active.push_back(r);
            // a cohort left without runs and without sweeps in flight closes
            if (k.members.empty() && k.joining.empty() && k.inflight == 0) {
                vp_cohort_close(k.h);
                for (cudaEvent_t& e : k.ev)
                    if (e) cudaEventDestroy(e);
                it = s->cohorts.erase(it);
            } else {
                ++it;
            }
        }
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
    for (auto& kv : s->cohorts) {
        CohortSlot& k = kv.second;
        if (k.h) vp_cohort_close(k.h);   // waits for its sweeps and lets go of its members
        for (cudaEvent_t& e : k.ev)
            if (e) cudaEventDestroy(e);
        k.h = nullptr;
    }
    s->cohorts.clear();
    for (auto& kv : s->reqs) {
        free_run(kv.second);
        delete kv.second;
    }
    delete s;
    return VP_OK;
}

extern "C" int vp_server_set_batching(vp_server* s, int32_t on) {
    if (!s) { vp_set_error("null argument"); return VP_E_ARG; }
    std::lock_guard<std::mutex> lk(s->mu);
    if (!s->reqs.empty()) { vp_set_error("set batching before the first vp_submit"); return VP_E_STATE; }
    s->batching = on != 0;
    return VP_OK;
}

extern "C" int vp_server_stats(vp_server* s, int64_t* launches, int64_t* run_sweeps) {
    if (!s) { vp_set_error("null argument"); return VP_E_ARG; }
    std::lock_guard<std::mutex> lk(s->mu);
    if (launches) *launches = s->launches;
    if (run_sweeps) *run_sweeps = s->run_sweeps;
    return VP_OK;
}
