// mpgpu_serve.cpp -- resident request loop for alignment jobs.
//
// Jobs are submitted from any host thread and run on worker threads, each
// with its own device context (streams, memory kept between its jobs).  A
// worker takes the oldest waiting job, runs its host structure passes, then
// asks for the job's device footprint out of the memory budget: jobs are
// admitted in order as memory frees up, and admitted jobs run concurrently
// on the device (their kernels overlap on separate streams).  Each job's
// matrix and vectors stay on the device across its iterations.  The device
// arithmetic of one job does not depend on the others, so a job's result is
// identical alone and in a mix.  Latency = submission to completion.
#include <chrono>
#include <condition_variable>
#include <cstdint>
#include <deque>
#include <functional>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/mpgpu.h"

int32_t pede_run_admitted(mpgpu_ctx *ctxIn, const mpgpu_steer *st, const mpgpu_job *job, mpgpu_result *res,
                          const std::function<bool(int64_t)> &admit);

namespace {
using Clock = std::chrono::steady_clock;
constexpr int64_t kServeStaging = (int64_t)8 << 30;

struct ServeJob {
    mpgpu_steer st;
    mpgpu_job job;
    mpgpu_result *res = nullptr;
    Clock::time_point tSubmit, tStart, tEnd;
    int64_t bytes = 0;
    int32_t rc = 0;
    bool admitted = false;
    bool done = false;
};
}  // namespace

struct mpgpu_server {
    int32_t device = 0;
    int64_t budget = 0, inUse = 0;
    std::mutex m;
    std::condition_variable cvWork, cvDone, cvMem;
    std::deque<int64_t> queue;          // waiting for a worker
    std::deque<int64_t> memQueue;       // waiting for memory, in admission order
    std::map<int64_t, ServeJob> jobs;
    int64_t next = 1;
    bool stop = false;
    std::vector<std::thread> workers;
    std::vector<mpgpu_ctx *> ctxs;
    std::string lastErr, lastErrOut;   // the last failed job's message, and the copy handed out

    void work(int w) {
        mpgpu_ctx *ctx = ctxs[w];
        for (;;) {
            int64_t id;
            {
                std::unique_lock<std::mutex> lk(m);
                cvWork.wait(lk, [&] { return stop || !queue.empty(); });
                if (queue.empty()) return;
                id = queue.front();
                queue.pop_front();
                jobs[id].tStart = Clock::now();
            }
            ServeJob *J;
            {
                std::lock_guard<std::mutex> lk(m);
                J = &jobs[id];
            }
            auto admit = [&](int64_t bytes) -> bool {
                std::unique_lock<std::mutex> lk(m);
                J->bytes = bytes;
                if (bytes > budget) return false;
                memQueue.push_back(id);
                cvMem.wait(lk, [&] { return memQueue.front() == id && inUse + bytes <= budget; });
                memQueue.pop_front();
                inUse += bytes;
                J->admitted = true;
                cvMem.notify_all();
                return true;
            };
            const int32_t rc = pede_run_admitted(ctx, &J->st, &J->job, J->res, admit);
            const std::string msg = rc ? mpgpu_last_error(ctx) : std::string();
            // the job's device memory goes back before its budget share does
            mpgpu_release(ctx);
            {
                std::lock_guard<std::mutex> lk(m);
                if (rc) lastErr = "ticket " + std::to_string(id) + ": status " + std::to_string(rc) + ": " + msg;
                if (J->admitted) inUse -= J->bytes;
                J->rc = rc;
                J->tEnd = Clock::now();
                J->done = true;
            }
            cvMem.notify_all();
            cvDone.notify_all();
        }
    }
};

extern "C" int32_t mpgpu_server_create(mpgpu_server **out, const mpgpu_server_cfg *cfg) {
    if (!out) return MPGPU_ERR_ARG;
    *out = nullptr;
    mpgpu_server *s = new mpgpu_server();
    s->device = cfg ? cfg->device : 0;
    const int32_t nw = (cfg && cfg->maxActive > 0) ? cfg->maxActive : 4;
    s->budget = (cfg && cfg->budgetBytes > 0) ? cfg->budgetBytes : (int64_t)150 << 30;
    for (int32_t w = 0; w < nw; ++w) {
        // a fixed staging size: the chunking of a job's update (and so the
        // order of its sums) must not depend on the memory other jobs hold
        mpgpu_cfg cc{s->device, 0, kServeStaging};
        mpgpu_ctx *ctx = nullptr;
        const int32_t rc = mpgpu_create(&ctx, &cc);
        if (rc) {
            for (mpgpu_ctx *c : s->ctxs) mpgpu_destroy(c);
            delete s;
            return rc;
        }
        s->ctxs.push_back(ctx);
    }
    for (int32_t w = 0; w < nw; ++w) s->workers.emplace_back([s, w] { s->work(w); });
    *out = s;
    return MPGPU_OK;
}

extern "C" int32_t mpgpu_server_submit(mpgpu_server *s, const mpgpu_steer *st, const mpgpu_job *job,
                                       mpgpu_result *res, int64_t *ticket) {
    if (!s || !st || !job || !res || !ticket) return MPGPU_ERR_ARG;
    std::lock_guard<std::mutex> lk(s->m);
    if (s->stop) return MPGPU_ERR_ARG;
    const int64_t id = s->next++;
    ServeJob &J = s->jobs[id];
    J.st = *st;
    J.job = *job;
    J.res = res;
    J.tSubmit = Clock::now();
    s->queue.push_back(id);
    *ticket = id;
    s->cvWork.notify_one();
    return MPGPU_OK;
}

extern "C" int32_t mpgpu_server_wait(mpgpu_server *s, int64_t ticket, double timeoutMs, double *msLatency,
                                     double *msQueue, int64_t *bytes) {
    if (!s) return MPGPU_ERR_ARG;
    std::unique_lock<std::mutex> lk(s->m);
    auto it = s->jobs.find(ticket);
    if (it == s->jobs.end()) return MPGPU_ERR_ARG;
    ServeJob &J = it->second;
    const auto pred = [&] { return J.done; };
    if (timeoutMs > 0.0) {
        if (!s->cvDone.wait_for(lk, std::chrono::duration<double, std::milli>(timeoutMs), pred))
            return MPGPU_ERR_TIMEOUT;
    } else {
        s->cvDone.wait(lk, pred);
    }
    const auto ms = [](Clock::duration d) { return std::chrono::duration<double, std::milli>(d).count(); };
    if (msLatency) *msLatency = ms(J.tEnd - J.tSubmit);
    if (msQueue) *msQueue = ms(J.tStart - J.tSubmit);
    if (bytes) *bytes = J.bytes;
    const int32_t rc = J.rc;
    s->jobs.erase(it);
    return rc;
}

extern "C" const char *mpgpu_server_last_error(mpgpu_server *s) {
    if (!s) return "";
    std::lock_guard<std::mutex> lk(s->m);
    s->lastErrOut = s->lastErr;
    return s->lastErrOut.c_str();
}

extern "C" int32_t mpgpu_server_destroy(mpgpu_server *s) {
    if (!s) return MPGPU_ERR_ARG;
    {
        std::lock_guard<std::mutex> lk(s->m);
        s->stop = true;
    }
    s->cvWork.notify_all();
    for (std::thread &t : s->workers) t.join();
    for (mpgpu_ctx *c : s->ctxs) mpgpu_destroy(c);
    delete s;
    return MPGPU_OK;
}
