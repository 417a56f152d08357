// Serving loop for many CG solves on different operators (afm_server_* in
// include/afm.h; no counterpart in the reference).
//
// A request carries its own operator (maps and element matrices set on the
// host) and load. Requests wait in a FIFO queue and are admitted while the
// server's HBM budget, the device's free memory and the slot limit allow.
// Admission finalises the operator on a worker thread (colouring, patch plan,
// upload of Ke and maps), so the polling thread never blocks on host work, and
// then drops the operator's host copy of the element matrices.
// An admitted request keeps all of its state on the device: Ke, maps, b, x
// and the Krylov vectors of its mixed-precision solve (afm_mixed.hpp). The
// server's progress thread keeps taking the next step of each request whose
// previous step has finished on the GPU (so progress never waits for the
// caller); each request runs on its own stream, so the kernels of all
// running requests overlap on the device, and requests that arrive while
// others run are admitted as soon as slots and memory free up (continuous
// batching). A finished request copies x back asynchronously, releases its
// device memory at once, and waits for afm_server_take.
//
// Each request's arithmetic is independent of the others (own operator, own
// vectors, deterministic kernels), so its result is the same alone and in
// any mix, bit for bit.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <future>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "afm_internal.hpp"
#include "afm_mixed.hpp"

namespace {

enum ReqState : int { RQ_QUEUED = 0, RQ_ADMITTING, RQ_RUNNING, RQ_COPYING, RQ_DONE };

struct Request {
    uint64_t id = 0;
    afm_operator* op = nullptr;
    std::vector<double> b;
    double rtol = 1e-8, inner_rtol = 0.1;
    uint64_t est_bytes = 0;
    int state = RQ_QUEUED;
    std::future<int> fin;
    double* d_bx = nullptr;  // b then x on the device
    std::vector<double> x;   // result on the host
    cudaEvent_t copied = nullptr;
    afm::MixedSolve ms;
    afm_solve_stats stats{};
    int status = AFM_SUCCESS;
    std::string message;
    double t_submit = 0, t_admit = 0, t_start = 0, t_done = 0;
};

double now_s() {
    using namespace std::chrono;
    return duration<double>(steady_clock::now().time_since_epoch()).count();
}

// Device bytes a request holds once admitted: element matrices (8 bytes per
// entry in every arena but FP32, plus the symmetric inner copy of at most 6
// bytes per stored pair), maps or patch index blocks, diagonal, the solver's
// FP64 and FP32 work vectors, b and x; 10% and 1 MB of slack.
uint64_t estimate_bytes(const afm_operator* op) {
    uint64_t ke = 0;
    for (uint32_t e = 0; e < op->n_elem; e++) {
        const uint64_t n = op->offsets[e + 1] - op->offsets[e];
        ke += n * n * 8 + 8 * n + 6 * n * (n / 2 + 1);
    }
    const uint64_t vec = (uint64_t)op->n_dofs * (8 * 8 + 7 * 4 + 3 * 8);
    return (ke + vec) * 11 / 10 + (1u << 20);
}

}  // namespace

struct afm_server {
    int device = 0;
    uint64_t budget = 0, in_use = 0, reserve = 0;
    uint32_t max_active = 0;
    uint64_t next_id = 1;
    std::deque<Request*> queue;
    std::vector<Request*> active;  // admitting, running or copying
    std::unordered_map<uint64_t, Request*> all;
    // finished operators are destroyed on a background thread: releasing
    // pinned host memory can wait for the whole device, which must not stall
    // the polling thread
    std::thread reaper;
    std::mutex mu;
    std::condition_variable cv;
    std::deque<afm_operator*> graveyard;
    bool stop = false;
    // requests advance on a progress thread of the server's own; state_mu
    // guards the queue, the active list and the request table
    std::thread progress;
    std::mutex state_mu;
    std::atomic<bool> running{false};
};

namespace {

void release_device(afm_server* s, Request* r) {
    if (r->d_bx && r->op) cudaFreeAsync(r->d_bx, r->op->stream);
    r->d_bx = nullptr;
    if (r->copied) cudaEventDestroy(r->copied);
    r->copied = nullptr;
    if (r->op) {
        std::lock_guard<std::mutex> lk(s->mu);
        s->graveyard.push_back(r->op);
        s->cv.notify_one();
    }
    r->op = nullptr;
}

void reap(afm_server* s) {
    cudaSetDevice(s->device);
    std::unique_lock<std::mutex> lk(s->mu);
    for (;;) {
        s->cv.wait(lk, [s] { return s->stop || !s->graveyard.empty(); });
        if (s->graveyard.empty() && s->stop) return;
        afm_operator* op = s->graveyard.front();
        s->graveyard.pop_front();
        lk.unlock();
        afm_destroy(op);
        lk.lock();
    }
}

void finish(afm_server* s, Request* r, int status, const char* msg) {
    r->status = status;
    if (msg) r->message = msg;
    r->state = RQ_DONE;
    r->t_done = now_s();
    release_device(s, r);
    s->in_use -= r->est_bytes;
}

// At most this many operators are finalised at once: each finalize runs
// OpenMP loops over all host cores, and more in parallel only contend.
constexpr int kMaxFinalizing = 4;

// admission: FIFO while the budget, free device memory and slots allow
int admit(afm_server* s) {
    int admitted = 0;
    int finalizing = 0;
    for (const Request* r : s->active) finalizing += (r->state == RQ_ADMITTING);
    while (!s->queue.empty() && s->active.size() < s->max_active && finalizing < kMaxFinalizing) {
        Request* r = s->queue.front();
        size_t free_b = 0, total_b = 0;
        if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) break;
        const bool fits = s->in_use + r->est_bytes <= s->budget && r->est_bytes + s->reserve <= free_b;
        if (!fits && !s->active.empty()) break;  // wait for memory to free up
        s->queue.pop_front();
        s->in_use += r->est_bytes;
        r->state = RQ_ADMITTING;
        r->t_admit = now_s();
        afm_operator* op = r->op;
        const int dev = s->device;
        r->fin = std::async(std::launch::async, [op, dev]() {
            cudaSetDevice(dev);
            const int st = afm_finalize(op);
            // the device arena holds the element matrices now; the server never finalizes again, so the
            // host copy goes (large requests would otherwise hold gigabytes of host memory until they end)
            if (st == AFM_SUCCESS) {
                std::vector<double>().swap(op->ke);
                op->ke_dirty = true;
            }
            return st;
        });
        s->active.push_back(r);
        finalizing++;
        admitted++;
    }
    return admitted;
}

int start(afm_server* s, Request* r) {
    (void)s;
    afm_operator* op = r->op;
    const size_t n = op->n_dofs;
    if (cudaMallocAsync((void**)&r->d_bx, 2 * n * sizeof(double), op->stream) != cudaSuccess) return AFM_ERR_OOM;
    if (cudaEventCreateWithFlags(&r->copied, cudaEventDisableTiming) != cudaSuccess) return AFM_ERR_CUDA;
    if (cudaMemcpyAsync(r->d_bx, r->b.data(), n * sizeof(double), cudaMemcpyHostToDevice, op->stream) != cudaSuccess ||
        cudaMemsetAsync(r->d_bx + n, 0, n * sizeof(double), op->stream) != cudaSuccess)
        return AFM_ERR_CUDA;
    r->ms = afm::MixedSolve{};
    r->ms.op = op;
    r->ms.d_b = r->d_bx;
    r->ms.d_x = r->d_bx + n;
    r->ms.rtol = r->rtol;
    r->ms.atol = 0.0;
    r->ms.inner_rtol = r->inner_rtol;
    r->ms.max_outer = 200;
    r->ms.max_inner = 20000;  // FP32 iterations per segment before the next FP64 update
    r->t_start = now_s();
    return afm::mixed_begin(r->ms);
}

}  // namespace

namespace {

// One round of progress (caller holds state_mu): admit, then take the next step
// of every admitted request whose previous step has finished on the GPU.
// Returns how many things changed.
int step(afm_server* s) {
    cudaSetDevice(s->device);
    int changes = admit(s);
    std::vector<Request*> still;
    still.reserve(s->active.size());
    for (Request* r : s->active) {
        if (r->state == RQ_ADMITTING &&
            r->fin.wait_for(std::chrono::seconds(0)) == std::future_status::ready) {
            const int st = r->fin.get();
            if (st != AFM_SUCCESS) {
                finish(s, r, st, "finalize failed");
                continue;
            }
            const int s2 = start(s, r);
            if (s2 != AFM_SUCCESS) {
                finish(s, r, s2, afm_last_error());
                continue;
            }
            r->state = RQ_RUNNING;
            changes++;
        }
        if (r->state == RQ_RUNNING) {
            int st = AFM_SUCCESS;
            while (st == AFM_SUCCESS && r->ms.phase != afm::MS_DONE && afm::mixed_ready(r->ms)) {
                st = afm::mixed_advance(r->ms);
                changes++;
            }
            if (st != AFM_SUCCESS) {
                afm::mixed_end(r->ms, nullptr);
                finish(s, r, st, afm_last_error());
                continue;
            }
            if (r->ms.phase == afm::MS_DONE) {
                // the solve's work has finished: a pageable copy returns quickly
                const size_t n = r->op->n_dofs;
                r->x.resize(n);
                cudaMemcpyAsync(r->x.data(), r->d_bx + n, n * sizeof(double), cudaMemcpyDeviceToHost, r->op->stream);
                cudaEventRecord(r->copied, r->op->stream);
                r->state = RQ_COPYING;
            }
        }
        if (r->state == RQ_COPYING && cudaEventQuery(r->copied) == cudaSuccess) {
            const int st = afm::mixed_end(r->ms, &r->stats);
            finish(s, r, st, st ? afm_last_error() : nullptr);
            continue;
        }
        still.push_back(r);
    }
    s->active.swap(still);
    changes += admit(s);
    return changes;
}

void run_progress(afm_server* s) {
    cudaSetDevice(s->device);
    while (s->running.load()) {
        int changes;
        {
            std::lock_guard<std::mutex> lk(s->state_mu);
            changes = step(s);
        }
        if (!changes) std::this_thread::sleep_for(std::chrono::microseconds(20));
    }
}

}  // namespace

extern "C" {

int afm_server_create(afm_server** out, int device, uint64_t hbm_budget_bytes, uint32_t max_active) {
    if (!out) return afm::set_error(AFM_ERR_INVALID_ARG, "out is null");
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return afm::set_error(AFM_ERR_CUDA, "no CUDA device");
    if (device < 0) cudaGetDevice(&device);
    if (device >= ndev) return afm::set_error(AFM_ERR_INVALID_ARG, "device %d of %d", device, ndev);
    if (cudaSetDevice(device) != cudaSuccess) return afm::set_error(AFM_ERR_CUDA, "cudaSetDevice(%d)", device);
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) return afm::set_error(AFM_ERR_CUDA, "cudaMemGetInfo");
    auto* s = new afm_server();
    s->device = device;
    s->budget = hbm_budget_bytes ? hbm_budget_bytes : (uint64_t)(free_b * 0.85);
    s->reserve = std::min<uint64_t>(total_b / 50, 2ull << 30);
    s->max_active = max_active ? max_active : 64;
    s->reaper = std::thread(reap, s);
    s->running = true;
    s->progress = std::thread(run_progress, s);
    *out = s;
    return afm::set_error(AFM_SUCCESS, "");
}

int afm_server_submit(afm_server* s, afm_operator* op, const double* b, double rtol, double inner_rtol, uint64_t* id) {
    if (!s || !op || !b || !id) return afm::set_error(AFM_ERR_INVALID_ARG, "null argument");
    if (!op->have_map) return afm::set_error(AFM_ERR_STATE, "operator without a map");
    if (op->device != s->device) return afm::set_error(AFM_ERR_INVALID_ARG, "operator on device %d", op->device);
    if (!(rtol > 0.0) || !(inner_rtol > 0.0) || inner_rtol >= 1.0)
        return afm::set_error(AFM_ERR_INVALID_ARG, "rtol %g, inner_rtol %g", rtol, inner_rtol);
    std::lock_guard<std::mutex> lk(s->state_mu);
    auto* r = new Request();
    r->id = s->next_id++;
    r->op = op;
    r->b.assign(b, b + op->n_dofs);
    r->rtol = rtol;
    r->inner_rtol = inner_rtol;
    r->est_bytes = estimate_bytes(op);
    r->t_submit = now_s();
    s->queue.push_back(r);
    s->all[r->id] = r;
    *id = r->id;
    return afm::set_error(AFM_SUCCESS, "");
}

int afm_server_poll(afm_server* s, uint32_t* n_queued, uint32_t* n_active) {
    if (!s) return afm::set_error(AFM_ERR_INVALID_ARG, "null server");
    std::lock_guard<std::mutex> lk(s->state_mu);
    step(s);
    if (n_queued) *n_queued = (uint32_t)s->queue.size();
    if (n_active) *n_active = (uint32_t)s->active.size();
    return afm::set_error(AFM_SUCCESS, "");
}

int afm_server_take(afm_server* s, uint64_t id, int* finished, double* x, afm_solve_stats* stats, double* times) {
    if (!s || !finished) return afm::set_error(AFM_ERR_INVALID_ARG, "null argument");
    *finished = 0;
    std::lock_guard<std::mutex> lk(s->state_mu);
    auto it = s->all.find(id);
    if (it == s->all.end()) return afm::set_error(AFM_ERR_INVALID_ARG, "unknown request %llu", (unsigned long long)id);
    Request* r = it->second;
    if (r->state != RQ_DONE) return afm::set_error(AFM_SUCCESS, "");
    *finished = 1;
    const int status = r->status;
    const std::string msg = r->message;
    if (x && r->x.size() == r->b.size()) memcpy(x, r->x.data(), r->x.size() * sizeof(double));
    if (stats) *stats = r->stats;
    if (times) {
        times[0] = r->t_submit;
        times[1] = r->t_admit;
        times[2] = r->t_start;
        times[3] = r->t_done;
    }
    s->all.erase(it);
    delete r;
    if (status != AFM_SUCCESS) return afm::set_error(status, "request failed: %s", msg.c_str());
    return afm::set_error(AFM_SUCCESS, "");
}

int afm_server_destroy(afm_server* s) {
    if (!s) return AFM_SUCCESS;
    s->running = false;
    if (s->progress.joinable()) s->progress.join();
    cudaSetDevice(s->device);
    for (Request* r : s->active)
        if (r->state == RQ_ADMITTING) r->fin.wait();
    cudaDeviceSynchronize();
    for (auto& kv : s->all) {
        Request* r = kv.second;
        if (r->ms.ev) afm::mixed_end(r->ms, nullptr);
        release_device(s, r);
        delete r;
    }
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
        s->cv.notify_one();
    }
    s->reaper.join();
    delete s;
    return AFM_SUCCESS;
}

}  // extern "C"
