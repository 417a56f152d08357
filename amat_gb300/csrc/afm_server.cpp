// Serving loop for many CG solves on different operators (afm_server_* in
// include/afm.h; no counterpart in the reference).
//
// A request carries its own operator (maps and element matrices set on the
// host) and load. Requests wait in a queue and are admitted (lane-sized ones
// first, the rest in arrival order) while the server's HBM budget, the
// device's free memory and the slot limit allow.
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
// Small requests (FP32 element matrices up to lane_max_bytes) run their FP32
// iterations in the serving lane instead (afm_lane.cu): whenever no lane
// launch is in flight, the progress thread gathers every solve waiting for
// FP32 iterations into one launch, one thread-block cluster per solve, that
// runs up to lane_iters iterations of each of them. Requests admitted while a
// launch runs join the next one, so the lane batches the matvecs of all active
// small solves without waiting for any of them to finish.
//
// Each request's arithmetic is independent of the others (own operator, own
// vectors, deterministic kernels, a lane cluster per request), so its result
// is the same alone and in any mix, bit for bit.
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
    uint64_t lane_bytes = 0;  // FP32 element-matrix bytes (lane eligibility, stream priority)
    int state = RQ_QUEUED;
    std::future<int> fin;
    double* d_bx = nullptr;  // b then x on the device
    std::vector<double> x;   // result on the host
    cudaEvent_t copied = nullptr;
    afm::MixedSolve ms;
    bool lane_candidate = false;         // small enough for the serving lane (decided at admission)
    afm::LaneSeg* d_lane_segs = nullptr; // the lane's view of the operator's segments
    uint32_t lane_nsegs = 0;
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
// FP64 and FP32 work vectors (and the FP64 inner vectors of formats 3 to 5),
// b and x; 10% and 1 MB of slack.
uint64_t estimate_bytes(const afm_operator* op) {
    uint64_t ke = 0;
    for (uint32_t e = 0; e < op->n_elem; e++) {
        const uint64_t n = op->offsets[e + 1] - op->offsets[e];
        ke += n * n * 8 + 8 * n + 6 * n * (n / 2 + 1);
    }
    const uint64_t vec = (uint64_t)op->n_dofs * (8 * 8 + 7 * 4 + 8 * 8 + 3 * 8);
    return (ke + vec) * 11 / 10 + (1u << 20);
}

// Bytes of FP32 element matrices the lane streams per product (hi plane).
uint64_t lane_bytes(const afm_operator* op) {
    uint64_t b = 0;
    for (uint32_t e = 0; e < op->n_elem; e++) {
        const uint64_t n = op->offsets[e + 1] - op->offsets[e];
        b += n * n * 4;
    }
    return b;
}

// Lane defaults: requests whose FP32 element matrices are at most 8 MB (a
// cluster of kLaneCtas SMs streams them in tens of microseconds, below the
// launch overheads of a per-request iteration), 32 iterations per launch.
constexpr uint64_t kLaneMaxBytes = 8ull << 20;
constexpr uint32_t kLaneIters = 32;

// Requests on their own streams with at least kFp64InnerDofs DoFs iterate in
// FP64 vectors on the corrected symmetric arena (format 4): the FP32
// recursion stalls on the large elastic requests of a serving mix (hex20
// elasticity 64^3, 3.3M DoF, under a random load: 100,053 FP32 iterations
// against 6,209 for FP64 CG; 6,385 in format 4, whose product takes 0.71 ms
// against 1.36 ms for the split product). Smaller ones keep the cheaper FP32
// recursion (format 1), which converges like format 4 up to ~0.5M DoF (hex20
// 32^3: 1.32x against 1.38x over FP64 CG; hex8 elasticity 48^3: 1.29x and 1.28x).
constexpr int kStreamInnerFormat = 4;
constexpr uint32_t kFp64InnerDofs = 1u << 20;

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
    // serving lane: one launch in flight at most, its job table in pinned
    // memory (rewritten only once the launch that read it has finished)
    uint64_t lane_max_bytes = kLaneMaxBytes;
    uint32_t lane_iters = kLaneIters;
    // symmetric inner format of the requests that run on their own streams
    int inner_format = kStreamInnerFormat;
    // stream priorities (lower numbers first): the lane and small requests
    // ahead of large ones, so that a small request's launches do not queue
    // behind the many launches a large request has in flight
    int prio_low = 0, prio_high = 0;
    bool priorities = true;
    cudaStream_t lane_stream = nullptr;
    cudaEvent_t lane_done = nullptr;
    bool lane_busy = false;
    afm::LaneJob* h_jobs = nullptr;
    afm::LaneJob* d_jobs = nullptr;
    afm_server_info info{};
};

namespace {

void release_device(afm_server* s, Request* r) {
    if (r->d_bx && r->op) cudaFreeAsync(r->d_bx, r->op->stream);
    r->d_bx = nullptr;
    if (r->d_lane_segs && r->op) cudaFreeAsync(r->d_lane_segs, r->op->stream);
    r->d_lane_segs = nullptr;
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
// OpenMP loops over all host cores, and more in parallel only contend. Small
// requests (the lane's) may use kExtraSmallFinalizing more slots, so that
// they do not wait behind the seconds-long finalizes of large meshes.
constexpr int kMaxFinalizing = 4;
constexpr int kExtraSmallFinalizing = 2;
// Admission order: lane-sized requests first (oldest first), then the rest
// in arrival order. Small requests then never wait behind the seconds-long
// finalizes of large meshes, while large requests still start in arrival
// order and overlap the rest of the mix (shortest-first throughout held
// them back until the end of a burst, where they ran with little overlap:
// 18.7 against 20.2 solves/s on the edge-8..32 mix).
bool is_small(const afm_server* s, const Request* r) {
    return s->lane_max_bytes > 0 && r->op->matfree_type != 2 && r->lane_bytes <= s->lane_max_bytes;
}

// Index in the queue of the next request to admit.
size_t next_in_queue(const afm_server* s) {
    for (size_t i = 0; i < s->queue.size(); i++)
        if (is_small(s, s->queue[i])) return i;
    return 0;
}

// admission while the budget, free device memory and slots allow
int admit(afm_server* s) {
    int admitted = 0;
    int finalizing = 0;
    for (const Request* r : s->active) finalizing += (r->state == RQ_ADMITTING);
    while (!s->queue.empty() && s->active.size() < s->max_active &&
           finalizing < kMaxFinalizing + kExtraSmallFinalizing) {
        const size_t k = next_in_queue(s);
        Request* r = s->queue[k];
        const bool small = is_small(s, r);
        if (!small && finalizing >= kMaxFinalizing) break;
        size_t free_b = 0, total_b = 0;
        if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) break;
        const bool fits = s->in_use + r->est_bytes <= s->budget && r->est_bytes + s->reserve <= free_b;
        if (!fits && !s->active.empty()) break;  // wait for memory to free up
        s->queue.erase(s->queue.begin() + (std::ptrdiff_t)k);
        s->in_use += r->est_bytes;
        r->state = RQ_ADMITTING;
        r->t_admit = now_s();
        afm_operator* op = r->op;
        // lane requests run colour segments (the lane reads their units), never patches
        r->lane_candidate = small;
        if (r->lane_candidate) afm_set_patch_mode(op, 0);
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

// The lane's segment table of a finalised operator (FP64_SPLIT arena in
// colour segments), uploaded on the operator's stream.
int build_lane_segs(Request* r) {
    afm_operator* op = r->op;
    std::vector<afm::LaneSeg> segs;
    std::vector<uint32_t> colors;
    for (const afm::Segment& g : op->segs) {
        if (g.units == 0) continue;
        afm::LaneSeg L{};
        L.ke = reinterpret_cast<const float*>(op->d_ke + g.ke_offset);  // hi plane first in every unit
        L.map = op->d_map + g.map_offset;
        L.unit_floats = g.unit_bytes / 4;
        L.n = g.n;
        L.regime = (uint32_t)g.regime;
        L.units = g.units;
        L.count = g.count;
        segs.push_back(L);
        colors.push_back(g.color);
    }
    // segments are colour-sorted: a cluster barrier after the last segment of each colour
    for (size_t k = 0; k < segs.size(); k++)
        segs[k].sync_after = (k + 1 == segs.size() || colors[k + 1] != colors[k]) ? 1u : 0u;
    r->lane_nsegs = (uint32_t)segs.size();
    if (segs.empty()) return AFM_SUCCESS;
    if (cudaMallocAsync((void**)&r->d_lane_segs, sizeof(afm::LaneSeg) * segs.size(), op->stream) != cudaSuccess)
        return AFM_ERR_OOM;
    if (cudaMemcpyAsync(r->d_lane_segs, segs.data(), sizeof(afm::LaneSeg) * segs.size(), cudaMemcpyHostToDevice,
                        op->stream) != cudaSuccess ||
        cudaStreamSynchronize(op->stream) != cudaSuccess)  // segs is a local vector
        return AFM_ERR_CUDA;
    return AFM_SUCCESS;
}

int start(afm_server* s, Request* r) {
    afm_operator* op = r->op;
    const size_t n = op->n_dofs;
    const bool lane = r->lane_candidate && op->precision == AFM_PREC_FP64_SPLIT && !op->use_patches &&
                      op->matfree_type != 2;
    // priority by size: one level per factor 8 of element-matrix bytes above 8 MB
    if (s->priorities && s->prio_high < s->prio_low) {
        int level = 0;
        for (uint64_t b = r->lane_bytes; b > (8ull << 20) && level < s->prio_low - s->prio_high; b >>= 3) level++;
        const int st = afm::set_stream_priority(op, s->prio_high + level);
        if (st != AFM_SUCCESS) return st;
    }
    if (lane) {
        const int st = build_lane_segs(r);
        if (st != AFM_SUCCESS) return st;
    }
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
    r->ms.lane = lane;
    if (!lane) afm_set_symmetric_inner(op, op->n_dofs >= kFp64InnerDofs ? s->inner_format : 1);
    r->t_start = now_s();
    if (lane) s->info.lane_requests++;
    else s->info.stream_requests++;
    return afm::mixed_begin(r->ms);
}

// Launches the FP32 iterations of every solve waiting for the lane (at most
// one launch in flight). Returns the number of solves launched.
int launch_lane_batch(afm_server* s) {
    if (s->lane_busy) {
        if (cudaEventQuery(s->lane_done) != cudaSuccess) return 0;
        s->lane_busy = false;
    }
    std::vector<Request*> batch;
    for (Request* r : s->active)
        if (r->state == RQ_RUNNING && r->ms.phase == afm::MS_LANE && afm::mixed_ready(r->ms) &&
            batch.size() < s->max_active)
            batch.push_back(r);
    if (batch.empty()) return 0;
    for (size_t i = 0; i < batch.size(); i++) {
        Request* r = batch[i];
        afm::LaneJob& J = s->h_jobs[i];
        afm::mixed_lane_job(r->ms, J);
        J.segs = r->d_lane_segs;
        J.n_segs = r->lane_nsegs;
        cudaStreamWaitEvent(s->lane_stream, r->ms.ev, 0);
    }
    cudaError_t e = cudaMemcpyAsync(s->d_jobs, s->h_jobs, sizeof(afm::LaneJob) * batch.size(),
                                    cudaMemcpyHostToDevice, s->lane_stream);
    if (e == cudaSuccess) e = afm::launch_lane(s->d_jobs, (uint32_t)batch.size(), s->lane_iters, s->lane_stream);
    int st = e == cudaSuccess ? AFM_SUCCESS : AFM_ERR_CUDA;
    for (Request* r : batch) {  // scalars to each solve's host mirror, then its event
        if (st == AFM_SUCCESS) st = afm::mixed_lane_record(r->ms, s->lane_stream);
        r->ms.phase = afm::MS_LANEITER;
    }
    if (st == AFM_SUCCESS) e = cudaEventRecord(s->lane_done, s->lane_stream);
    if (st != AFM_SUCCESS || e != cudaSuccess) {
        if (e == cudaSuccess) e = cudaGetLastError();
        for (Request* r : batch) {
            afm::mixed_end(r->ms, nullptr);
            finish(s, r, AFM_ERR_CUDA, cudaGetErrorString(e));
        }
        std::vector<Request*> still;
        for (Request* r : s->active)
            if (r->state != RQ_DONE) still.push_back(r);
        s->active.swap(still);
        return (int)batch.size();
    }
    s->lane_busy = true;
    s->info.lane_launches++;
    s->info.lane_solve_launches += batch.size();
    s->info.lane_max_batch = std::max<uint32_t>(s->info.lane_max_batch, (uint32_t)batch.size());
    return (int)batch.size();
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
            while (st == AFM_SUCCESS && r->ms.phase != afm::MS_DONE && r->ms.phase != afm::MS_LANE &&
                   afm::mixed_ready(r->ms)) {
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
    changes += launch_lane_batch(s);
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
    cudaDeviceGetStreamPriorityRange(&s->prio_low, &s->prio_high);
    if (cudaStreamCreateWithPriority(&s->lane_stream, cudaStreamNonBlocking, s->prio_high) != cudaSuccess ||
        cudaEventCreateWithFlags(&s->lane_done, cudaEventDisableTiming) != cudaSuccess ||
        cudaMallocHost((void**)&s->h_jobs, sizeof(afm::LaneJob) * s->max_active) != cudaSuccess ||
        cudaMalloc((void**)&s->d_jobs, sizeof(afm::LaneJob) * s->max_active) != cudaSuccess) {
        if (s->d_jobs) cudaFree(s->d_jobs);
        if (s->h_jobs) cudaFreeHost(s->h_jobs);
        if (s->lane_done) cudaEventDestroy(s->lane_done);
        if (s->lane_stream) cudaStreamDestroy(s->lane_stream);
        delete s;
        return afm::set_error(AFM_ERR_CUDA, "serving lane resources");
    }
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
    r->lane_bytes = lane_bytes(op);
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
    cudaFree(s->d_jobs);
    cudaFreeHost(s->h_jobs);
    cudaEventDestroy(s->lane_done);
    cudaStreamDestroy(s->lane_stream);
    delete s;
    return AFM_SUCCESS;
}

int afm_server_set_lane(afm_server* s, uint64_t max_ke_bytes, uint32_t iters_per_launch) {
    if (!s) return afm::set_error(AFM_ERR_INVALID_ARG, "null server");
    if (iters_per_launch == 0 || iters_per_launch > 4096)
        return afm::set_error(AFM_ERR_INVALID_ARG, "iters_per_launch %u (1 to 4096)", iters_per_launch);
    std::lock_guard<std::mutex> lk(s->state_mu);
    s->lane_max_bytes = max_ke_bytes;
    s->lane_iters = iters_per_launch;
    return afm::set_error(AFM_SUCCESS, "");
}

int afm_server_set_priorities(afm_server* s, int enable) {
    if (!s || (enable != 0 && enable != 1)) return afm::set_error(AFM_ERR_INVALID_ARG, "server or enable %d", enable);
    std::lock_guard<std::mutex> lk(s->state_mu);
    s->priorities = enable == 1;
    return afm::set_error(AFM_SUCCESS, "");
}

int afm_server_set_inner_format(afm_server* s, int format) {
    if (!s) return afm::set_error(AFM_ERR_INVALID_ARG, "null server");
    if (format < 0 || format > 5) return afm::set_error(AFM_ERR_INVALID_ARG, "inner format %d (0 to 5)", format);
    std::lock_guard<std::mutex> lk(s->state_mu);
    s->inner_format = format;
    return afm::set_error(AFM_SUCCESS, "");
}

int afm_server_get_info(afm_server* s, afm_server_info* info) {
    if (!s || !info) return afm::set_error(AFM_ERR_INVALID_ARG, "null argument");
    std::lock_guard<std::mutex> lk(s->state_mu);
    *info = s->info;
    return afm::set_error(AFM_SUCCESS, "");
}

}  // extern "C"
