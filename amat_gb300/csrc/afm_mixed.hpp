// Resumable mixed-precision solve (afm_solve_cg_mixed_device): FP32
// Jacobi-PCG recursion on the operator's FP32 products (symmetric FP32 copy,
// hi plane of the split arena, or matrix-free kernels) with FP64 reliable
// updates, written as a state machine whose every step only enqueues work on
// the operator's stream and records an event. afm_solve_cg_mixed_device
// drives it by waiting on the event; the serving loop (afm_server.cpp) drives
// many at once by polling their events, so their kernels overlap on the GPU.
#pragma once

#include <cuda_runtime.h>

#include <cmath>
#include <vector>

#include "afm_internal.hpp"

namespace afm {

enum MixedPhase : int {
    MS_IDLE = 0,
    MS_NORMB,     // ||b|| in flight
    MS_RESID,     // FP64 true residual in flight
    MS_SEGSTART,  // start of an FP32 segment (init or reliable update) in flight
    MS_ITER,      // a captured batch of FP32 iterations in flight
    MS_DONE,
    MS_LANE,      // serving lane: FP32 iterations wait for the next lane launch (afm_lane.cu)
    MS_LANEITER   // serving lane: a lane launch with this solve's iterations in flight
};

struct MixedSolve {
    afm_operator* op = nullptr;
    const double* d_b = nullptr;
    double* d_x = nullptr;
    double rtol = 0.0, atol = 0.0, inner_rtol = 0.0;
    int max_outer = 0, max_inner = 0;
    // progress
    int phase = MS_IDLE;
    int outer = 0, inner_total = 0, stall = 0, status = AFM_ERR_MAXIT;
    double bn = 0.0, tol = 0.0, rn = 0.0, best = HUGE_VAL, inner_tol = 0.0;
    // the FP32 segment runs on sigma times the FP64 residual (sigma = 2^k with
    // ||sigma r|| in [0.5, 1)), so that tiny or huge loads stay in FP32's range
    double sigma = 1.0;
    bool fresh = true;
    // the FP32 iterations run in the serving lane: the owner of the solve
    // launches them (launch_lane) for every solve in MS_LANE, records ev on the
    // lane's stream and sets MS_LANEITER; no symmetric inner arena is built
    bool lane = false;
    // symmetric inner format 3: the inner recursion in FP64 vectors with the
    // double-float products of the corrected symmetric arena (set by mixed_begin)
    bool inner64 = false;
    cudaEvent_t ev = nullptr, e0 = nullptr, e1 = nullptr;
    // each FP64 residual of the solve: inner iterations so far and ||r|| / ||b||
    std::vector<int> trace_iters;
    std::vector<double> trace_res;
};

// Checks the arguments, allocates the work vectors and enqueues the set-up.
int mixed_begin(MixedSolve& m);
// True when the work enqueued by the last step has completed.
bool mixed_ready(const MixedSolve& m);
// Takes the next step (call only when mixed_ready and not in MS_LANE): reads
// the scalars of the finished work and enqueues the next, or moves to MS_DONE.
int mixed_advance(MixedSolve& m);
// The FP32 vectors, scalars and error flags of the solve, as a lane job (the
// caller fills segs and n_segs). After the launch, the caller copies the
// device scalars to the host mirror (mixed_lane_record) on the lane's stream.
void mixed_lane_job(const MixedSolve& m, LaneJob& J);
int mixed_lane_record(MixedSolve& m, cudaStream_t lane_stream);
// Fills stats (device time between begin and done), releases the events and
// returns the solve's status.
int mixed_end(MixedSolve& m, afm_solve_stats* stats);

}  // namespace afm
