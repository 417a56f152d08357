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

#include "afm_internal.hpp"

namespace afm {

enum MixedPhase : int {
    MS_IDLE = 0,
    MS_NORMB,     // ||b|| in flight
    MS_RESID,     // FP64 true residual in flight
    MS_SEGSTART,  // start of an FP32 segment (init or reliable update) in flight
    MS_ITER,      // a captured batch of FP32 iterations in flight
    MS_DONE
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
    cudaEvent_t ev = nullptr, e0 = nullptr, e1 = nullptr;
};

// Checks the arguments, allocates the work vectors and enqueues the set-up.
int mixed_begin(MixedSolve& m);
// True when the work enqueued by the last step has completed.
bool mixed_ready(const MixedSolve& m);
// Takes the next step (call only when mixed_ready): reads the scalars of the
// finished work and enqueues the next, or moves to MS_DONE.
int mixed_advance(MixedSolve& m);
// Fills stats (device time between begin and done), releases the events and
// returns the solve's status.
int mixed_end(MixedSolve& m, afm_solve_stats* stats);

}  // namespace afm
