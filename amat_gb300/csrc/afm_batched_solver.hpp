// Launchers of the batched CG kernels (afm_batched_solver.cu).
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

namespace afm {

constexpr int kBBlocks = 1024;  // row chunks of the column reductions

// Per-column scalar slots: sc[j * kBSlots + slot].
// B_BN: ||b_j||; B_TRR: ||b_j - A x_j||^2 in FP64 at the last residual check;
// B_CONV: column j meets its FP64 tolerance; B_RZOLD: r.z of the step before
// the last update; B_GAMMA: coefficient of a reliable update (mixed-precision
// solve).
enum : int {
    B_RZ = 0, B_ALPHA, B_BETA, B_RR, B_BB, B_TOL, B_ITER, B_FLAG, B_DONE, B_CONV, B_TRR, B_BN, B_RZOLD, B_GAMMA,
    kBSlots = 16
};

template <typename T>
cudaError_t launch_bset_constrained(T* v, const T* u, const uint32_t* idx, uint32_t nc, uint32_t ld, uint32_t R,
                                    cudaStream_t st);
template <typename T>
cudaError_t launch_bcg_init(const T* b, const T* q, const T* dinv, T* r, T* z, T* p, size_t n, uint32_t ld,
                            uint32_t R, double* sc, double* part, double rtol, double atol, cudaStream_t st);
template <typename T>
cudaError_t launch_bcg_step_scalars(const T* p, const T* q, size_t n, uint32_t ld, uint32_t R, double* sc,
                                    double* part, cudaStream_t st);
// remaining: device counter of columns still iterating after this step
template <typename T>
cudaError_t launch_bcg_update(T* x, T* r, T* z, T* p, const T* q, const T* dinv, size_t n, uint32_t ld, uint32_t R,
                              double* sc, double* part, double maxit, unsigned int* remaining, cudaStream_t st);
// Mixed-precision block solve. bstore_norm: sc[B_BN] = ||a_j|| of an FP64 block.
// bcheck: sc[B_TRR] = ||a_j||^2 of the FP64 residual block and sc[B_CONV] =
// (||a_j|| <= max(rtol sc[B_BN], atol)).
cudaError_t launch_bstore_norm(const double* a, size_t n, uint32_t R, double* sc, double* part, cudaStream_t st);
cudaError_t launch_bcheck(const double* a, size_t n, uint32_t R, double* sc, double* part, double rtol, double atol,
                          cudaStream_t st);
// Reliable update of the FP32 block recursion from the FP64 residual block
// (a finished column keeps its last direction p_k): r = fl32(r64),
// z = dinv r, p = z + beta (p - gamma z) with beta = r.z / r_k.z_k and
// gamma = r.p / r.z (p = z where the column's recursion broke down); per
// column rz, rr, target inner_rtol ||r||, iteration count cleared, done where
// B_CONV is set.
cudaError_t launch_breliable(const double* r64, float* r, float* z, float* p, const float* dinv, size_t n, uint32_t R,
                             double* sc, double* part, double inner_rtol, cudaStream_t st);
// part[block * R + j]: partial ||a_j||^2 (sum over kBBlocks in fixed order)
template <typename T>
cudaError_t launch_bnorm2(const T* a, size_t n, uint32_t ld, uint32_t R, double* part, cudaStream_t st);

}  // namespace afm
