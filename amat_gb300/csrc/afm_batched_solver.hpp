// Launchers of the batched CG kernels (afm_batched_solver.cu).
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

namespace afm {

constexpr int kBBlocks = 256;  // row chunks of the column reductions

// Per-column scalar slots: sc[j * kBSlots + slot].
enum : int { B_RZ = 0, B_ALPHA, B_BETA, B_RR, B_BB, B_TOL, B_ITER, B_FLAG, B_DONE, kBSlots = 12 };

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
// part[block * R + j]: partial ||a_j||^2 (sum over kBBlocks in fixed order)
template <typename T>
cudaError_t launch_bnorm2(const T* a, size_t n, uint32_t ld, uint32_t R, double* part, cudaStream_t st);

}  // namespace afm
