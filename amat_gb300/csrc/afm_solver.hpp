// Launchers of the vector / CG kernels (afm_solver.cu).
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

namespace afm {

constexpr int kRedBlocks = 512;
constexpr int kRedThreads = 256;

// Scalar slots of the solver state (device array of kScalarSlots doubles,
// followed by kPartialSlots reduction partials).
enum : int { S_RZ = 0, S_PQ, S_ALPHA, S_BETA, S_RR, S_ZZ, S_BB, S_DB, S_FLAG, kScalarSlots = 16 };
constexpr int kPartialSlots = 5 * kRedBlocks;

cudaError_t launch_dots(const double* a, const double* b, size_t n, double* part, cudaStream_t st);
cudaError_t launch_cg_init(const double* b, const double* q, const double* dinv, double* r, double* z, double* p,
                           size_t n, double* sc, double* part, cudaStream_t st);
cudaError_t launch_cg_alpha(const double* p, const double* q, size_t n, double* sc, double* part, cudaStream_t st);
cudaError_t launch_cg_update(double* x, double* r, double* z, double* p, const double* q, const double* dinv,
                             size_t n, double* sc, double* part, cudaStream_t st);
cudaError_t launch_invert(double* dinv, const double* d, size_t n, cudaStream_t st);
cudaError_t launch_axpby(double* y, const double* x, double a, double b, size_t n, cudaStream_t st);

}  // namespace afm
