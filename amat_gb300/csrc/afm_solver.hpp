// Launchers of the vector / CG kernels (afm_solver.cu).
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

namespace afm {

constexpr int kRedBlocks = 512;
constexpr int kRedThreads = 256;

// Blocks of a reduction over n entries: about 2048 entries per block, at
// least 1 and at most kRedBlocks (a function of n only: deterministic sums).
inline uint32_t red_blocks(size_t n) {
    const size_t b = (n + 2047) / 2048;
    return (uint32_t)(b < 1 ? 1 : (b > (size_t)kRedBlocks ? (size_t)kRedBlocks : b));
}

// Scalar slots of the solver state (device array of kScalarSlots doubles,
// followed by kPartialSlots reduction partials).
// S_TOL, S_MAXIT, S_NORM are set by the host before the iterations; the
// kernels keep S_ITER and raise S_DONE on convergence (monitored norm <=
// S_TOL), on S_MAXIT iterations (when > 0) or on breakdown (S_FLAG), after
// which further iterations leave every vector unchanged. That lets a captured
// graph run several iterations without reading anything back.
// S_RZOLD keeps r.z of the step before the last update (the reliable update
// of the mixed-precision solve needs it); S_GAMMA is that update's
// orthogonalisation coefficient.
enum : int {
    S_RZ = 0, S_PQ, S_ALPHA, S_BETA, S_RR, S_ZZ, S_BB, S_DB, S_FLAG,
    S_DONE, S_TOL, S_ITER, S_MAXIT, S_NORM, S_RZOLD, S_GAMMA,
    kScalarSlots = 16
};
constexpr int kPartialSlots = 5 * kRedBlocks;

// T = double (FP64 CG) or float (inner CG of the mixed-precision solve);
// step scalars are FP64 in both; dot products accumulate in FP64 (double) or
// in compensated FP32 (float) and are reduced across threads in FP64.
template <typename T>
cudaError_t launch_set_constrained(T* v, const T* u, const uint32_t* idx, uint32_t n, cudaStream_t st);
template <typename T>
cudaError_t launch_cg_init(const T* b, const T* q, const T* dinv, T* r, T* z, T* p, size_t n, double* sc,
                           double* part, cudaStream_t st);
template <typename T>
cudaError_t launch_cg_alpha(const T* p, const T* q, size_t n, double* sc, double* part, cudaStream_t st);
template <typename T>
cudaError_t launch_cg_update(T* x, T* r, T* z, T* p, const T* q, const T* dinv, size_t n, double* sc, double* part,
                             cudaStream_t st);
template <typename T>
cudaError_t launch_invert(T* dinv, const double* d, size_t n, cudaStream_t st);
// sc[S_PQ] = ||a||^2 (no CG bookkeeping)
template <typename T>
cudaError_t launch_norm2(const T* a, size_t n, double* sc, double* part, cudaStream_t st);
// Reliable update of the FP32 recursion (after a segment stopped on S_DONE,
// p is still the last direction p_k): r = fl32(r64), z = dinv r,
// p = z + beta (p - gamma z) with beta = r.z / r_k.z_k and gamma = r.p / r.z,
// so that the new residual is orthogonal to the kept direction again;
// sc[S_RZ], sc[S_RR], sc[S_ZZ] of the new residual; S_DONE and S_ITER cleared.
// The recursion runs on the residual times a power of two: sigma is the new
// segment's scale (r = fl32(sigma r64)), rho = sigma / the previous segment's.
// T = float (the FP32 recursion) or double (the FP64-vector recursion of
// symmetric inner format 3).
template <typename T>
cudaError_t launch_cg_reliable(const double* r64, T* r, T* z, T* p, const T* dinv, size_t n, double* sc,
                               double* part, double sigma, double rho, cudaStream_t st);
cudaError_t launch_axpby(double* y, const double* x, double a, double b, size_t n, cudaStream_t st);
// out = fl32(scale in), or scale in for a double out
cudaError_t launch_to_f32(float* out, const double* in, size_t n, cudaStream_t st, double scale = 1.0);
cudaError_t launch_to_f32(double* out, const double* in, size_t n, cudaStream_t st, double scale = 1.0);
// x += inv d, d = 0
cudaError_t launch_add_f32(double* x, float* d, size_t n, cudaStream_t st, double inv = 1.0);
cudaError_t launch_add_f32(double* x, double* d, size_t n, cudaStream_t st, double inv = 1.0);

// Words of the u-scale buffer of an operator (afm_operator::d_usc): [0] max|u|
// of the last single-vector split product, [1] block counter, [2, 2 +
// kRedBlocks) block maxima, then kMaxUmaxCols per-column maxima of a batched
// split product.
constexpr int kMaxUmaxCols = 256;
constexpr int kUscWords = 2 + kRedBlocks + kMaxUmaxCols;
constexpr int kUscColsOffset = 2 + kRedBlocks;
// w[0] = max over the unmasked i < n of |u[i]| (double bits) and vz[0 .. nv) =
// 0, in one launch (mask may be null; w[1] must be 0 before the first launch
// and is left 0).
cudaError_t launch_umax(const double* u, const uint8_t* mask, size_t n, double* vz, size_t nv,
                        unsigned long long* w, cudaStream_t st);
// cm[j] = max over the unmasked rows of |U(:, j)|, j < R <= kMaxUmaxCols.
cudaError_t launch_umax_cols(const double* U, const uint8_t* mask, size_t rows, uint32_t R, uint32_t ld,
                             unsigned long long* cm, cudaStream_t st);

}  // namespace afm
