// Batched Jacobi-PCG: one CG per right-hand side, all advanced in lockstep
// over n_dofs x ld blocks (column j of every block belongs to solve j).
// Every column has its own FP64 scalars (rz, alpha, beta, norms, done flag);
// a finished column is frozen (alpha = beta = 0) while the others continue.
// Column reductions are deterministic: a fixed grid of kBRows-row chunks per
// block, a fixed in-block order, then a fixed-order sum over the blocks.
#include <cuda_runtime.h>
#include <stdint.h>

#include "afm_batched_solver.hpp"

namespace afm {

namespace {

constexpr int kBThreads = 256;

// Block (rows r of columns j): thread (ry, j) with ry in [0, kBThreads / R).
template <typename T>
__device__ __forceinline__ void row_col(uint32_t R, uint32_t& ry, uint32_t& j, uint32_t& rstep) {
    rstep = kBThreads / R;
    ry = threadIdx.x / R;
    j = threadIdx.x % R;
}

// Sums v over the rstep row lanes of the block for every column; result in
// sh[j] (fixed order).
__device__ __forceinline__ void col_reduce(double v, uint32_t R, uint32_t ry, uint32_t j, uint32_t rstep, double* sh) {
    sh[ry * R + j] = v;
    __syncthreads();
    if (ry == 0) {
        double s = 0.0;
        for (uint32_t y = 0; y < rstep; y++) s += sh[y * R + j];
        sh[j] = s;
    }
    __syncthreads();
}

// partials of up to 3 column dot products: part[(q * kBBlocks + block) * R + j]
template <typename T, int Q>
__global__ void __launch_bounds__(kBThreads) k_bdots(const T* __restrict__ a, const T* __restrict__ b,
                                                     const T* __restrict__ c, size_t n, uint32_t ld, uint32_t R,
                                                     double* part) {
    __shared__ double sh[kBThreads];
    uint32_t ry, j, rstep;
    row_col<T>(R, ry, j, rstep);
    double s0 = 0, s1 = 0, s2 = 0;
    if (ry < rstep && j < R) {
        const size_t chunk = (n + kBBlocks - 1) / kBBlocks;
        const size_t r0 = (size_t)blockIdx.x * chunk, r1 = min(n, r0 + chunk);
        for (size_t i = r0 + ry; i < r1; i += rstep) {
            const double x = a[i * ld + j];
            s0 = __fma_rn(x, (double)b[i * ld + j], s0);
            if (Q > 1) s1 = __fma_rn(x, x, s1);
            if (Q > 2) s2 = __fma_rn((double)c[i * ld + j], (double)c[i * ld + j], s2);
        }
    }
    double v[3] = {s0, s1, s2};
    for (int q = 0; q < Q; q++) {
        col_reduce(ry < rstep ? v[q] : 0.0, R, ry, j, rstep, sh);
        if (ry == 0 && j < R) part[((size_t)q * kBBlocks + blockIdx.x) * R + j] = sh[j];
        __syncthreads();
    }
}

__device__ __forceinline__ double bsum(const double* part, uint32_t q, uint32_t R, uint32_t j) {
    double s = 0.0;
    for (int b = 0; b < kBBlocks; b++) s += part[((size_t)q * kBBlocks + b) * R + j];
    return s;
}

// init: r = b - q, z = dinv r, p = z; per column rz, rr, bb
template <typename T>
__global__ void __launch_bounds__(kBThreads) k_binit(const T* __restrict__ b, const T* __restrict__ q,
                                                     const T* __restrict__ dinv, T* __restrict__ r, T* __restrict__ z,
                                                     T* __restrict__ p, size_t n, uint32_t ld, uint32_t R,
                                                     double* part) {
    __shared__ double sh[kBThreads];
    uint32_t ry, j, rstep;
    row_col<T>(R, ry, j, rstep);
    double rz = 0, rr = 0, bb = 0;
    if (ry < rstep && j < R) {
        const size_t chunk = (n + kBBlocks - 1) / kBBlocks;
        const size_t r0 = (size_t)blockIdx.x * chunk, r1 = min(n, r0 + chunk);
        for (size_t i = r0 + ry; i < r1; i += rstep) {
            const size_t k = i * ld + j;
            const T bi = b[k];
            const T ri = bi - q[k];
            const T zi = dinv[i] * ri;
            r[k] = ri;
            z[k] = zi;
            p[k] = zi;
            rz = __fma_rn((double)ri, (double)zi, rz);
            rr = __fma_rn((double)ri, (double)ri, rr);
            bb = __fma_rn((double)bi, (double)bi, bb);
        }
    }
    double v[3] = {rz, rr, bb};
    for (int qq = 0; qq < 3; qq++) {
        col_reduce(ry < rstep ? v[qq] : 0.0, R, ry, j, rstep, sh);
        if (ry == 0 && j < R) part[((size_t)qq * kBBlocks + blockIdx.x) * R + j] = sh[j];
        __syncthreads();
    }
}

// scalars: sc[j * kBSlots + slot]
__global__ void k_binit_final(double* sc, const double* part, uint32_t R, double rtol, double atol) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= R) return;
    double* c = sc + (size_t)j * kBSlots;
    const double rz = bsum(part, 0, R, j), rr = bsum(part, 1, R, j), bb = bsum(part, 2, R, j);
    c[B_RZ] = rz;
    c[B_RR] = rr;
    c[B_BB] = bb;
    c[B_ITER] = 0.0;
    c[B_FLAG] = (rz < 0.0 || rz != rz) ? 1.0 : 0.0;
    c[B_TOL] = fmax(rtol * sqrt(bb), atol);
    c[B_DONE] = (c[B_FLAG] != 0.0 || sqrt(rr) <= c[B_TOL]) ? 1.0 : 0.0;
}

__global__ void k_balpha(double* sc, const double* part, uint32_t R) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= R) return;
    double* c = sc + (size_t)j * kBSlots;
    const double pq = bsum(part, 0, R, j);
    if (c[B_DONE] != 0.0) {
        c[B_ALPHA] = 0.0;
        return;
    }
    if (!(pq > 0.0)) {
        c[B_FLAG] = 1.0;
        c[B_DONE] = 1.0;
        c[B_ALPHA] = 0.0;
    } else {
        c[B_ALPHA] = c[B_RZ] / pq;
    }
}

// x += alpha p, r -= alpha q, z = dinv r; partials of r.z, r.r
template <typename T>
__global__ void __launch_bounds__(kBThreads) k_bupdate(T* __restrict__ x, T* __restrict__ r, T* __restrict__ z,
                                                       const T* __restrict__ p, const T* __restrict__ q,
                                                       const T* __restrict__ dinv, size_t n, uint32_t ld, uint32_t R,
                                                       const double* sc, double* part) {
    __shared__ double sh[kBThreads];
    uint32_t ry, j, rstep;
    row_col<T>(R, ry, j, rstep);
    double rz = 0, rr = 0;
    if (ry < rstep && j < R) {
        const T alpha = (T)sc[(size_t)j * kBSlots + B_ALPHA];
        const size_t chunk = (n + kBBlocks - 1) / kBBlocks;
        const size_t r0 = (size_t)blockIdx.x * chunk, r1 = min(n, r0 + chunk);
        for (size_t i = r0 + ry; i < r1; i += rstep) {
            const size_t k = i * ld + j;
            x[k] = alpha * p[k] + x[k];
            const T ri = -alpha * q[k] + r[k];
            const T zi = dinv[i] * ri;
            r[k] = ri;
            z[k] = zi;
            rz = __fma_rn((double)ri, (double)zi, rz);
            rr = __fma_rn((double)ri, (double)ri, rr);
        }
    }
    double v[2] = {rz, rr};
    for (int qq = 0; qq < 2; qq++) {
        col_reduce(ry < rstep ? v[qq] : 0.0, R, ry, j, rstep, sh);
        if (ry == 0 && j < R) part[((size_t)qq * kBBlocks + blockIdx.x) * R + j] = sh[j];
        __syncthreads();
    }
}

__global__ void k_bbeta(double* sc, const double* part, uint32_t R, double maxit, unsigned int* remaining) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= R) return;
    double* c = sc + (size_t)j * kBSlots;
    if (c[B_DONE] != 0.0) {
        c[B_BETA] = 0.0;
        return;
    }
    const double rz = bsum(part, 0, R, j), rr = bsum(part, 1, R, j);
    c[B_BETA] = (c[B_RZ] != 0.0) ? rz / c[B_RZ] : 0.0;
    c[B_RZOLD] = c[B_RZ];
    c[B_RZ] = rz;
    c[B_RR] = rr;
    const double it = c[B_ITER] + 1.0;
    c[B_ITER] = it;
    if (rz < 0.0 || rz != rz) {
        c[B_FLAG] = 1.0;
        c[B_DONE] = 1.0;
    } else if (sqrt(rr) <= c[B_TOL] || it >= maxit) {
        c[B_DONE] = 1.0;
    }
    if (c[B_DONE] == 0.0) atomicAdd(remaining, 1u);
}

template <typename T>
__global__ void __launch_bounds__(kBThreads) k_bp(T* __restrict__ p, const T* __restrict__ z, size_t n, uint32_t ld,
                                                  uint32_t R, const double* sc) {
    const size_t total = n * (size_t)R;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < total; k += stride) {
        const size_t i = k / R;
        const uint32_t j = (uint32_t)(k % R);
        // a finished column keeps its last direction
        if (sc[(size_t)j * kBSlots + B_DONE] != 0.0) continue;
        const T beta = (T)sc[(size_t)j * kBSlots + B_BETA];
        p[i * ld + j] = beta * p[i * ld + j] + z[i * ld + j];
    }
}

__global__ void k_bstore_norm(double* sc, const double* part, uint32_t R) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= R) return;
    sc[(size_t)j * kBSlots + B_BN] = sqrt(bsum(part, 0, R, j));
}

__global__ void k_bcheck(double* sc, const double* part, uint32_t R, double rtol, double atol) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= R) return;
    double* c = sc + (size_t)j * kBSlots;
    const double rr = bsum(part, 0, R, j);
    c[B_TRR] = rr;
    c[B_CONV] = (sqrt(rr) <= fmax(rtol * c[B_BN], atol)) ? 1.0 : 0.0;
}

__global__ void __launch_bounds__(kBThreads) k_breliable(const double* __restrict__ r64, float* __restrict__ r,
                                                         float* __restrict__ z, const float* __restrict__ p,
                                                         const float* __restrict__ dinv, size_t n, uint32_t R,
                                                         double* part) {
    __shared__ double sh[kBThreads];
    uint32_t ry, j, rstep;
    row_col<float>(R, ry, j, rstep);
    double rz = 0, rr = 0, rp = 0;
    if (ry < rstep && j < R) {
        const size_t chunk = (n + kBBlocks - 1) / kBBlocks;
        const size_t r0 = (size_t)blockIdx.x * chunk, r1 = min(n, r0 + chunk);
        for (size_t i = r0 + ry; i < r1; i += rstep) {
            const size_t k = i * R + j;
            const float ri = (float)r64[k];
            const float zi = dinv[i] * ri;
            r[k] = ri;
            z[k] = zi;
            rz = __fma_rn((double)ri, (double)zi, rz);
            rr = __fma_rn((double)ri, (double)ri, rr);
            rp = __fma_rn((double)ri, (double)p[k], rp);
        }
    }
    double v[3] = {rz, rr, rp};
    for (int qq = 0; qq < 3; qq++) {
        col_reduce(ry < rstep ? v[qq] : 0.0, R, ry, j, rstep, sh);
        if (ry == 0 && j < R) part[((size_t)qq * kBBlocks + blockIdx.x) * R + j] = sh[j];
        __syncthreads();
    }
}

__global__ void k_breliable_final(double* sc, const double* part, uint32_t R, double inner_rtol) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= R) return;
    double* c = sc + (size_t)j * kBSlots;
    const double rz = bsum(part, 0, R, j), rr = bsum(part, 1, R, j), rp = bsum(part, 2, R, j);
    const bool restart = c[B_FLAG] != 0.0;  // the recursion broke down: fresh direction
    const bool bad = (rz < 0.0 || rz != rz);
    c[B_BETA] = (!restart && !bad && c[B_RZOLD] > 0.0) ? rz / c[B_RZOLD] : 0.0;
    c[B_GAMMA] = (!restart && !bad && rz > 0.0) ? rp / rz : 0.0;
    c[B_RZ] = rz;
    c[B_RR] = rr;
    c[B_ITER] = 0.0;
    c[B_FLAG] = bad ? 1.0 : 0.0;
    c[B_TOL] = inner_rtol * sqrt(rr);
    c[B_DONE] = (c[B_CONV] != 0.0 || c[B_FLAG] != 0.0 || rr == 0.0) ? 1.0 : 0.0;
}

// p = z + beta (p - gamma z) per column
__global__ void __launch_bounds__(kBThreads) k_breliable_p(float* __restrict__ p, const float* __restrict__ z, size_t n,
                                                           uint32_t R, const double* sc) {
    const size_t total = n * (size_t)R;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < total; k += stride) {
        const uint32_t j = (uint32_t)(k % R);
        const double* c = sc + (size_t)j * kBSlots;
        const float beta = (float)c[B_BETA];
        p[k] = __fmaf_rn(beta, p[k], (float)(1.0 - c[B_BETA] * c[B_GAMMA]) * z[k]);
    }
}

template <typename T>
__global__ void k_bset_constrained(T* v, const T* u, const uint32_t* idx, uint32_t nc, uint32_t ld, uint32_t R) {
    const size_t total = (size_t)nc * R;
    const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= total) return;
    const uint32_t c = idx[k / R];
    const uint32_t j = (uint32_t)(k % R);
    v[(size_t)c * ld + j] = u[(size_t)c * ld + j];
}

unsigned grid_for(size_t n) {
    size_t g = (n + kBThreads - 1) / kBThreads;
    return (unsigned)(g > 4096 ? 4096 : (g == 0 ? 1 : g));
}

}  // namespace

template <typename T>
cudaError_t launch_bset_constrained(T* v, const T* u, const uint32_t* idx, uint32_t nc, uint32_t ld, uint32_t R,
                                    cudaStream_t st) {
    if (nc == 0) return cudaSuccess;
    const size_t total = (size_t)nc * R;
    k_bset_constrained<T><<<(unsigned)((total + 255) / 256), 256, 0, st>>>(v, u, idx, nc, ld, R);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_bcg_init(const T* b, const T* q, const T* dinv, T* r, T* z, T* p, size_t n, uint32_t ld,
                            uint32_t R, double* sc, double* part, double rtol, double atol, cudaStream_t st) {
    k_binit<T><<<kBBlocks, kBThreads, 0, st>>>(b, q, dinv, r, z, p, n, ld, R, part);
    k_binit_final<<<(R + 63) / 64, 64, 0, st>>>(sc, part, R, rtol, atol);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_bcg_step_scalars(const T* p, const T* q, size_t n, uint32_t ld, uint32_t R, double* sc,
                                    double* part, cudaStream_t st) {
    k_bdots<T, 1><<<kBBlocks, kBThreads, 0, st>>>(p, q, nullptr, n, ld, R, part);
    k_balpha<<<(R + 63) / 64, 64, 0, st>>>(sc, part, R);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_bcg_update(T* x, T* r, T* z, T* p, const T* q, const T* dinv, size_t n, uint32_t ld, uint32_t R,
                              double* sc, double* part, double maxit, unsigned int* remaining, cudaStream_t st) {
    k_bupdate<T><<<kBBlocks, kBThreads, 0, st>>>(x, r, z, p, q, dinv, n, ld, R, sc, part);
    cudaMemsetAsync(remaining, 0, sizeof(unsigned int), st);
    k_bbeta<<<(R + 63) / 64, 64, 0, st>>>(sc, part, R, maxit, remaining);
    k_bp<T><<<grid_for(n * R), kBThreads, 0, st>>>(p, z, n, ld, R, sc);
    return cudaGetLastError();
}

cudaError_t launch_bstore_norm(const double* a, size_t n, uint32_t R, double* sc, double* part, cudaStream_t st) {
    k_bdots<double, 1><<<kBBlocks, kBThreads, 0, st>>>(a, a, nullptr, n, R, R, part);
    k_bstore_norm<<<(R + 63) / 64, 64, 0, st>>>(sc, part, R);
    return cudaGetLastError();
}

cudaError_t launch_bcheck(const double* a, size_t n, uint32_t R, double* sc, double* part, double rtol, double atol,
                          cudaStream_t st) {
    k_bdots<double, 1><<<kBBlocks, kBThreads, 0, st>>>(a, a, nullptr, n, R, R, part);
    k_bcheck<<<(R + 63) / 64, 64, 0, st>>>(sc, part, R, rtol, atol);
    return cudaGetLastError();
}

cudaError_t launch_breliable(const double* r64, float* r, float* z, float* p, const float* dinv, size_t n, uint32_t R,
                             double* sc, double* part, double inner_rtol, cudaStream_t st) {
    k_breliable<<<kBBlocks, kBThreads, 0, st>>>(r64, r, z, p, dinv, n, R, part);
    k_breliable_final<<<(R + 63) / 64, 64, 0, st>>>(sc, part, R, inner_rtol);
    k_breliable_p<<<grid_for(n * R), kBThreads, 0, st>>>(p, z, n, R, sc);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_bnorm2(const T* a, size_t n, uint32_t ld, uint32_t R, double* out_part, cudaStream_t st) {
    k_bdots<T, 1><<<kBBlocks, kBThreads, 0, st>>>(a, a, nullptr, n, ld, R, out_part);
    return cudaGetLastError();
}

#define AFM_BATCHED_INSTANCES(T)                                                                                    \
    template cudaError_t launch_bset_constrained<T>(T*, const T*, const uint32_t*, uint32_t, uint32_t, uint32_t,    \
                                                    cudaStream_t);                                                  \
    template cudaError_t launch_bcg_init<T>(const T*, const T*, const T*, T*, T*, T*, size_t, uint32_t, uint32_t,   \
                                            double*, double*, double, double, cudaStream_t);                        \
    template cudaError_t launch_bcg_step_scalars<T>(const T*, const T*, size_t, uint32_t, uint32_t, double*,        \
                                                    double*, cudaStream_t);                                         \
    template cudaError_t launch_bcg_update<T>(T*, T*, T*, T*, const T*, const T*, size_t, uint32_t, uint32_t,       \
                                              double*, double*, double, unsigned int*, cudaStream_t);               \
    template cudaError_t launch_bnorm2<T>(const T*, size_t, uint32_t, uint32_t, double*, cudaStream_t);

AFM_BATCHED_INSTANCES(double)
AFM_BATCHED_INSTANCES(float)

}  // namespace afm
