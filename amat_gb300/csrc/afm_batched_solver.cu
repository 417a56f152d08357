// Batched Jacobi-PCG: one CG per right-hand side, all advanced in lockstep
// over n_dofs x ld blocks (column j of every block belongs to solve j).
// Every column has its own FP64 scalars (rz, alpha, beta, norms, done flag);
// a finished column is frozen (alpha = beta = 0) while the others continue.
// Column reductions are deterministic: a fixed grid of kBBlocks row chunks, a
// fixed in-block order, then a fixed tree over the block partials per column.
// Every thread moves 16 bytes of one row per access.
#include <cuda_runtime.h>
#include <stdint.h>

#include "afm_batched_solver.hpp"

namespace afm {

namespace {

constexpr int kBThreads = 256;
constexpr int kFinThreads = 128;

// Thread geometry of the row-chunk kernels: block b owns a contiguous chunk
// of rows; a thread owns VEC = 16 / sizeof(T) consecutive columns (one 16-byte
// access), tpr = R / VEC threads cover a row and rstep = kBThreads / tpr rows
// are in flight per pass.
template <typename T>
struct Geo {
    static constexpr uint32_t VEC = 16 / sizeof(T);
    uint32_t tpr, rstep, ry, col;
    bool active;
    size_t r0, r1;
    __device__ Geo(size_t n, uint32_t R) {
        tpr = R / VEC;
        rstep = kBThreads / tpr;
        ry = threadIdx.x / tpr;
        col = (threadIdx.x % tpr) * VEC;
        active = ry < rstep;
        const size_t chunk = (n + gridDim.x - 1) / gridDim.x;
        r0 = (size_t)blockIdx.x * chunk;
        r1 = r0 + chunk < n ? r0 + chunk : n;
    }
};

template <typename T>
__device__ __forceinline__ void ldv(const T* p, T* x) {
    if constexpr (sizeof(T) == 4) {
        const float4 t = *reinterpret_cast<const float4*>(p);
        x[0] = t.x, x[1] = t.y, x[2] = t.z, x[3] = t.w;
    } else {
        const double2 t = *reinterpret_cast<const double2*>(p);
        x[0] = t.x, x[1] = t.y;
    }
}
template <typename T>
__device__ __forceinline__ void stv(T* p, const T* x) {
    if constexpr (sizeof(T) == 4)
        *reinterpret_cast<float4*>(p) = make_float4(x[0], x[1], x[2], x[3]);
    else
        *reinterpret_cast<double2*>(p) = make_double2(x[0], x[1]);
}

// Column sums of the block for Q quantities (acc[q][v] of this thread's VEC
// columns), in a fixed order over the block's rows; block partials at
// part[(q * gridDim.x + block) * R + column].
template <typename T, int Q>
__device__ __forceinline__ void block_cols(const double (&acc)[Q][16 / sizeof(T)], const Geo<T>& g, uint32_t R,
                                           double* part, double* sh) {
    constexpr uint32_t VEC = Geo<T>::VEC;
#pragma unroll
    for (int q = 0; q < Q; q++) {
        if (g.active)
#pragma unroll
            for (uint32_t v = 0; v < VEC; v++) sh[g.ry * R + g.col + v] = acc[q][v];
        __syncthreads();
        if (g.active && g.ry == 0)
#pragma unroll
            for (uint32_t v = 0; v < VEC; v++) {
                double s = 0.0;
                for (uint32_t y = 0; y < g.rstep; y++) s += sh[y * R + g.col + v];
                part[((size_t)q * gridDim.x + blockIdx.x) * R + g.col + v] = s;
            }
        __syncthreads();
    }
}

// Sum over the nb block partials of quantity q, column j (one block per
// column, fixed tree); valid in thread 0.
__device__ __forceinline__ double col_total(const double* part, uint32_t q, uint32_t j, uint32_t R, uint32_t nb,
                                            double* sh) {
    double s = 0.0;
    for (uint32_t b = threadIdx.x; b < nb; b += kFinThreads) s += part[((size_t)q * nb + b) * R + j];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int w = kFinThreads / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
        __syncthreads();
    }
    const double r = sh[0];
    __syncthreads();
    return r;
}

// per column a.b (a == b: squared norms)
template <typename T>
__global__ void __launch_bounds__(kBThreads) k_bdots(const T* __restrict__ a, const T* __restrict__ b, size_t n,
                                                     uint32_t ld, uint32_t R, double* part) {
    __shared__ double sh[kBThreads * 4];
    const Geo<T> g(n, R);
    constexpr uint32_t VEC = Geo<T>::VEC;
    double acc[1][VEC] = {};
    if (g.active)
        for (size_t i = g.r0 + g.ry; i < g.r1; i += g.rstep) {
            T x[VEC], y[VEC];
            ldv(a + i * ld + g.col, x);
            ldv(b + i * ld + g.col, y);
#pragma unroll
            for (uint32_t v = 0; v < VEC; v++) acc[0][v] = __fma_rn((double)x[v], (double)y[v], acc[0][v]);
        }
    block_cols<T, 1>(acc, g, R, part, sh);
}

// init: r = b - q, z = dinv r, p = z; per column rz, rr, bb
template <typename T>
__global__ void __launch_bounds__(kBThreads) k_binit(const T* __restrict__ b, const T* __restrict__ q,
                                                     const T* __restrict__ dinv, T* __restrict__ r, T* __restrict__ z,
                                                     T* __restrict__ p, size_t n, uint32_t ld, uint32_t R,
                                                     double* part) {
    __shared__ double sh[kBThreads * 4];
    const Geo<T> g(n, R);
    constexpr uint32_t VEC = Geo<T>::VEC;
    double acc[3][VEC] = {};
    if (g.active)
        for (size_t i = g.r0 + g.ry; i < g.r1; i += g.rstep) {
            const size_t k = i * ld + g.col;
            T bi[VEC], qi[VEC], ri[VEC], zi[VEC];
            ldv(b + k, bi);
            ldv(q + k, qi);
            const T di = dinv[i];
#pragma unroll
            for (uint32_t v = 0; v < VEC; v++) {
                ri[v] = bi[v] - qi[v];
                zi[v] = di * ri[v];
                acc[0][v] = __fma_rn((double)ri[v], (double)zi[v], acc[0][v]);
                acc[1][v] = __fma_rn((double)ri[v], (double)ri[v], acc[1][v]);
                acc[2][v] = __fma_rn((double)bi[v], (double)bi[v], acc[2][v]);
            }
            stv(r + k, ri);
            stv(z + k, zi);
            stv(p + k, zi);
        }
    block_cols<T, 3>(acc, g, R, part, sh);
}

// scalars: sc[j * kBSlots + slot]; one block per column
__global__ void __launch_bounds__(kFinThreads) k_binit_final(double* sc, const double* part, uint32_t R, uint32_t nb,
                                                             double rtol, double atol) {
    __shared__ double sh[kFinThreads];
    const uint32_t j = blockIdx.x;
    const double rz = col_total(part, 0, j, R, nb, sh);
    const double rr = col_total(part, 1, j, R, nb, sh);
    const double bb = col_total(part, 2, j, R, nb, sh);
    if (threadIdx.x) return;
    double* c = sc + (size_t)j * kBSlots;
    c[B_RZ] = rz;
    c[B_RR] = rr;
    c[B_BB] = bb;
    c[B_ITER] = 0.0;
    c[B_FLAG] = (rz < 0.0 || rz != rz) ? 1.0 : 0.0;
    c[B_TOL] = fmax(rtol * sqrt(bb), atol);
    c[B_DONE] = (c[B_FLAG] != 0.0 || sqrt(rr) <= c[B_TOL]) ? 1.0 : 0.0;
}

__global__ void __launch_bounds__(kFinThreads) k_balpha(double* sc, const double* part, uint32_t R, uint32_t nb) {
    __shared__ double sh[kFinThreads];
    const uint32_t j = blockIdx.x;
    const double pq = col_total(part, 0, j, R, nb, sh);
    if (threadIdx.x) return;
    double* c = sc + (size_t)j * kBSlots;
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
    __shared__ double sh[kBThreads * 4];
    const Geo<T> g(n, R);
    constexpr uint32_t VEC = Geo<T>::VEC;
    double acc[2][VEC] = {};
    if (g.active) {
        T alpha[VEC];
#pragma unroll
        for (uint32_t v = 0; v < VEC; v++) alpha[v] = (T)sc[(size_t)(g.col + v) * kBSlots + B_ALPHA];
        for (size_t i = g.r0 + g.ry; i < g.r1; i += g.rstep) {
            const size_t k = i * ld + g.col;
            T xi[VEC], ri[VEC], pi[VEC], qi[VEC], zi[VEC];
            ldv(x + k, xi);
            ldv(r + k, ri);
            ldv(p + k, pi);
            ldv(q + k, qi);
            const T di = dinv[i];
#pragma unroll
            for (uint32_t v = 0; v < VEC; v++) {
                xi[v] = alpha[v] * pi[v] + xi[v];
                ri[v] = -alpha[v] * qi[v] + ri[v];
                zi[v] = di * ri[v];
                acc[0][v] = __fma_rn((double)ri[v], (double)zi[v], acc[0][v]);
                acc[1][v] = __fma_rn((double)ri[v], (double)ri[v], acc[1][v]);
            }
            stv(x + k, xi);
            stv(r + k, ri);
            stv(z + k, zi);
        }
    }
    block_cols<T, 2>(acc, g, R, part, sh);
}

__global__ void __launch_bounds__(kFinThreads) k_bbeta(double* sc, const double* part, uint32_t R, uint32_t nb,
                                                       double maxit, unsigned int* remaining) {
    __shared__ double sh[kFinThreads];
    const uint32_t j = blockIdx.x;
    const double rz = col_total(part, 0, j, R, nb, sh);
    const double rr = col_total(part, 1, j, R, nb, sh);
    if (threadIdx.x) return;
    double* c = sc + (size_t)j * kBSlots;
    if (c[B_DONE] != 0.0) {
        c[B_BETA] = 0.0;
        return;
    }
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

// p = beta p + z per column; a finished column keeps its last direction
template <typename T>
__global__ void __launch_bounds__(kBThreads) k_bp(T* __restrict__ p, const T* __restrict__ z, size_t n, uint32_t ld,
                                                  uint32_t R, const double* sc) {
    const Geo<T> g(n, R);
    constexpr uint32_t VEC = Geo<T>::VEC;
    if (!g.active) return;
    T beta[VEC];
    bool run[VEC], any = false;
#pragma unroll
    for (uint32_t v = 0; v < VEC; v++) {
        const double* c = sc + (size_t)(g.col + v) * kBSlots;
        run[v] = c[B_DONE] == 0.0;
        beta[v] = (T)c[B_BETA];
        any = any || run[v];
    }
    if (!any) return;
    for (size_t i = g.r0 + g.ry; i < g.r1; i += g.rstep) {
        const size_t k = i * ld + g.col;
        T pi[VEC], zi[VEC];
        ldv(p + k, pi);
        ldv(z + k, zi);
#pragma unroll
        for (uint32_t v = 0; v < VEC; v++)
            if (run[v]) pi[v] = beta[v] * pi[v] + zi[v];
        stv(p + k, pi);
    }
}

__global__ void __launch_bounds__(kFinThreads) k_bstore_norm(double* sc, const double* part, uint32_t R,
                                                             uint32_t nb) {
    __shared__ double sh[kFinThreads];
    const uint32_t j = blockIdx.x;
    const double s = col_total(part, 0, j, R, nb, sh);
    if (threadIdx.x == 0) sc[(size_t)j * kBSlots + B_BN] = sqrt(s);
}

__global__ void __launch_bounds__(kFinThreads) k_bcheck(double* sc, const double* part, uint32_t R, uint32_t nb,
                                                        double rtol, double atol) {
    __shared__ double sh[kFinThreads];
    const uint32_t j = blockIdx.x;
    const double rr = col_total(part, 0, j, R, nb, sh);
    if (threadIdx.x) return;
    double* c = sc + (size_t)j * kBSlots;
    c[B_TRR] = rr;
    c[B_CONV] = (sqrt(rr) <= fmax(rtol * c[B_BN], atol)) ? 1.0 : 0.0;
}

__global__ void __launch_bounds__(kBThreads) k_breliable(const double* __restrict__ r64, float* __restrict__ r,
                                                         float* __restrict__ z, const float* __restrict__ p,
                                                         const float* __restrict__ dinv, size_t n, uint32_t R,
                                                         double* part) {
    __shared__ double sh[kBThreads * 4];
    const Geo<float> g(n, R);
    constexpr uint32_t VEC = Geo<float>::VEC;
    double acc[3][VEC] = {};
    if (g.active)
        for (size_t i = g.r0 + g.ry; i < g.r1; i += g.rstep) {
            const size_t k = i * R + g.col;
            double t0[2], t1[2];
            ldv(r64 + k, t0);
            ldv(r64 + k + 2, t1);
            const float ri[4] = {(float)t0[0], (float)t0[1], (float)t1[0], (float)t1[1]};
            float zi[4], pi[4];
            ldv(p + k, pi);
            const float di = dinv[i];
#pragma unroll
            for (uint32_t v = 0; v < VEC; v++) {
                zi[v] = di * ri[v];
                acc[0][v] = __fma_rn((double)ri[v], (double)zi[v], acc[0][v]);
                acc[1][v] = __fma_rn((double)ri[v], (double)ri[v], acc[1][v]);
                acc[2][v] = __fma_rn((double)ri[v], (double)pi[v], acc[2][v]);
            }
            stv(r + k, ri);
            stv(z + k, zi);
        }
    block_cols<float, 3>(acc, g, R, part, sh);
}

__global__ void __launch_bounds__(kFinThreads) k_breliable_final(double* sc, const double* part, uint32_t R,
                                                                 uint32_t nb, double inner_rtol) {
    __shared__ double sh[kFinThreads];
    const uint32_t j = blockIdx.x;
    const double rz = col_total(part, 0, j, R, nb, sh);
    const double rr = col_total(part, 1, j, R, nb, sh);
    const double rp = col_total(part, 2, j, R, nb, sh);
    if (threadIdx.x) return;
    double* c = sc + (size_t)j * kBSlots;
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
    const Geo<float> g(n, R);
    constexpr uint32_t VEC = Geo<float>::VEC;
    if (!g.active) return;
    float beta[VEC], cz[VEC];
#pragma unroll
    for (uint32_t v = 0; v < VEC; v++) {
        const double* c = sc + (size_t)(g.col + v) * kBSlots;
        beta[v] = (float)c[B_BETA];
        cz[v] = (float)(1.0 - c[B_BETA] * c[B_GAMMA]);
    }
    for (size_t i = g.r0 + g.ry; i < g.r1; i += g.rstep) {
        const size_t k = i * R + g.col;
        float pi[VEC], zi[VEC];
        ldv(p + k, pi);
        ldv(z + k, zi);
#pragma unroll
        for (uint32_t v = 0; v < VEC; v++) pi[v] = __fmaf_rn(beta[v], pi[v], cz[v] * zi[v]);
        stv(p + k, pi);
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
    k_binit_final<<<R, kFinThreads, 0, st>>>(sc, part, R, kBBlocks, rtol, atol);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_bcg_step_scalars(const T* p, const T* q, size_t n, uint32_t ld, uint32_t R, double* sc,
                                    double* part, cudaStream_t st) {
    k_bdots<T><<<kBBlocks, kBThreads, 0, st>>>(p, q, n, ld, R, part);
    k_balpha<<<R, kFinThreads, 0, st>>>(sc, part, R, kBBlocks);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_bcg_update(T* x, T* r, T* z, T* p, const T* q, const T* dinv, size_t n, uint32_t ld, uint32_t R,
                              double* sc, double* part, double maxit, unsigned int* remaining, cudaStream_t st) {
    k_bupdate<T><<<kBBlocks, kBThreads, 0, st>>>(x, r, z, p, q, dinv, n, ld, R, sc, part);
    cudaMemsetAsync(remaining, 0, sizeof(unsigned int), st);
    k_bbeta<<<R, kFinThreads, 0, st>>>(sc, part, R, kBBlocks, maxit, remaining);
    k_bp<T><<<kBBlocks, kBThreads, 0, st>>>(p, z, n, ld, R, sc);
    return cudaGetLastError();
}

cudaError_t launch_bstore_norm(const double* a, size_t n, uint32_t R, double* sc, double* part, cudaStream_t st) {
    k_bdots<double><<<kBBlocks, kBThreads, 0, st>>>(a, a, n, R, R, part);
    k_bstore_norm<<<R, kFinThreads, 0, st>>>(sc, part, R, kBBlocks);
    return cudaGetLastError();
}

cudaError_t launch_bcheck(const double* a, size_t n, uint32_t R, double* sc, double* part, double rtol, double atol,
                          cudaStream_t st) {
    k_bdots<double><<<kBBlocks, kBThreads, 0, st>>>(a, a, n, R, R, part);
    k_bcheck<<<R, kFinThreads, 0, st>>>(sc, part, R, kBBlocks, rtol, atol);
    return cudaGetLastError();
}

cudaError_t launch_breliable(const double* r64, float* r, float* z, float* p, const float* dinv, size_t n, uint32_t R,
                             double* sc, double* part, double inner_rtol, cudaStream_t st) {
    k_breliable<<<kBBlocks, kBThreads, 0, st>>>(r64, r, z, p, dinv, n, R, part);
    k_breliable_final<<<R, kFinThreads, 0, st>>>(sc, part, R, kBBlocks, inner_rtol);
    k_breliable_p<<<kBBlocks, kBThreads, 0, st>>>(p, z, n, R, sc);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_bnorm2(const T* a, size_t n, uint32_t ld, uint32_t R, double* out_part, cudaStream_t st) {
    k_bdots<T><<<kBBlocks, kBThreads, 0, st>>>(a, a, n, ld, R, out_part);
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
