// Vector kernels around the AFM matvec: boundary-condition wrapping of
// MatMult_mf and the Jacobi-preconditioned CG of the example drivers' solve
// (examples/include/solve.hpp:75-127), all in FP64 on the device.
//
// Reductions are deterministic: a fixed grid of kRedBlocks x kRedThreads
// threads sums fixed strided slices in index order, each block reduces in a
// fixed tree, and one block reduces the kRedBlocks partials in a fixed tree.
// The result depends only on n, never on the device or on timing.
#include <cuda_runtime.h>
#include <stdint.h>

#include "afm_solver.hpp"

namespace afm {

namespace {

__device__ __forceinline__ double block_sum(double x, double* sh) {
    const int t = threadIdx.x;
    sh[t] = x;
    __syncthreads();
    for (int s = kRedThreads / 2; s > 0; s >>= 1) {
        if (t < s) sh[t] += sh[t + s];
        __syncthreads();
    }
    const double r = sh[0];
    __syncthreads();
    return r;
}

__global__ void __launch_bounds__(kRedThreads) k_set_constrained(double* v, const double* u, const uint32_t* idx,
                                                                 uint32_t n) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) v[idx[k]] = u[idx[k]];
}

__global__ void __launch_bounds__(kRedThreads) k_scatter_values(double* v, const double* vals, const uint32_t* idx,
                                                                uint32_t n) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) v[idx[k]] = vals[k];
}

// part[j*kRedBlocks + block] = partial sums of the requested products
// (which: bit0 a.b, bit1 a.a, bit2 b.b).
__global__ void __launch_bounds__(kRedThreads) k_dots(const double* __restrict__ a, const double* __restrict__ b,
                                                      size_t n, double* part) {
    __shared__ double sh[kRedThreads];
    double ab = 0.0, aa = 0.0, bb = 0.0;
    const size_t stride = (size_t)kRedBlocks * kRedThreads;
    for (size_t i = (size_t)blockIdx.x * kRedThreads + threadIdx.x; i < n; i += stride) {
        const double x = a[i], y = b[i];
        ab = __fma_rn(x, y, ab);
        aa = __fma_rn(x, x, aa);
        bb = __fma_rn(y, y, bb);
    }
    ab = block_sum(ab, sh);
    aa = block_sum(aa, sh);
    bb = block_sum(bb, sh);
    if (threadIdx.x == 0) {
        part[blockIdx.x] = ab;
        part[kRedBlocks + blockIdx.x] = aa;
        part[2 * kRedBlocks + blockIdx.x] = bb;
    }
}

__device__ __forceinline__ double final_sum(const double* part, double* sh) {
    double s = 0.0;
    for (int i = threadIdx.x; i < kRedBlocks; i += kRedThreads) s += part[i];
    return block_sum(s, sh);
}

// r = b - q, z = dinv r, p = z; partials of r.z, r.r, z.z, b.b, (dinv b).(dinv b)
__global__ void __launch_bounds__(kRedThreads) k_cg_init(const double* __restrict__ b, const double* __restrict__ q,
                                                         const double* __restrict__ dinv, double* __restrict__ r,
                                                         double* __restrict__ z, double* __restrict__ p, size_t n,
                                                         double* part) {
    __shared__ double sh[kRedThreads];
    double rz = 0, rr = 0, zz = 0, bb = 0, db = 0;
    const size_t stride = (size_t)kRedBlocks * kRedThreads;
    for (size_t i = (size_t)blockIdx.x * kRedThreads + threadIdx.x; i < n; i += stride) {
        const double bi = b[i], di = dinv[i];
        const double ri = bi - q[i];
        const double zi = di * ri;
        r[i] = ri;
        z[i] = zi;
        p[i] = zi;
        rz = __fma_rn(ri, zi, rz);
        rr = __fma_rn(ri, ri, rr);
        zz = __fma_rn(zi, zi, zz);
        bb = __fma_rn(bi, bi, bb);
        const double t = di * bi;
        db = __fma_rn(t, t, db);
    }
    double v[5] = {rz, rr, zz, bb, db};
    for (int j = 0; j < 5; j++) {
        const double s = block_sum(v[j], sh);
        if (threadIdx.x == 0) part[j * kRedBlocks + blockIdx.x] = s;
    }
}

__global__ void __launch_bounds__(kRedThreads) k_cg_init_final(double* sc, const double* part) {
    __shared__ double sh[kRedThreads];
    const double rz = final_sum(part, sh);
    const double rr = final_sum(part + kRedBlocks, sh);
    const double zz = final_sum(part + 2 * kRedBlocks, sh);
    const double bb = final_sum(part + 3 * kRedBlocks, sh);
    const double db = final_sum(part + 4 * kRedBlocks, sh);
    if (threadIdx.x == 0) {
        sc[S_RZ] = rz;
        sc[S_RR] = rr;
        sc[S_ZZ] = zz;
        sc[S_BB] = bb;
        sc[S_DB] = db;
        sc[S_FLAG] = (rz < 0.0 || rz != rz) ? 1.0 : 0.0;
    }
}

// alpha = rz / (p.q); flag on p.q <= 0 or NaN
__global__ void __launch_bounds__(kRedThreads) k_cg_alpha(double* sc, const double* part) {
    __shared__ double sh[kRedThreads];
    const double pq = final_sum(part, sh);
    if (threadIdx.x == 0) {
        sc[S_PQ] = pq;
        if (!(pq > 0.0)) {
            sc[S_FLAG] = 1.0;
            sc[S_ALPHA] = 0.0;
        } else {
            sc[S_ALPHA] = sc[S_RZ] / pq;
        }
    }
}

// x += alpha p, r -= alpha q, z = dinv r; partials of r.z, r.r, z.z
__global__ void __launch_bounds__(kRedThreads) k_cg_update(double* __restrict__ x, double* __restrict__ r,
                                                           double* __restrict__ z, const double* __restrict__ p,
                                                           const double* __restrict__ q,
                                                           const double* __restrict__ dinv, size_t n,
                                                           const double* sc, double* part) {
    __shared__ double sh[kRedThreads];
    const double alpha = sc[S_ALPHA];
    double rz = 0, rr = 0, zz = 0;
    const size_t stride = (size_t)kRedBlocks * kRedThreads;
    for (size_t i = (size_t)blockIdx.x * kRedThreads + threadIdx.x; i < n; i += stride) {
        x[i] = __fma_rn(alpha, p[i], x[i]);
        const double ri = __fma_rn(-alpha, q[i], r[i]);
        const double zi = dinv[i] * ri;
        r[i] = ri;
        z[i] = zi;
        rz = __fma_rn(ri, zi, rz);
        rr = __fma_rn(ri, ri, rr);
        zz = __fma_rn(zi, zi, zz);
    }
    rz = block_sum(rz, sh);
    rr = block_sum(rr, sh);
    zz = block_sum(zz, sh);
    if (threadIdx.x == 0) {
        part[blockIdx.x] = rz;
        part[kRedBlocks + blockIdx.x] = rr;
        part[2 * kRedBlocks + blockIdx.x] = zz;
    }
}

// beta = rz_new / rz
__global__ void __launch_bounds__(kRedThreads) k_cg_beta(double* sc, const double* part) {
    __shared__ double sh[kRedThreads];
    const double rz = final_sum(part, sh);
    const double rr = final_sum(part + kRedBlocks, sh);
    const double zz = final_sum(part + 2 * kRedBlocks, sh);
    if (threadIdx.x == 0) {
        const double old = sc[S_RZ];
        sc[S_BETA] = (old != 0.0) ? rz / old : 0.0;
        sc[S_RZ] = rz;
        sc[S_RR] = rr;
        sc[S_ZZ] = zz;
        if (rz < 0.0 || rz != rz) sc[S_FLAG] = 1.0;
    }
}

__global__ void __launch_bounds__(kRedThreads) k_cg_p(double* __restrict__ p, const double* __restrict__ z, size_t n,
                                                      const double* sc) {
    const double beta = sc[S_BETA];
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
        p[i] = __fma_rn(beta, p[i], z[i]);
}

__global__ void __launch_bounds__(kRedThreads) k_invert(double* __restrict__ dinv, const double* __restrict__ d,
                                                        size_t n) {
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) dinv[i] = 1.0 / d[i];
}

__global__ void __launch_bounds__(kRedThreads) k_axpby(double* __restrict__ y, const double* __restrict__ x,
                                                       double a, double b, size_t n) {
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
        y[i] = __fma_rn(a, x[i], b * y[i]);
}

inline unsigned grid_for(size_t n) {
    size_t g = (n + kRedThreads - 1) / kRedThreads;
    if (g > 4096) g = 4096;
    if (g == 0) g = 1;
    return (unsigned)g;
}

}  // namespace

cudaError_t launch_set_constrained(double* v, const double* u, const uint32_t* idx, uint32_t n, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    k_set_constrained<<<(n + kRedThreads - 1) / kRedThreads, kRedThreads, 0, st>>>(v, u, idx, n);
    return cudaGetLastError();
}

cudaError_t launch_scatter_values(double* v, const double* vals, const uint32_t* idx, uint32_t n, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    k_scatter_values<<<(n + kRedThreads - 1) / kRedThreads, kRedThreads, 0, st>>>(v, vals, idx, n);
    return cudaGetLastError();
}

cudaError_t launch_dots(const double* a, const double* b, size_t n, double* part, cudaStream_t st) {
    k_dots<<<kRedBlocks, kRedThreads, 0, st>>>(a, b, n, part);
    return cudaGetLastError();
}

cudaError_t launch_cg_init(const double* b, const double* q, const double* dinv, double* r, double* z, double* p,
                           size_t n, double* sc, double* part, cudaStream_t st) {
    k_cg_init<<<kRedBlocks, kRedThreads, 0, st>>>(b, q, dinv, r, z, p, n, part);
    k_cg_init_final<<<1, kRedThreads, 0, st>>>(sc, part);
    return cudaGetLastError();
}

cudaError_t launch_cg_alpha(const double* p, const double* q, size_t n, double* sc, double* part, cudaStream_t st) {
    k_dots<<<kRedBlocks, kRedThreads, 0, st>>>(p, q, n, part);
    k_cg_alpha<<<1, kRedThreads, 0, st>>>(sc, part);
    return cudaGetLastError();
}

cudaError_t launch_cg_update(double* x, double* r, double* z, double* p, const double* q, const double* dinv,
                             size_t n, double* sc, double* part, cudaStream_t st) {
    k_cg_update<<<kRedBlocks, kRedThreads, 0, st>>>(x, r, z, p, q, dinv, n, sc, part);
    k_cg_beta<<<1, kRedThreads, 0, st>>>(sc, part);
    k_cg_p<<<grid_for(n), kRedThreads, 0, st>>>(p, z, n, sc);
    return cudaGetLastError();
}

cudaError_t launch_invert(double* dinv, const double* d, size_t n, cudaStream_t st) {
    k_invert<<<grid_for(n), kRedThreads, 0, st>>>(dinv, d, n);
    return cudaGetLastError();
}

cudaError_t launch_axpby(double* y, const double* x, double a, double b, size_t n, cudaStream_t st) {
    k_axpby<<<grid_for(n), kRedThreads, 0, st>>>(y, x, a, b, n);
    return cudaGetLastError();
}

}  // namespace afm
