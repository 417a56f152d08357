// Vector kernels around the AFM matvec: boundary-condition wrapping of
// MatMult_mf and the Jacobi-preconditioned CG of the example drivers' solve
// (examples/include/solve.hpp:75-127). Vectors are T = double (the FP64 CG)
// or T = float (the inner CG of the mixed-precision solve); every dot product
// and step scalar is accumulated and held in FP64.
//
// Reductions are deterministic: a grid of nb = red_blocks(n) x kRedThreads
// threads sums fixed strided slices in index order, each block reduces in a
// fixed tree, and one block reduces the nb partials in a fixed tree. The
// result depends only on n, never on the device or on timing. (nb grows with
// n up to kRedBlocks, so a small solve occupies few SMs.)
#include <cuda_runtime.h>
#include <stdint.h>

#include "afm_solver.hpp"
#include "afm_internal.hpp"

namespace afm {

namespace {

// Sum over the block in a fixed tree: shuffles within each warp, then over
// the warps' sums (sh holds at least 33 doubles).
__device__ __forceinline__ double block_sum(double x, double* sh) {
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) sh[w] = x;
    __syncthreads();
    if (w == 0) {
        double r = lane < kRedThreads / 32 ? sh[lane] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) r += __shfl_down_sync(0xffffffffu, r, o);
        if (lane == 0) sh[32] = r;
    }
    __syncthreads();
    const double r = sh[32];
    __syncthreads();
    return r;
}

__device__ __forceinline__ double final_sum(const double* part, double* sh, uint32_t nb) {
    double s = 0.0;
    for (uint32_t i = threadIdx.x; i < nb; i += kRedThreads) s += part[i];
    return block_sum(s, sh);
}

#define kStride ((size_t)gridDim.x * kRedThreads)

// Dot-product accumulators of one thread. FP64 vectors: FP64 fused
// multiply-adds. FP32 vectors: compensated FP32 arithmetic (Ogita, Rump &
// Oishi, "Accurate sum and dot product", 2005, Dot2: TwoProduct by FMA and
// TwoSum, about twice FP32 precision per thread), which keeps the FP32
// recursion off GB300's FP64 pipe (1/64 of the FP32 rate). The _rn intrinsics
// keep the compiler from fusing the steps.
template <typename T>
struct DotAcc;
template <>
struct DotAcc<double> {
    double s = 0.0;
    __device__ __forceinline__ void add(double x, double y) { s = __fma_rn(x, y, s); }
    __device__ __forceinline__ double value() const { return s; }
};
template <>
struct DotAcc<float> {
    float hi = 0.0f, lo = 0.0f;
    __device__ __forceinline__ void add(float x, float y) {
        const float p = __fmul_rn(x, y);
        const float e = __fmaf_rn(x, y, -p);
        const float t = __fadd_rn(hi, p);
        const float bp = __fsub_rn(t, hi);
        const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(t, bp)), __fsub_rn(p, bp));
        hi = t;
        lo = __fadd_rn(lo, __fadd_rn(err, e));
    }
    __device__ __forceinline__ double value() const { return (double)hi + (double)lo; }
};

// Strided loops visit i = i0, i0 + stride, ... in index order; kUnroll of
// them load before any is used, so that each thread keeps several memory
// requests in flight (the order of every sum is unchanged).
constexpr int kUnroll = 4;



template <typename T>
__global__ void __launch_bounds__(kRedThreads) k_set_constrained(T* v, const T* u, const uint32_t* idx, uint32_t n) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) v[idx[k]] = u[idx[k]];
}

// part[block]: partial sums of a.b
template <typename T>
__global__ void __launch_bounds__(kRedThreads) k_dot(const T* __restrict__ a, const T* __restrict__ b, size_t n,
                                                     double* part) {
    __shared__ double sh[kRedThreads];
    DotAcc<T> ab;
    size_t i = (size_t)blockIdx.x * kRedThreads + threadIdx.x;
    for (; i + (kUnroll - 1) * kStride < n; i += kUnroll * kStride) {
        T x[kUnroll], y[kUnroll];
#pragma unroll
        for (int q = 0; q < kUnroll; q++) {
            x[q] = a[i + q * kStride];
            y[q] = b[i + q * kStride];
        }
#pragma unroll
        for (int q = 0; q < kUnroll; q++) ab.add(x[q], y[q]);
    }
    for (; i < n; i += kStride) ab.add(a[i], b[i]);
    const double s = block_sum(ab.value(), sh);
    if (threadIdx.x == 0) part[blockIdx.x] = s;
}

// r = b - q, z = dinv r, p = z; partials of r.z, r.r, z.z, b.b, (dinv b).(dinv b)
template <typename T>
__global__ void __launch_bounds__(kRedThreads) k_cg_init(const T* __restrict__ b, const T* __restrict__ q,
                                                         const T* __restrict__ dinv, T* __restrict__ r,
                                                         T* __restrict__ z, T* __restrict__ p, size_t n, double* part) {
    __shared__ double sh[kRedThreads];
    double rz = 0, rr = 0, zz = 0, bb = 0, db = 0;
    for (size_t i = (size_t)blockIdx.x * kRedThreads + threadIdx.x; i < n; i += kStride) {
        const T bi = b[i], di = dinv[i];
        const T ri = bi - q[i];
        const T zi = di * ri;
        r[i] = ri;
        z[i] = zi;
        p[i] = zi;
        rz = __fma_rn((double)ri, (double)zi, rz);
        rr = __fma_rn((double)ri, (double)ri, rr);
        zz = __fma_rn((double)zi, (double)zi, zz);
        bb = __fma_rn((double)bi, (double)bi, bb);
        const double t = (double)di * (double)bi;
        db = __fma_rn(t, t, db);
    }
    double v[5] = {rz, rr, zz, bb, db};
    for (int j = 0; j < 5; j++) {
        const double s = block_sum(v[j], sh);
        if (threadIdx.x == 0) part[j * kRedBlocks + blockIdx.x] = s;
    }
}

__global__ void __launch_bounds__(kRedThreads) k_cg_init_final(double* sc, const double* part, uint32_t nb) {
    __shared__ double sh[kRedThreads];
    const double rz = final_sum(part, sh, nb);
    const double rr = final_sum(part + kRedBlocks, sh, nb);
    const double zz = final_sum(part + 2 * kRedBlocks, sh, nb);
    const double bb = final_sum(part + 3 * kRedBlocks, sh, nb);
    const double db = final_sum(part + 4 * kRedBlocks, sh, nb);
    if (threadIdx.x == 0) {
        sc[S_RZ] = rz;
        sc[S_RR] = rr;
        sc[S_ZZ] = zz;
        sc[S_BB] = bb;
        sc[S_DB] = db;
        sc[S_FLAG] = (rz < 0.0 || rz != rz) ? 1.0 : 0.0;
        sc[S_DONE] = 0.0;
        sc[S_ITER] = 0.0;
    }
}

// Reliable update of the FP32 recursion of the mixed-precision solve, pass 1:
// r = fl32(sigma r64) (the FP64 true residual in the new segment's scale),
// z = dinv r; partials of r.z, r.r, z.z and r.p (p = the last direction p_k,
// still in the previous segment's scale)
template <typename T>
__global__ void __launch_bounds__(kRedThreads) k_cg_reliable(const double* __restrict__ r64, T* __restrict__ r,
                                                             T* __restrict__ z, const T* __restrict__ p,
                                                             const T* __restrict__ dinv, size_t n, double* part,
                                                             double sigma) {
    __shared__ double sh[kRedThreads];
    double rz = 0, rr = 0, zz = 0, rp = 0;
    for (size_t i = (size_t)blockIdx.x * kRedThreads + threadIdx.x; i < n; i += kStride) {
        const T ri = (T)(r64[i] * sigma);
        const T zi = dinv[i] * ri;
        r[i] = ri;
        z[i] = zi;
        rz = __fma_rn((double)ri, (double)zi, rz);
        rr = __fma_rn((double)ri, (double)ri, rr);
        zz = __fma_rn((double)zi, (double)zi, zz);
        rp = __fma_rn((double)ri, (double)p[i], rp);
    }
    double v[4] = {rz, rr, zz, rp};
    for (int j = 0; j < 4; j++) {
        const double s = block_sum(v[j], sh);
        if (threadIdx.x == 0) part[j * kRedBlocks + blockIdx.x] = s;
    }
}

// pass 2 (one block): beta = r.z / (rho r_k.z_k), gamma = r.p / r.z; S_DONE,
// S_ITER cleared. rho = sigma_new / sigma_old, the change of the residual's
// scale: with r, z in the new scale and p, r_k.z_k in the old one,
// p = z + beta (p - gamma z) is the scaled form of the unscaled update.
__global__ void __launch_bounds__(kRedThreads) k_cg_reliable_final(double* sc, const double* part, uint32_t nb,
                                                                   double rho) {
    __shared__ double sh[kRedThreads];
    const double rz = final_sum(part, sh, nb);
    const double rr = final_sum(part + kRedBlocks, sh, nb);
    const double zz = final_sum(part + 2 * kRedBlocks, sh, nb);
    const double rp = final_sum(part + 3 * kRedBlocks, sh, nb);
    if (threadIdx.x == 0) {
        const double old = sc[S_RZOLD];
        const bool bad = (rz < 0.0 || rz != rz);
        sc[S_BETA] = (!bad && old > 0.0) ? rz / (old * rho) : 0.0;
        sc[S_GAMMA] = (!bad && rz > 0.0) ? rp / rz : 0.0;
        sc[S_RZ] = rz;
        sc[S_RR] = rr;
        sc[S_ZZ] = zz;
        sc[S_FLAG] = bad ? 1.0 : 0.0;
        sc[S_DONE] = 0.0;
        sc[S_ITER] = 0.0;
    }
}

// pass 3: p = z + beta (p - gamma z)
__device__ __forceinline__ float fma_rn(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double fma_rn(double a, double b, double c) { return __fma_rn(a, b, c); }

template <typename T>
__global__ void __launch_bounds__(kRedThreads) k_cg_reliable_p(T* __restrict__ p, const T* __restrict__ z,
                                                               size_t n, const double* sc) {
    const T beta = (T)sc[S_BETA];
    const T c = (T)(1.0 - sc[S_BETA] * sc[S_GAMMA]);
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
        p[i] = fma_rn(beta, p[i], c * z[i]);
}

// alpha = rz / (p.q); flag on p.q <= 0 or NaN
__global__ void __launch_bounds__(kRedThreads) k_cg_alpha(double* sc, const double* part, uint32_t nb) {
    __shared__ double sh[kRedThreads];
    const double pq = final_sum(part, sh, nb);
    if (threadIdx.x == 0) {
        if (sc[S_DONE] != 0.0) {  // finished earlier: this iteration changes nothing
            sc[S_ALPHA] = 0.0;
            return;
        }
        sc[S_PQ] = pq;
        if (!(pq > 0.0)) {
            sc[S_FLAG] = 1.0;
            sc[S_DONE] = 1.0;
            sc[S_ALPHA] = 0.0;
        } else {
            sc[S_ALPHA] = sc[S_RZ] / pq;
        }
    }
}

// sc[S_PQ] = sum of the partials (a plain reduction, no CG bookkeeping)
__global__ void __launch_bounds__(kRedThreads) k_sum(double* sc, const double* part, uint32_t nb) {
    __shared__ double sh[kRedThreads];
    const double s = final_sum(part, sh, nb);
    if (threadIdx.x == 0) sc[S_PQ] = s;
}

// x += alpha p, r -= alpha q, z = dinv r; partials of r.z, r.r, z.z
template <typename T>
__global__ void __launch_bounds__(kRedThreads) k_cg_update(T* __restrict__ x, T* __restrict__ r, T* __restrict__ z,
                                                           const T* __restrict__ p, const T* __restrict__ q,
                                                           const T* __restrict__ dinv, size_t n, const double* sc,
                                                           double* part) {
    __shared__ double sh[kRedThreads];
    const T alpha = (T)sc[S_ALPHA];
    DotAcc<T> rz, rr, zz;
    auto step = [&](size_t i, T xi, T pi, T qi, T ri0, T di) {
        x[i] = alpha * pi + xi;
        const T ri = -alpha * qi + ri0;
        const T zi = di * ri;
        r[i] = ri;
        z[i] = zi;
        rz.add(ri, zi);
        rr.add(ri, ri);
        zz.add(zi, zi);
    };
    size_t i = (size_t)blockIdx.x * kRedThreads + threadIdx.x;
    for (; i + (kUnroll - 1) * kStride < n; i += kUnroll * kStride) {
        T xv[kUnroll], pv[kUnroll], qv[kUnroll], rv[kUnroll], dv[kUnroll];
#pragma unroll
        for (int k = 0; k < kUnroll; k++) {
            const size_t j = i + k * kStride;
            xv[k] = x[j], pv[k] = p[j], qv[k] = q[j], rv[k] = r[j], dv[k] = dinv[j];
        }
#pragma unroll
        for (int k = 0; k < kUnroll; k++) step(i + k * kStride, xv[k], pv[k], qv[k], rv[k], dv[k]);
    }
    for (; i < n; i += kStride) step(i, x[i], p[i], q[i], r[i], dinv[i]);
    const double v[3] = {rz.value(), rr.value(), zz.value()};
    for (int j = 0; j < 3; j++) {
        const double t = block_sum(v[j], sh);
        if (threadIdx.x == 0) part[j * kRedBlocks + blockIdx.x] = t;
    }
}

// beta = rz_new / rz
__global__ void __launch_bounds__(kRedThreads) k_cg_beta(double* sc, const double* part, uint32_t nb) {
    __shared__ double sh[kRedThreads];
    const double rz = final_sum(part, sh, nb);
    const double rr = final_sum(part + kRedBlocks, sh, nb);
    const double zz = final_sum(part + 2 * kRedBlocks, sh, nb);
    if (threadIdx.x == 0) {
        if (sc[S_DONE] != 0.0) {
            sc[S_BETA] = 0.0;
            return;
        }
        const double old = sc[S_RZ];
        sc[S_BETA] = (old != 0.0) ? rz / old : 0.0;
        sc[S_RZOLD] = old;
        sc[S_RZ] = rz;
        sc[S_RR] = rr;
        sc[S_ZZ] = zz;
        const double it = sc[S_ITER] + 1.0;
        sc[S_ITER] = it;
        const double nrm = sqrt(sc[S_NORM] != 0.0 ? zz : rr);
        if (rz < 0.0 || rz != rz || nrm != nrm) {
            sc[S_FLAG] = 1.0;
            sc[S_DONE] = 1.0;
        } else if (nrm <= sc[S_TOL] || (sc[S_MAXIT] > 0.0 && it >= sc[S_MAXIT])) {
            sc[S_DONE] = 1.0;
        }
    }
}

template <typename T>
__global__ void __launch_bounds__(kRedThreads) k_cg_p(T* __restrict__ p, const T* __restrict__ z, size_t n,
                                                      const double* sc) {
    // a finished solve keeps its last direction (the mixed-precision solve
    // continues from it after a reliable update)
    if (sc[S_DONE] != 0.0) return;
    const T beta = (T)sc[S_BETA];
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) p[i] = beta * p[i] + z[i];
}

template <typename T>
__global__ void __launch_bounds__(kRedThreads) k_invert(T* __restrict__ dinv, const double* __restrict__ d,
                                                        size_t n) {
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) dinv[i] = (T)(1.0 / d[i]);
}

__global__ void __launch_bounds__(kRedThreads) k_axpby(double* __restrict__ y, const double* __restrict__ x,
                                                       double a, double b, size_t n) {
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
        y[i] = __fma_rn(a, x[i], b * y[i]);
}

// out = (T)(scale in64) (scale a power of two: exact before the rounding)
template <typename T>
__global__ void __launch_bounds__(kRedThreads) k_to_f32(T* __restrict__ out, const double* __restrict__ in,
                                                        size_t n, double scale) {
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) out[i] = (T)(in[i] * scale);
}

// x64 += inv d, d = 0 (inv a power of two)
template <typename T>
__global__ void __launch_bounds__(kRedThreads) k_add_f32(double* __restrict__ x, T* __restrict__ d, size_t n,
                                                         double inv) {
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        x[i] += (double)d[i] * inv;
        d[i] = (T)0;
    }
}

// |x| as the bits of a non-negative double: ordered like the values, with
// NaN above infinity, so that an integer max propagates both.
__device__ __forceinline__ unsigned long long abs_bits(double x) {
    return (unsigned long long)__double_as_longlong(x) & 0x7fffffffffffffffull;
}

__device__ __forceinline__ unsigned long long warp_max(unsigned long long m) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long y = __shfl_down_sync(0xffffffffu, m, o);
        m = y > m ? y : m;
    }
    return m;
}

// w[0] = max |u[i]| over the DoFs not masked (mask[i] != 0: a constrained DoF
// that the product reads as zero), as double bits; vz[0 .. nv) = 0 on the way.
// The grid's blocks leave their maxima in w[2 + block]; the last block to
// finish (counted in the low word of w[1]) reduces them, writes w[0] and
// resets the counter, so one launch does it all and repeats cleanly inside a
// captured graph. The maximum is exact, hence independent of the order.
__global__ void __launch_bounds__(kRedThreads) k_umax(const double* __restrict__ u, const uint8_t* __restrict__ mask,
                                                      size_t n, double* __restrict__ vz, size_t nv,
                                                      unsigned long long* __restrict__ w) {
    __shared__ unsigned long long sh[kRedThreads / 32];
    __shared__ bool last;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    const size_t i0 = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long m = 0;
    for (size_t i = i0; i < n; i += stride) {
        const unsigned long long b = abs_bits(u[i]);
        if ((!mask || !mask[i]) && b > m) m = b;
    }
    if (vz)
        for (size_t i = i0; i < nv; i += stride) vz[i] = 0.0;
    m = warp_max(m);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) sh[wid] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long bm = 0;
        for (int k = 0; k < kRedThreads / 32; k++) bm = sh[k] > bm ? sh[k] : bm;
        w[2 + blockIdx.x] = bm;
        __threadfence();
        const unsigned prev = atomicAdd(reinterpret_cast<unsigned*>(w + 1), 1u);
        last = (prev == gridDim.x - 1);
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    unsigned long long r = 0;
    for (uint32_t k = threadIdx.x; k < gridDim.x; k += blockDim.x) {
        const unsigned long long b = __ldcg(w + 2 + k);
        r = b > r ? b : r;
    }
    r = warp_max(r);
    if (lane == 0) sh[wid] = r;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long bm = 0;
        for (int k = 0; k < kRedThreads / 32; k++) bm = sh[k] > bm ? sh[k] : bm;
        w[0] = bm;
        *reinterpret_cast<unsigned*>(w + 1) = 0u;
    }
}

// cm[j] = max over the unmasked rows i of |U[i ld + j]|, j < R (double bits;
// cm zeroed before the launch). Per block in shared memory, then one global
// atomic max per column.
__global__ void __launch_bounds__(kRedThreads) k_umax_cols(const double* __restrict__ U, const uint8_t* __restrict__ mask,
                                                           size_t rows, uint32_t R, uint32_t ld,
                                                           unsigned long long* __restrict__ cm) {
    __shared__ unsigned long long sm[kMaxUmaxCols];
    for (uint32_t j = threadIdx.x; j < R; j += blockDim.x) sm[j] = 0;
    __syncthreads();
    const size_t total = rows * R, stride = (size_t)gridDim.x * blockDim.x;
    for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < total; q += stride) {
        const size_t i = q / R;
        const uint32_t j = (uint32_t)(q % R);
        if (mask && mask[i]) continue;
        const unsigned long long b = abs_bits(U[i * ld + j]);
        if (b) atomicMax(sm + j, b);
    }
    __syncthreads();
    for (uint32_t j = threadIdx.x; j < R; j += blockDim.x)
        if (sm[j]) atomicMax(cm + j, sm[j]);
}

// Combine pass of one-launch patches: v[dof[i]] = the entries of shared DoF
// i in the combine buffer, summed in patch order (the first entry, then each
// next one added), one thread per shared DoF. Waits for the patch launch
// (programmatic dependence) before reading.
template <typename VO>
__global__ void __launch_bounds__(kRedThreads) k_patch_combine(VO* __restrict__ v, const VO* __restrict__ pv,
                                                               const uint32_t* __restrict__ dof,
                                                               const uint32_t* __restrict__ off,
                                                               const uint32_t* __restrict__ idx, uint32_t nb) {
    asm volatile("griddepcontrol.wait;" ::: "memory");
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nb; i += stride) {
        const uint32_t k0 = off[i], k1 = off[i + 1];
        VO s = pv[idx[k0]];
        for (uint32_t k = k0 + 1; k < k1; k++) s += pv[idx[k]];
        v[dof[i]] = s;
    }
}

inline unsigned grid_for(size_t n) {
    size_t g = (n + kRedThreads - 1) / kRedThreads;
    if (g > 4096) g = 4096;
    if (g == 0) g = 1;
    return (unsigned)g;
}

}  // namespace

template <typename T>
cudaError_t launch_set_constrained(T* v, const T* u, const uint32_t* idx, uint32_t n, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    k_set_constrained<T><<<(n + kRedThreads - 1) / kRedThreads, kRedThreads, 0, st>>>(v, u, idx, n);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_cg_init(const T* b, const T* q, const T* dinv, T* r, T* z, T* p, size_t n, double* sc,
                           double* part, cudaStream_t st) {
    const uint32_t nb = red_blocks(n);
    k_cg_init<T><<<nb, kRedThreads, 0, st>>>(b, q, dinv, r, z, p, n, part);
    k_cg_init_final<<<1, kRedThreads, 0, st>>>(sc, part, nb);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_cg_alpha(const T* p, const T* q, size_t n, double* sc, double* part, cudaStream_t st) {
    const uint32_t nb = red_blocks(n);
    k_dot<T><<<nb, kRedThreads, 0, st>>>(p, q, n, part);
    k_cg_alpha<<<1, kRedThreads, 0, st>>>(sc, part, nb);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_cg_update(T* x, T* r, T* z, T* p, const T* q, const T* dinv, size_t n, double* sc, double* part,
                             cudaStream_t st) {
    const uint32_t nb = red_blocks(n);
    k_cg_update<T><<<nb, kRedThreads, 0, st>>>(x, r, z, p, q, dinv, n, sc, part);
    k_cg_beta<<<1, kRedThreads, 0, st>>>(sc, part, nb);
    k_cg_p<T><<<grid_for(n), kRedThreads, 0, st>>>(p, z, n, sc);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_invert(T* dinv, const double* d, size_t n, cudaStream_t st) {
    k_invert<T><<<grid_for(n), kRedThreads, 0, st>>>(dinv, d, n);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_norm2(const T* a, size_t n, double* sc, double* part, cudaStream_t st) {
    const uint32_t nb = red_blocks(n);
    k_dot<T><<<nb, kRedThreads, 0, st>>>(a, a, n, part);
    k_sum<<<1, kRedThreads, 0, st>>>(sc, part, nb);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_cg_reliable(const double* r64, T* r, T* z, T* p, const T* dinv, size_t n, double* sc,
                               double* part, double sigma, double rho, cudaStream_t st) {
    const uint32_t nb = red_blocks(n);
    k_cg_reliable<T><<<nb, kRedThreads, 0, st>>>(r64, r, z, p, dinv, n, part, sigma);
    k_cg_reliable_final<<<1, kRedThreads, 0, st>>>(sc, part, nb, rho);
    k_cg_reliable_p<T><<<grid_for(n), kRedThreads, 0, st>>>(p, z, n, sc);
    return cudaGetLastError();
}
template cudaError_t launch_cg_reliable<float>(const double*, float*, float*, float*, const float*, size_t, double*,
                                               double*, double, double, cudaStream_t);
template cudaError_t launch_cg_reliable<double>(const double*, double*, double*, double*, const double*, size_t,
                                                double*, double*, double, double, cudaStream_t);

cudaError_t launch_axpby(double* y, const double* x, double a, double b, size_t n, cudaStream_t st) {
    k_axpby<<<grid_for(n), kRedThreads, 0, st>>>(y, x, a, b, n);
    return cudaGetLastError();
}

cudaError_t launch_to_f32(float* out, const double* in, size_t n, cudaStream_t st, double scale) {
    k_to_f32<float><<<grid_for(n), kRedThreads, 0, st>>>(out, in, n, scale);
    return cudaGetLastError();
}

cudaError_t launch_to_f32(double* out, const double* in, size_t n, cudaStream_t st, double scale) {
    k_to_f32<double><<<grid_for(n), kRedThreads, 0, st>>>(out, in, n, scale);
    return cudaGetLastError();
}

cudaError_t launch_add_f32(double* x, float* d, size_t n, cudaStream_t st, double inv) {
    k_add_f32<float><<<grid_for(n), kRedThreads, 0, st>>>(x, d, n, inv);
    return cudaGetLastError();
}

cudaError_t launch_add_f32(double* x, double* d, size_t n, cudaStream_t st, double inv) {
    k_add_f32<double><<<grid_for(n), kRedThreads, 0, st>>>(x, d, n, inv);
    return cudaGetLastError();
}

cudaError_t launch_patch_combine(int vo_bytes, void* v, const void* pv, const uint32_t* dof, const uint32_t* off,
                                 const uint32_t* idx, uint32_t nb, cudaStream_t st) {
    if (nb == 0) return cudaSuccess;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid_for(nb));
    cfg.blockDim = dim3(kRedThreads);
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    if (vo_bytes == 8)
        return cudaLaunchKernelEx(&cfg, k_patch_combine<double>, static_cast<double*>(v),
                                  static_cast<const double*>(pv), dof, off, idx, nb);
    return cudaLaunchKernelEx(&cfg, k_patch_combine<float>, static_cast<float*>(v), static_cast<const float*>(pv),
                              dof, off, idx, nb);
}

cudaError_t launch_umax(const double* u, const uint8_t* mask, size_t n, double* vz, size_t nv,
                        unsigned long long* w, cudaStream_t st) {
    k_umax<<<red_blocks(n > nv ? n : nv), kRedThreads, 0, st>>>(u, mask, n, vz, nv, w);
    return cudaGetLastError();
}

cudaError_t launch_umax_cols(const double* U, const uint8_t* mask, size_t rows, uint32_t R, uint32_t ld,
                             unsigned long long* cm, cudaStream_t st) {
    if (R == 0 || R > (uint32_t)kMaxUmaxCols) return cudaErrorInvalidValue;
    cudaError_t e = cudaMemsetAsync(cm, 0, sizeof(unsigned long long) * R, st);
    if (e != cudaSuccess) return e;
    k_umax_cols<<<grid_for(rows * R), kRedThreads, 0, st>>>(U, mask, rows, R, ld, cm);
    return cudaGetLastError();
}

#define AFM_SOLVER_INSTANCES(T)                                                                                       \
    template cudaError_t launch_set_constrained<T>(T*, const T*, const uint32_t*, uint32_t, cudaStream_t);            \
    template cudaError_t launch_cg_init<T>(const T*, const T*, const T*, T*, T*, T*, size_t, double*, double*,        \
                                           cudaStream_t);                                                             \
    template cudaError_t launch_cg_alpha<T>(const T*, const T*, size_t, double*, double*, cudaStream_t);              \
    template cudaError_t launch_cg_update<T>(T*, T*, T*, T*, const T*, const T*, size_t, double*, double*,            \
                                             cudaStream_t);                                                           \
    template cudaError_t launch_invert<T>(T*, const double*, size_t, cudaStream_t);                                   \
    template cudaError_t launch_norm2<T>(const T*, size_t, double*, double*, cudaStream_t);

AFM_SOLVER_INSTANCES(double)
AFM_SOLVER_INSTANCES(float)

}  // namespace afm
