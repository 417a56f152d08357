// Serving lane: one launch runs the FP32 Jacobi-PCG iterations of many served
// solves. Each request is one thread-block cluster of kLaneCtas CTAs; the
// cluster runs whole iterations on its own (q = A p colour by colour, p.q, the
// x, r, z updates with r.z, r.r, z.z, then p), separated by hardware cluster
// barriers, with the partial sums of every dot product exchanged through
// distributed shared memory. A launch of n requests replaces n x iters x
// (colours + 5) launches of the per-request path, whose small requests are
// bound by launch latency.
//
// The iteration is the one of cg_step<float> (afm_capi.cpp) and the solver
// kernels (afm_solver.cu): alpha = r.z / p.q, x += alpha p, r -= alpha q,
// z = D^-1 r, beta = r.z_new / r.z, p = z + beta p, with the same stopping
// rules on S_TOL / S_MAXIT and breakdown flags; the products read the hi
// plane of the split arena (FP32 Ke) with constrained columns as zero and
// constrained rows q = p (MatMult_mf form). Every sum runs in a fixed order
// that depends only on the request (its size and the cluster shape), never on
// the other requests of the launch or on timing, so a request's result is the
// same alone and in any mix, bit for bit.
//
// No thread waits on a flag: the only waits are the cluster barriers, which
// every thread of the cluster reaches the same number of times (the loop
// bounds and the stop decision are computed identically by all CTAs).
#include <cooperative_groups.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "afm_internal.hpp"
#include "afm_solver.hpp"

namespace cg = cooperative_groups;

namespace afm {

namespace {

constexpr uint32_t kLaneWarps = kLaneThreads / 32;
constexpr uint32_t kClusterThreads = kLaneCtas * kLaneThreads;
constexpr uint32_t kClusterWarps = kLaneCtas * kLaneWarps;

// Compensated FP32 dot accumulator (Dot2 of Ogita, Rump & Oishi, 2005), the
// arithmetic of the per-request path's FP32 dot products.
struct Dot2 {
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

__device__ __forceinline__ void bounds_error(int* err, uint32_t d, uint32_t n) {
    if (atomicOr(err, kErrBounds) == 0) {
        err[1] = 7;
        err[2] = (int)blockIdx.x;
        err[3] = (int)threadIdx.x;
        err[4] = (int)d;
        err[5] = (int)n;
        err[6] = 0;
    }
}

// One element of a warp-per-element segment (column-major Ke, entry (r, c)
// at c n + r): lane l holds rows l, l + 32, l + 64 and the same entries of u.
template <int NR>
__device__ __forceinline__ void wpe_element(const float* __restrict__ ke, const uint32_t* __restrict__ map,
                                            uint32_t n, const float* __restrict__ p, float* __restrict__ q,
                                            uint32_t n_dofs, int* err) {
    const uint32_t lane = threadIdx.x & 31;
    float u[NR], acc[NR];
    uint32_t d[NR];
#pragma unroll
    for (int k = 0; k < NR; k++) {
        const uint32_t i = lane + 32 * k;
        u[k] = 0.0f;
        acc[k] = 0.0f;
        d[k] = 0xffffffffu;
        if (i < n) {
            const uint32_t m = map[i];
            const uint32_t g = m & kDofMask;
            if (g < n_dofs) {
                d[k] = g;
                u[k] = (m & kBcFlag) ? 0.0f : p[g];
            } else {
                bounds_error(err, g, n_dofs);
            }
        }
    }
#pragma unroll
    for (int kb = 0; kb < NR; kb++) {
        const uint32_t c1 = min(n, 32u * (kb + 1));
#pragma unroll 4
        for (uint32_t c = 32u * kb; c < c1; c++) {
            const float uc = __shfl_sync(0xffffffffu, u[kb], c & 31);
            const float* col = ke + (size_t)c * n;
#pragma unroll
            for (int k = 0; k < NR; k++) {
                const uint32_t r = lane + 32 * k;
                if (r < n) acc[k] = fmaf(col[r], uc, acc[k]);
            }
        }
    }
#pragma unroll
    for (int k = 0; k < NR; k++)
        if (d[k] != 0xffffffffu) q[d[k]] += acc[k];
}

// One element slot of a thread-per-element unit (entry (r, c) of slot l at
// (r n + c) 32 + l, map entry i of slot l at i 32 + l).
__device__ __forceinline__ void tpe_slot(const float* __restrict__ ke, const uint32_t* __restrict__ map, uint32_t n,
                                         const float* __restrict__ p, float* __restrict__ q, uint32_t n_dofs,
                                         int* err) {
    const uint32_t l = threadIdx.x & 31;
    float u[kTpeMaxN];
    uint32_t d[kTpeMaxN];
    bool ok = true;
#pragma unroll
    for (uint32_t i = 0; i < kTpeMaxN; i++) {
        u[i] = 0.0f;
        d[i] = 0;
        if (i < n) {
            const uint32_t m = map[i * kTpeWidth + l];
            const uint32_t g = m & kDofMask;
            if (g < n_dofs) {
                d[i] = g;
                u[i] = (m & kBcFlag) ? 0.0f : p[g];
            } else {
                bounds_error(err, g, n_dofs);
                ok = false;
            }
        }
    }
    if (!ok) return;
#pragma unroll
    for (uint32_t r = 0; r < kTpeMaxN; r++) {
        if (r >= n) break;
        float acc = 0.0f;
        const float* row = ke + (size_t)r * n * kTpeWidth + l;
#pragma unroll
        for (uint32_t c = 0; c < kTpeMaxN; c++)
            if (c < n) acc = fmaf(row[(size_t)c * kTpeWidth], u[c], acc);
        q[d[r]] += acc;
    }
}

// Sum of up to three doubles over the CTA in a fixed tree; the results land in
// out[0 .. nv) of this CTA's shared memory (read by the cluster after a barrier).
template <int NV>
__device__ __forceinline__ void cta_sums(const double (&v)[NV], double* warp_part, double* out) {
    const uint32_t lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    double x[NV];
#pragma unroll
    for (int j = 0; j < NV; j++) {
        x[j] = v[j];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x[j] += __shfl_down_sync(0xffffffffu, x[j], o);
        if (lane == 0) warp_part[j * kLaneWarps + w] = x[j];
    }
    __syncthreads();
    if (w == 0) {
#pragma unroll
        for (int j = 0; j < NV; j++) {
            double s = lane < kLaneWarps ? warp_part[j * kLaneWarps + lane] : 0.0;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
            if (lane == 0) out[j] = s;
        }
    }
}

// Sum of slot j of every CTA's out[] in rank order (after a cluster barrier).
__device__ __forceinline__ double cluster_sum(cg::cluster_group& cl, double* out, int j) {
    double s = 0.0;
#pragma unroll
    for (uint32_t k = 0; k < kLaneCtas; k++) s += cl.map_shared_rank(out, k)[j];
    return s;
}

__global__ void __cluster_dims__(kLaneCtas, 1, 1) __launch_bounds__(kLaneThreads, 1)
    afm_lane_kernel(const LaneJob* __restrict__ jobs, uint32_t iters) {
    cg::cluster_group cl = cg::this_cluster();
    __shared__ double warp_part[3 * kLaneWarps];
    __shared__ double out[4];  // this CTA's partials: p.q | r.z, r.r, z.z
    const LaneJob J = jobs[blockIdx.x / kLaneCtas];
    const uint32_t rank = cl.block_rank();
    const uint32_t gt = rank * kLaneThreads + threadIdx.x;
    const uint32_t gw = rank * kLaneWarps + (threadIdx.x >> 5);
    const uint32_t n = J.n_dofs;
    float* __restrict__ x = J.x;
    float* __restrict__ r = J.r;
    float* __restrict__ z = J.z;
    float* __restrict__ p = J.p;
    float* __restrict__ q = J.q;
    const float* __restrict__ dinv = J.dinv;
    const uint8_t* __restrict__ bc = J.bcmask;
    const double* sc = J.sc;

    double rz = sc[S_RZ], pq = sc[S_PQ], alpha = sc[S_ALPHA], beta = sc[S_BETA], rr = sc[S_RR], zz = sc[S_ZZ];
    double rzold = sc[S_RZOLD], it = sc[S_ITER], flag = sc[S_FLAG], done = sc[S_DONE];
    const double tol = sc[S_TOL], maxit = sc[S_MAXIT], norm = sc[S_NORM];

    for (uint32_t i = gt; i < n; i += kClusterThreads) q[i] = 0.0f;
    cl.sync();

    for (uint32_t k = 0; k < iters && done == 0.0; k++) {
        // q = A p, colour by colour (elements of a colour share no DoF)
        for (uint32_t s = 0; s < J.n_segs; s++) {
            const LaneSeg S = J.segs[s];
            if (S.regime == REG_WPE) {
                for (uint32_t e = gw; e < S.count; e += kClusterWarps) {
                    const float* ke = S.ke + (size_t)e * S.unit_floats;
                    const uint32_t* mp = S.map + (size_t)e * S.n;
                    if (S.n <= 32)
                        wpe_element<1>(ke, mp, S.n, p, q, n, J.err);
                    else if (S.n <= 64)
                        wpe_element<2>(ke, mp, S.n, p, q, n, J.err);
                    else
                        wpe_element<3>(ke, mp, S.n, p, q, n, J.err);
                }
            } else {
                for (uint32_t u = gw; u < S.units; u += kClusterWarps) {
                    const uint32_t slot = u * kTpeWidth + (threadIdx.x & 31);
                    if (slot < S.count)
                        tpe_slot(S.ke + (size_t)u * S.unit_floats, S.map + (size_t)u * S.n * kTpeWidth, S.n, p, q,
                                 n, J.err);
                }
            }
            if (S.sync_after) cl.sync();
        }
        // p.q with q = p on constrained rows
        {
            Dot2 a;
            for (uint32_t i = gt; i < n; i += kClusterThreads) {
                const float pi = p[i];
                const float qi = (bc && bc[i]) ? pi : q[i];
                a.add(pi, qi);
            }
            const double v[1] = {a.value()};
            cta_sums<1>(v, warp_part, out);
        }
        cl.sync();
        const double pq_new = cluster_sum(cl, out, 0);
        if (!(pq_new > 0.0)) {
            pq = pq_new;
            flag = 1.0;
            done = 1.0;
            alpha = 0.0;
        } else {
            pq = pq_new;
            alpha = rz / pq_new;
        }
        // x += alpha p, r -= alpha q, z = D^-1 r; q cleared for the next product
        {
            const float al = (float)alpha;
            Dot2 a_rz, a_rr, a_zz;
            for (uint32_t i = gt; i < n; i += kClusterThreads) {
                const float pi = p[i];
                const float qi = (bc && bc[i]) ? pi : q[i];
                x[i] = al * pi + x[i];
                const float ri = -al * qi + r[i];
                const float zi = dinv[i] * ri;
                r[i] = ri;
                z[i] = zi;
                q[i] = 0.0f;
                a_rz.add(ri, zi);
                a_rr.add(ri, ri);
                a_zz.add(zi, zi);
            }
            const double v[3] = {a_rz.value(), a_rr.value(), a_zz.value()};
            cta_sums<3>(v, warp_part, out + 1);
        }
        cl.sync();
        const double rz_new = cluster_sum(cl, out, 1), rr_new = cluster_sum(cl, out, 2),
                     zz_new = cluster_sum(cl, out, 3);
        if (done != 0.0) {
            beta = 0.0;
        } else {
            beta = (rz != 0.0) ? rz_new / rz : 0.0;
            rzold = rz;
            rz = rz_new;
            rr = rr_new;
            zz = zz_new;
            it += 1.0;
            const double nrm = sqrt(norm != 0.0 ? zz_new : rr_new);
            if (rz_new < 0.0 || rz_new != rz_new || nrm != nrm) {
                flag = 1.0;
                done = 1.0;
            } else if (nrm <= tol || (maxit > 0.0 && it >= maxit)) {
                done = 1.0;
            }
        }
        // p = z + beta p (a finished solve keeps its last direction)
        if (done == 0.0) {
            const float be = (float)beta;
            for (uint32_t i = gt; i < n; i += kClusterThreads) p[i] = be * p[i] + z[i];
        }
        cl.sync();
    }
    if (rank == 0 && threadIdx.x == 0) {
        double* w = J.sc;
        {
            w[S_RZ] = rz;
            w[S_PQ] = pq;
            w[S_ALPHA] = alpha;
            w[S_BETA] = beta;
            w[S_RR] = rr;
            w[S_ZZ] = zz;
            w[S_RZOLD] = rzold;
            w[S_ITER] = it;
            w[S_FLAG] = flag;
            w[S_DONE] = done;
            w[S_TOL] = tol;
            w[S_MAXIT] = maxit;
            w[S_NORM] = norm;
        }
    }
    cl.sync();  // no CTA leaves while another may still read its shared memory
}

}  // namespace

cudaError_t launch_lane(const LaneJob* d_jobs, uint32_t n_jobs, uint32_t iters, cudaStream_t st) {
    if (n_jobs == 0 || iters == 0) return cudaSuccess;
    afm_lane_kernel<<<n_jobs * kLaneCtas, kLaneThreads, 0, st>>>(d_jobs, iters);
    return cudaGetLastError();
}

}  // namespace afm
