// Batched (multi right-hand side) AFM product V = K U for elements with more
// than 16 DoFs: U and V are n_dofs x ld, row-major (the R = nrhs values of one
// DoF are contiguous). Each streamed element matrix is used for all R columns:
// per element V_e (n x R) += Ke (n x n) U_e (n x R).
//
// Warp per element. Ke arrives through the TMA ring of the single-vector
// kernels (one element per slot, column-major, entry (r, c) at c n + r). The
// warp gathers U_e (n rows of R contiguous values) into its own shared
// buffer with cp.async, one element ahead (double buffer), so the gather
// overlaps the product of the previous element. Lane tile: RT rows x CT
// columns of V_e in registers; per column c of Ke the lane reads RT entries of
// Ke and CT entries of U_e from shared memory and does RT CT multiply-adds.
// The tiles of one element cover V_e once (ceil(n / RT) x R / CT tiles, dealt
// round robin to the 32 lanes). Scatter: colour-exclusive V = V_old + V_e with
// 16-byte vector loads and stores; no atomics, deterministic.
#pragma once

#include "afm_matvec.cuh"

namespace afm {

// Per-warp shared buffer (one parity): the element's map (n uint32, 16-byte
// padded) and U_e (n x R values).
__host__ __device__ inline uint32_t batch_map_bytes(uint32_t n) { return (n * 4u + 15u) & ~15u; }
__host__ __device__ inline uint32_t batch_buf_bytes(uint32_t n, uint32_t nrhs, uint32_t vt) {
    return batch_map_bytes(n) + ((n * nrhs * vt + 15u) & ~15u);
}

__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_addr(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// 16-byte vector access to CT consecutive values of a row of V
template <typename VT, int CT>
struct RowVec;
template <int CT>
struct RowVec<float, CT> {
    static __device__ __forceinline__ void load(const float* p, float* x) {
#pragma unroll
        for (int y = 0; y < CT; y += 4) {
            const float4 t = *reinterpret_cast<const float4*>(p + y);
            x[y] = t.x, x[y + 1] = t.y, x[y + 2] = t.z, x[y + 3] = t.w;
        }
    }
    static __device__ __forceinline__ void store(float* p, const float* x) {
#pragma unroll
        for (int y = 0; y < CT; y += 4) *reinterpret_cast<float4*>(p + y) = make_float4(x[y], x[y + 1], x[y + 2], x[y + 3]);
    }
};
template <int CT>
struct RowVec<double, CT> {
    static __device__ __forceinline__ void load(const double* p, double* x) {
#pragma unroll
        for (int y = 0; y < CT; y += 2) {
            const double2 t = *reinterpret_cast<const double2*>(p + y);
            x[y] = t.x, x[y + 1] = t.y;
        }
    }
    static __device__ __forceinline__ void store(double* p, const double* x) {
#pragma unroll
        for (int y = 0; y < CT; y += 2) *reinterpret_cast<double2*>(p + y) = make_double2(x[y], x[y + 1]);
    }
};

template <int NT, typename A, int RT, int CT>
__global__ void __launch_bounds__(9 * 32, 1) afm_batched_kernel(BatchArgs a, RingLayout L, uint32_t n_rt) {
    using VT = typename A::VT;
    using UT = typename A::UT;
    const uint32_t n = NT ? NT : n_rt;
    extern __shared__ __align__(128) unsigned char smem[];
    uint64_t* full = reinterpret_cast<uint64_t*>(smem + L.bars_offset());
    uint64_t* empty = full + L.stages;
    volatile int* abort = reinterpret_cast<volatile int*>(empty + L.stages);
    volatile uint32_t* tag = reinterpret_cast<volatile uint32_t*>(smem + L.tags_offset());
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t NW = L.warps, S = L.stages;

    const uint32_t per = a.units / gridDim.x, rem = a.units % gridDim.x;
    const uint32_t begin = blockIdx.x * per + min(blockIdx.x, rem);
    const uint32_t cnt = per + (blockIdx.x < rem ? 1u : 0u);

    if (threadIdx.x == 0) {
        for (uint32_t s = 0; s < S; s++) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
            tag[s] = 0xffffffffu;
        }
        *abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();

    if (warp == NW) {  // producer
        if (lane == 0) {
            const uint64_t pol = l2_evict_first_policy();
            uint32_t issued = 0;
            for (uint32_t i = 0; i < cnt; i++) {
                const uint32_t s = i % S;
                if (i >= S && !mbar_wait_abortable(&empty[s], ((i / S) - 1) & 1, abort, a.wait_ns)) break;
                tag[s] = i;
                mbar_arrive_expect_tx(&full[s], a.copy_bytes);
                bulk_load(smem + (size_t)s * L.slot_bytes, a.ke + (size_t)(begin + i) * a.unit_bytes, a.copy_bytes,
                          &full[s], pol);
                issued = i + 1;
            }
            allow_dependent_launch();
            if (*abort) atomicOr(a.err, kErrTimeout);
            drain_ring(full, S, issued);
        }
        return;
    }

    if (a.probe && blockIdx.x == 0 && warp == 0 && !probe_wait(a.probe, a.wait_ns)) *abort = 1;
    const uint32_t R = a.nrhs, ld = a.ld;
    const uint32_t ctiles = R / CT, tiles = ((n + RT - 1) / RT) * ctiles;
    constexpr uint32_t kChunk = 16 / sizeof(VT);  // values per 16-byte copy
    const uint32_t row_chunks = R / kChunk;
    const uint32_t bb = batch_buf_bytes(n, R, (uint32_t)sizeof(VT));
    unsigned char* wbuf = smem + L.ubuf_offset() + (size_t)warp * 2 * bb;
    const VT* __restrict__ U = static_cast<const VT*>(a.u);
    VT* __restrict__ V = static_cast<VT*>(a.v);

    // map and U_e of element i into buffer p (cp.async, one commit group)
    auto prefetch = [&](uint32_t i, uint32_t p) {
        unsigned char* b = wbuf + (size_t)p * bb;
        uint32_t* mp = reinterpret_cast<uint32_t*>(b);
        VT* ub = reinterpret_cast<VT*>(b + batch_map_bytes(n));
        const uint32_t* gm = a.map + (size_t)(begin + i) * n;
        for (uint32_t c = lane; c < n; c += 32) mp[c] = __ldg(gm + c);
        __syncwarp();
        for (uint32_t q = lane; q < n * row_chunks; q += 32) {
            const uint32_t c = q / row_chunks, k = q % row_chunks;
            const uint32_t row = mp[c] & kDofMask;
            VT* dst = ub + (size_t)c * R + k * kChunk;
            const VT* src = U + (size_t)row * ld + k * kChunk;
            const uint32_t off = (uint32_t)(reinterpret_cast<unsigned char*>(dst) - smem);
            if (row >= a.n_dofs)
                report_bad(a.err, 1, row, c, begin + i);
            else if (off + 16 > a.smem_total || (off & 15))
                report_bad(a.err, 2, off, c, k);
            else if (reinterpret_cast<uintptr_t>(src) & 15)
                report_bad(a.err, 3, row, k, (uint32_t)(reinterpret_cast<uintptr_t>(src) & 0xffffffffu));
            else
                cp_async16(dst, src);
        }
        cp_async_commit();
    };

    uint32_t i = warp, par = 0;
    if (i < cnt) prefetch(i, 0);
    wait_prior_grid();
    for (; i < cnt; i += NW, par ^= 1) {
        if (i + NW < cnt)
            prefetch(i + NW, par ^ 1);
        else
            cp_async_commit();  // keep one group per iteration
        cp_async_wait<1>();
        __syncwarp();
        const unsigned char* b = wbuf + (size_t)par * bb;
        const uint32_t* mp = reinterpret_cast<const uint32_t*>(b);
        const VT* ub = reinterpret_cast<const VT*>(b + batch_map_bytes(n));
        const uint32_t s = i % S;
        const bool ok = __all_sync(0xffffffffu, ring_wait(&full[s], &tag[s], i, (i / S) & 1, abort, a.wait_ns));
        const unsigned char* ks = smem + (size_t)s * L.slot_bytes;
        const uint32_t ub_end = (uint32_t)(reinterpret_cast<const unsigned char*>(ub) - smem) + n * R * sizeof(VT);
        if (ub_end > a.smem_total || s >= S) report_bad(a.err, 6, ub_end, s, i);
        for (uint32_t t = lane; t < tiles && ok && ub_end <= a.smem_total; t += 32) {
            const uint32_t r0 = (t / ctiles) * RT, j0 = (t % ctiles) * CT;
            int usk[CT];  // per-column u scale of the split arithmetic
#pragma unroll
            for (int y = 0; y < CT; y++) usk[y] = load_uscale<A>(a.umax + j0 + y);
            typename A::Acc acc[RT][CT];
#pragma unroll
            for (int x = 0; x < RT; x++)
#pragma unroll
                for (int y = 0; y < CT; y++) acc[x][y] = A::zero();
#pragma unroll 2
            for (uint32_t c = 0; c < n; c++) {
                typename A::KT kk[RT];
#pragma unroll
                for (int x = 0; x < RT; x++)
                    kk[x] = A::kload(ks, (size_t)c * n + min(r0 + x, n - 1), a.plane);
                VT uv[CT];
                RowVec<VT, CT>::load(ub + (size_t)c * R + j0, uv);
                const bool zero = a.bc_mode && (mp[c] & kBcFlag);
                UT us[CT];
#pragma unroll
                for (int y = 0; y < CT; y++) us[y] = stage_s<A>(zero ? VT(0) : uv[y], usk[y]);
#pragma unroll
                for (int x = 0; x < RT; x++)
#pragma unroll
                    for (int y = 0; y < CT; y++) A::fma(acc[x][y], kk[x], us[y]);
            }
            if (!*abort) {
#pragma unroll
                for (int x = 0; x < RT; x++) {
                    if (r0 + x < n) {
                        const uint32_t d = mp[r0 + x] & kDofMask;
                        VT* row = V + (size_t)d * ld + j0;
                        if (d >= a.n_dofs || (reinterpret_cast<uintptr_t>(row) & 15) || j0 + CT > R) {
                            report_bad(a.err, 4, d, j0, begin + i);
                            continue;
                        }
                        VT old[CT];
                        RowVec<VT, CT>::load(row, old);
#pragma unroll
                        for (int y = 0; y < CT; y++) old[y] = old[y] + finish_s<A>(acc[x][y], usk[y]);
                        RowVec<VT, CT>::store(row, old);
                    }
                }
            }
        }
        __syncwarp();
        if (ok && lane == 0) mbar_arrive(&empty[s]);
    }
    cp_async_wait<0>();
    if (lane == 0 && *abort) atomicOr(a.err, kErrTimeout);
}

}  // namespace afm
