// Batched (multi right-hand-side) AFM product V = K U for the warp-group
// regime (n > 16): U and V are n_dofs x R, row-major with leading dimension
// ld (the R values of one DoF are contiguous). Each streamed element matrix is
// used for all R columns: per element V_e (n x R) += Ke (n x n) U_e (n x R).
//
// Same TMA ring as the single-vector kernels (one element per unit, Ke
// column-major). ng element groups per CTA; a group of gthreads threads owns
// one element at a time. U_e is staged in shared memory (double buffer, the
// next element gathered while this one is multiplied). Thread tile: 4 rows x
// TR columns of V_e; per column c of Ke it loads 4 Ke entries and TR entries
// of U_e and does 4 TR multiply-adds. Colour-exclusive scatter as in the
// single-vector kernels: V = V_old + V_e, no atomics, deterministic.
#pragma once

#include "afm_matvec.cuh"

namespace afm {

struct BatchGeom {
    uint32_t ng;        // element groups per CTA
    uint32_t gthreads;  // threads per group (multiple of 32)
    uint32_t rtiles;    // ceil(n / 4)
    uint32_t ctiles;    // nrhs / TR
};

// shared bytes of one group's U_e buffer (both parities)
__host__ __device__ inline uint32_t batch_ubuf_bytes(uint32_t n, uint32_t nrhs, uint32_t ut) {
    return 2 * ((n * nrhs * ut + 127) / 128 * 128);
}

template <int NT, typename A, int TR>
__global__ void __launch_bounds__(544, 1) afm_batched_kernel(BatchArgs a, RingLayout L, BatchGeom G, uint32_t n_rt) {
    using UT = typename A::UT;
    using VT = typename A::VT;
    using Acc = typename A::Acc;
    const uint32_t n = NT ? NT : n_rt;
    extern __shared__ __align__(128) unsigned char smem[];
    uint64_t* full = reinterpret_cast<uint64_t*>(smem + L.bars_offset());
    uint64_t* empty = full + L.stages;
    volatile int* abort = reinterpret_cast<volatile int*>(empty + L.stages);
    const uint32_t ub = batch_ubuf_bytes(n, a.nrhs, sizeof(UT)) / 2;  // one parity
    const uint32_t tid = threadIdx.x;
    const uint32_t consumers = G.ng * G.gthreads;
    const uint32_t S = L.stages;

    const uint32_t per = a.units / gridDim.x, rem = a.units % gridDim.x;
    const uint32_t begin = blockIdx.x * per + min(blockIdx.x, rem);
    const uint32_t cnt = per + (blockIdx.x < rem ? 1u : 0u);

    if (tid == 0) {
        for (uint32_t s = 0; s < S; s++) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], G.gthreads / 32);
        }
        *abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();

    if (tid >= consumers) {  // producer warp
        if ((tid & 31) == 0) {
            const uint64_t pol = l2_evict_first_policy();
            uint32_t issued = 0;
            for (uint32_t i = 0; i < cnt; i++) {
                const uint32_t s = i % S;
                if (i >= S && !mbar_wait_abortable(&empty[s], ((i / S) - 1) & 1, abort)) break;
                mbar_arrive_expect_tx(&full[s], a.copy_bytes);
                bulk_load(smem + (size_t)s * L.slot_bytes, a.ke + (size_t)(begin + i) * a.unit_bytes, a.copy_bytes,
                          &full[s], pol);
                issued = i + 1;
            }
            allow_dependent_launch();
            if (*abort) {
                atomicOr(a.err, kErrTimeout);
                const uint32_t first = issued > S ? issued - S : 0;
                const unsigned long long t0 = globaltimer_ns();
                for (uint32_t i = first; i < issued; i++)
                    while (!mbar_try_wait(&full[i % S], (i / S) & 1) && globaltimer_ns() - t0 < kWaitLimitNs) {
                    }
            }
        }
        return;
    }

    const uint32_t grp = tid / G.gthreads, t = tid % G.gthreads;
    const uint32_t bar_id = 1 + grp;
    const uint32_t R = a.nrhs, ld = a.ld;
    unsigned char* ubase = smem + L.ubuf_offset() + (size_t)grp * 2 * ub;
    auto ubuf = [&](uint32_t p) { return reinterpret_cast<UT*>(ubase + (size_t)p * ub); };
    const VT* __restrict__ U = static_cast<const VT*>(a.u);
    VT* __restrict__ V = static_cast<VT*>(a.v);
    const uint64_t keep = l2_evict_last_policy();
    const uint32_t tiles = G.rtiles * G.ctiles;
    const uint32_t nu = n * R;  // entries of U_e

    // stage U_e of element i (group-cooperative, coalesced rows of R values)
    auto gather = [&](uint32_t i, UT* dst) {
        const uint32_t* mp = a.map + (size_t)(begin + i) * n;
        for (uint32_t k = t; k < nu; k += G.gthreads) {
            const uint32_t c = k / R, j = k % R;
            const uint32_t m = __ldg(mp + c);
            VT x = ld_nc_hint(U + (size_t)(m & kDofMask) * ld + j, keep);
            if (a.bc_mode && (m & kBcFlag)) x = VT(0);
            dst[k] = A::stage(x);
        }
    };

    uint32_t i = grp;
    if (i < cnt) gather(i, ubuf(0));
    wait_prior_grid();
    named_barrier(bar_id, G.gthreads);
    for (uint32_t k = 0; i < cnt; i += G.ng, k++) {
        const uint32_t par = k & 1;
        const uint32_t s = i % S;
        const bool ok = mbar_wait_abortable(&full[s], (i / S) & 1, abort);
        const unsigned char* ks = smem + (size_t)s * L.slot_bytes;
        const UT* uu = ubuf(par);
        const uint32_t* mp = a.map + (size_t)(begin + i) * n;
        for (uint32_t tile = t; tile < tiles && ok; tile += G.gthreads) {
            const uint32_t rb = tile / G.ctiles, cb = tile % G.ctiles;
            const uint32_t r0 = 4 * rb, j0 = TR * cb;
            Acc acc[4][TR];
#pragma unroll
            for (int x = 0; x < 4; x++)
#pragma unroll
                for (int y = 0; y < TR; y++) acc[x][y] = A::zero();
#pragma unroll 4
            for (uint32_t c = 0; c < n; c++) {
                typename A::KT kk[4];
#pragma unroll
                for (int x = 0; x < 4; x++)
                    kk[x] = (r0 + x < n) ? A::kload(ks, (size_t)c * n + r0 + x, a.plane) : A::kload(ks, 0, a.plane);
                UT uv[TR];
#pragma unroll
                for (int y = 0; y < TR; y++) uv[y] = uu[(size_t)c * R + j0 + y];
#pragma unroll
                for (int x = 0; x < 4; x++)
#pragma unroll
                    for (int y = 0; y < TR; y++) A::fma(acc[x][y], kk[x], uv[y]);
            }
#pragma unroll
            for (int x = 0; x < 4; x++) {
                if (r0 + x < n && !*abort) {
                    const uint32_t d = __ldg(mp + r0 + x) & kDofMask;
                    VT* row = V + (size_t)d * ld + j0;
#pragma unroll
                    for (int y = 0; y < TR; y++) st_hint(row + y, ld_hint(row + y, keep) + A::finish(acc[x][y]), keep);
                }
            }
        }
        // every warp of the group is done with this slot and this u buffer
        __syncwarp();
        if (ok && (t & 31) == 0) mbar_arrive(&empty[s]);
        if (i + G.ng < cnt) gather(i + G.ng, ubuf(par ^ 1));
        named_barrier(bar_id, G.gthreads);
    }
    if ((t & 31) == 0 && *abort) atomicOr(a.err, kErrTimeout);
}

}  // namespace afm
