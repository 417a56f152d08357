// Patch kernel for small elements (n <= kPatchMaxN): v += sum over the patches
// of one patch colour of P_p^T (sum over the patch's elements of P_e^T Ke P_e) P_p u;
// or, in one launch over every patch, the same sums written out: straight to
// v for a DoF that only this patch lists, to the patch's slice of a combine
// buffer for a shared DoF (kSharedFlag), which a second pass adds up in patch
// order (the colour order of the per-colour launches, hence the same bits).
//
// A patch is a compact group of up to 128 elements, grown breadth first over
// shared DoFs when the operator is finalised. Patches of one
// colour share no DoF. Per patch an index block is stored:
//   glob[ndof]           sorted global DoF ids (kBcFlag on constrained DoFs,
//                        kSharedFlag on DoFs that other patches list too)
//   lmap[units][n][32]   uint16 local DoF index of column c of element slot
//   csr_off[ndof + 1]    uint16: contributions of local DoF d are
//   slot[...]            slot[csr_off[d] .. csr_off[d+1]), each r * cap + e
//                        (row r of element slot e; cap = 32 units)
// and the patch's Ke as units of 32 element slots in the thread-per-element
// layout (entry (r, c) of slot l at (r n + c) 32 + l, or at the packed
// triangle index for the symmetric inner arena; empty slots are zero). The
// patch's units start at unit0 of whichever arena the launch streams.
//
// CTA = G consumer groups of GW warps + 1 producer warp; group g takes the
// CTA's patches g, g + G, ... (G patches in flight per SM, so one patch's
// gather and reduce latency hides behind the others' products). The producer's elected lane copies each
// patch's index block into the group's buffer (one bulk copy) and streams
// its Ke units through the shared ring. A group: gathers u of the patch's
// DoFs into shared memory once; each lane multiplies one element slot and
// writes its n products to a shared buffer; then each DoF sums its
// contributions in the stored order and adds the sum to v at L2 (red.add,
// one per DoF and colour: no two patches of a colour share a DoF, so no
// update races). The order of every sum is fixed by the index block and the
// colour order, so v is bit-reproducible. u and v cross HBM about once per
// patch instead of once per element colour.
#pragma once

#include "afm_matvec.cuh"

namespace afm {

// G consumer groups of GW warps: 8 groups of 2 warps for FP32 (or 4 when the
// shared memory of 8 would leave the ring too few slots), 4 groups of 2 warps
// for 8-byte entries (or 2 groups of 4 when their 25.6 KB units would leave
// the ring too few slots). A group's patch passes through phases bound by
// memory latency (the index block, the gather of u), so the patches in flight
// per SM, not the multiply, set the kernel's pace.
constexpr uint32_t kPatchMaxGroups = 8;
constexpr int kBatch = 8;  // global loads a thread keeps in flight in the gather

// Shared-memory layout: ring slots, mbarriers (full[S], empty[S], idx_full[8],
// idx_empty[8]) and the abort flag, the slot tags (ring_wait), then per group:
// index block, staged u, element products.
struct PatchLayout {
    uint32_t slot_bytes, stages, groups;
    uint32_t idx_bytes, us_bytes, ve_bytes;  // per group, 16-byte multiples
    __host__ __device__ uint32_t bars_offset() const { return slot_bytes * stages; }
    __host__ __device__ uint32_t tags_offset() const {
        return bars_offset() + 16u * stages + 16u * kPatchMaxGroups + 16u;
    }
    __host__ __device__ uint32_t group_offset() const { return tags_offset() + ((4u * stages + 15u) & ~15u); }
    __host__ __device__ uint32_t group_bytes() const { return idx_bytes + us_bytes + ve_bytes; }
    __host__ __device__ uint32_t total() const { return group_offset() + groups * group_bytes(); }
};

// v[i] += x at L2, round to nearest (the f32 form flushes subnormal values
// to zero)
__device__ __forceinline__ void red_add(float* p, float x) {
    asm volatile("red.global.add.f32 [%0], %1;" ::"l"(p), "f"(x) : "memory");
}
__device__ __forceinline__ void red_add(double* p, double x) {
    asm volatile("red.global.add.f64 [%0], %1;" ::"l"(p), "d"(x) : "memory");
}

template <int NT, typename A, int G, int GW>
__global__ void __launch_bounds__((G * GW + 1) * 32, 1) afm_patch_kernel(PatchArgs a, PatchLayout L, uint32_t n_rt) {
    constexpr uint32_t kPatchGroups = G;
    constexpr uint32_t kPatchGroupWarps = GW;
    constexpr uint32_t kPatchGroupThreads = kPatchGroupWarps * 32;
    using KT = typename A::KT;
    using UT = typename A::UT;
    using VT = typename A::VT;
    using VO = typename A::VO;
    constexpr int NM = NT ? NT : 12;
    const uint32_t n = NT ? NT : n_rt;
    extern __shared__ __align__(128) unsigned char smem[];
    uint64_t* full = reinterpret_cast<uint64_t*>(smem + L.bars_offset());
    uint64_t* empty = full + L.stages;
    uint64_t* idx_full = empty + L.stages;
    uint64_t* idx_empty = idx_full + kPatchMaxGroups;
    volatile int* abort = reinterpret_cast<volatile int*>(idx_empty + kPatchMaxGroups);
    volatile uint32_t* tag = reinterpret_cast<volatile uint32_t*>(smem + L.tags_offset());
    const uint32_t tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t S = L.stages;

    const uint32_t per = a.count / gridDim.x, rem = a.count % gridDim.x;
    const uint32_t begin = blockIdx.x * per + min(blockIdx.x, rem);
    const uint32_t cnt = per + (blockIdx.x < rem ? 1u : 0u);
    const PatchDesc* __restrict__ desc = a.desc + begin;

    if (tid == 0) {
        for (uint32_t s = 0; s < S; s++) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
            tag[s] = 0xffffffffu;
        }
        for (uint32_t g = 0; g < kPatchGroups; g++) {
            mbar_init(&idx_full[g], 1);
            mbar_init(&idx_empty[g], 1);
        }
        *abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();

    if (warp == kPatchGroups * kPatchGroupWarps) {  // producer
        if (lane == 0) {
            const uint64_t pol = l2_evict_first_policy();
            uint32_t issued = 0;  // Ke units
            uint32_t idx_issued[kPatchGroups] = {};
            bool stop = false;
            for (uint32_t k = 0; k < cnt && !stop; k++) {
                const uint32_t g = k % kPatchGroups, j = k / kPatchGroups;
                const PatchDesc d = desc[k];
                if (j >= 1 && !mbar_wait_abortable(&idx_empty[g], (j - 1) & 1, abort, a.wait_ns)) break;
                mbar_arrive_expect_tx(&idx_full[g], d.idx_bytes);
                bulk_load(smem + L.group_offset() + g * L.group_bytes(), a.idx + d.idx_off, d.idx_bytes,
                          &idx_full[g], pol);
                idx_issued[g] = j + 1;
                // 8-byte entries: the group's next index block into L2 now, so that its copy (issued once
                // this patch is done) does not wait on HBM (measured: split tet10 product 1.115 -> 1.065 ms;
                // the FP32 kernels, with twice the groups, ran slower with it)
                if (sizeof(VT) == 8 && k + kPatchGroups < cnt) {
                    const PatchDesc d2 = desc[k + kPatchGroups];
                    bulk_prefetch_l2(a.idx + d2.idx_off, d2.idx_bytes);
                }
                for (uint32_t u = 0; u < d.units; u++) {
                    const uint32_t s = issued % S;
                    if (issued >= S && !mbar_wait_abortable(&empty[s], ((issued / S) - 1) & 1, abort, a.wait_ns)) {
                        stop = true;
                        break;
                    }
                    tag[s] = issued;
                    mbar_arrive_expect_tx(&full[s], a.copy_bytes);
                    bulk_load(smem + (size_t)s * L.slot_bytes, a.ke + (uint64_t)(d.unit0 + u) * a.unit_bytes,
                              a.copy_bytes, &full[s], pol);
                    issued++;
                }
            }
            allow_dependent_launch();
            if (*abort) atomicOr(a.err, kErrTimeout);
            // wait (bounded) for the copies still in flight before the CTA exits
            drain_ring(full, S, issued);
            const unsigned long long t0 = globaltimer_ns();
            for (uint32_t g = 0; g < kPatchGroups; g++)
                if (idx_issued[g])
                    while (!mbar_try_wait(&idx_full[g], (idx_issued[g] - 1) & 1) &&
                           globaltimer_ns() - t0 < kDrainLimitNs) {
                    }
        }
        return;
    }

    if (a.probe && blockIdx.x == 0 && warp == 0 && !probe_wait(a.probe, a.wait_ns)) *abort = 1;
    const uint32_t g = warp / kPatchGroupWarps, wg = warp % kPatchGroupWarps, t = tid % kPatchGroupThreads;
    const uint32_t bar_id = 1 + g;
    unsigned char* gbase = smem + L.group_offset() + g * L.group_bytes();
    UT* us = reinterpret_cast<UT*>(gbase + L.idx_bytes);
    // element products stay in the accumulator format (a double-float pair
    // for the split arithmetic) until one finish per DoF: on GB300 every FP64
    // instruction costs as much as 64 FP32 ones
    using Acc = typename A::Acc;
    Acc* ve = reinterpret_cast<Acc*>(gbase + L.idx_bytes + L.us_bytes);
    const VT* __restrict__ u = static_cast<const VT*>(a.u);
    VO* __restrict__ v = static_cast<VO*>(a.v);
    VO* __restrict__ pv = static_cast<VO*>(a.pv);
    const uint64_t keep = l2_evict_last_policy();
    // the scale was written by a launch that completed before this matvec's first launch
    const int usk = load_uscale<A>(a.umax);

    // ring index of this group's first unit: units of the patches before it
    uint32_t base = 0;
    for (uint32_t k = 0; k < g && k < cnt; k++) base += desc[k].units;
    bool waited_prior = false;
    for (uint32_t k = g; k < cnt; k += kPatchGroups) {
        const PatchDesc d = desc[k];
        const uint32_t j = k / kPatchGroups;
        const bool iok = __all_sync(0xffffffffu, mbar_wait_abortable(&idx_full[g], j & 1, abort, a.wait_ns));
        const uint32_t* glob = reinterpret_cast<const uint32_t*>(gbase);
        const uint16_t* lmap = reinterpret_cast<const uint16_t*>(gbase + patch_lmap_off(d.ndof));
        const uint16_t* coff = reinterpret_cast<const uint16_t*>(gbase + patch_csr_off(d.ndof, d.units, n));
        const uint16_t* slot = reinterpret_cast<const uint16_t*>(gbase + patch_slot_off(d.ndof, d.units, n));
        const uint32_t cap = d.units * 32u;

        // u of the patch's DoFs, once; kBatch independent loads in flight per
        // thread before any of them is used (in-order issue would otherwise
        // pay one memory latency per DoF)
        if (iok)
            for (uint32_t i0 = t; i0 < d.ndof; i0 += kPatchGroupThreads * kBatch) {
                uint32_t m[kBatch];
                VT x[kBatch];
#pragma unroll
                for (int q = 0; q < kBatch; q++) {
                    const uint32_t i = i0 + q * kPatchGroupThreads;
                    m[q] = i < d.ndof ? glob[i] : 0u;
                    x[q] = i < d.ndof ? ld_nc_hint(u + (m[q] & kPatchDofMask), keep) : VT(0);
                }
#pragma unroll
                for (int q = 0; q < kBatch; q++) {
                    const uint32_t i = i0 + q * kPatchGroupThreads;
                    if (i < d.ndof) us[i] = stage_s<A>((a.bc_mode && (m[q] & kBcFlag)) ? VT(0) : x[q], usk);
                }
            }
        named_barrier(bar_id, kPatchGroupThreads);

        // element products: lane l of warp w takes slot (unit w + W i, lane l)
        for (uint32_t un = wg; un < d.units; un += kPatchGroupWarps) {
            const uint32_t ii = base + un, s = ii % S;
            const bool ok = __all_sync(0xffffffffu, iok && ring_wait(&full[s], &tag[s], ii, (ii / S) & 1, abort, a.wait_ns));
            if (ok) {
                const unsigned char* ks = smem + (size_t)s * L.slot_bytes;
                UT ul[NM];
#pragma unroll
                for (int c = 0; c < NM; c++)
                    if (c < (int)n) ul[c] = us[lmap[(un * n + c) * 32u + lane]];
                const uint32_t e = un * 32u + lane;
#pragma unroll
                for (int r = 0; r < NM; r++) {
                    if (r < (int)n) {
                        typename A::Acc acc = A::zero();
#pragma unroll
                        for (int c = 0; c < NM; c++)
                            if (c < (int)n) A::fma(acc, A::kload(ks, (size_t)tpe_entry<A>(r, c, n) * 32u + lane, a.plane),
                                              ul[c]);
                        ve[r * cap + e] = acc;
                    }
                }
            }
            __syncwarp();
            if (ok && lane == 0) mbar_arrive(&empty[s]);
        }
        named_barrier(bar_id, kPatchGroupThreads);

        // each DoF sums its contributions in stored order; one v update, as
        // a reduction performed at L2 (red.add: no load, no wait). Patches of
        // one colour share no DoF and colour launches are ordered, so every v
        // entry still receives v + sum once per colour, in colour order.
        if (!waited_prior) {
            wait_prior_grid();
            waited_prior = true;
        }
        if (iok && !*abort)
            for (uint32_t i = t; i < d.ndof; i += kPatchGroupThreads) {
                Acc sum = A::zero();
                const uint32_t q1 = coff[i + 1];
                for (uint32_t c = coff[i]; c < q1; c++) A::combine(sum, ve[slot[c]]);
                const VO val = finish_s<A>(sum, usk);
                const uint32_t g = glob[i];
                if (pv == nullptr)
                    red_add(v + (g & kPatchDofMask), val);
                else if (g & kSharedFlag)
                    pv[d.pv_off + i] = val;  // added to v by the combine pass, in patch order
                else
                    v[g & kPatchDofMask] = val;  // the only patch that lists this DoF
            }
        named_barrier(bar_id, kPatchGroupThreads);
        if (t == 0) mbar_arrive(&idx_empty[g]);
        // skip the other groups' patches up to this group's next one
        for (uint32_t k2 = k; k2 < k + kPatchGroups && k2 < cnt; k2++) base += desc[k2].units;
    }
    if (!waited_prior) wait_prior_grid();
    if (t == 0 && *abort) atomicOr(a.err, kErrTimeout);
}

}  // namespace afm
