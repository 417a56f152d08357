// Instantiation and dispatch of the matvec kernels for one arithmetic policy
// (included by afm_mv_fp64.cu, afm_mv_split.cu, afm_mv_fp32.cu, which define
// ARITH and LAUNCH_FN so that the three compile in parallel).
#include "afm_matvec.cuh"

namespace afm {

namespace {

// Element sizes with a compile-time specialisation; any other n <= 16 (TPE)
// or <= kMaxN (WPE) runs the run-time-n instance (template argument 0).
template <int NT, bool WPE, bool DUP>
void* kernel_ptr() {
    if constexpr (WPE) {
        if constexpr (DUP)
            return (void*)afm_wpe_kernel<NT, ARITH, true>;
        else
            return (void*)afm_wpg_kernel<NT, ARITH>;
    } else {
        return (void*)afm_tpe_kernel<NT, ARITH, DUP>;
    }
}

void* pick_kernel(int regime, uint32_t n, bool dup) {
    if (regime == REG_TPE) {
        if (dup) return kernel_ptr<0, false, true>();
        switch (n) {
            case 4: return kernel_ptr<4, false, false>();
            case 8: return kernel_ptr<8, false, false>();
            case 10: return kernel_ptr<10, false, false>();
            default: return kernel_ptr<0, false, false>();
        }
    }
    if (dup) return kernel_ptr<0, true, true>();
    switch (n) {
        case 20: return kernel_ptr<20, true, false>();
        case 24: return kernel_ptr<24, true, false>();
        case 30: return kernel_ptr<30, true, false>();
        case 60: return kernel_ptr<60, true, false>();
        default: return kernel_ptr<0, true, false>();
    }
}

}  // namespace

static uint32_t stages_for(uint32_t slot_bytes, uint32_t extra) {
    if (extra + 16 >= kSmemBudget) return 0;
    uint32_t st = (kSmemBudget - extra - 16) / (slot_bytes + 16);
    return st > 16 ? 16 : st;
}

// Ring layout and (for the warp-group kernel) group geometry of a segment.
static RingLayout ring_layout(const Segment& s, bool dup, GroupGeom* geom) {
    RingLayout L;
    const size_t ut = sizeof(typename ARITH::UT), acc = sizeof(typename ARITH::Acc);
    L.slot_bytes = (uint32_t)((s.unit_bytes + kSlotAlign - 1) / kSlotAlign * kSlotAlign);
    L.ubuf_bytes = 0;
    L.extra_bytes = 0;
    if (s.regime == REG_WPE && !dup) {
        GroupGeom G;
        G.gr = (s.n + 31) / 32;
        G.gc = G.gr >= 3 ? 1 : 4 / G.gr;
        G.g = G.gr * G.gc;
        const uint32_t ub = wpg_ubuf_bytes(s.n, (uint32_t)ut);
        const uint32_t pstride = (G.gc > 1 ? G.gc - 1 : 1) * s.n;
        for (G.ng = 16 / G.g; G.ng >= 1; G.ng--) {
            L.extra_bytes = G.ng * 2 * ub + G.ng * 2 * pstride * (uint32_t)acc;
            L.stages = stages_for(L.slot_bytes, L.extra_bytes);
            if (L.stages >= G.ng + 2 || G.ng == 1) break;
        }
        L.warps = G.ng * G.g;
        L.ubuf_bytes = ub;
        if (geom) *geom = G;
        return L;
    }
    L.warps = (s.regime == REG_TPE) ? 8u : (s.n <= 32 ? 8u : 4u);
    L.ubuf_bytes = (s.regime == REG_WPE) ? (uint32_t)((s.n * ut + 15) / 16 * 16) : 0u;
    L.extra_bytes = L.ubuf_bytes * L.warps;
    L.stages = stages_for(L.slot_bytes, L.extra_bytes);
    // keep at least two slots in flight beyond the ones the consumers hold
    while (L.warps > 1 && L.stages < L.warps + 2) {
        L.warps = L.warps / 2;
        L.extra_bytes = L.ubuf_bytes * L.warps;
        L.stages = stages_for(L.slot_bytes, L.extra_bytes);
    }
    return L;
}

cudaError_t LAUNCH_FN(const Segment& s, const SegArgs& a, int sm_count, bool dup, cudaStream_t stream) {
    if (s.units == 0) return cudaSuccess;
    GroupGeom G{1, 1, 1, 1};
    const RingLayout L = ring_layout(s, dup, &G);
    if (L.stages < 2) return cudaErrorInvalidConfiguration;
    void* fn = pick_kernel(s.regime, s.n, dup);
    const uint32_t smem = L.total();
    static thread_local int configured_dev = -1;
    int dev = 0;
    cudaGetDevice(&dev);
    if (configured_dev != dev) {
        for (int reg = 0; reg < 2; reg++)
            for (uint32_t nn : {4u, 8u, 10u, 20u, 24u, 30u, 60u, 0u})
                for (int d = 0; d < 2; d++) {
                    void* f = pick_kernel(reg, nn == 0 ? 7u : nn, d != 0);
                    cudaError_t e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                         (int)(kSmemBudget + 1024));
                    if (e != cudaSuccess) return e;
                }
        configured_dev = dev;
    }
    uint32_t grid = s.units < (uint32_t)sm_count ? s.units : (uint32_t)sm_count;
    dim3 block((L.warps + 1) * 32);
    uint32_t n_rt = s.n;
    SegArgs args = a;
    RingLayout Lc = L;
    if (s.regime == REG_WPE && !dup) {
        void* params[] = {&args, &Lc, &G, &n_rt};
        return cudaLaunchKernel(fn, dim3(grid), block, params, smem, stream);
    }
    void* params[] = {&args, &Lc, &n_rt};
    return cudaLaunchKernel(fn, dim3(grid), block, params, smem, stream);
}

size_t SMEM_FN(const Segment& s) { return ring_layout(s, false, nullptr).total(); }

}  // namespace afm
