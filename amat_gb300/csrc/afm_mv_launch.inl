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
    if constexpr (WPE)
        return (void*)afm_wpe_kernel<NT, ARITH, DUP>;
    else
        return (void*)afm_tpe_kernel<NT, ARITH, DUP>;
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

static RingLayout ring_layout(const Segment& s, size_t ut_bytes) {
    RingLayout L;
    L.slot_bytes = (uint32_t)((s.unit_bytes + kSlotAlign - 1) / kSlotAlign * kSlotAlign);
    L.warps = (s.regime == REG_TPE) ? 8u : (s.n <= 32 ? 8u : 4u);
    L.ubuf_bytes = (s.regime == REG_WPE) ? (uint32_t)((s.n * ut_bytes + 15) / 16 * 16) : 0u;
    uint32_t fixed = L.ubuf_bytes * L.warps;
    uint32_t st = (kSmemBudget - fixed) / (L.slot_bytes + 16);
    if (st > 16) st = 16;
    // keep at least two slots in flight beyond the ones the consumers hold
    while (L.warps > 1 && st < L.warps + 2) {
        L.warps = L.warps / 2;
        fixed = L.ubuf_bytes * L.warps;
        st = (kSmemBudget - fixed) / (L.slot_bytes + 16);
        if (st > 16) st = 16;
    }
    L.stages = st;
    return L;
}

cudaError_t LAUNCH_FN(const Segment& s, const SegArgs& a, int sm_count, bool dup, cudaStream_t stream) {
    if (s.units == 0) return cudaSuccess;
    const RingLayout L = ring_layout(s, sizeof(typename ARITH::UT));
    if (L.stages < 2) return cudaErrorInvalidConfiguration;
    void* fn = pick_kernel(s.regime, s.n, dup);
    const uint32_t smem = L.total();
    static thread_local int configured_dev = -1;
    int dev = 0;
    cudaGetDevice(&dev);
    if (configured_dev != dev) {
        // every instance may take the whole budget
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
    void* params[] = {&args, (void*)&L, &n_rt};
    return cudaLaunchKernel(fn, dim3(grid), block, params, smem, stream);
}

size_t SMEM_FN(const Segment& s) { return ring_layout(s, sizeof(typename ARITH::UT)).total(); }

}  // namespace afm
