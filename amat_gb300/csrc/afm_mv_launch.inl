// Instantiation and dispatch of the matvec kernels for one arithmetic policy
// (included by afm_mv_fp64.cu, afm_mv_split.cu, afm_mv_fp32.cu and
// afm_mv_f32sym.cu, which define ARITH and LAUNCH_FN so that they compile in
// parallel; BATCH_FN is left undefined where there is no batched product).
#include <algorithm>

#include "afm_batched.cuh"
#include "afm_patch.cuh"

namespace afm {

namespace {

// Element sizes with a compile-time specialisation; any other n <= 16 (TPE)
// or <= kMaxN (WPE) runs the run-time-n instance (template argument 0).
template <int NT, bool WPE, bool DUP, bool CH = false>
void* kernel_ptr() {
    if constexpr (ARITH::kSym && (!WPE || DUP)) {
        return nullptr;  // the symmetric arena has element units for the warp-group kernel only
    } else if constexpr (WPE) {
        if constexpr (DUP)
            return (void*)afm_wpe_kernel<NT, ARITH, true>;
        else
            return (void*)afm_wpg_kernel<NT, ARITH, CH>;
    } else {
        return (void*)afm_tpe_kernel<NT, ARITH, DUP>;
    }
}

// chunked: warp-group launches whose ring slots hold several units (small
// elements; hex20's units fill a slot alone and keep the single-unit kernel)
void* pick_kernel(int regime, uint32_t n, bool dup, bool chunked = false) {
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
    if (chunked) {
        switch (n) {
            case 20: return kernel_ptr<20, true, false, true>();
            case 24: return kernel_ptr<24, true, false, true>();
            case 30: return kernel_ptr<30, true, false, true>();
            default: return kernel_ptr<0, true, false, true>();
        }
    }
    switch (n) {
        case 20: return kernel_ptr<20, true, false>();
        case 24: return kernel_ptr<24, true, false>();
        case 30: return kernel_ptr<30, true, false>();
        case 60: return kernel_ptr<60, true, false>();
        default: return kernel_ptr<0, true, false>();
    }
}

}  // namespace

// Ring stages that fit beside `extra` bytes: per stage the slot, two
// mbarriers and a tag; 32 bytes for the flag word and the tags' padding. Up to
// kMaxStages: under full load an element matrix copy takes microseconds to
// land, and each SM needs ~200 KB of copies in flight to keep HBM busy, which
// small slots reach only with many stages.
constexpr uint32_t kMaxStages = 32;
static uint32_t stages_for(uint32_t slot_bytes, uint32_t extra) {
    if (extra + 32 >= kSmemBudget) return 0;
    uint32_t st = (kSmemBudget - extra - 32) / (slot_bytes + 20);
    return st > kMaxStages ? kMaxStages : st;
}

// Warp-group kernel: ring slots hold up to kMaxChunk consecutive element
// units, about kChunkBytes per bulk copy. One copy per small unit (a few KB)
// is issue-bound: every kernel on units of 1-8 KB moved ~0.6-0.7 G elements/s
// whatever its bytes per element (hex8 elasticity, tet10 elasticity, FP32 and
// split), against ~0.2 G/s of 28.8 KB hex20 units at the HBM roof.
constexpr uint32_t kMaxChunk = 8;
constexpr uint32_t kChunkBytes = 16384;

// Ring layout and (for the warp-group kernel) group geometry of a segment;
// unit_bytes: the stride between units (chunks need whole units copied).
static RingLayout ring_layout(const Segment& s, uint64_t copy_bytes, uint64_t unit_bytes, bool dup,
                              GroupGeom* geom, bool fused = false) {
    RingLayout L;
    const size_t ut = sizeof(typename ARITH::UT), acc = sizeof(typename ARITH::Acc);
    L.slot_bytes = (uint32_t)((copy_bytes + kSlotAlign - 1) / kSlotAlign * kSlotAlign);
    L.ubuf_bytes = 0;
    L.extra_bytes = 0;
    L.chunk = 1;
    if (s.regime == REG_WPE && !dup) {
        GroupGeom G;
        G.gr = (s.n + 31) / 32;
        G.gc = wpg_gc(G.gr, (uint32_t)ut);
        G.g = G.gr * G.gc;
        const uint32_t ub = wpg_ubuf_bytes(ARITH::kSym ? 2 * s.n : s.n, (uint32_t)ut);  // u staged twice (symmetric)
        const uint32_t pstride = (G.gc > 1 ? G.gc - 1 : 1) * s.n;
        // groups of one warp synchronise with __syncwarp; larger groups take one named barrier each (ids 1..15;
        // a fused launch keeps id 15 for its grid barrier)
        const uint32_t ng_max =
            G.g == 1 ? ARITH::kWpgWarps : std::min<uint32_t>(ARITH::kWpgWarps / G.g, fused ? 14u : 15u);
        const uint32_t emax = copy_bytes == unit_bytes
                                  ? std::max<uint32_t>(1u, std::min<uint32_t>(kMaxChunk, (uint32_t)(kChunkBytes / copy_bytes)))
                                  : 1u;
        // the largest chunk that keeps every element group (up to ARITH::kWpgWarps consumer warps) and
        // stages >= groups + 2; with single units, fewer groups if needed
        for (uint32_t E = emax; E >= 1; E--) {
            L.chunk = E;
            L.slot_bytes = (uint32_t)((E * copy_bytes + kSlotAlign - 1) / kSlotAlign * kSlotAlign);
            for (G.ng = ng_max; G.ng >= 1; G.ng--) {
                L.extra_bytes = G.ng * 2 * ub + G.ng * 2 * pstride * (uint32_t)acc;
                L.stages = stages_for(L.slot_bytes, L.extra_bytes);
                if (L.stages >= G.ng + 2 || G.ng == 1) break;
            }
            if (G.ng == ng_max && L.stages >= G.ng + 2) break;
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

cudaError_t LAUNCH_FN(const Segment& s, const SegArgs& a, int sm_count, bool dup, bool pdl, cudaStream_t stream) {
    if (s.units == 0) return cudaSuccess;
    GroupGeom G{1, 1, 1, 1};
    const RingLayout L = ring_layout(s, a.copy_bytes, a.unit_bytes, dup, &G);
    if (L.stages < 2) return cudaErrorInvalidConfiguration;
    void* fn = pick_kernel(s.regime, s.n, dup, L.chunk > 1);
    if (!fn) return cudaErrorInvalidValue;
    const uint32_t smem = L.total();
    // at least 4 elements (2 thread-per-element units) per CTA: a small segment occupies few SMs
    // and leaves the rest to concurrent work (other operators' streams)
    const uint32_t per_cta = s.regime == REG_TPE ? 2u : 4u;
    const uint32_t want = (s.units + per_cta - 1) / per_cta;
    uint32_t grid = want < (uint32_t)sm_count ? want : (uint32_t)sm_count;
    dim3 block((L.warps + 1) * 32);
    uint32_t n_rt = s.n;
    SegArgs args = a;
    RingLayout Lc = L;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = pdl ? 1 : 0;
    if (s.regime == REG_WPE && !dup) {
        void* params[] = {&args, &Lc, &G, &n_rt};
        return cudaLaunchKernelExC(&cfg, fn, params);
    }
    void* params[] = {&args, &Lc, &n_rt};
    return cudaLaunchKernelExC(&cfg, fn, params);
}

#ifdef BATCH_FN
// ---- batched (multi right-hand side) product, warp per element -------------

namespace {
template <int NT, int RT, int CT>
void* batch_kernel_ptr() {
    return (void*)afm_batched_kernel<NT, ARITH, RT, CT>;
}
template <int RT, int CT>
void* batch_kernel_n(uint32_t n) {
    return n == 24 ? batch_kernel_ptr<24, RT, CT>() : batch_kernel_ptr<0, RT, CT>();
}
// lane tile rows x columns: (2, 8), (4, 4), (4, 8), (6, 8)
void* pick_batch_kernel(uint32_t n, int rt, int ct) {
    if (ct == 4) return rt == 4 ? batch_kernel_n<4, 4>(n) : nullptr;
    if (ct != 8) return nullptr;
    switch (rt) {
        case 2: return batch_kernel_n<2, 8>(n);
        case 4: return batch_kernel_n<4, 8>(n);
        case 6: return batch_kernel_n<6, 8>(n);
        default: return nullptr;
    }
}
}  // namespace

// ct: columns per lane tile (4 or 8); rt: rows per lane tile (2, 4 or 6).
cudaError_t BATCH_FN(const Segment& s, const BatchArgs& a, int sm_count, int ct, int rt, bool pdl,
                     cudaStream_t stream) {
    if (s.units == 0) return cudaSuccess;
    void* fn = pick_batch_kernel(s.n, rt, ct);
    if (s.regime != REG_WPE || !fn || a.nrhs % ct != 0) return cudaErrorInvalidValue;
    RingLayout L;
    L.slot_bytes = (a.copy_bytes + kSlotAlign - 1) / kSlotAlign * kSlotAlign;
    L.ubuf_bytes = batch_buf_bytes(s.n, a.nrhs, (uint32_t)sizeof(typename ARITH::VT));
    // Consumers take elements round robin and wait on full[i % S] by parity,
    // which tells only two consecutive phases apart: a warp must never reach a
    // slot whose previous round is still loading, so the ring keeps at least
    // two stages more than there are consumer warps (as ring_layout does).
    for (L.warps = 8; L.warps >= 1; L.warps--) {
        L.extra_bytes = L.warps * 2 * L.ubuf_bytes;
        L.stages = stages_for(L.slot_bytes, L.extra_bytes);
        if (L.stages >= L.warps + 2) break;
    }
    if (L.warps == 0 || L.stages < L.warps + 2) return cudaErrorInvalidConfiguration;
    cudaLaunchConfig_t cfg = {};
    const uint32_t want = (s.units + 3) / 4;  // at least 4 elements per CTA
    cfg.gridDim = dim3(want < (uint32_t)sm_count ? want : (uint32_t)sm_count);
    cfg.blockDim = dim3((L.warps + 1) * 32);
    cfg.dynamicSmemBytes = L.total();
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = pdl ? 1 : 0;
    BatchArgs args = a;
    args.smem_total = L.total();
    uint32_t n_rt = s.n;
    void* params[] = {&args, &L, &n_rt};
    return cudaLaunchKernelExC(&cfg, fn, params);
}

#endif  // BATCH_FN

// ---- patch path (small elements) -----------------------------------------

namespace {
// consumer groups (G) of GW warps of the patch kernel for this arithmetic
// (see afm_patch.cuh): FP32 tries 8 groups of 2 warps, then 4; 8-byte entries
// 4 groups of 2 warps, then 2 of 4 (their 25.6 KB units leave few ring slots).
constexpr bool kF32Patch = sizeof(typename ARITH::VT) == 4;
constexpr uint32_t kMinPatchStages = kF32Patch ? 6 : 5;  // ring slots below which fewer groups are used

// warps per group for G groups
constexpr int patch_gw(int G) { return kF32Patch ? 2 : (G == 4 ? 2 : 4); }

template <int G>
void* patch_kernel_g(uint32_t n) {
    constexpr int GW = patch_gw(G);
    switch (n) {
        case 4: return (void*)afm_patch_kernel<4, ARITH, G, GW>;
        case 8: return (void*)afm_patch_kernel<8, ARITH, G, GW>;
        case 10: return (void*)afm_patch_kernel<10, ARITH, G, GW>;
        default: return (void*)afm_patch_kernel<0, ARITH, G, GW>;
    }
}

void* pick_patch_kernel(uint32_t n, uint32_t groups) {
    if constexpr (kF32Patch) return groups == 8 ? patch_kernel_g<8>(n) : patch_kernel_g<4>(n);
    else return groups == 4 ? patch_kernel_g<4>(n) : patch_kernel_g<2>(n);
}

PatchLayout patch_layout_g(const PatchPlanGeom& pg, uint32_t copy_bytes, uint32_t groups) {
    PatchLayout L;
    L.groups = groups;
    L.slot_bytes = (copy_bytes + kSlotAlign - 1) / kSlotAlign * kSlotAlign;
    L.idx_bytes = patch_r16(pg.max_idx);
    L.us_bytes = patch_r16(pg.max_ndof * (uint32_t)sizeof(typename ARITH::UT));
    L.ve_bytes = patch_r16(pg.n * pg.max_slots * (uint32_t)sizeof(typename ARITH::Acc));
    const uint32_t fixed = 16 * kPatchMaxGroups + 16 + 16 + L.groups * L.group_bytes();
    L.stages = 0;
    if (fixed < kSmemBudget) {
        const uint32_t st = (kSmemBudget - fixed) / (L.slot_bytes + 20);
        L.stages = st > kMaxStages ? kMaxStages : st;
    }
    return L;
}

PatchLayout patch_layout(const PatchPlanGeom& pg, uint32_t copy_bytes) {
    const uint32_t more = kF32Patch ? 8 : 4, fewer = kF32Patch ? 4 : 2;
    const PatchLayout L = patch_layout_g(pg, copy_bytes, more);
    if (L.stages >= kMinPatchStages) return L;
    return patch_layout_g(pg, copy_bytes, fewer);
}
}  // namespace

cudaError_t PATCH_FN(const PatchPlanGeom& pg, const PatchArgs& a, int sm_count, bool pdl, cudaStream_t stream) {
    if (a.count == 0) return cudaSuccess;
    PatchLayout L = patch_layout(pg, a.copy_bytes);
    if (L.stages < 2 || pg.n == 0 || pg.n > kPatchMaxN) return cudaErrorInvalidConfiguration;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(a.count < (uint32_t)sm_count ? a.count : (uint32_t)sm_count);
    cfg.blockDim = dim3((L.groups * patch_gw((int)L.groups) + 1) * 32);
    cfg.dynamicSmemBytes = L.total();
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = pdl ? 1 : 0;
    PatchArgs args = a;
    uint32_t n_rt = pg.n;
    void* params[] = {&args, &L, &n_rt};
    return cudaLaunchKernelExC(&cfg, pick_patch_kernel(pg.n, L.groups), params);
}

size_t PATCH_SMEM_FN(const PatchPlanGeom& pg, uint32_t copy_bytes) {
    const PatchLayout L = patch_layout(pg, copy_bytes);
    return L.stages >= 2 ? L.total() : 0;
}

size_t SMEM_FN(const Segment& s) { return ring_layout(s, s.unit_bytes, s.unit_bytes, false, nullptr).total(); }

#ifdef FUSED_FN
namespace {
template <int NT, bool CH>
void* fused_ptr() {
    return (void*)afm_wpg_fused_kernel<NT, ARITH, CH>;
}
void* pick_fused_kernel(uint32_t n, bool chunked) {
    if (chunked) {
        switch (n) {
            case 24: return fused_ptr<24, true>();
            case 30: return fused_ptr<30, true>();
            default: return fused_ptr<0, true>();
        }
    }
    switch (n) {
        case 24: return fused_ptr<24, false>();
        case 30: return fused_ptr<30, false>();
        case 60: return fused_ptr<60, false>();
        default: return fused_ptr<0, false>();
    }
}
}  // namespace

// The colours segs[0 .. ncol) of a segment plan whose elements share one size
// (warp-group regime) in one cooperative launch: one CTA per SM, each taking
// the share of every colour that a launch of that colour alone would give it,
// a grid barrier between colours (gbar: ncol - 1 counters, zero at launch).
// a.ke and a.map: the arena and map bases; the colours' offsets come from segs.
cudaError_t FUSED_FN(const Segment* segs, uint32_t ncol, const SegArgs& a, unsigned* gbar, int sm_count,
                     cudaStream_t stream) {
    if (ncol == 0 || ncol > kMaxFusedColours || segs[0].regime != REG_WPE) return cudaErrorInvalidValue;
    GroupGeom G{1, 1, 1, 1};
    const RingLayout L = ring_layout(segs[0], a.copy_bytes, a.unit_bytes, false, &G, true);
    if (L.stages < 2) return cudaErrorInvalidConfiguration;
    void* fn = pick_fused_kernel(segs[0].n, L.chunk > 1);
    ColourTable T{};
    T.ncol = ncol;
    T.gbar = gbar;
    for (uint32_t c = 0; c < ncol; c++) {
        if (segs[c].n != segs[0].n || segs[c].regime != REG_WPE) return cudaErrorInvalidValue;
        T.ke_off[c] = segs[c].ke_offset;
        T.map_off[c] = segs[c].map_offset;
        T.units[c] = segs[c].units;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((uint32_t)sm_count);
    cfg.blockDim = dim3((L.warps + 1) * 32);
    cfg.dynamicSmemBytes = L.total();
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    SegArgs args = a;
    RingLayout Lc = L;
    uint32_t n_rt = segs[0].n;
    void* params[] = {&args, &Lc, &G, &n_rt, &T};
    return cudaLaunchKernelExC(&cfg, fn, params);
}
#endif  // FUSED_FN

#define AFM_CAT2(a, b) a##b
#define AFM_CAT(a, b) AFM_CAT2(a, b)
// Launch geometry of a warp-group segment (host checks): out = chunk,
// stages, consumer warps, element groups, column groups, dynamic shared
// memory bytes.
void AFM_CAT(SMEM_FN, _geom)(const Segment& s, uint64_t copy_bytes, uint64_t unit_bytes, uint32_t* out) {
    GroupGeom G{1, 1, 1, 1};
    const RingLayout L = ring_layout(s, copy_bytes, unit_bytes, false, &G);
    out[0] = L.chunk;
    out[1] = L.stages;
    out[2] = L.warps;
    out[3] = G.ng;
    out[4] = G.gc;
    out[5] = L.total();
}

// Raises the dynamic shared-memory limit of every kernel instance on the
// current device; called once per device before any launch or capture.
cudaError_t CONFIG_FN() {
    for (int reg = 0; reg < 2; reg++)
        for (uint32_t nn : {4u, 8u, 10u, 20u, 24u, 30u, 60u, 0u})
            for (int d = 0; d < 2; d++)
                for (int ch = 0; ch < 2; ch++) {
                    void* f = pick_kernel(reg, nn == 0 ? 7u : nn, d != 0, ch != 0);
                    if (!f) continue;
                    cudaError_t e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                         (int)(kSmemBudget + 1024));
                    if (e != cudaSuccess) return e;
                }
    for (uint32_t nn : {4u, 8u, 10u, 0u})
        for (uint32_t gg : {2u, 4u, 8u}) {
            cudaError_t e = cudaFuncSetAttribute(pick_patch_kernel(nn, gg),
                                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(kSmemBudget + 1024));
            if (e != cudaSuccess) return e;
        }
#ifdef FUSED_FN
    for (uint32_t nn : {24u, 30u, 60u, 7u})
        for (int ch = 0; ch < 2; ch++) {
            cudaError_t e = cudaFuncSetAttribute(pick_fused_kernel(nn, ch != 0),
                                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(kSmemBudget + 1024));
            if (e != cudaSuccess) return e;
        }
#endif
#ifdef BATCH_FN
    const int tiles[4][2] = {{2, 8}, {4, 4}, {4, 8}, {6, 8}};
    for (const auto& t : tiles)
        for (uint32_t nn : {24u, 7u}) {
            cudaError_t e = cudaFuncSetAttribute(pick_batch_kernel(nn, t[0], t[1]),
                                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(kSmemBudget + 1024));
            if (e != cudaSuccess) return e;
        }
#endif
    return cudaSuccess;
}


}  // namespace afm
