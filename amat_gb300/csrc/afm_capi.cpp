// Host runtime of the GB300 AFM operator: the C ABI of include/afm.h.
//
// Set-up mirrors par::Maps / par::aMatFree on one rank; finalize colours the
// elements (the reference's greedy first-fit, include/meshGraph.hpp:59-193),
// sorts them by (colour, n, element id), lays the DoF map and element
// matrices out for the device kernels and uploads them once. Every matvec is
// then one launch per (colour, n) segment, in colour order, on the operator's
// stream: no host round trip, no atomics.
#include <cuda_runtime.h>
#include <stdarg.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <numeric>
#include <string>
#include <type_traits>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

#include "afm_batched_solver.hpp"
#include "afm_internal.hpp"
#include "afm_mixed.hpp"
#include "afm_shape.hpp"
#include "afm_solver.hpp"

namespace afm {
cudaError_t launch_segment_fp64(const Segment& s, const SegArgs& a, int sm_count, bool dup, bool pdl,
                                 cudaStream_t st);
cudaError_t launch_segment_split(const Segment& s, const SegArgs& a, int sm_count, bool dup, bool pdl,
                                 cudaStream_t st);
cudaError_t launch_segment_fp32(const Segment& s, const SegArgs& a, int sm_count, bool dup, bool pdl,
                                 cudaStream_t st);
cudaError_t launch_batched_fp64(const Segment& s, const BatchArgs& a, int sm_count, int tr, int ng, bool pdl,
                                cudaStream_t st);
cudaError_t launch_batched_split(const Segment& s, const BatchArgs& a, int sm_count, int tr, int ng, bool pdl,
                                 cudaStream_t st);
cudaError_t launch_fused_split(const Segment* segs, uint32_t ncol, const SegArgs& a, unsigned* gbar, int sm_count,
                               cudaStream_t st);
bool batched_tc_supported(uint32_t n, uint32_t nrhs);
cudaError_t launch_batched_tc(const Segment& s, const BatchArgs& a, int sm_count, bool pdl, cudaStream_t stream);
cudaError_t launch_batched_fp32(const Segment& s, const BatchArgs& a, int sm_count, int tr, int ng, bool pdl,
                                cudaStream_t st);
cudaError_t configure_kernels_fp64();
cudaError_t configure_kernels_split();
cudaError_t configure_kernels_fp32();
cudaError_t launch_patches_fp64(const PatchPlanGeom& pg, const PatchArgs& a, int sm_count, bool pdl, cudaStream_t st);
cudaError_t launch_patches_split(const PatchPlanGeom& pg, const PatchArgs& a, int sm_count, bool pdl, cudaStream_t st);
cudaError_t launch_patches_fp32(const PatchPlanGeom& pg, const PatchArgs& a, int sm_count, bool pdl, cudaStream_t st);
cudaError_t launch_segment_f32sym(const Segment& s, const SegArgs& a, int sm_count, bool dup, bool pdl,
                                  cudaStream_t st);
cudaError_t launch_patches_f32sym(const PatchPlanGeom& pg, const PatchArgs& a, int sm_count, bool pdl,
                                  cudaStream_t st);
cudaError_t configure_kernels_f32sym();
cudaError_t launch_segment_f32symx(const Segment& s, const SegArgs& a, int sm_count, bool dup, bool pdl,
                                   cudaStream_t st);
cudaError_t launch_patches_f32symx(const PatchPlanGeom& pg, const PatchArgs& a, int sm_count, bool pdl,
                                   cudaStream_t st);
cudaError_t configure_kernels_f32symx();
size_t patch_smem_f32symx(const PatchPlanGeom& pg, uint32_t copy_bytes);
size_t segment_smem_f32symx(const Segment& s);
cudaError_t launch_segment_splitsymx(const Segment& s, const SegArgs& a, int sm_count, bool dup, bool pdl,
                                     cudaStream_t st);
cudaError_t launch_patches_splitsymx(const PatchPlanGeom& pg, const PatchArgs& a, int sm_count, bool pdl,
                                     cudaStream_t st);
cudaError_t configure_kernels_splitsymx();
cudaError_t launch_segment_f32symc(const Segment& s, const SegArgs& a, int sm_count, bool dup, bool pdl,
                                   cudaStream_t st);
cudaError_t launch_patches_f32symc(const PatchPlanGeom& pg, const PatchArgs& a, int sm_count, bool pdl,
                                   cudaStream_t st);
cudaError_t configure_kernels_f32symc();
size_t patch_smem_f32symc(const PatchPlanGeom& pg, uint32_t copy_bytes);
size_t segment_smem_f32symc(const Segment& s);
size_t patch_smem_splitsymx(const PatchPlanGeom& pg, uint32_t copy_bytes);
size_t segment_smem_splitsymx(const Segment& s);
size_t patch_smem_f32sym(const PatchPlanGeom& pg, uint32_t copy_bytes);
size_t segment_smem_f32sym(const Segment& s);
size_t patch_smem_fp64(const PatchPlanGeom& pg, uint32_t copy_bytes);
size_t patch_smem_split(const PatchPlanGeom& pg, uint32_t copy_bytes);
size_t patch_smem_fp32(const PatchPlanGeom& pg, uint32_t copy_bytes);

void segment_smem_fp64_geom(const Segment& s, uint64_t copy_bytes, uint64_t unit_bytes, uint32_t* out);
void segment_smem_split_geom(const Segment& s, uint64_t copy_bytes, uint64_t unit_bytes, uint32_t* out);
void segment_smem_fp32_geom(const Segment& s, uint64_t copy_bytes, uint64_t unit_bytes, uint32_t* out);
void segment_smem_f32sym_geom(const Segment& s, uint64_t copy_bytes, uint64_t unit_bytes, uint32_t* out);
void segment_smem_f32symx_geom(const Segment& s, uint64_t copy_bytes, uint64_t unit_bytes, uint32_t* out);
void segment_smem_splitsymx_geom(const Segment& s, uint64_t copy_bytes, uint64_t unit_bytes, uint32_t* out);
void segment_smem_f32symc_geom(const Segment& s, uint64_t copy_bytes, uint64_t unit_bytes, uint32_t* out);

cudaError_t launch_patches(int prec, const PatchPlanGeom& pg, const PatchArgs& a, int sm_count, bool pdl,
                           cudaStream_t stream) {
    switch (prec) {
        case AFM_PREC_FP64: return launch_patches_fp64(pg, a, sm_count, pdl, stream);
        case AFM_PREC_FP64_SPLIT: return launch_patches_split(pg, a, sm_count, pdl, stream);
        case kPrecF32Sym: return launch_patches_f32sym(pg, a, sm_count, pdl, stream);
        case kPrecF32SymX: return launch_patches_f32symx(pg, a, sm_count, pdl, stream);
        case kPrecSplitSymX: return launch_patches_splitsymx(pg, a, sm_count, pdl, stream);
        case kPrecF32SymC: return launch_patches_f32symc(pg, a, sm_count, pdl, stream);
        default: return launch_patches_fp32(pg, a, sm_count, pdl, stream);
    }
}

size_t patch_smem_bytes(int prec, const PatchPlanGeom& pg, uint32_t copy_bytes) {
    switch (prec) {
        case AFM_PREC_FP64: return patch_smem_fp64(pg, copy_bytes);
        case AFM_PREC_FP64_SPLIT: return patch_smem_split(pg, copy_bytes);
        case kPrecF32Sym: return patch_smem_f32sym(pg, copy_bytes);
        case kPrecF32SymX: return patch_smem_f32symx(pg, copy_bytes);
        case kPrecSplitSymX: return patch_smem_splitsymx(pg, copy_bytes);
        case kPrecF32SymC: return patch_smem_f32symc(pg, copy_bytes);
        default: return patch_smem_fp32(pg, copy_bytes);
    }
}

size_t segment_smem_fp64(const Segment& s);
size_t segment_smem_split(const Segment& s);
size_t segment_smem_fp32(const Segment& s);

cudaError_t launch_segment(const Segment& s, int prec, const SegArgs& a, int sm_count, bool dup, bool pdl,
                           cudaStream_t stream) {
    switch (prec) {
        case AFM_PREC_FP64: return launch_segment_fp64(s, a, sm_count, dup, pdl, stream);
        case AFM_PREC_FP64_SPLIT: return launch_segment_split(s, a, sm_count, dup, pdl, stream);
        case kPrecF32Sym: return launch_segment_f32sym(s, a, sm_count, dup, pdl, stream);
        case kPrecF32SymX: return launch_segment_f32symx(s, a, sm_count, dup, pdl, stream);
        case kPrecSplitSymX: return launch_segment_splitsymx(s, a, sm_count, dup, pdl, stream);
        case kPrecF32SymC: return launch_segment_f32symc(s, a, sm_count, dup, pdl, stream);
        default: return launch_segment_fp32(s, a, sm_count, dup, pdl, stream);
    }
}

size_t segment_smem_bytes(const Segment& s, int prec) {
    switch (prec) {
        case AFM_PREC_FP64: return segment_smem_fp64(s);
        case AFM_PREC_FP64_SPLIT: return segment_smem_split(s);
        case kPrecF32Sym: return segment_smem_f32sym(s);
        case kPrecF32SymX: return segment_smem_f32symx(s);
        case kPrecSplitSymX: return segment_smem_splitsymx(s);
        case kPrecF32SymC: return segment_smem_f32symc(s);
        default: return segment_smem_fp32(s);
    }
}
}  // namespace afm

using namespace afm;

namespace {
thread_local std::string g_last_error;
}

int afm::set_error(int status, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return status;
}

namespace {

int fail(int status, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return status;
}

int ok() {
    g_last_error.clear();
    return AFM_SUCCESS;
}

#define AFM_CUDA(call)                                                                                    \
    do {                                                                                                  \
        cudaError_t e_ = (call);                                                                          \
        if (e_ != cudaSuccess)                                                                            \
            return fail(e_ == cudaErrorMemoryAllocation ? AFM_ERR_OOM : AFM_ERR_CUDA, "%s: %s (%s:%d)", #call, \
                        cudaGetErrorString(e_), __FILE__, __LINE__);                                      \
    } while (0)

#define AFM_CHECK_OP(op)                                                                    \
    do {                                                                                    \
        if (!(op)) return fail(AFM_ERR_INVALID_ARG, "null operator");                       \
    } while (0)

struct DeviceGuard {
    int prev = -1;
    explicit DeviceGuard(int dev) {
        cudaGetDevice(&prev);
        if (prev != dev) cudaSetDevice(dev);
    }
    ~DeviceGuard() {
        int cur = -1;
        cudaGetDevice(&cur);
        if (prev >= 0 && cur != prev) cudaSetDevice(prev);
    }
};

size_t entry_bytes(int prec) { return prec == AFM_PREC_FP32 ? 4 : 8; }

uint64_t round16(uint64_t b) { return (b + 15) / 16 * 16; }

// The operator's device buffers are stream-ordered allocations on its own
// stream: releasing them (finalize again, destroy) never synchronises the
// device, so other operators' work keeps running. Work a caller enqueued on
// its own streams with this operator must be ordered before such a release.
template <typename T>
cudaError_t dalloc(afm_operator* op, T** p, size_t bytes) {
    return cudaMallocAsync((void**)p, bytes, op->stream);
}
template <typename T>
void dfree(afm_operator* op, T*& p) {
    if (p) cudaFreeAsync(p, op->stream);
    p = nullptr;
}

void drop_graph(afm_operator::CgGraph& g);

void free_device(afm_operator* op) {
    drop_graph(op->cg64);
    drop_graph(op->cg32);
    drop_graph(op->cg64i);
    drop_graph(op->bcg64);
    drop_graph(op->bcg32);
    op->batch_tune.clear();
    dfree(op, op->d_bwork);
    dfree(op, op->d_bsc);
    op->bwork_elems = 0;
    op->bsc_elems = 0;
    op->generation++;
    dfree(op, op->d_ke);
    dfree(op, op->d_map);
    dfree(op, op->d_diag);
    dfree(op, op->d_bc_idx);
    dfree(op, op->d_bc_val);
    dfree(op, op->d_bcmask);
    dfree(op, op->d_gbar);
    op->fused_ok = false;
    dfree(op, op->d_work);
    dfree(op, op->d_work32);
    dfree(op, op->d_work64i);
    dfree(op, op->d_patch_desc);
    dfree(op, op->d_patch_idx);
    dfree(op, op->d_pv);
    dfree(op, op->d_shared_dof);
    dfree(op, op->d_shared_off);
    dfree(op, op->d_shared_idx);
    dfree(op, op->d_sym);
    dfree(op, op->d_vx);
    dfree(op, op->d_csr_rp);
    dfree(op, op->d_csr_cols);
    dfree(op, op->d_csr_vals);
    op->csr_nnz = 0;
    dfree(op, op->d_free_xe64);
    dfree(op, op->d_free_xe32);
    dfree(op, op->d_free_ref64);
    dfree(op, op->d_free_ref32);
    op->work_elems = 0;
    op->work32_elems = 0;
    op->work64i_elems = 0;
}

// Greedy first-fit colouring in element order (include/meshGraph.hpp:59-109)
// of the graph "elements sharing a DoF" (mesh2Graph, 132-155). Integer work,
// identical result to the reference for the same map.
uint32_t color_elements(uint32_t n_dofs, uint32_t n_elem, const std::vector<uint32_t>& offs,
                        const std::vector<uint32_t>& map, std::vector<uint32_t>& colors) {
    std::vector<uint32_t> cnt((size_t)n_dofs + 1, 0);
    for (uint32_t e = 0; e < n_elem; e++)
        for (uint32_t k = offs[e]; k < offs[e + 1]; k++) cnt[map[k] + 1]++;
    for (uint32_t d = 0; d < n_dofs; d++) cnt[d + 1] += cnt[d];
    std::vector<uint32_t> fill(cnt.begin(), cnt.end() - 1);
    std::vector<uint32_t> d2e(offs[n_elem]);
    for (uint32_t e = 0; e < n_elem; e++)
        for (uint32_t k = offs[e]; k < offs[e + 1]; k++) d2e[fill[map[k]]++] = e;
    colors.assign(n_elem, UINT32_MAX);
    std::vector<uint32_t> used(64, 0);
    uint32_t ncol = n_elem ? 1 : 0;
    for (uint32_t e = 0; e < n_elem; e++) {
        for (uint32_t k = offs[e]; k < offs[e + 1]; k++) {
            const uint32_t d = map[k];
            for (uint32_t j = cnt[d]; j < cnt[d + 1]; j++) {
                const uint32_t f = d2e[j];
                if (f != e && colors[f] != UINT32_MAX) {
                    if (colors[f] >= used.size()) used.resize(colors[f] * 2 + 2, 0);
                    used[colors[f]] = e + 1;
                }
            }
        }
        uint32_t c = 0;
        while (c < used.size() && used[c] == e + 1) c++;
        if (c >= used.size()) used.resize(c * 2 + 2, 0);
        colors[e] = c;
        if (c + 1 > ncol) ncol = c + 1;
    }
    return ncol;
}

template <typename KT>
inline void put_entry(unsigned char* base, size_t idx, double x);
template <>
inline void put_entry<double>(unsigned char* base, size_t idx, double x) {
    reinterpret_cast<double*>(base)[idx] = x;
}
template <>
inline void put_entry<float>(unsigned char* base, size_t idx, double x) {
    reinterpret_cast<float*>(base)[idx] = (float)x;
}
// Split entries: hi = fl32(x) in the unit's hi plane, lo = fl32(x - hi) in
// the lo plane that follows it, so the hi plane alone is the FP32 matrix.
struct SplitPair {};
template <>
inline void put_entry<SplitPair>(unsigned char* base, size_t idx, double x) {
    (void)base, (void)idx, (void)x;  // planar: written by put_split
}
inline void put_split(unsigned char* base, size_t idx, size_t plane, double x) {
    const float h = (float)x;
    const float l = (float)(x - (double)h);
    reinterpret_cast<float*>(base)[idx] = h;
    reinterpret_cast<float*>(base)[idx + plane] = l;
}

// Writes element e (at offset `rel` inside segment s) into the host image of
// the segment's arena chunk starting at chunk_base (unit index u0).
template <typename KT>
void layout_element(const afm_operator* op, const Segment& s, uint32_t e, uint64_t rel, uint64_t u0,
                    unsigned char* chunk) {
    const uint32_t n = s.n;
    const double* k = op->ke.data() + op->kofs[e];
    constexpr bool split = std::is_same<KT, SplitPair>::value;
    if (s.regime == REG_WPE) {
        unsigned char* dst = chunk + (rel - u0) * s.unit_bytes;
        for (uint32_t c = 0; c < n; c++)
            for (uint32_t r = 0; r < n; r++) {
                if (split)
                    put_split(dst, (size_t)c * n + r, s.plane, k[(size_t)r * n + c]);
                else
                    put_entry<KT>(dst, (size_t)c * n + r, k[(size_t)r * n + c]);
            }
    } else {
        const uint64_t unit = rel / kTpeWidth, lane = rel % kTpeWidth;
        unsigned char* dst = chunk + (unit - u0) * s.unit_bytes;
        for (uint32_t r = 0; r < n; r++)
            for (uint32_t c = 0; c < n; c++) {
                const size_t idx = ((size_t)r * n + c) * kTpeWidth + lane;
                if (split)
                    put_split(dst, idx, s.plane, k[(size_t)r * n + c]);
                else
                    put_entry<KT>(dst, idx, k[(size_t)r * n + c]);
            }
    }
}

// Patch plan of the small-element path (afm_patch.cuh). Patches grow
// breadth first over shared DoFs from the lowest unassigned element, up to
// 128 elements and kPatchMaxDofs distinct DoFs; patches get first-fit colours
// in creation order (no two patches of a colour share a DoF). Fills the
// element slots (op->perm, kNoElement for empty slots), one TPE-layout
// segment covering every slot, the patch descriptors and index blocks.
// Returns false (and leaves the operator to the colour-segment path) when the
// patches need more than 64 colours or do not fit the shared memory.
bool build_patch_plan(afm_operator* op, uint32_t n, int prec, std::vector<PatchDesc>& desc,
                      std::vector<unsigned char>& idx) {
    // patch size: 128 elements, or down to 32 on meshes too small to give every SM several patches
    uint32_t P = 128;
    const uint64_t slots = 4ull * (uint64_t)std::max(op->sm_count, 1);
    while (P > 32 && (uint64_t)op->n_elem < slots * P) P /= 2;
    const uint32_t NE = op->n_elem, ND = op->n_dofs;
    const uint32_t* off = op->offsets.data();
    const uint32_t* map = op->map.data();
    // DoF -> elements
    std::vector<uint64_t> doff((size_t)ND + 1, 0);
    for (uint32_t x : op->map) doff[(size_t)x + 1]++;
    for (size_t d = 0; d < ND; d++) doff[d + 1] += doff[d];
    std::vector<uint32_t> del(op->map.size());
    {
        std::vector<uint64_t> pos(doff.begin(), doff.end() - 1);
        for (uint32_t e = 0; e < NE; e++)
            for (uint32_t i = off[e]; i < off[e + 1]; i++) del[pos[map[i]]++] = e;
    }
    // breadth-first patches
    std::vector<int32_t> owner(NE, -1);
    std::vector<uint32_t> dstamp(ND, UINT32_MAX), qstamp(NE, UINT32_MAX), queue;
    std::vector<uint32_t> pel, poff(1, 0);
    pel.reserve(NE);
    uint32_t np = 0;
    for (uint32_t seed = 0; seed < NE; seed++) {
        if (owner[seed] >= 0) continue;
        queue.clear();
        queue.push_back(seed);
        qstamp[seed] = np;
        uint32_t cnt = 0, nd = 0;
        for (size_t h = 0; h < queue.size() && cnt < P; h++) {
            const uint32_t e = queue[h];
            const uint32_t* m = map + off[e];
            uint32_t add = 0;
            for (uint32_t i = 0; i < n; i++) add += (dstamp[m[i]] != np);
            if (nd + add > kPatchMaxDofs) continue;
            owner[e] = (int32_t)np;
            cnt++;
            nd += add;
            pel.push_back(e);
            for (uint32_t i = 0; i < n; i++) dstamp[m[i]] = np;
            for (uint32_t i = 0; i < n; i++)
                for (uint64_t k = doff[m[i]]; k < doff[(size_t)m[i] + 1]; k++) {
                    const uint32_t f = del[k];
                    if (owner[f] < 0 && qstamp[f] != np) {
                        qstamp[f] = np;
                        queue.push_back(f);
                    }
                }
        }
        poff.push_back((uint32_t)pel.size());
        np++;
    }
    // first-fit patch colours
    std::vector<uint64_t> dmask(ND, 0);
    std::vector<uint32_t> pcol(np);
    uint32_t ncol = 0;
    for (uint32_t q = 0; q < np; q++) {
        uint64_t forb = 0;
        for (uint32_t k = poff[q]; k < poff[q + 1]; k++)
            for (uint32_t i = off[pel[k]]; i < off[pel[k] + 1]; i++) forb |= dmask[map[i]];
        if (forb == ~0ull) return false;
        const uint32_t c = (uint32_t)__builtin_ctzll(~forb);
        pcol[q] = c;
        ncol = std::max(ncol, c + 1);
        for (uint32_t k = poff[q]; k < poff[q + 1]; k++)
            for (uint32_t i = off[pel[k]]; i < off[pel[k] + 1]; i++) dmask[map[i]] |= 1ull << c;
    }
    std::vector<uint32_t> order(np);
    std::iota(order.begin(), order.end(), 0u);
    std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) { return pcol[a] < pcol[b]; });
    op->patch_color_first.assign(ncol + 1, 0);
    for (uint32_t q = 0; q < np; q++) op->patch_color_first[pcol[q] + 1]++;
    for (uint32_t c = 0; c < ncol; c++) op->patch_color_first[c + 1] += op->patch_color_first[c];

    // sizes: local DoFs, units and index bytes per patch (colour order)
    auto local_dofs = [&](uint32_t q, std::vector<uint32_t>& ld) {
        ld.clear();
        for (uint32_t k = poff[q]; k < poff[q + 1]; k++)
            for (uint32_t i = off[pel[k]]; i < off[pel[k] + 1]; i++) ld.push_back(map[i]);
        std::sort(ld.begin(), ld.end());
        ld.erase(std::unique(ld.begin(), ld.end()), ld.end());
    };
    desc.assign(np, PatchDesc{});
#pragma omp parallel
    {
        std::vector<uint32_t> ld;
#pragma omp for schedule(dynamic, 64)
        for (int64_t x = 0; x < (int64_t)np; x++) {
            const uint32_t q = order[x];
            local_dofs(q, ld);
            PatchDesc& d = desc[x];
            d.elems = poff[q + 1] - poff[q];
            d.units = (d.elems + 31) / 32;
            d.ndof = (uint32_t)ld.size();
            d.idx_bytes = patch_slot_off(d.ndof, d.units, n) + patch_r16(d.elems * n * 2);
        }
    }
    const size_t eb = entry_bytes(prec);
    Segment s;
    s.color = 0;
    s.n = n;
    s.regime = REG_TPE;
    s.first_pos = 0;
    s.unit_bytes = round16((uint64_t)n * n * eb * kTpeWidth);
    if (prec == AFM_PREC_FP64_SPLIT) {
        s.plane = n * n * kTpeWidth;
        s.unit_bytes = 2ull * s.plane * 4;
    }
    PatchPlanGeom& G = op->patch_geom;
    G = PatchPlanGeom{};
    G.n = n;
    uint64_t units = 0, ib = 0;
    uint64_t pv = 0;
    for (PatchDesc& d : desc) {
        d.unit0 = (uint32_t)units;
        d.pv_off = (uint32_t)pv;
        pv += d.ndof;
        d.ke_off = units * s.unit_bytes;
        d.idx_off = ib;
        units += d.units;
        ib += d.idx_bytes;
        G.max_slots = std::max(G.max_slots, d.units * 32);
        G.max_ndof = std::max(G.max_ndof, d.ndof);
        G.max_idx = std::max(G.max_idx, d.idx_bytes);
    }
    if (patch_smem_bytes(prec, G, (uint32_t)s.unit_bytes) == 0) return false;
    if (pv > 0xffffffffull || ND > kPatchDofMask) return false;
    s.units = (uint32_t)units;
    s.count = (uint32_t)(units * kTpeWidth);
    s.ke_offset = 0;
    s.map_offset = 0;

    // DoFs that more than one patch lists: their patch sums are combined in a
    // second pass (one-launch mode); the others are written straight to v
    std::vector<uint32_t> npatch(ND, 0);
    {
        std::vector<uint32_t> ld;
        for (uint32_t x = 0; x < np; x++) {
            local_dofs(order[x], ld);
            for (uint32_t g : ld) npatch[g]++;
        }
    }
    // element slots and index blocks
    std::vector<uint8_t> is_bc(ND, 0);
    for (uint32_t d : op->bc_unique) is_bc[d] = 1;
    op->perm.assign((size_t)units * kTpeWidth, kNoElement);
    idx.assign(ib, 0);
#pragma omp parallel
    {
        std::vector<uint32_t> ld, cntd;
#pragma omp for schedule(dynamic, 64)
        for (int64_t x = 0; x < (int64_t)np; x++) {
            const uint32_t q = order[x];
            const PatchDesc& d = desc[x];
            local_dofs(q, ld);
            const uint64_t slot0 = d.ke_off / s.unit_bytes * kTpeWidth;
            for (uint32_t el = 0; el < d.elems; el++) op->perm[slot0 + el] = pel[poff[q] + el];
            unsigned char* blk = idx.data() + d.idx_off;
            uint32_t* glob = reinterpret_cast<uint32_t*>(blk);
            uint16_t* lmap = reinterpret_cast<uint16_t*>(blk + patch_lmap_off(d.ndof));
            uint16_t* coff = reinterpret_cast<uint16_t*>(blk + patch_csr_off(d.ndof, d.units, n));
            uint16_t* slot = reinterpret_cast<uint16_t*>(blk + patch_slot_off(d.ndof, d.units, n));
            for (uint32_t k = 0; k < d.ndof; k++)
                glob[k] = ld[k] | (is_bc[ld[k]] ? kBcFlag : 0u) | (npatch[ld[k]] > 1 ? kSharedFlag : 0u);
            auto loc = [&](uint32_t g) {
                return (uint32_t)(std::lower_bound(ld.begin(), ld.end(), g) - ld.begin());
            };
            cntd.assign(d.ndof + 1, 0);
            for (uint32_t el = 0; el < d.elems; el++) {
                const uint32_t* m = map + off[pel[poff[q] + el]];
                const uint32_t un = el / 32, lane = el % 32;
                for (uint32_t c = 0; c < n; c++) {
                    const uint32_t l = loc(m[c]);
                    lmap[((size_t)un * n + c) * 32 + lane] = (uint16_t)l;
                    cntd[l + 1]++;
                }
            }
            for (uint32_t k = 0; k < d.ndof; k++) cntd[k + 1] += cntd[k];
            for (uint32_t k = 0; k <= d.ndof; k++) coff[k] = (uint16_t)cntd[k];
            const uint32_t cap = d.units * 32;
            for (uint32_t el = 0; el < d.elems; el++) {
                const uint32_t* m = map + off[pel[poff[q] + el]];
                for (uint32_t r = 0; r < n; r++) slot[cntd[loc(m[r])]++] = (uint16_t)(r * cap + el);
            }
        }
    }
    // combine lists: per shared DoF (ascending), its entries pv_off + local index in patch order, which
    // is colour order, so the sums are added in the order of the one-launch-per-colour mode
    op->pv_count = pv;
    op->shared_dof.clear();
    op->shared_off.assign(1, 0);
    op->shared_idx.clear();
    {
        std::vector<uint32_t> first((size_t)ND + 1, 0);
        for (uint32_t g = 0; g < ND; g++)
            if (npatch[g] > 1) {
                op->shared_dof.push_back(g);
                first[g + 1] = npatch[g];
            }
        for (uint32_t g = 0; g < ND; g++) first[g + 1] += first[g];
        op->shared_idx.assign(first[ND], 0);
        std::vector<uint32_t> fill(first.begin(), first.end() - 1);
        std::vector<uint32_t> ld;
        for (uint32_t x = 0; x < np; x++) {
            local_dofs(order[x], ld);
            for (uint32_t k = 0; k < (uint32_t)ld.size(); k++)
                if (npatch[ld[k]] > 1) op->shared_idx[fill[ld[k]]++] = desc[x].pv_off + k;
        }
        for (uint32_t g : op->shared_dof) op->shared_off.push_back(first[g + 1]);
    }
    op->n_shared = (uint32_t)op->shared_dof.size();
    op->segs.assign(1, s);
    op->n_patches = np;
    return true;
}

// Colour-sorted element order (colour, then element size) and one segment
// per (colour, size) with its arena and map offsets.
void build_segments(afm_operator* op, int prec) {
    op->perm.resize(op->n_elem);
    std::iota(op->perm.begin(), op->perm.end(), 0u);
    std::stable_sort(op->perm.begin(), op->perm.end(), [&](uint32_t a, uint32_t b) {
        if (op->colors[a] != op->colors[b]) return op->colors[a] < op->colors[b];
        const uint32_t na = op->offsets[a + 1] - op->offsets[a], nb = op->offsets[b + 1] - op->offsets[b];
        return na < nb;
    });

    op->segs.clear();
    const size_t eb = entry_bytes(prec);
    uint64_t ke_off = 0, map_off = 0;
    for (uint32_t p = 0; p < op->n_elem;) {
        const uint32_t e = op->perm[p];
        Segment s;
        s.color = op->colors[e];
        s.n = op->offsets[e + 1] - op->offsets[e];
        s.regime = (s.n <= kTpeMaxN) ? REG_TPE : REG_WPE;
        s.first_pos = p;
        uint32_t q = p;
        while (q < op->n_elem) {
            const uint32_t f = op->perm[q];
            if (op->colors[f] != s.color || op->offsets[f + 1] - op->offsets[f] != s.n) break;
            q++;
        }
        s.count = q - p;
        if (s.regime == REG_TPE) {
            s.units = (s.count + kTpeWidth - 1) / kTpeWidth;
            s.unit_bytes = round16((uint64_t)s.n * s.n * eb * kTpeWidth);
            if (prec == AFM_PREC_FP64_SPLIT) {
                s.plane = s.n * s.n * kTpeWidth;
                s.unit_bytes = 2ull * s.plane * 4;
            }
        } else {
            s.units = s.count;
            s.unit_bytes = round16((uint64_t)s.n * s.n * eb);
            if (prec == AFM_PREC_FP64_SPLIT) {
                s.plane = (s.n * s.n + 3) / 4 * 4;  // 16-byte aligned planes
                s.unit_bytes = 2ull * s.plane * 4;
            }
        }
        s.ke_offset = ke_off;
        s.map_offset = map_off;
        ke_off += s.unit_bytes * s.units;
        map_off += (uint64_t)s.units * (s.regime == REG_TPE ? kTpeWidth : 1) * s.n;
        map_off = (map_off + 3) / 4 * 4;  // keep 16-byte alignment of each segment's map
        op->segs.push_back(s);
        p = q;
    }
    op->ke_bytes = ke_off;
    op->map_bytes = map_off * sizeof(uint32_t);
}

// True when every element matrix is symmetric to within 1e-6 of its largest
// diagonal entry (exactly, for an element whose diagonal is zero).
bool ke_is_symmetric(const afm_operator* op) {
    int sym = 1;
#pragma omp parallel for schedule(static) reduction(&& : sym)
    for (int64_t e = 0; e < (int64_t)op->n_elem; e++) {
        if (!sym) continue;
        const uint32_t n = op->offsets[e + 1] - op->offsets[e];
        const double* k = op->ke.data() + op->kofs[e];
        double dmax = 0.0;
        for (uint32_t r = 0; r < n; r++) dmax = std::max(dmax, std::fabs(k[(size_t)r * n + r]));
        const double tol = 1e-6 * dmax;
        for (uint32_t r = 0; r < n && sym; r++)
            for (uint32_t c = r + 1; c < n; c++)
                if (!(std::fabs(k[(size_t)r * n + c] - k[(size_t)c * n + r]) <= tol)) {
                    sym = 0;
                    break;
                }
    }
    return sym != 0;
}

// Layout of the symmetric inner arena in format `mode` (1: FP32, 2: FP32 +
// BF16 correction plane): patch units hold the packed triangle of 32 element
// slots (S = n (n + 1) / 2 x 32 entries), element units the n/2 + 1 wrapped
// diagonals (S = (n/2 + 1) n); the correction plane follows the FP32 plane
// at a 16-byte boundary.
void layout_sym(afm_operator* op, int mode) {
    uint64_t off = 0;
    for (Segment& s : op->segs) {
        const uint64_t S = s.regime == REG_TPE ? (uint64_t)s.n * (s.n + 1) / 2 * kTpeWidth
                                               : (uint64_t)(s.n / 2 + 1) * s.n;
        const uint64_t P = (S + 3) / 4 * 4;
        s.sym_plane = mode == 2 ? (uint32_t)P : 0;
        s.sym_unit_bytes = mode == 2 ? round16(P * 4 + S * 2) : round16(S * 4);
        s.sym_offset = off;
        off += s.sym_unit_bytes * s.units;
    }
    op->sym_bytes = off;
}

// Format of the symmetric inner arena the operator's FP32 products use (0:
// none, they read the hi plane).
int sym_format(const afm_operator* op) { return op->sym_ok ? op->sym_mode : 0; }

// The arena the format needs: formats 3 to 5 (FP64 inner vectors) read the
// corrected arena of format 2.
int sym_arena(const afm_operator* op) {
    const int f = sym_format(op);
    return f >= 3 ? 2 : f;
}

// Builds the symmetric inner arena in the operator's format on its stream
// (once per format); work enqueued afterwards on `st` is ordered after it.
// Call outside stream capture.
int ensure_sym(afm_operator* op, cudaStream_t st) {
    const int fmt = sym_arena(op);
    if (!fmt) return AFM_SUCCESS;
    if (op->d_sym && op->sym_built == fmt) return AFM_SUCCESS;
    dfree(op, op->d_sym);
    dfree(op, op->d_vx);
    op->sym_built = 0;
    layout_sym(op, fmt);
    if (fmt == 2) AFM_CUDA(dalloc(op, &op->d_vx, sizeof(double) * std::max<uint32_t>(op->n_dofs, 1)));
    AFM_CUDA(dalloc(op, &op->d_sym, op->sym_bytes));
    AFM_CUDA(cudaMemsetAsync(op->d_sym, 0, op->sym_bytes, op->stream));
    for (const Segment& s : op->segs) {
        const cudaError_t e = build_sym_segment(s, op->d_ke, op->d_sym, op->sm_count, op->stream);
        if (e != cudaSuccess) {
            dfree(op, op->d_sym);
            return fail(AFM_ERR_CUDA, "symmetric arena: %s", cudaGetErrorString(e));
        }
    }
    op->sym_built = fmt;
    op->generation++;  // captured FP32 iterations switch to the new arena
    if (st != op->stream) {
        cudaEvent_t ev;
        AFM_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
        cudaEventRecord(ev, op->stream);
        cudaStreamWaitEvent(st, ev, 0);
        cudaEventDestroy(ev);
    }
    return AFM_SUCCESS;
}

int upload_arena(afm_operator* op) {
    // staging in pinned memory, chunks of up to 256 MB of whole units (no more
    // than the arena: pinning is slow and small operators need little)
    uint64_t largest = 0;
    for (const Segment& s : op->segs) largest = std::max<uint64_t>(largest, s.unit_bytes);
    const size_t kChunk = (size_t)std::max<uint64_t>(std::min<uint64_t>(256ull << 20, op->ke_bytes), largest);
    unsigned char* stage = nullptr;
    if (kChunk == 0) return AFM_SUCCESS;
    AFM_CUDA(cudaMallocHost((void**)&stage, kChunk));
    int status = AFM_SUCCESS;
    for (const Segment& s : op->segs) {
        if (s.units == 0) continue;
        const uint64_t units_per_chunk = std::max<uint64_t>(1, kChunk / s.unit_bytes);
        if (s.unit_bytes > kChunk) {
            status = fail(AFM_ERR_INVALID_ARG, "element matrix larger than staging chunk");
            break;
        }
        for (uint64_t u0 = 0; u0 < s.units; u0 += units_per_chunk) {
            const uint64_t u1 = std::min<uint64_t>(s.units, u0 + units_per_chunk);
            const size_t bytes = (size_t)((u1 - u0) * s.unit_bytes);
            // the previous chunk's copy must finish before the buffer is reused
            cudaError_t e = cudaStreamSynchronize(op->stream);
            if (e != cudaSuccess) {
                status = fail(AFM_ERR_CUDA, "upload: %s", cudaGetErrorString(e));
                break;
            }
            memset(stage, 0, bytes);
            const uint64_t el0 = (s.regime == REG_WPE) ? u0 : u0 * kTpeWidth;
            const uint64_t el1 = std::min<uint64_t>(s.count, (s.regime == REG_WPE) ? u1 : u1 * kTpeWidth);
#pragma omp parallel for schedule(static)
            for (int64_t rel = (int64_t)el0; rel < (int64_t)el1; rel++) {
                const uint32_t e = op->perm[s.first_pos + rel];
                if (e == kNoElement) continue;  // empty slot of a patch
                if (op->precision == AFM_PREC_FP64)
                    layout_element<double>(op, s, e, rel, u0, stage);
                else if (op->precision == AFM_PREC_FP64_SPLIT)
                    layout_element<SplitPair>(op, s, e, rel, u0, stage);
                else
                    layout_element<float>(op, s, e, rel, u0, stage);
            }
            e = cudaMemcpyAsync(op->d_ke + s.ke_offset + u0 * s.unit_bytes, stage, bytes, cudaMemcpyHostToDevice,
                                op->stream);
            if (e != cudaSuccess) {
                status = fail(AFM_ERR_CUDA, "upload: %s", cudaGetErrorString(e));
                break;
            }
        }
        if (status != AFM_SUCCESS) break;
    }
    cudaStreamSynchronize(op->stream);
    cudaFreeHost(stage);
    return status;
}

int ensure_work(afm_operator* op, size_t vectors) {
    const size_t need = vectors * (size_t)std::max<uint32_t>(op->n_dofs, 1);
    if (op->work_elems >= need) return AFM_SUCCESS;
    dfree(op, op->d_work);
    op->work_elems = 0;
    AFM_CUDA(dalloc(op, &op->d_work, need * sizeof(double)));
    op->work_elems = need;
    return AFM_SUCCESS;
}

int ensure_work64i(afm_operator* op, size_t vectors) {
    const size_t need = vectors * (size_t)std::max<uint32_t>(op->n_dofs, 1);
    if (op->work64i_elems >= need) return AFM_SUCCESS;
    dfree(op, op->d_work64i);
    op->work64i_elems = 0;
    AFM_CUDA(dalloc(op, &op->d_work64i, need * sizeof(double)));
    op->work64i_elems = need;
    return AFM_SUCCESS;
}

int ensure_work32(afm_operator* op, size_t vectors) {
    const size_t need = vectors * (size_t)std::max<uint32_t>(op->n_dofs, 1);
    if (op->work32_elems >= need) return AFM_SUCCESS;
    dfree(op, op->d_work32);
    op->work32_elems = 0;
    AFM_CUDA(dalloc(op, &op->d_work32, need * sizeof(float)));
    op->work32_elems = need;
    return AFM_SUCCESS;
}

int check_device_error(afm_operator* op) {
    int h[kErrWords] = {0};
    AFM_CUDA(cudaMemcpyAsync(h, op->d_err, sizeof(h), cudaMemcpyDeviceToHost, op->stream));
    AFM_CUDA(cudaStreamSynchronize(op->stream));
    if (h[0]) cudaMemsetAsync(op->d_err, 0, sizeof(h), op->stream);
    if (h[0] & kErrBounds)
        return fail(AFM_ERR_INTERNAL, "device bounds check %d failed (block %d, thread %d: %d %d %d)", h[1], h[2],
                    h[3], h[4], h[5], h[6]);
    if (h[0] & kErrTimeout) return fail(AFM_ERR_TIMEOUT, "a device wait exceeded its time limit");
    return AFM_SUCCESS;
}

// v = K u (bc_mode 0) or the product of MatMult_mf without the final v_c = u_c
// (bc_mode 1: constrained columns of u read as zero), device arrays.
// Matrix-free product (method 2): one launch per colour.
int enqueue_free(afm_operator* op, void* d_v, const void* d_u, int bc_mode, cudaStream_t st, bool f32) {
    AFM_CUDA(cudaMemsetAsync(d_v, 0, (size_t)op->n_dofs * (f32 ? 4 : 8), st));
    const double E = op->elem_E, nu = op->elem_nu;
    FreeArgs a;
    a.xe = f32 ? (const void*)op->d_free_xe32 : (const void*)op->d_free_xe64;
    a.map = op->d_map;
    a.ref = f32 ? (const void*)op->d_free_ref32 : (const void*)op->d_free_ref64;
    a.u = d_u;
    a.v = d_v;
    a.nq = op->free_nq;
    a.bc_mode = bc_mode;
    a.lam = E * nu / (1.0 + nu) / (1.0 - 2.0 * nu);
    a.mu = 0.5 * E / (1.0 + nu);
    for (size_t c = 0; c + 1 < op->free_color_first.size(); c++) {
        a.first = op->free_color_first[c];
        a.count = op->free_color_first[c + 1] - a.first;
        AFM_CUDA(launch_free(op->elem_kind, f32, a, op->sm_count, st));
    }
    return AFM_SUCCESS;
}

int enqueue_matvec(afm_operator* op, void* d_v, const void* d_u, int bc_mode, cudaStream_t st, bool f32 = false,
                   bool inner64 = false) {
    if (op->matfree_type == 2) return enqueue_free(op, d_v, d_u, bc_mode, st, f32);
    // f32: FP32 product on float vectors, from the symmetric inner arena once
    // built, else from an FP32 arena or the hi plane of a split arena (half of
    // each unit is copied). inner64: FP64 vectors on the corrected symmetric
    // arena (it must be built): format 3, double-float products of the FP64 u;
    // format 4, the products of format 2 on u rounded to FP32, summed into v
    // in FP64; format 5, as 4 with the element rows summed in plain FP32.
    const bool sym = (f32 || inner64) && op->d_sym != nullptr;
    const bool symx = sym && op->sym_built == 2;
    if (inner64 && !symx) return fail(AFM_ERR_STATE, "FP64 inner product without the corrected symmetric arena");
    const bool inner_f32u = inner64 && sym_format(op) >= 4;
    if (inner_f32u) {
        if (op->work64i_elems < 8ull * op->n_dofs) return fail(AFM_ERR_STATE, "format 4 product without its buffer");
        float* u32 = reinterpret_cast<float*>(op->d_work64i + 7ull * op->n_dofs);
        AFM_CUDA(launch_to_f32(u32, static_cast<const double*>(d_u), op->n_dofs, st));
        d_u = u32;
    }
    const int kprec = inner64 ? (inner_f32u ? (sym_format(op) == 5 ? kPrecF32SymC : kPrecF32SymX) : kPrecSplitSymX)
                              : sym ? (symx ? kPrecF32SymX : kPrecF32Sym) : f32 ? AFM_PREC_FP32 : op->precision;
    const size_t vbytes = (size_t)op->n_dofs * (f32 || kprec == AFM_PREC_FP32 ? 4 : 8);
    // the corrected format's FP32 products sum into an FP64 vector, rounded to FP32 at the end
    const bool via_vx = symx && !inner64;
    float* const d_v32 = static_cast<float*>(d_v);
    if (via_vx) d_v = op->d_vx;
    // split arithmetic: max|u| for the launches' power-of-two u scale (and v = 0) in one launch, before
    // the first element launch, which waits for it in full; other arithmetic: v = 0
    const bool scaled = kprec == AFM_PREC_FP64_SPLIT || kprec == kPrecSplitSymX;
    if (scaled)
        AFM_CUDA(launch_umax(static_cast<const double*>(d_u), bc_mode ? op->d_bcmask : nullptr, op->n_dofs,
                             static_cast<double*>(d_v), op->n_dofs, op->d_usc, st));
    else
        AFM_CUDA(cudaMemsetAsync(d_v, 0, via_vx ? (size_t)op->n_dofs * 8 : vbytes, st));
    bool first = true;
    if (op->use_patches) {
        const Segment& s = op->segs[0];
        // one launch over every patch plus the combine pass, or one launch per patch colour
        const bool one = op->patch_one_launch;
        const size_t launches = one ? 1 : op->patch_color_first.size() - 1;
        for (size_t c = 0; c < launches; c++) {
            PatchArgs a;
            a.desc = op->d_patch_desc + (one ? 0 : op->patch_color_first[c]);
            a.count = one ? op->n_patches : op->patch_color_first[c + 1] - op->patch_color_first[c];
            a.pv = one ? (void*)op->d_pv : nullptr;
            a.ke = sym ? op->d_sym : op->d_ke;
            a.idx = op->d_patch_idx;
            a.u = d_u;
            a.v = d_v;
            a.unit_bytes = sym ? s.sym_unit_bytes : s.unit_bytes;
            a.copy_bytes = (uint32_t)a.unit_bytes;
            a.plane = sym ? s.sym_plane : s.plane;
            if (f32 && !sym && op->precision == AFM_PREC_FP64_SPLIT) a.copy_bytes = s.plane * 4;
            a.bc_mode = bc_mode;
            a.err = op->d_err;
            a.umax = op->d_usc;
            a.wait_ns = op->wait_ns;
            a.probe = op->wait_probe ? op->d_err + (kErrWords - 1) : nullptr;
            AFM_CUDA(launch_patches(kprec, op->patch_geom, a, op->sm_count, !first, st));
            first = false;
        }
        if (one)
            AFM_CUDA(launch_patch_combine((f32 && !symx) ? 4 : 8, d_v, op->d_pv, op->d_shared_dof,
                                          op->d_shared_off, op->d_shared_idx, op->n_shared, st));
        if (via_vx) AFM_CUDA(launch_to_f32(d_v32, op->d_vx, op->n_dofs, st));
        return AFM_SUCCESS;
    }
    // split products of a plan with one element size: every colour in one cooperative launch (outside
    // stream capture: captured solve iterations keep the colour launches)
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (op->fused && op->fused_ok && kprec == AFM_PREC_FP64_SPLIT && !sym && !f32 &&
        cudaStreamIsCapturing(st, &cap) == cudaSuccess && cap == cudaStreamCaptureStatusNone) {
        const Segment& s0 = op->segs[0];
        SegArgs a;
        a.ke = op->d_ke;
        a.map = op->d_map;
        a.u = d_u;
        a.v = d_v;
        a.units = s0.units;
        a.count = s0.count;
        a.unit_bytes = s0.unit_bytes;
        a.copy_bytes = (uint32_t)s0.unit_bytes;
        a.plane = s0.plane;
        a.bc_mode = bc_mode;
        a.err = op->d_err;
        a.umax = op->d_usc;
        a.wait_ns = op->wait_ns;
        a.probe = op->wait_probe ? op->d_err + (kErrWords - 1) : nullptr;
        AFM_CUDA(cudaMemsetAsync(op->d_gbar, 0, sizeof(unsigned) * op->segs.size(), st));
        AFM_CUDA(launch_fused_split(op->segs.data(), (uint32_t)op->segs.size(), a, op->d_gbar, op->sm_count, st));
        return AFM_SUCCESS;
    }
    for (const Segment& s : op->segs) {
        if (s.units == 0) continue;
        SegArgs a;
        a.ke = sym ? op->d_sym + s.sym_offset : op->d_ke + s.ke_offset;
        a.map = op->d_map + s.map_offset;
        a.u = d_u;
        a.v = d_v;
        a.units = s.units;
        a.count = s.count;
        a.unit_bytes = sym ? s.sym_unit_bytes : s.unit_bytes;
        a.copy_bytes = (uint32_t)a.unit_bytes;
        a.plane = sym ? s.sym_plane : s.plane;
        if (f32 && !sym && op->precision == AFM_PREC_FP64_SPLIT) a.copy_bytes = s.plane * 4;
        a.bc_mode = bc_mode;
        a.err = op->d_err;
        a.umax = op->d_usc;
        a.wait_ns = op->wait_ns;
        a.probe = op->wait_probe ? op->d_err + (kErrWords - 1) : nullptr;
        // every launch after the first may overlap its prologue with the previous one's tail
        AFM_CUDA(launch_segment(s, kprec, a, op->sm_count, op->dup_in_element, !first, st));
        first = false;
    }
    if (via_vx) AFM_CUDA(launch_to_f32(d_v32, op->d_vx, op->n_dofs, st));
    return AFM_SUCCESS;
}

cudaStream_t pick_stream(afm_operator* op, void* stream) {
    return stream ? (cudaStream_t)stream : op->stream;
}

// ---- batched (multi right-hand side) products ------------------------------

int enqueue_matvec_batched(afm_operator* op, void* d_V, const void* d_U, uint32_t nrhs, uint32_t ld, int bc_mode,
                           cudaStream_t st, bool f32, int tr, int ng) {
    const int kprec = f32 ? AFM_PREC_FP32 : op->precision;
    const size_t vb = (kprec == AFM_PREC_FP32 ? 4 : 8);
    AFM_CUDA(cudaMemsetAsync(d_V, 0, (size_t)op->n_dofs * ld * vb, st));
    // split arithmetic: max|U(:, j)| of every column for the per-column u scale
    if (kprec == AFM_PREC_FP64_SPLIT)
        AFM_CUDA(launch_umax_cols(static_cast<const double*>(d_U), bc_mode ? op->d_bcmask : nullptr, op->n_dofs,
                                  nrhs, ld, op->d_usc + kUscColsOffset, st));
    bool first = true;
    for (const Segment& s : op->segs) {
        if (s.units == 0) continue;
        BatchArgs a;
        a.ke = op->d_ke + s.ke_offset;
        a.map = op->d_map + s.map_offset;
        a.u = d_U;
        a.v = d_V;
        a.units = s.units;
        a.count = s.count;
        a.unit_bytes = s.unit_bytes;
        a.copy_bytes = (uint32_t)s.unit_bytes;
        a.plane = s.plane;
        if (f32 && op->precision == AFM_PREC_FP64_SPLIT) a.copy_bytes = s.plane * 4;
        a.nrhs = nrhs;
        a.ld = ld;
        a.bc_mode = bc_mode;
        a.err = op->d_err;
        a.n_dofs = op->n_dofs;
        a.umax = op->d_usc + kUscColsOffset;
        a.wait_ns = op->wait_ns;
        a.probe = op->wait_probe ? op->d_err + (kErrWords - 1) : nullptr;
        cudaError_t e;
        if (kprec == AFM_PREC_FP64)
            e = launch_batched_fp64(s, a, op->sm_count, tr, ng, !first, st);
        else if (kprec == AFM_PREC_FP64_SPLIT)
            e = launch_batched_split(s, a, op->sm_count, tr, ng, !first, st);
        else if (tr == 0)  // the tensor-core kernel
            e = launch_batched_tc(s, a, op->sm_count, !first, st);
        else
            e = launch_batched_fp32(s, a, op->sm_count, tr, ng, !first, st);
        if (e != cudaSuccess) return fail(AFM_ERR_CUDA, "batched launch (n=%u, tr=%d, ng=%d): %s", s.n, tr, ng,
                                          cudaGetErrorString(e));
        first = false;
    }
    return AFM_SUCCESS;
}

int check_batched(afm_operator* op, uint32_t nrhs, uint32_t ld) {
    if (!op->finalized) return fail(AFM_ERR_STATE, "batched product before finalize");
    if (op->matfree_type == 2) return fail(AFM_NOT_IMPLEMENTED, "batched product of a matrix-free (method 2) operator");
    if (nrhs == 0 || nrhs > 256 || nrhs % 4 != 0 || ld < nrhs || ld % 4 != 0)
        return fail(AFM_ERR_INVALID_ARG, "nrhs %u (multiple of 4, <= 256), ld %u (>= nrhs, multiple of 4)", nrhs, ld);
    for (const Segment& s : op->segs)
        if (s.units && s.regime != REG_WPE)
            return fail(AFM_NOT_IMPLEMENTED, "batched product needs elements with more than %u DoFs", kTpeMaxN);
    if (op->dup_in_element) return fail(AFM_NOT_IMPLEMENTED, "batched product with a DoF listed twice in an element");
    return AFM_SUCCESS;
}

// Every segment of the operator can run the tensor-core FP32 kernel for nrhs.
bool batched_tc_all(afm_operator* op, uint32_t nrhs) {
    for (const Segment& s : op->segs)
        if (s.units && !batched_tc_supported(s.n, nrhs)) return false;
    return true;
}

// The project's autotuner: the first batched call for (nrhs, ld, arithmetic)
// times every (columns per thread tile, element groups per CTA) candidate on
// the caller's data, three runs each, and keeps the fastest for the operator.
// allow_tc = false leaves the tensor-core kernel out: the mixed block CG's
// FP32 recursion takes the CUDA-core kernels, whose products are IEEE FP32
// (the 3xTF32 products drop the lo x lo term and accumulate in the tensor
// pipe; on hex20 elasticity they raised the inner iterations by 58% and cost
// more time than the faster product saved). Its choice is kept under its own key.
int batch_tuning(afm_operator* op, void* d_V, const void* d_U, uint32_t nrhs, uint32_t ld, bool f32, cudaStream_t st,
                 int* tr, int* ng, bool allow_tc = true) {
    const int kprec = f32 ? AFM_PREC_FP32 : op->precision;
    const uint64_t key = ((uint64_t)nrhs << 40) | ((uint64_t)ld << 8) | (uint64_t)kprec | (allow_tc ? 0u : 0x80u);
    for (const auto& t : op->batch_tune)
        if (t.key == key) {
            *tr = t.tr;
            *ng = t.ng;
            return AFM_SUCCESS;
        }
    // (columns, rows) of the lane tile; (0, 0): the tensor-core kernel (FP32 products)
    std::vector<std::pair<int, int>> cand = {{8, 6}, {8, 4}, {8, 2}, {4, 4}};
    if (f32 && allow_tc && batched_tc_all(op, nrhs)) cand.insert(cand.begin(), {0, 0});
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = 1e30f;
    int btr = 4, bng = 2;
    for (auto c : cand) {
        if (c.first != 0 && nrhs % (uint32_t)c.first) continue;  // a lane tile must divide the columns
        int s = enqueue_matvec_batched(op, d_V, d_U, nrhs, ld, 0, st, f32, c.first, c.second);  // warm-up
        if (s) {
            g_last_error.clear();
            continue;
        }
        enqueue_matvec_batched(op, d_V, d_U, nrhs, ld, 0, st, f32, c.first, c.second);  // a second warm-up
        cudaEventRecord(e0, st);
        for (int r = 0; r < 3; r++) enqueue_matvec_batched(op, d_V, d_U, nrhs, ld, 0, st, f32, c.first, c.second);
        cudaEventRecord(e1, st);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best) {
            best = ms;
            btr = c.first;
            bng = c.second;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (best >= 1e30f) return fail(AFM_ERR_CUDA, "no batched kernel configuration runs");
    op->batch_tune.push_back({key, btr, bng, best / 3.0f});
    *tr = btr;
    *ng = bng;
    return AFM_SUCCESS;
}

template <typename T>
int batched_product(afm_operator* op, T* d_V, const T* d_U, uint32_t nrhs, uint32_t ld, int bc_mode, void* stream) {
    const bool f32 = std::is_same<T, float>::value;
    int s = check_batched(op, nrhs, ld);
    if (s) return s;
    if (f32 && op->precision != AFM_PREC_FP32 && op->precision != AFM_PREC_FP64_SPLIT)
        return fail(AFM_ERR_STATE, "FP32 product needs an FP32 or FP64_SPLIT operator");
    if (!f32 && op->precision == AFM_PREC_FP32) return fail(AFM_ERR_STATE, "FP32 operator: use the _f32 entry");
    if (!d_V || !d_U || (const void*)d_V == (const void*)d_U) return fail(AFM_ERR_INVALID_ARG, "bad blocks");
    if (((uintptr_t)d_V | (uintptr_t)d_U) % 16) return fail(AFM_ERR_INVALID_ARG, "blocks must be 16-byte aligned");
    DeviceGuard g(op->device);
    cudaStream_t st = pick_stream(op, stream);
    int tr = 4, ng = 2;
    s = batch_tuning(op, d_V, d_U, nrhs, ld, f32, st, &tr, &ng);
    if (s) return s;
    s = enqueue_matvec_batched(op, d_V, d_U, nrhs, ld, bc_mode, st, f32, tr, ng);
    if (s) return s;
    if (bc_mode) AFM_CUDA(launch_bset_constrained(d_V, d_U, op->d_bc_idx, op->n_bc, ld, nrhs, st));
    return ok();
}

int ensure_bwork(afm_operator* op, size_t doubles) {
    if (op->bwork_elems >= doubles) return AFM_SUCCESS;
    dfree(op, op->d_bwork);
    op->bwork_elems = 0;
    AFM_CUDA(dalloc(op, &op->d_bwork, doubles * sizeof(double)));
    op->bwork_elems = doubles;
    return AFM_SUCCESS;
}

int ensure_bscalars(afm_operator* op, uint32_t nrhs) {
    const size_t need = (size_t)nrhs * kBSlots + (size_t)kBBlocks * nrhs * 3;
    if (op->bsc_elems < need) {
        dfree(op, op->d_bsc);
        op->bsc_elems = 0;
        AFM_CUDA(dalloc(op, &op->d_bsc, need * sizeof(double)));
        op->bsc_elems = need;
    }
    if (!op->d_bremain) AFM_CUDA(dalloc(op, &op->d_bremain, sizeof(unsigned int)));
    if (!op->h_bremain) AFM_CUDA(cudaMallocHost((void**)&op->h_bremain, sizeof(unsigned int)));
    return AFM_SUCCESS;
}

template <typename T>
struct BVectors {
    T *r, *z, *p, *q, *dinv, *x;
};

// Batched CG iterations after launch_bcg_init, as captured graphs of `batch`
// steps; stops when the device counts no column still iterating.
template <typename T>
int run_bcg(afm_operator* op, const BVectors<T>& V, uint32_t R, double maxit, int tr, int ng, int* iters,
            bool* breakdown = nullptr) {
    cudaStream_t st = op->stream;
    const size_t n = op->n_dofs;
    double* sc = op->d_bsc;
    double* part = op->d_bsc + (size_t)R * kBSlots;
    unsigned int* remaining = op->d_bremain;
    const bool f32 = std::is_same<T, float>::value;
    const int batch = 4;
    auto step = [&]() -> int {
        int s = enqueue_matvec_batched(op, V.q, V.p, R, R, 1, st, f32, tr, ng);
        if (s) return s;
        AFM_CUDA(launch_bset_constrained(V.q, V.p, op->d_bc_idx, op->n_bc, R, R, st));
        AFM_CUDA(launch_bcg_step_scalars(V.p, V.q, n, R, R, sc, part, st));
        AFM_CUDA(launch_bcg_update(V.x, V.r, V.z, V.p, V.q, V.dinv, n, R, R, sc, part, maxit, remaining, st));
        return AFM_SUCCESS;
    };
    afm_operator::CgGraph& gc = f32 ? op->bcg32 : op->bcg64;
    const void* key[6] = {V.r, V.x, V.q, (const void*)(uintptr_t)R, (const void*)(uintptr_t)(tr * 16 + ng),
                          (const void*)(uintptr_t)maxit};
    bool same = gc.exec && gc.gen == op->generation;
    for (int i = 0; i < 6 && same; i++) same = (gc.key[i] == key[i]);
    if (!same) {
        drop_graph(gc);
        AFM_CUDA(cudaStreamSynchronize(st));
        AFM_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        int s = AFM_SUCCESS;
        for (int i = 0; i < batch && s == AFM_SUCCESS; i++) s = step();
        if (s == AFM_SUCCESS && cudaMemcpyAsync(op->h_bremain, remaining, sizeof(unsigned int),
                                                cudaMemcpyDeviceToHost, st) != cudaSuccess)
            s = fail(AFM_ERR_CUDA, "capture: counter copy");
        cudaGraph_t graph = nullptr;
        const cudaError_t ec = cudaStreamEndCapture(st, &graph);
        if (s != AFM_SUCCESS) {
            if (graph) cudaGraphDestroy(graph);
            return s;
        }
        if (ec != cudaSuccess) return fail(AFM_ERR_CUDA, "stream capture: %s", cudaGetErrorString(ec));
        const cudaError_t ei = cudaGraphInstantiate(&gc.exec, graph, 0);
        cudaGraphDestroy(graph);
        if (ei != cudaSuccess) {
            gc.exec = nullptr;
            return fail(AFM_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(ei));
        }
        gc.batch = batch;
        gc.gen = op->generation;
        for (int i = 0; i < 6; i++) gc.key[i] = key[i];
    }
    for (;;) {
        AFM_CUDA(cudaGraphLaunch(gc.exec, st));
        AFM_CUDA(cudaStreamSynchronize(st));
        if (*op->h_bremain == 0) break;
    }
    std::vector<double> h((size_t)R * kBSlots);
    AFM_CUDA(cudaMemcpy(h.data(), sc, h.size() * sizeof(double), cudaMemcpyDeviceToHost));
    int it = 0;
    bool flag = false;
    for (uint32_t j = 0; j < R; j++) {
        it = std::max(it, (int)h[(size_t)j * kBSlots + B_ITER]);
        flag = flag || h[(size_t)j * kBSlots + B_FLAG] != 0.0;
    }
    *iters = it;
    if (breakdown) *breakdown = flag;
    return AFM_SUCCESS;
}

// max over columns of ||b_j - A x_j|| / ||b_j|| in FP64 (split or FP64 arena)
int batched_residual(afm_operator* op, const double* d_B, const double* d_X, uint32_t R, double* q, double* worst,
                     int tr64, int ng64) {
    cudaStream_t st = op->stream;
    const size_t n = op->n_dofs;
    int s = enqueue_matvec_batched(op, q, d_X, R, R, 1, st, false, tr64, ng64);
    if (s) return s;
    AFM_CUDA(launch_bset_constrained(q, d_X, op->d_bc_idx, op->n_bc, R, R, st));
    AFM_CUDA(launch_axpby(q, d_B, 1.0, -1.0, n * R, st));  // q = b - A x
    double* part = op->d_bsc + (size_t)R * kBSlots;
    AFM_CUDA(launch_bnorm2(q, n, R, R, part, st));
    std::vector<double> hp((size_t)kBBlocks * R), hb((size_t)kBBlocks * R);
    AFM_CUDA(cudaMemcpyAsync(hp.data(), part, hp.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
    AFM_CUDA(launch_bnorm2(d_B, n, R, R, part, st));
    AFM_CUDA(cudaMemcpyAsync(hb.data(), part, hb.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
    AFM_CUDA(cudaStreamSynchronize(st));
    double w = 0.0;
    for (uint32_t j = 0; j < R; j++) {
        double rr = 0.0, bb = 0.0;
        for (int b = 0; b < kBBlocks; b++) {
            rr += hp[(size_t)b * R + j];
            bb += hb[(size_t)b * R + j];
        }
        w = std::max(w, bb > 0 ? std::sqrt(rr / bb) : std::sqrt(rr));
    }
    *worst = w;
    return AFM_SUCCESS;
}


// CG work vectors: residual r, preconditioned z, direction p, product q,
// inverse diagonal, iterate x.
template <typename T>
struct CgVectors {
    T *r, *z, *p, *q, *dinv, *x;
};

template <typename T>
int cg_step(afm_operator* op, const CgVectors<T>& V, cudaStream_t st);
template <>
int cg_step<double>(afm_operator* op, const CgVectors<double>& V, cudaStream_t st) {
    int s = enqueue_matvec(op, V.q, V.p, 1, st);
    if (s) return s;
    AFM_CUDA(launch_set_constrained(V.q, V.p, op->d_bc_idx, op->n_bc, st));
    double* sc = op->d_scalars;
    double* part = sc + kScalarSlots;
    AFM_CUDA(launch_cg_alpha(V.p, V.q, op->n_dofs, sc, part, st));
    AFM_CUDA(launch_cg_update(V.x, V.r, V.z, V.p, V.q, V.dinv, op->n_dofs, sc, part, st));
    return AFM_SUCCESS;
}
template <>
int cg_step<float>(afm_operator* op, const CgVectors<float>& V, cudaStream_t st) {
    int s = enqueue_matvec(op, V.q, V.p, 1, st, true);
    if (s) return s;
    AFM_CUDA(launch_set_constrained(V.q, V.p, op->d_bc_idx, op->n_bc, st));
    double* sc = op->d_scalars;
    double* part = sc + kScalarSlots;
    AFM_CUDA(launch_cg_alpha(V.p, V.q, op->n_dofs, sc, part, st));
    AFM_CUDA(launch_cg_update(V.x, V.r, V.z, V.p, V.q, V.dinv, op->n_dofs, sc, part, st));
    return AFM_SUCCESS;
}

// One iteration of the FP64-vector inner recursion (symmetric inner format
// 3): the double-float product of the corrected symmetric arena.
int cg_step_inner64(afm_operator* op, const CgVectors<double>& V, cudaStream_t st) {
    int s = enqueue_matvec(op, V.q, V.p, 1, st, false, true);
    if (s) return s;
    AFM_CUDA(launch_set_constrained(V.q, V.p, op->d_bc_idx, op->n_bc, st));
    double* sc = op->d_scalars;
    double* part = sc + kScalarSlots;
    AFM_CUDA(launch_cg_alpha(V.p, V.q, op->n_dofs, sc, part, st));
    AFM_CUDA(launch_cg_update(V.x, V.r, V.z, V.p, V.q, V.dinv, op->n_dofs, sc, part, st));
    return AFM_SUCCESS;
}

void drop_graph(afm_operator::CgGraph& g) {
    if (g.exec) cudaGraphExecDestroy(g.exec);
    g = afm_operator::CgGraph();
}

// Runs CG iterations after launch_cg_init until the device marks the solve
// done (monitored norm <= tol, maxit iterations, or breakdown). The iterations
// run as a captured CUDA graph of `batch` steps followed by a copy of the
// scalars to the pinned host mirror: one host round trip per batch instead of
// one per iteration. Steps after convergence leave every vector unchanged, so
// the result equals the iteration-by-iteration loop.
// The captured CG iteration batch of gc for the vectors V (re-captured when
// the vectors, the batch size or the operator's device buffers changed). The
// graph ends with a copy of the scalars to the pinned host mirror. The stream
// must be idle.
template <typename T>
int ensure_cg_graph(afm_operator* op, afm_operator::CgGraph& gc, const CgVectors<T>& V, bool inner64 = false) {
    cudaStream_t st = op->stream;
    double* h = op->h_scalars;
    const int batch = op->n_dofs > (1u << 20) ? 4 : 8;
    const void* key[6] = {V.r, V.z, V.p, V.q, V.dinv, V.x};
    bool same = gc.exec && gc.batch == batch && gc.gen == op->generation;
    for (int i = 0; i < 6 && same; i++) same = (gc.key[i] == key[i]);
    if (same) return AFM_SUCCESS;
    drop_graph(gc);
    AFM_CUDA(cudaStreamSynchronize(st));
    AFM_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    int s = AFM_SUCCESS;
    for (int i = 0; i < batch && s == AFM_SUCCESS; i++) {
        if constexpr (std::is_same<T, double>::value)
            s = inner64 ? cg_step_inner64(op, V, st) : cg_step<T>(op, V, st);
        else
            s = cg_step<T>(op, V, st);
    }
    if (s == AFM_SUCCESS &&
        cudaMemcpyAsync(h, op->d_scalars, sizeof(double) * kScalarSlots, cudaMemcpyDeviceToHost, st) != cudaSuccess)
        s = fail(AFM_ERR_CUDA, "capture: scalar copy");
    cudaGraph_t graph = nullptr;
    const cudaError_t ec = cudaStreamEndCapture(st, &graph);
    if (s != AFM_SUCCESS) {
        if (graph) cudaGraphDestroy(graph);
        return s;
    }
    if (ec != cudaSuccess) return fail(AFM_ERR_CUDA, "stream capture: %s", cudaGetErrorString(ec));
    const cudaError_t ei = cudaGraphInstantiate(&gc.exec, graph, 0);
    cudaGraphDestroy(graph);
    if (ei != cudaSuccess) {
        gc.exec = nullptr;
        return fail(AFM_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(ei));
    }
    gc.batch = batch;
    gc.gen = op->generation;
    for (int i = 0; i < 6; i++) gc.key[i] = key[i];
    return AFM_SUCCESS;
}

template <typename T>
int run_cg_iterations(afm_operator* op, afm_operator::CgGraph& gc, const CgVectors<T>& V, double tol, int maxit,
                      int norm_type, int* iters, int* status) {
    cudaStream_t st = op->stream;
    double* h = op->h_scalars;
    const double n0 = std::sqrt(norm_type ? h[S_ZZ] : h[S_RR]);
    *iters = 0;
    if (h[S_FLAG] != 0.0 || std::isnan(n0)) {
        *status = AFM_ERR_BREAKDOWN;
        return AFM_SUCCESS;
    }
    if (n0 <= tol) {
        *status = AFM_SUCCESS;
        return AFM_SUCCESS;
    }
    if (maxit <= 0) {
        *status = AFM_ERR_MAXIT;
        return AFM_SUCCESS;
    }
    // solver controls (device copies of tol, maxit, norm)
    h[S_TOL] = tol;
    h[S_MAXIT] = (double)maxit;
    h[S_NORM] = (double)norm_type;
    AFM_CUDA(cudaMemcpyAsync(op->d_scalars + S_DONE, h + S_DONE, sizeof(double) * (S_NORM - S_DONE + 1),
                             cudaMemcpyHostToDevice, st));
    int s = ensure_cg_graph<T>(op, gc, V);
    if (s) return s;
    for (;;) {
        AFM_CUDA(cudaGraphLaunch(gc.exec, st));
        AFM_CUDA(cudaStreamSynchronize(st));
        if (h[S_DONE] != 0.0) break;
    }
    *iters = (int)h[S_ITER];
    const double nrm = std::sqrt(norm_type ? h[S_ZZ] : h[S_RR]);
    if (h[S_FLAG] != 0.0)
        *status = AFM_ERR_BREAKDOWN;
    else if (nrm <= tol)
        *status = AFM_SUCCESS;
    else
        *status = AFM_ERR_MAXIT;
    return AFM_SUCCESS;
}

// Stopping rule of the FP64 updates of the mixed-precision solves. The
// residual norm of CG is not monotone (it can rise or plateau for a few
// hundred iterations), so a solve stops early only after kIrMaxStall
// consecutive updates without a new smallest FP64 residual; max_outer bounds
// the rest.
constexpr int kIrMaxStall = 10;

// Power of two sigma with sigma x in [0.5, 1) for x > 0 (1 otherwise), its
// exponent clamped so that sigma and 1 / sigma stay normal doubles.
double residual_scale(double x) {
    if (!(x > 0.0) || !std::isfinite(x)) return 1.0;
    int e = 0;
    std::frexp(x, &e);
    e = std::max(-1000, std::min(1000, e));
    return std::ldexp(1.0, -e);
}

bool ir_progress(double rn, double* best, int* stall) {
    if (rn < *best) {
        *best = rn;
        *stall = 0;
        return true;
    }
    return ++*stall < kIrMaxStall;
}

}  // namespace

// ---- resumable mixed-precision solve (afm_mixed.hpp) ------------------------

namespace afm {

namespace {

struct MixedVectors {
    double *r64, *q64;
    float* b32;
    CgVectors<float> V;
    double* b64;         // format 3: the inner right-hand side and vectors in FP64
    CgVectors<double> D;
};

MixedVectors mixed_vectors(afm_operator* op) {
    const size_t n = op->n_dofs;
    float* b32 = op->d_work32;
    double* b64 = op->d_work64i;
    MixedVectors W{op->d_work + 2 * n, op->d_work + 5 * n, b32,
                   CgVectors<float>{b32 + n, b32 + 2 * n, b32 + 3 * n, b32 + 4 * n, b32 + 6 * n, b32 + 5 * n},
                   b64, CgVectors<double>{}};
    if (b64) W.D = CgVectors<double>{b64 + n, b64 + 2 * n, b64 + 3 * n, b64 + 4 * n, b64 + 6 * n, b64 + 5 * n};
    return W;
}

int mixed_record(MixedSolve& m) {
    AFM_CUDA(cudaMemcpyAsync(m.op->h_scalars, m.op->d_scalars, sizeof(double) * kScalarSlots,
                             cudaMemcpyDeviceToHost, m.op->stream));
    AFM_CUDA(cudaEventRecord(m.ev, m.op->stream));
    return AFM_SUCCESS;
}

// FP64 true residual r = b - A x (split arena, MatMult_mf semantics), ||r||^2 into S_PQ
int mixed_residual(MixedSolve& m) {
    afm_operator* op = m.op;
    const MixedVectors W = mixed_vectors(op);
    const size_t n = op->n_dofs;
    cudaStream_t st = op->stream;
    int s = afm_matmult_bc_device(op, W.q64, m.d_x, st);
    if (s) return s;
    AFM_CUDA(cudaMemcpyAsync(W.r64, m.d_b, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
    AFM_CUDA(launch_axpby(W.r64, W.q64, -1.0, 1.0, n, st));
    AFM_CUDA(launch_norm2(W.r64, n, op->d_scalars, op->d_scalars + kScalarSlots, st));
    m.phase = MS_RESID;
    return mixed_record(m);
}

int mixed_finish(MixedSolve& m, int status) {
    m.status = status;
    m.phase = MS_DONE;
    AFM_CUDA(cudaEventRecord(m.e1, m.op->stream));
    return AFM_SUCCESS;
}

// the FP32 segment ended: x += x_s, then the FP64 residual
int mixed_segment_end(MixedSolve& m, int iters, int seg_status) {
    m.inner_total += iters;
    m.fresh = (seg_status == AFM_ERR_BREAKDOWN);
    const MixedVectors W = mixed_vectors(m.op);
    if (m.inner64)
        AFM_CUDA(launch_add_f32(m.d_x, W.D.x, m.op->n_dofs, m.op->stream, 1.0 / m.sigma));
    else
        AFM_CUDA(launch_add_f32(m.d_x, W.V.x, m.op->n_dofs, m.op->stream, 1.0 / m.sigma));
    m.outer++;
    return mixed_residual(m);
}

}  // namespace

int mixed_begin(MixedSolve& m) {
    afm_operator* op = m.op;
    AFM_CHECK_OP(op);
    if (!op->finalized) return fail(AFM_ERR_STATE, "solve before finalize");
    if (op->precision != AFM_PREC_FP64_SPLIT && op->matfree_type != 2)
        return fail(AFM_ERR_STATE, "mixed-precision solve needs an FP64_SPLIT or matrix-free operator");
    if (!m.d_b || !m.d_x) return fail(AFM_ERR_INVALID_ARG, "null vector");
    DeviceGuard g(op->device);
    int s = ensure_work(op, 8);
    if (s) return s;
    m.inner64 = !m.lane && op->matfree_type != 2 && sym_format(op) >= 3;
    s = m.inner64 ? ensure_work64i(op, 8) : ensure_work32(op, 7);
    if (s) return s;
    if (!m.lane) {
        s = ensure_sym(op, op->stream);  // once per operator, before the timed solve
        if (s) return s;
    }
    if (m.inner64 && op->sym_built != 2) return fail(AFM_ERR_STATE, "symmetric inner format 3 needs symmetric Ke");
    AFM_CUDA(cudaEventCreateWithFlags(&m.ev, cudaEventDisableTiming));
    AFM_CUDA(cudaEventCreate(&m.e0));
    AFM_CUDA(cudaEventCreate(&m.e1));
    const MixedVectors W = mixed_vectors(op);
    const size_t n = op->n_dofs;
    cudaStream_t st = op->stream;
    AFM_CUDA(cudaEventRecord(m.e0, st));
    if (m.inner64) {
        AFM_CUDA(launch_invert(W.D.dinv, op->d_diag, n, st));
        AFM_CUDA(cudaMemsetAsync(W.D.x, 0, n * sizeof(double), st));
    } else {
        AFM_CUDA(launch_invert(W.V.dinv, op->d_diag, n, st));
        AFM_CUDA(cudaMemsetAsync(W.V.x, 0, n * sizeof(float), st));
    }
    AFM_CUDA(launch_norm2(m.d_b, n, op->d_scalars, op->d_scalars + kScalarSlots, st));
    m.phase = MS_NORMB;
    return mixed_record(m);
}

bool mixed_ready(const MixedSolve& m) { return m.ev && cudaEventQuery(m.ev) == cudaSuccess; }

int mixed_lane_record(MixedSolve& m, cudaStream_t lane_stream) {
    AFM_CUDA(cudaMemcpyAsync(m.op->h_scalars, m.op->d_scalars, sizeof(double) * kScalarSlots,
                             cudaMemcpyDeviceToHost, lane_stream));
    AFM_CUDA(cudaEventRecord(m.ev, lane_stream));
    m.phase = MS_LANEITER;
    return AFM_SUCCESS;
}

void mixed_lane_job(const MixedSolve& m, LaneJob& J) {
    afm_operator* op = m.op;
    const MixedVectors W = mixed_vectors(op);
    J.x = W.V.x;
    J.r = W.V.r;
    J.z = W.V.z;
    J.p = W.V.p;
    J.q = W.V.q;
    J.dinv = W.V.dinv;
    J.bcmask = op->d_bcmask;
    J.sc = op->d_scalars;
    J.err = op->d_err;
    J.n_dofs = op->n_dofs;
}

int mixed_advance(MixedSolve& m) {
    afm_operator* op = m.op;
    DeviceGuard g(op->device);
    double* h = op->h_scalars;
    const size_t n = op->n_dofs;
    cudaStream_t st = op->stream;
    const MixedVectors W = mixed_vectors(op);
    double* sc = op->d_scalars;
    double* part = sc + kScalarSlots;
    switch (m.phase) {
        case MS_NORMB:
            m.bn = std::sqrt(h[S_PQ]);
            m.tol = std::max(m.rtol * m.bn, m.atol);
            return mixed_residual(m);
        case MS_RESID: {
            m.rn = std::sqrt(h[S_PQ]);
            m.trace_iters.push_back(m.inner_total);
            m.trace_res.push_back(m.bn > 0 ? m.rn / m.bn : m.rn);
            if (std::isnan(m.rn)) return mixed_finish(m, AFM_ERR_BREAKDOWN);
            if (m.rn <= m.tol) return mixed_finish(m, AFM_SUCCESS);
            if (!ir_progress(m.rn, &m.best, &m.stall) || m.outer >= m.max_outer)
                return mixed_finish(m, AFM_ERR_MAXIT);
            // the segment's scale: a power of two that brings ||r|| into [0.5, 1) (exact)
            const double sigma = residual_scale(m.rn);
            if (m.fresh && m.inner64) {
                // FP64-vector Jacobi-PCG on A d = sigma r from d = 0
                AFM_CUDA(launch_to_f32(W.b64, W.r64, n, st, sigma));
                AFM_CUDA(cudaMemsetAsync(W.D.q, 0, n * sizeof(double), st));
                AFM_CUDA(launch_cg_init(W.b64, W.D.q, W.D.dinv, W.D.r, W.D.z, W.D.p, n, sc, part, st));
            } else if (m.fresh) {
                // FP32 Jacobi-PCG on A d = sigma r from d = 0
                AFM_CUDA(launch_to_f32(W.b32, W.r64, n, st, sigma));
                AFM_CUDA(cudaMemsetAsync(W.V.q, 0, n * sizeof(float), st));
                AFM_CUDA(launch_cg_init(W.b32, W.V.q, W.V.dinv, W.V.r, W.V.z, W.V.p, n, sc, part, st));
            } else if (m.inner64) {
                // reliable update: the recursion continues from the true residual
                AFM_CUDA(launch_cg_reliable(W.r64, W.D.r, W.D.z, W.D.p, W.D.dinv, n, sc, part, sigma,
                                            sigma / m.sigma, st));
            } else {
                AFM_CUDA(launch_cg_reliable(W.r64, W.V.r, W.V.z, W.V.p, W.V.dinv, n, sc, part, sigma,
                                            sigma / m.sigma, st));
            }
            m.sigma = sigma;
            // the segment ends once the FP32 residual has dropped by inner_rtol
            m.inner_tol = std::max(m.inner_rtol * m.rn, m.tol);
            m.phase = MS_SEGSTART;
            return mixed_record(m);
        }
        case MS_SEGSTART: {
            const double n0 = std::sqrt(h[S_RR]) / m.sigma;
            if (h[S_FLAG] != 0.0 || std::isnan(n0)) return mixed_segment_end(m, 0, AFM_ERR_BREAKDOWN);
            if (n0 <= m.inner_tol) return mixed_segment_end(m, 0, AFM_SUCCESS);
            if (m.max_inner <= 0) return mixed_segment_end(m, 0, AFM_ERR_MAXIT);
            h[S_TOL] = m.inner_tol * m.sigma;
            h[S_MAXIT] = (double)m.max_inner;
            h[S_NORM] = 0.0;
            AFM_CUDA(cudaMemcpyAsync(sc + S_DONE, h + S_DONE, sizeof(double) * (S_NORM - S_DONE + 1),
                                     cudaMemcpyHostToDevice, st));
            if (m.lane) {  // the iterations join the next lane launch
                AFM_CUDA(cudaEventRecord(m.ev, st));
                m.phase = MS_LANE;
                return AFM_SUCCESS;
            }
            int s = m.inner64 ? ensure_cg_graph<double>(op, op->cg64i, W.D, true)
                              : ensure_cg_graph<float>(op, op->cg32, W.V);
            if (s) return s;
            AFM_CUDA(cudaGraphLaunch(m.inner64 ? op->cg64i.exec : op->cg32.exec, st));
            AFM_CUDA(cudaEventRecord(m.ev, st));
            m.phase = MS_ITER;
            return AFM_SUCCESS;
        }
        case MS_LANEITER:
            // the solve's stream continues after the lane launch
            AFM_CUDA(cudaStreamWaitEvent(st, m.ev, 0));
            if (h[S_DONE] == 0.0) {
                m.phase = MS_LANE;
                return AFM_SUCCESS;
            }
            [[fallthrough]];
        case MS_ITER: {
            if (h[S_DONE] == 0.0) {
                AFM_CUDA(cudaGraphLaunch(m.inner64 ? op->cg64i.exec : op->cg32.exec, st));
                AFM_CUDA(cudaEventRecord(m.ev, st));
                return AFM_SUCCESS;
            }
            const double nrm = std::sqrt(h[S_RR]) / m.sigma;
            const int seg = h[S_FLAG] != 0.0 ? AFM_ERR_BREAKDOWN : (nrm <= m.inner_tol ? AFM_SUCCESS : AFM_ERR_MAXIT);
            return mixed_segment_end(m, (int)h[S_ITER], seg);
        }
        default:
            return fail(AFM_ERR_STATE, "mixed solve step in phase %d", m.phase);
    }
}

int mixed_end(MixedSolve& m, afm_solve_stats* stats) {
    int s = AFM_SUCCESS;
    float ms = 0.f;
    if (m.phase == MS_DONE && m.op) {
        DeviceGuard g(m.op->device);
        if (cudaEventSynchronize(m.e1) == cudaSuccess) cudaEventElapsedTime(&ms, m.e0, m.e1);
        s = check_device_error(m.op);
    }
    if (m.ev) cudaEventDestroy(m.ev);
    if (m.e0) cudaEventDestroy(m.e0);
    if (m.e1) cudaEventDestroy(m.e1);
    m.ev = m.e0 = m.e1 = nullptr;
    if (m.op) {
        m.op->trace_iters = m.trace_iters;
        m.op->trace_res = m.trace_res;
    }
    if (s) return s;
    if (m.phase != MS_DONE) return fail(AFM_ERR_STATE, "mixed solve not finished");
    if (stats) {
        stats->iterations = m.inner_total;
        stats->status = m.status;
        stats->rel_residual = m.bn > 0 ? m.rn / m.bn : m.rn;
        stats->residual_norm = m.rn;
        stats->seconds = ms * 1e-3;
        stats->refinements = m.outer;
    }
    if (m.status != AFM_SUCCESS)
        return fail(m.status, m.status == AFM_ERR_MAXIT ? "refinement stopped after %d steps"
                                                        : "breakdown after %d steps",
                    m.outer);
    return ok();
}

}  // namespace afm

int afm::set_stream_priority(afm_operator* op, int priority) {
    AFM_CHECK_OP(op);
    DeviceGuard g(op->device);
    cudaStream_t st = nullptr;
    AFM_CUDA(cudaStreamCreateWithPriority(&st, cudaStreamNonBlocking, priority));
    if (cudaStreamSynchronize(op->stream) != cudaSuccess) {
        cudaStreamDestroy(st);
        return fail(AFM_ERR_CUDA, "stream priority: %s", cudaGetErrorString(cudaGetLastError()));
    }
    cudaStreamDestroy(op->stream);
    op->stream = st;
    drop_graph(op->cg64);  // no captured iteration keeps the old stream's work order
    drop_graph(op->cg32);
    drop_graph(op->cg64i);
    return ok();
}

extern "C" {

const char* afm_last_error(void) { return g_last_error.c_str(); }

const char* afm_status_string(int s) {
    switch (s) {
        case AFM_SUCCESS: return "SUCCESS";
        case AFM_INDEX_OUT_OF_BOUNDS: return "INDEX_OUT_OF_BOUNDS";
        case AFM_UNKNOWN_ELEMENT_TYPE: return "UNKNOWN_ELEMENT_TYPE";
        case AFM_UNKNOWN_ELEMENT_STATUS: return "UNKNOWN_ELEMENT_STATUS";
        case AFM_NULL_L2G_MAP: return "NULL_L2G_MAP";
        case AFM_GHOST_NODE_NOT_FOUND: return "GHOST_NODE_NOT_FOUND";
        case AFM_UNKNOWN_MAT_TYPE: return "UNKNOWN_MAT_TYPE";
        case AFM_WRONG_COMMUNICATION: return "WRONG_COMMUNICATION";
        case AFM_UNKNOWN_DOF_TYPE: return "UNKNOWN_DOF_TYPE";
        case AFM_UNKNOWN_CONSTRAINT: return "UNKNOWN_CONSTRAINT";
        case AFM_UNKNOWN_BC_METH: return "UNKNOWN_BC_METH";
        case AFM_NOT_IMPLEMENTED: return "NOT_IMPLEMENTED";
        case AFM_GLOBAL_DOF_ID_NOT_FOUND: return "GLOBAL_DOF_ID_NOT_FOUND";
        case AFM_ERR_CUDA: return "ERR_CUDA";
        case AFM_ERR_OOM: return "ERR_OOM";
        case AFM_ERR_TIMEOUT: return "ERR_TIMEOUT";
        case AFM_ERR_BREAKDOWN: return "ERR_BREAKDOWN";
        case AFM_ERR_STATE: return "ERR_STATE";
        case AFM_ERR_INVALID_ARG: return "ERR_INVALID_ARG";
        case AFM_ERR_MAXIT: return "ERR_MAXIT";
        case AFM_ERR_INTERNAL: return "ERR_INTERNAL";
        default: return "UNKNOWN_STATUS";
    }
}

int afm_create(afm_operator** out, int bc_method, int device) {
    if (!out) return fail(AFM_ERR_INVALID_ARG, "out is null");
    *out = nullptr;
    if (bc_method != AFM_BC_IMATRIX && bc_method != AFM_BC_PENALTY)
        return fail(AFM_UNKNOWN_BC_METH, "unknown BC method %d", bc_method);
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0)
        return fail(AFM_ERR_CUDA, "no CUDA device: %s", e != cudaSuccess ? cudaGetErrorString(e) : "count 0");
    if (device < 0) AFM_CUDA(cudaGetDevice(&device));
    if (device >= ndev) return fail(AFM_ERR_INVALID_ARG, "device %d of %d", device, ndev);
    cudaDeviceProp prop;
    AFM_CUDA(cudaGetDeviceProperties(&prop, device));
    if (!(prop.major == 10 && prop.minor == 3))
        return fail(AFM_ERR_CUDA, "device %d is sm_%d%d; this library is built for sm_103a only", device,
                    prop.major, prop.minor);
    DeviceGuard g(device);
    // kernels' shared-memory limits, before any launch or graph capture
    if (configure_kernels_fp64() != cudaSuccess || configure_kernels_split() != cudaSuccess ||
        configure_kernels_fp32() != cudaSuccess || configure_kernels_f32sym() != cudaSuccess ||
        configure_kernels_f32symx() != cudaSuccess || configure_kernels_splitsymx() != cudaSuccess ||
        configure_kernels_f32symc() != cudaSuccess)
        return fail(AFM_ERR_CUDA, "kernel configuration failed on device %d", device);
    auto* op = new afm_operator();
    op->device = device;
    op->bc_method = bc_method;
    op->sm_count = prop.multiProcessorCount;
    if (cudaStreamCreateWithFlags(&op->stream, cudaStreamNonBlocking) != cudaSuccess ||
        dalloc(op, &op->d_err, sizeof(int) * kErrWords) != cudaSuccess ||
        dalloc(op, &op->d_usc, sizeof(unsigned long long) * kUscWords) != cudaSuccess ||
        dalloc(op, &op->d_scalars, sizeof(double) * (kScalarSlots + kPartialSlots)) != cudaSuccess ||
        cudaMallocHost((void**)&op->h_scalars, sizeof(double) * kScalarSlots) != cudaSuccess) {
        afm_destroy(op);
        return fail(AFM_ERR_CUDA, "afm_create: stream or buffer allocation failed");
    }
    cudaMemsetAsync(op->d_err, 0, sizeof(int) * kErrWords, op->stream);
    cudaMemsetAsync(op->d_usc, 0, sizeof(unsigned long long) * kUscWords, op->stream);
    cudaStreamSynchronize(op->stream);
    *out = op;
    return ok();
}

int afm_destroy(afm_operator* op) {
    if (!op) return ok();
    {
        DeviceGuard g(op->device);
        if (op->stream) cudaStreamSynchronize(op->stream);
        free_device(op);
        if (op->stream) {
            dfree(op, op->d_err);
            dfree(op, op->d_usc);
            dfree(op, op->d_scalars);
            dfree(op, op->d_bremain);
            cudaStreamSynchronize(op->stream);
        }
        if (op->h_scalars) cudaFreeHost(op->h_scalars);
        if (op->h_bremain) cudaFreeHost(op->h_bremain);
        if (op->stream) cudaStreamDestroy(op->stream);
    }
    delete op;
    return ok();
}

int afm_set_matfree_type(afm_operator* op, int t) {
    AFM_CHECK_OP(op);
    if (t != 1 && t != 2 && t != 3) return fail(AFM_UNKNOWN_MAT_TYPE, "MATFREE_TYPE %d not provided (1, 2 or 3)", t);
    if ((t == 2) != (op->matfree_type == 2)) op->finalized = false;
    op->matfree_type = t;
    return ok();
}

int afm_set_precision(afm_operator* op, int p) {
    AFM_CHECK_OP(op);
    if (p < AFM_PREC_FP64 || p > AFM_PREC_AUTO) return fail(AFM_ERR_INVALID_ARG, "precision %d", p);
    op->precision_req = p;
    op->finalized = false;
    return ok();
}

int afm_set_patch_mode(afm_operator* op, int mode) {
    AFM_CHECK_OP(op);
    if (mode < 0 || mode > 3) return fail(AFM_ERR_INVALID_ARG, "patch mode %d (0 to 3)", mode);
    op->patch_mode = mode;
    op->finalized = false;
    return ok();
}

int afm_set_wait_limit(afm_operator* op, double seconds) {
    AFM_CHECK_OP(op);
    if (!(seconds >= 1e-9 && seconds <= 600.0)) return fail(AFM_ERR_INVALID_ARG, "wait limit %g s (1e-9 .. 600)", seconds);
    const unsigned long long ns = (unsigned long long)std::llround(seconds * 1e9);
    if (ns != op->wait_ns) {
        op->wait_ns = ns;
        op->generation++;  // captured iterations hold the old limit in their launch arguments
    }
    return ok();
}

int afm_set_wait_probe(afm_operator* op, int enable) {
    AFM_CHECK_OP(op);
    if (enable != 0 && enable != 1) return fail(AFM_ERR_INVALID_ARG, "wait probe %d (0 or 1)", enable);
    if (op->wait_probe != (enable == 1)) {
        op->wait_probe = enable == 1;
        op->generation++;  // captured iterations hold the hook in their launch arguments
    }
    return ok();
}

int afm_set_fused_colours(afm_operator* op, int enable) {
    AFM_CHECK_OP(op);
    if (enable != 0 && enable != 1) return fail(AFM_ERR_INVALID_ARG, "fused colours %d (0 or 1)", enable);
    op->fused = enable == 1;
    return ok();
}

int afm_set_symmetric_inner(afm_operator* op, int format) {
    AFM_CHECK_OP(op);
    if (format < 0 || format > 5) return fail(AFM_ERR_INVALID_ARG, "symmetric inner format %d (0 to 5)", format);
    op->sym_mode = format;
    if (op->d_sym && op->sym_built != sym_arena(op)) {
        DeviceGuard g(op->device);
        dfree(op, op->d_sym);
        dfree(op, op->d_vx);
        op->sym_built = 0;
        op->generation++;  // captured FP32 iterations leave the old arena
    }
    return ok();
}

int afm_set_map(afm_operator* op, uint32_t n_elements, const uint32_t* dof_offsets, uint32_t dofs_per_element,
                const uint32_t* e2r, uint32_t n_all_dofs, const uint64_t* r2g, uint64_t owned_begin,
                uint64_t owned_end, uint64_t n_global) {
    AFM_CHECK_OP(op);
    if (n_elements > 0 && !e2r) return fail(AFM_ERR_INVALID_ARG, "element_to_rank_map is null");
    if (n_global == 0 || n_global > kDofMask) return fail(AFM_ERR_INVALID_ARG, "n_global_dofs %llu", (unsigned long long)n_global);
    // one rank owns [0, n_global-1]; the reference's m_uiNumDofs = end - begin + 1 (include/maps.hpp:413)
    if (owned_begin != 0 || owned_end + 1 != n_global || n_all_dofs != n_global)
        return fail(AFM_WRONG_COMMUNICATION, "maps need ghost exchange: owned [%llu, %llu], %u local of %llu global",
                    (unsigned long long)owned_begin, (unsigned long long)owned_end, n_all_dofs,
                    (unsigned long long)n_global);
    std::vector<uint32_t> offs((size_t)n_elements + 1, 0);
    for (uint32_t e = 0; e < n_elements; e++) {
        const uint32_t n = dof_offsets ? dof_offsets[e + 1] - dof_offsets[e] : dofs_per_element;
        if (dof_offsets && dof_offsets[e + 1] < dof_offsets[e])
            return fail(AFM_ERR_INVALID_ARG, "dof_offsets not monotone at element %u", e);
        if (n == 0 || n > kMaxN) return fail(AFM_NOT_IMPLEMENTED, "element %u has %u DoFs (1..%u supported)", e, n, kMaxN);
        if ((uint64_t)offs[e] + n > 0xffffffffull) return fail(AFM_ERR_INVALID_ARG, "map too large");
        offs[e + 1] = offs[e] + n;
    }
    const uint32_t base = dof_offsets ? dof_offsets[0] : 0;
    std::vector<uint32_t> map(offs[n_elements]);
    for (uint32_t k = 0; k < offs[n_elements]; k++) {
        const uint32_t l = e2r[base + k];
        if (l >= n_all_dofs) return fail(AFM_INDEX_OUT_OF_BOUNDS, "local DoF %u >= %u", l, n_all_dofs);
        const uint64_t gid = r2g ? r2g[l] : l;
        if (gid >= n_global) return fail(AFM_GLOBAL_DOF_ID_NOT_FOUND, "global DoF %llu >= %llu", (unsigned long long)gid, (unsigned long long)n_global);
        map[k] = (uint32_t)gid;
    }
    op->n_elem = n_elements;
    op->n_dofs = (uint32_t)n_global;
    op->offsets.swap(offs);
    op->map.swap(map);
    op->nmax = 0;
    op->dup_in_element = false;
    op->kofs.assign((size_t)n_elements + 1, 0);
    std::vector<uint32_t> tmp;
    for (uint32_t e = 0; e < n_elements; e++) {
        const uint32_t n = op->offsets[e + 1] - op->offsets[e];
        op->nmax = std::max(op->nmax, n);
        op->kofs[e + 1] = op->kofs[e] + (uint64_t)n * n;
        tmp.assign(op->map.begin() + op->offsets[e], op->map.begin() + op->offsets[e + 1]);
        std::sort(tmp.begin(), tmp.end());
        if (std::adjacent_find(tmp.begin(), tmp.end()) != tmp.end()) op->dup_in_element = true;
    }
    // the host element-matrix store is allocated by the first set_element_matrix (a matrix-free
    // operator never needs it)
    op->ke.clear();
    op->ke.shrink_to_fit();
    op->xe.clear();
    op->have_map = true;
    op->finalized = false;
    op->ke_dirty = true;
    return ok();
}

int afm_set_bdr_map(afm_operator* op, const uint64_t* constrained, const double* values, uint32_t n) {
    AFM_CHECK_OP(op);
    if (!op->have_map) return fail(AFM_ERR_STATE, "set_bdr_map before set_map");
    if (n > 0 && (!constrained || !values)) return fail(AFM_ERR_INVALID_ARG, "null constraint arrays");
    for (uint32_t i = 0; i < n; i++)
        if (constrained[i] >= op->n_dofs)
            return fail(AFM_GLOBAL_DOF_ID_NOT_FOUND, "constrained DoF %llu >= %u", (unsigned long long)constrained[i], op->n_dofs);
    op->constrained.assign(constrained, constrained + n);
    op->values.assign(values, values + n);
    op->bc_unique.assign(constrained, constrained + n);
    std::sort(op->bc_unique.begin(), op->bc_unique.end());
    op->bc_unique.erase(std::unique(op->bc_unique.begin(), op->bc_unique.end()), op->bc_unique.end());
    op->finalized = false;
    return ok();
}

namespace {
// Host store of the element matrices (zeros until set), n_elem blocks of n^2 entries.
int ensure_ke_store(afm_operator* op) {
    const uint64_t need = op->kofs.empty() ? 0 : op->kofs[op->n_elem];
    if (op->ke.size() == need) return AFM_SUCCESS;
    try {
        op->ke.assign(need, 0.0);
    } catch (...) {
        return fail(AFM_ERR_OOM, "host element-matrix store of %llu entries", (unsigned long long)need);
    }
    return AFM_SUCCESS;
}
}  // namespace

int afm_set_element_matrix(afm_operator* op, uint32_t eid, const double* e_mat, uint32_t bi, uint32_t bj,
                           uint32_t bd) {
    AFM_CHECK_OP(op);
    if (!op->have_map) return fail(AFM_ERR_STATE, "set_element_matrix before set_map");
    if (int st = ensure_ke_store(op)) return st;
    if (eid >= op->n_elem) return fail(AFM_INDEX_OUT_OF_BOUNDS, "element %u >= %u", eid, op->n_elem);
    if (!e_mat || bd == 0 || bi >= bd || bj >= bd) return fail(AFM_ERR_INVALID_ARG, "bad block (%u,%u) of %u", bi, bj, bd);
    const uint32_t n = op->offsets[eid + 1] - op->offsets[eid];
    if (n % bd) return fail(AFM_ERR_INVALID_ARG, "element %u: %u DoFs not divisible into %u blocks", eid, n, bd);
    const uint32_t nb = n / bd;
    double* k = op->ke.data() + op->kofs[eid];
    for (uint32_t r = 0; r < nb; r++)
        for (uint32_t c = 0; c < nb; c++) k[(size_t)(bi * nb + r) * n + (bj * nb + c)] = e_mat[(size_t)r * nb + c];
    op->ke_dirty = true;
    op->finalized = false;
    return ok();
}

int afm_set_element_matrices(afm_operator* op, uint32_t first, uint32_t count, const double* ke) {
    AFM_CHECK_OP(op);
    if (!op->have_map) return fail(AFM_ERR_STATE, "set_element_matrices before set_map");
    if ((uint64_t)first + count > op->n_elem) return fail(AFM_INDEX_OUT_OF_BOUNDS, "elements %u+%u > %u", first, count, op->n_elem);
    if (count && !ke) return fail(AFM_ERR_INVALID_ARG, "ke is null");
    if (int st = ensure_ke_store(op)) return st;
    const uint64_t a = op->kofs[first], b = op->kofs[(size_t)first + count];
    memcpy(op->ke.data() + a, ke, (size_t)(b - a) * sizeof(double));
    op->ke_dirty = true;
    op->finalized = false;
    return ok();
}

namespace {

// Matrix-free finalize (method 2): colours, the colour-sorted element order
// with its DoF map and node coordinates (FP64 and FP32), the reference-element
// tables, and the Jacobi diagonal and trace from the element kernels on the
// host (each diagonal entry summed exactly as the stored-Ke element kernel
// sums it, so both operators give the same diagonal).
int finalize_free(afm_operator* op) {
    if (op->elem_kind < 0) return fail(AFM_ERR_STATE, "MATFREE_TYPE::FREE needs afm_set_element_kind");
    afm_shape::Kind K;
    if (!afm_shape::kind_info(op->elem_kind, &K)) return fail(AFM_UNKNOWN_ELEMENT_TYPE, "kind %d", op->elem_kind);
    const uint32_t nn = (uint32_t)K.nodes, n = nn * (uint32_t)K.dpn;
    for (uint32_t e = 0; e < op->n_elem; e++)
        if (op->offsets[e + 1] - op->offsets[e] != n)
            return fail(AFM_ERR_INVALID_ARG, "element %u has %u DoFs, kind %d needs %u", e,
                        op->offsets[e + 1] - op->offsets[e], op->elem_kind, n);
    if (op->xe.size() != (size_t)op->n_elem * nn * 3) return fail(AFM_ERR_STATE, "element coordinates not set");
    DeviceGuard g(op->device);
    AFM_CUDA(cudaStreamSynchronize(op->stream));
    free_device(op);
    op->finalized = false;
    op->precision = AFM_PREC_FP64;  // FP64 products in FP64 arithmetic, _f32 products in FP32
    op->use_patches = false;
    op->n_patches = 0;
    op->patch_color_first.clear();
    op->segs.clear();
    op->sym_ok = false;
    op->ke_symmetric = false;
    op->n_colors = color_elements(op->n_dofs, op->n_elem, op->offsets, op->map, op->colors);
    op->perm.resize(op->n_elem);
    std::iota(op->perm.begin(), op->perm.end(), 0u);
    std::stable_sort(op->perm.begin(), op->perm.end(),
                     [&](uint32_t a, uint32_t b) { return op->colors[a] < op->colors[b]; });
    op->free_color_first.assign(op->n_colors + 1, 0);
    for (uint32_t e = 0; e < op->n_elem; e++) op->free_color_first[op->colors[e] + 1]++;
    for (uint32_t c = 0; c < op->n_colors; c++) op->free_color_first[c + 1] += op->free_color_first[c];
    std::vector<uint8_t> is_bc(op->n_dofs, 0);
    for (uint32_t d : op->bc_unique) is_bc[d] = 1;
    std::vector<uint32_t> hmap((size_t)op->n_elem * n);
    std::vector<double> x64((size_t)op->n_elem * nn * 3);
    std::vector<float> x32(x64.size());
#pragma omp parallel for schedule(static)
    for (int64_t p = 0; p < (int64_t)op->n_elem; p++) {
        const uint32_t e = op->perm[p];
        for (uint32_t i = 0; i < n; i++) {
            const uint32_t d = op->map[op->offsets[e] + i];
            hmap[(size_t)p * n + i] = d | (is_bc[d] ? kBcFlag : 0u);
        }
        for (uint32_t k = 0; k < nn * 3; k++) {
            x64[(size_t)p * nn * 3 + k] = op->xe[(size_t)e * nn * 3 + k];
            x32[(size_t)p * nn * 3 + k] = (float)op->xe[(size_t)e * nn * 3 + k];
        }
    }
    // reference tables: dN of every node at every quadrature point, then the weights
    std::vector<double> q;
    afm_shape::quadrature(K.tet, op->elem_ngt, q);
    const uint32_t nq = (uint32_t)(q.size() / 4);
    std::vector<double> r64((size_t)nq * (nn * 3 + 1));
    for (uint32_t t = 0; t < nq; t++) {
        K.shape(&q[4 * t], nullptr, &r64[(size_t)t * nn * 3]);
        r64[(size_t)nq * nn * 3 + t] = q[4 * t + 3];
    }
    std::vector<float> r32(r64.begin(), r64.end());
    op->free_nq = nq;
    // Jacobi diagonal and trace in element order (mat_get_diagonal, include/aMatFree.hpp:998-1056)
    const double E = op->elem_E, nu = op->elem_nu;
    const double lam = E * nu / (1.0 + nu) / (1.0 - 2.0 * nu), mu = 0.5 * E / (1.0 + nu);
    std::vector<double> kd((size_t)op->n_elem * n, 0.0);
    int bad = 0;
#pragma omp parallel for schedule(static) reduction(| : bad)
    for (int64_t e = 0; e < (int64_t)op->n_elem; e++) {
        double dNx[3 * 20], detJ;
        double* k = kd.data() + (size_t)e * n;
        const double* xe = op->xe.data() + (size_t)e * nn * 3;
        for (size_t t = 0; t < q.size(); t += 4) {
            if (!afm_shape::gradients(K, xe, &q[t], nullptr, dNx, &detJ)) {
                bad = 1;
                break;
            }
            const double w = detJ * q[t + 3];
            for (uint32_t a = 0; a < nn; a++) {
                const double* ga = dNx + 3 * a;
                const double gg = ga[0] * ga[0] + ga[1] * ga[1] + ga[2] * ga[2];
                if (K.dpn == 1) {
                    k[a] += gg * w;
                } else {
                    for (int i = 0; i < 3; i++) {
                        double v = lam * ga[i] * ga[i] + mu * ga[i] * ga[i];
                        v += mu * gg;
                        k[3 * a + i] += v * w;
                    }
                }
            }
        }
    }
    if (bad) return fail(AFM_ERR_INVALID_ARG, "an element has a non-positive Jacobian");
    op->diag_host.assign(op->n_dofs, 0.0);
    op->trace = 0.0;
    for (uint32_t e = 0; e < op->n_elem; e++)
        for (uint32_t r = 0; r < n; r++) {
            op->diag_host[op->map[op->offsets[e] + r]] += kd[(size_t)e * n + r];
            op->trace += kd[(size_t)e * n + r];
        }
    const double bc_diag = (op->bc_method == AFM_BC_PENALTY) ? 100.0 * op->trace : 1.0;
    for (uint32_t d : op->map)
        if (is_bc[d]) op->diag_host[d] = bc_diag;
    // uploads
    op->ke_bytes = 0;
    op->map_bytes = hmap.size() * sizeof(uint32_t);
    op->n_bc = (uint32_t)op->constrained.size();
    AFM_CUDA(dalloc(op, &op->d_map, std::max<size_t>(op->map_bytes, 16)));
    AFM_CUDA(dalloc(op, &op->d_diag, sizeof(double) * std::max<uint32_t>(op->n_dofs, 1)));
    AFM_CUDA(dalloc(op, &op->d_bc_idx, sizeof(uint32_t) * std::max<uint32_t>(op->n_bc, 1)));
    AFM_CUDA(dalloc(op, &op->d_bc_val, sizeof(double) * std::max<uint32_t>(op->n_bc, 1)));
    AFM_CUDA(dalloc(op, &op->d_free_xe64, sizeof(double) * std::max<size_t>(x64.size(), 1)));
    AFM_CUDA(dalloc(op, &op->d_free_xe32, sizeof(float) * std::max<size_t>(x32.size(), 1)));
    AFM_CUDA(dalloc(op, &op->d_free_ref64, sizeof(double) * r64.size()));
    AFM_CUDA(dalloc(op, &op->d_free_ref32, sizeof(float) * r32.size()));
    std::vector<uint32_t> bci(op->constrained.begin(), op->constrained.end());
    cudaStream_t st = op->stream;
    AFM_CUDA(cudaMemcpyAsync(op->d_map, hmap.data(), op->map_bytes, cudaMemcpyHostToDevice, st));
    AFM_CUDA(cudaMemcpyAsync(op->d_diag, op->diag_host.data(), sizeof(double) * op->n_dofs, cudaMemcpyHostToDevice,
                             st));
    if (op->n_bc) {
        AFM_CUDA(cudaMemcpyAsync(op->d_bc_idx, bci.data(), sizeof(uint32_t) * op->n_bc, cudaMemcpyHostToDevice, st));
        AFM_CUDA(cudaMemcpyAsync(op->d_bc_val, op->values.data(), sizeof(double) * op->n_bc, cudaMemcpyHostToDevice,
                                 st));
    }
    AFM_CUDA(cudaMemcpyAsync(op->d_free_xe64, x64.data(), sizeof(double) * x64.size(), cudaMemcpyHostToDevice, st));
    AFM_CUDA(cudaMemcpyAsync(op->d_free_xe32, x32.data(), sizeof(float) * x32.size(), cudaMemcpyHostToDevice, st));
    AFM_CUDA(cudaMemcpyAsync(op->d_free_ref64, r64.data(), sizeof(double) * r64.size(), cudaMemcpyHostToDevice, st));
    AFM_CUDA(cudaMemcpyAsync(op->d_free_ref32, r32.data(), sizeof(float) * r32.size(), cudaMemcpyHostToDevice, st));
    AFM_CUDA(cudaStreamSynchronize(st));
    op->ke_dirty = false;
    op->finalized = true;
    return ok();
}

}  // namespace

int afm_set_element_kind(afm_operator* op, int kind, double E, double nu, uint32_t ngt) {
    AFM_CHECK_OP(op);
    afm_shape::Kind K;
    if (!afm_shape::kind_info(kind, &K)) return fail(AFM_UNKNOWN_ELEMENT_TYPE, "element kind %d", kind);
    if (ngt < 1 || ngt > 3) return fail(AFM_ERR_INVALID_ARG, "%u Gauss points per direction (1 to 3)", ngt);
    if (K.dpn == 3 && !(E > 0.0 && nu > -1.0 && nu < 0.5)) return fail(AFM_ERR_INVALID_ARG, "E %g, nu %g", E, nu);
    if ((uint32_t)K.nodes != op->elem_nodes) op->xe.clear();
    op->elem_kind = kind;
    op->elem_E = E;
    op->elem_nu = nu;
    op->elem_ngt = ngt;
    op->elem_nodes = (uint32_t)K.nodes;
    op->finalized = false;
    return ok();
}

int afm_set_element_coords(afm_operator* op, uint32_t first, uint32_t count, const double* xe) {
    AFM_CHECK_OP(op);
    if (!op->have_map) return fail(AFM_ERR_STATE, "set_element_coords before set_map");
    if (op->elem_kind < 0) return fail(AFM_ERR_STATE, "set_element_coords before set_element_kind");
    if ((uint64_t)first + count > op->n_elem) return fail(AFM_INDEX_OUT_OF_BOUNDS, "elements %u+%u > %u", first, count, op->n_elem);
    if (count && !xe) return fail(AFM_ERR_INVALID_ARG, "xe is null");
    const size_t per = (size_t)op->elem_nodes * 3;
    if (op->xe.size() != (size_t)op->n_elem * per) op->xe.assign((size_t)op->n_elem * per, 0.0);
    memcpy(op->xe.data() + (size_t)first * per, xe, sizeof(double) * per * count);
    op->finalized = false;
    return ok();
}

int afm_finalize(afm_operator* op) {
    AFM_CHECK_OP(op);
    if (!op->have_map) return fail(AFM_ERR_STATE, "finalize before set_map");
    if (op->matfree_type == 2) return finalize_free(op);
    if (int st = ensure_ke_store(op)) return st;
    DeviceGuard g(op->device);
    AFM_CUDA(cudaStreamSynchronize(op->stream));
    free_device(op);
    op->finalized = false;

    // precision
    int prec = op->precision_req;
    if (prec == AFM_PREC_AUTO) {
        // the split arithmetic's range: each element's largest |entry| in [1e-30, 1e30] (an all-zero element
        // too); smaller entries of an element, such as the round-off residue of exact zeros that quadrature
        // leaves (~1e-35 in tet10 elasticity), lose at most FP32-subnormal-sized amounts, far below the
        // element's 2^-44 bound
        int fits = 1;
#pragma omp parallel for schedule(static) reduction(&& : fits)
        for (int64_t e = 0; e < (int64_t)op->n_elem; e++) {
            double mx = 0.0;
            bool finite = true;
            for (uint64_t k = op->kofs[e]; k < op->kofs[e + 1]; k++) {
                const double x = op->ke[k];
                finite = finite && std::isfinite(x);
                mx = std::max(mx, std::fabs(x));
            }
            fits = fits && finite && (mx == 0.0 || (mx >= 1e-30 && mx <= 1e30));
        }
        prec = fits ? AFM_PREC_FP64_SPLIT : AFM_PREC_FP64;
    }
    op->precision = prec;
    if (prec == AFM_PREC_FP64_SPLIT) {
        // the pair hi + lo of every entry must be FP32 numbers
        for (double x : op->ke)
            if (!std::isfinite(x) || std::fabs(x) > 1e38)
                return fail(AFM_ERR_INVALID_ARG, "FP64_SPLIT: element matrix entry %g outside the FP32 range", x);
    }

    // colouring (the reference's greedy colouring, also the segment order)
    op->n_colors = color_elements(op->n_dofs, op->n_elem, op->offsets, op->map, op->colors);

    // small elements of one size: patch plan
    std::vector<PatchDesc> pdesc;
    std::vector<unsigned char> pidx;
    op->use_patches = false;
    op->n_patches = 0;
    op->patch_color_first.clear();
    op->segs.clear();
    {
        bool uniform = op->n_elem > 0;
        const uint32_t n0 = op->n_elem ? op->offsets[1] - op->offsets[0] : 0;
        for (uint32_t e = 0; e < op->n_elem && uniform; e++) uniform = (op->offsets[e + 1] - op->offsets[e] == n0);
        if (op->patch_mode && uniform && !op->dup_in_element && n0 >= 1 && n0 <= kPatchMaxN)
            op->use_patches = build_patch_plan(op, n0, prec, pdesc, pidx);
        if (!op->use_patches) op->segs.clear();
    }

    // colour-sorted order and segments (elements not run as patches)
    if (!op->use_patches) {
        build_segments(op, prec);
    } else {
        op->ke_bytes = (uint64_t)op->segs[0].units * op->segs[0].unit_bytes;
        op->map_bytes = 0;  // the patch index blocks replace the map
    }
    const uint64_t map_off = op->map_bytes / sizeof(uint32_t);

    // device map with constrained columns flagged
    std::vector<uint8_t> is_bc(op->n_dofs, 0);
    for (uint32_t d : op->bc_unique) is_bc[d] = 1;
    std::vector<uint32_t> hmap(map_off, 0);
    for (const Segment& s : op->segs) {
        if (op->use_patches) break;
        for (uint32_t rel = 0; rel < s.count; rel++) {
            const uint32_t e = op->perm[s.first_pos + rel];
            for (uint32_t i = 0; i < s.n; i++) {
                uint32_t d = op->map[op->offsets[e] + i];
                if (is_bc[d]) d |= kBcFlag;
                size_t at;
                if (s.regime == REG_WPE)
                    at = s.map_offset + (size_t)rel * s.n + i;
                else
                    at = s.map_offset + ((size_t)(rel / kTpeWidth) * s.n + i) * kTpeWidth + rel % kTpeWidth;
                hmap[at] = d;
            }
        }
    }

    // Jacobi diagonal in element order (mat_get_diagonal_ghosted,
    // include/aMatFree.hpp:998-1056), trace (749-785), BC rows (4310-4338)
    op->diag_host.assign(op->n_dofs, 0.0);
    op->trace = 0.0;
    for (uint32_t e = 0; e < op->n_elem; e++) {
        const uint32_t n = op->offsets[e + 1] - op->offsets[e];
        const double* k = op->ke.data() + op->kofs[e];
        for (uint32_t r = 0; r < n; r++) {
            op->diag_host[op->map[op->offsets[e] + r]] += k[(size_t)r * n + r];
            op->trace += k[(size_t)r * n + r];
        }
    }
    // apply_bc_diagonal reaches constrained DoFs through the elements, so a
    // constrained DoF of no element keeps its (zero) sum
    const double bc_diag = (op->bc_method == AFM_BC_PENALTY) ? 100.0 * op->trace : 1.0;
    for (uint32_t d : op->map)
        if (is_bc[d]) op->diag_host[d] = bc_diag;

    // uploads
    AFM_CUDA(dalloc(op, &op->d_ke, std::max<size_t>(op->ke_bytes, 16)));
    AFM_CUDA(dalloc(op, &op->d_map, std::max<size_t>(op->map_bytes, 16)));
    AFM_CUDA(dalloc(op, &op->d_diag, sizeof(double) * std::max<uint32_t>(op->n_dofs, 1)));
    op->n_bc = (uint32_t)op->constrained.size();
    AFM_CUDA(dalloc(op, &op->d_bc_idx, sizeof(uint32_t) * std::max<uint32_t>(op->n_bc, 1)));
    AFM_CUDA(dalloc(op, &op->d_bc_val, sizeof(double) * std::max<uint32_t>(op->n_bc, 1)));
    std::vector<uint32_t> bci(op->constrained.begin(), op->constrained.end());
    AFM_CUDA(cudaMemcpyAsync(op->d_map, hmap.data(), op->map_bytes, cudaMemcpyHostToDevice, op->stream));
    AFM_CUDA(cudaMemcpyAsync(op->d_diag, op->diag_host.data(), sizeof(double) * op->n_dofs, cudaMemcpyHostToDevice,
                             op->stream));
    if (!op->bc_unique.empty()) {
        AFM_CUDA(dalloc(op, &op->d_bcmask, std::max<uint32_t>(op->n_dofs, 1)));
        AFM_CUDA(cudaMemcpyAsync(op->d_bcmask, is_bc.data(), op->n_dofs, cudaMemcpyHostToDevice, op->stream));
    }
    if (op->n_bc) {
        AFM_CUDA(cudaMemcpyAsync(op->d_bc_idx, bci.data(), sizeof(uint32_t) * op->n_bc, cudaMemcpyHostToDevice,
                                 op->stream));
        AFM_CUDA(cudaMemcpyAsync(op->d_bc_val, op->values.data(), sizeof(double) * op->n_bc,
                                 cudaMemcpyHostToDevice, op->stream));
    }
    // every colour of a split product in one cooperative launch (afm_set_fused_colours, off by default): a
    // segment plan whose elements share one size in the warp-group regime. Measured slower than one launch
    // per colour (hex20 64^3: 1.438 against 1.359 ms; hex8 elasticity 48^3: 0.179 against 0.172 ms)
    op->fused_ok = false;
    if (!op->use_patches && !op->dup_in_element && prec == AFM_PREC_FP64_SPLIT && !op->segs.empty() &&
        op->segs.size() <= kMaxFusedColours) {
        bool same = true;
        for (const Segment& g : op->segs)
            same = same && g.regime == REG_WPE && g.n == op->segs[0].n && g.units > 0;
        if (same) {
            AFM_CUDA(dalloc(op, &op->d_gbar, sizeof(unsigned) * kMaxFusedColours));
            op->fused_ok = true;
        }
    }
    // one launch for every patch colour when the colours are small (a launch per colour would leave
    // most SMs idle between colours), else one launch per colour
    op->patch_one_launch = false;
    if (op->use_patches) {
        const size_t ncol = std::max<size_t>(op->patch_color_first.size() - 1, 1);
        const bool small = op->n_patches / ncol < 16ull * (uint64_t)std::max(op->sm_count, 1);
        op->patch_one_launch = op->patch_mode == 3 || (op->patch_mode == 1 && small);
    }
    if (op->patch_one_launch) {
        AFM_CUDA(dalloc(op, &op->d_pv, sizeof(double) * std::max<size_t>(op->pv_count, 1)));
        AFM_CUDA(dalloc(op, &op->d_shared_dof, sizeof(uint32_t) * std::max<size_t>(op->shared_dof.size(), 1)));
        AFM_CUDA(dalloc(op, &op->d_shared_off, sizeof(uint32_t) * op->shared_off.size()));
        AFM_CUDA(dalloc(op, &op->d_shared_idx, sizeof(uint32_t) * std::max<size_t>(op->shared_idx.size(), 1)));
        AFM_CUDA(cudaMemcpyAsync(op->d_shared_dof, op->shared_dof.data(), sizeof(uint32_t) * op->shared_dof.size(),
                                 cudaMemcpyHostToDevice, op->stream));
        AFM_CUDA(cudaMemcpyAsync(op->d_shared_off, op->shared_off.data(), sizeof(uint32_t) * op->shared_off.size(),
                                 cudaMemcpyHostToDevice, op->stream));
        AFM_CUDA(cudaMemcpyAsync(op->d_shared_idx, op->shared_idx.data(), sizeof(uint32_t) * op->shared_idx.size(),
                                 cudaMemcpyHostToDevice, op->stream));
    }
    if (op->use_patches) {
        op->patch_idx_bytes = pidx.size();
        AFM_CUDA(dalloc(op, &op->d_patch_desc, sizeof(PatchDesc) * std::max<size_t>(pdesc.size(), 1)));
        AFM_CUDA(dalloc(op, &op->d_patch_idx, std::max<size_t>(pidx.size(), 16)));
        AFM_CUDA(cudaMemcpyAsync(op->d_patch_desc, pdesc.data(), sizeof(PatchDesc) * pdesc.size(),
                                 cudaMemcpyHostToDevice, op->stream));
        AFM_CUDA(cudaMemcpyAsync(op->d_patch_idx, pidx.data(), pidx.size(), cudaMemcpyHostToDevice, op->stream));
    }
    AFM_CUDA(cudaStreamSynchronize(op->stream));
    int st = upload_arena(op);
    if (st != AFM_SUCCESS) return st;

    // symmetric inner arena (built on the first FP32 product): split arena,
    // symmetric Ke, and elements that run as patches or on the warp-group kernel
    op->ke_symmetric = false;
    op->sym_ok = false;
    op->sym_bytes = 0;
    op->sym_built = 0;
    if (prec == AFM_PREC_FP64_SPLIT && !op->dup_in_element && op->n_elem > 0) {
        op->ke_symmetric = ke_is_symmetric(op);
        bool covered = true;
        if (!op->use_patches)
            for (const Segment& s : op->segs)
                if (s.units && s.regime != REG_WPE) covered = false;
        op->sym_ok = op->ke_symmetric && covered;
    }
    op->ke_dirty = false;
    op->finalized = true;
    return ok();
}

int afm_matvec_device(afm_operator* op, double* d_v, const double* d_u, void* stream) {
    AFM_CHECK_OP(op);
    if (!op->finalized) return fail(AFM_ERR_STATE, "matvec before finalize");
    if (op->precision == AFM_PREC_FP32) return fail(AFM_ERR_STATE, "FP32 operator: use afm_matvec_device_f32");
    if (!d_v || !d_u) return fail(AFM_ERR_INVALID_ARG, "null vector");
    if (d_v == (double*)d_u) return fail(AFM_ERR_INVALID_ARG, "v and u must not alias");
    DeviceGuard g(op->device);
    int s = enqueue_matvec(op, d_v, d_u, 0, pick_stream(op, stream));
    return s == AFM_SUCCESS ? ok() : s;
}

int afm_matvec_device_f32(afm_operator* op, float* d_v, const float* d_u, void* stream) {
    AFM_CHECK_OP(op);
    if (!op->finalized) return fail(AFM_ERR_STATE, "matvec before finalize");
    if (op->precision != AFM_PREC_FP32 && op->precision != AFM_PREC_FP64_SPLIT && op->matfree_type != 2)
        return fail(AFM_ERR_STATE, "FP32 product needs an FP32, FP64_SPLIT or matrix-free operator");
    if (!d_v || !d_u || (void*)d_v == (const void*)d_u) return fail(AFM_ERR_INVALID_ARG, "bad vectors");
    DeviceGuard g(op->device);
    cudaStream_t st = pick_stream(op, stream);
    int s = ensure_sym(op, st);
    if (s) return s;
    s = enqueue_matvec(op, d_v, d_u, 0, st, true);
    return s == AFM_SUCCESS ? ok() : s;
}

int afm_matvec_inner_device(afm_operator* op, double* d_v, const double* d_u, void* stream) {
    AFM_CHECK_OP(op);
    if (!op->finalized) return fail(AFM_ERR_STATE, "matvec before finalize");
    if (op->precision != AFM_PREC_FP64_SPLIT || op->matfree_type == 2 || sym_format(op) < 3)
        return fail(AFM_ERR_STATE, "the FP64 inner product needs an FP64_SPLIT operator in symmetric inner format 3 to 5");
    if (!d_v || !d_u || (void*)d_v == (const void*)d_u) return fail(AFM_ERR_INVALID_ARG, "bad vectors");
    DeviceGuard g(op->device);
    cudaStream_t st = pick_stream(op, stream);
    int s = ensure_sym(op, st);
    if (s) return s;
    s = ensure_work64i(op, 8);
    if (s) return s;
    s = enqueue_matvec(op, d_v, d_u, 0, st, false, true);
    return s == AFM_SUCCESS ? ok() : s;
}

int afm_matvec(afm_operator* op, double* v, const double* u, int is_ghosted) {
    (void)is_ghosted;
    AFM_CHECK_OP(op);
    if (!op->finalized) return fail(AFM_ERR_STATE, "matvec before finalize");
    if (!v || !u) return fail(AFM_ERR_INVALID_ARG, "null vector");
    if (op->precision == AFM_PREC_FP32) return fail(AFM_ERR_STATE, "FP32 operator: use afm_matvec_device_f32");
    DeviceGuard g(op->device);
    int s = ensure_work(op, 2);
    if (s) return s;
    double* du = op->d_work;
    double* dv = op->d_work + op->n_dofs;
    const size_t bytes = sizeof(double) * op->n_dofs;
    AFM_CUDA(cudaMemcpyAsync(du, u, bytes, cudaMemcpyHostToDevice, op->stream));
    s = enqueue_matvec(op, dv, du, 0, op->stream);
    if (s) return s;
    AFM_CUDA(cudaMemcpyAsync(v, dv, bytes, cudaMemcpyDeviceToHost, op->stream));
    s = check_device_error(op);
    return s == AFM_SUCCESS ? ok() : s;
}

int afm_matmult_bc_device(afm_operator* op, double* d_v, const double* d_u, void* stream) {
    AFM_CHECK_OP(op);
    if (!op->finalized) return fail(AFM_ERR_STATE, "matmult before finalize");
    if (op->precision == AFM_PREC_FP32) return fail(AFM_ERR_STATE, "FP32 operator");
    if (!d_v || !d_u || d_v == (double*)d_u) return fail(AFM_ERR_INVALID_ARG, "bad vectors");
    DeviceGuard g(op->device);
    cudaStream_t st = pick_stream(op, stream);
    int s = enqueue_matvec(op, d_v, d_u, 1, st);
    if (s) return s;
    AFM_CUDA(launch_set_constrained(d_v, d_u, op->d_bc_idx, op->n_bc, st));
    return ok();
}

int afm_matmult_bc(afm_operator* op, double* v, const double* u) {
    AFM_CHECK_OP(op);
    if (!op->finalized) return fail(AFM_ERR_STATE, "matmult before finalize");
    if (!v || !u) return fail(AFM_ERR_INVALID_ARG, "null vector");
    DeviceGuard g(op->device);
    int s = ensure_work(op, 2);
    if (s) return s;
    double* du = op->d_work;
    double* dv = op->d_work + op->n_dofs;
    const size_t bytes = sizeof(double) * op->n_dofs;
    AFM_CUDA(cudaMemcpyAsync(du, u, bytes, cudaMemcpyHostToDevice, op->stream));
    s = afm_matmult_bc_device(op, dv, du, op->stream);
    if (s) return s;
    AFM_CUDA(cudaMemcpyAsync(v, dv, bytes, cudaMemcpyDeviceToHost, op->stream));
    s = check_device_error(op);
    return s == AFM_SUCCESS ? ok() : s;
}

int afm_matmult_bc_device_f32(afm_operator* op, float* d_v, const float* d_u, void* stream) {
    AFM_CHECK_OP(op);
    if (!op->finalized) return fail(AFM_ERR_STATE, "matmult before finalize");
    if (op->precision != AFM_PREC_FP32 && op->precision != AFM_PREC_FP64_SPLIT && op->matfree_type != 2)
        return fail(AFM_ERR_STATE, "FP32 product needs an FP32, FP64_SPLIT or matrix-free operator");
    if (!d_v || !d_u || (void*)d_v == (const void*)d_u) return fail(AFM_ERR_INVALID_ARG, "bad vectors");
    DeviceGuard g(op->device);
    cudaStream_t st = pick_stream(op, stream);
    int s = ensure_sym(op, st);
    if (s) return s;
    s = enqueue_matvec(op, d_v, d_u, 1, st, true);
    if (s) return s;
    AFM_CUDA(launch_set_constrained(d_v, d_u, op->d_bc_idx, op->n_bc, st));
    return ok();
}

int afm_get_diagonal(afm_operator* op, double* diag) {
    AFM_CHECK_OP(op);
    if (!op->finalized) return fail(AFM_ERR_STATE, "get_diagonal before finalize");
    if (!diag) return fail(AFM_ERR_INVALID_ARG, "null diag");
    memcpy(diag, op->diag_host.data(), sizeof(double) * op->n_dofs);
    return ok();
}

int afm_get_trace(afm_operator* op, double* trace) {
    AFM_CHECK_OP(op);
    if (!op->finalized) return fail(AFM_ERR_STATE, "get_trace before finalize");
    if (!trace) return fail(AFM_ERR_INVALID_ARG, "null trace");
    *trace = op->trace;
    return ok();
}

int afm_apply_bc_rhs(afm_operator* op, double* rhs) {
    AFM_CHECK_OP(op);
    if (!op->finalized) return fail(AFM_ERR_STATE, "apply_bc before finalize");
    if (!rhs) return fail(AFM_ERR_INVALID_ARG, "null rhs");
    if (op->bc_method == AFM_BC_PENALTY) {
        const double pen = 100.0 * op->trace;
        for (size_t i = 0; i < op->constrained.size(); i++) rhs[op->constrained[i]] = pen * op->values[i];
        return ok();
    }
    if (op->precision == AFM_PREC_FP32) return fail(AFM_ERR_STATE, "FP32 operator");
    // K_fc U_c as K g with g = U_c on constrained DoFs and 0 elsewhere (the
    // assembled operator's route, include/aMatBased.hpp:366-410)
    std::vector<double> g(op->n_dofs, 0.0), kg(op->n_dofs);
    std::vector<uint8_t> is_bc(op->n_dofs, 0);
    for (size_t i = 0; i < op->constrained.size(); i++) {
        g[op->constrained[i]] = op->values[i];
        is_bc[op->constrained[i]] = 1;
    }
    int s = afm_matvec(op, kg.data(), g.data(), 1);
    if (s) return s;
    for (size_t i = 0; i < op->constrained.size(); i++) rhs[op->constrained[i]] = op->values[i];
    for (uint32_t d = 0; d < op->n_dofs; d++)
        if (!is_bc[d]) rhs[d] = -kg[d] + rhs[d];
    return ok();
}

int afm_solve_cg_device(afm_operator* op, const double* d_b, double* d_x, double rtol, double atol, int maxit,
                        int norm_type, afm_solve_stats* stats) {
    AFM_CHECK_OP(op);
    if (!op->finalized) return fail(AFM_ERR_STATE, "solve before finalize");
    if (op->precision == AFM_PREC_FP32) return fail(AFM_ERR_STATE, "FP32 operator: use the mixed-precision solve");
    if (!d_b || !d_x) return fail(AFM_ERR_INVALID_ARG, "null vector");
    if (norm_type != AFM_CG_NORM_UNPRECONDITIONED && norm_type != AFM_CG_NORM_PRECONDITIONED)
        return fail(AFM_ERR_INVALID_ARG, "norm type %d", norm_type);
    DeviceGuard g(op->device);
    int s = ensure_work(op, 8);
    if (s) return s;
    const size_t n = op->n_dofs;
    CgVectors<double> V{op->d_work + 2 * n, op->d_work + 3 * n, op->d_work + 4 * n, op->d_work + 5 * n,
                        op->d_work + 6 * n, d_x};
    double* sc = op->d_scalars;
    double* part = op->d_scalars + kScalarSlots;
    cudaStream_t st = op->stream;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, st);
    AFM_CUDA(launch_invert(V.dinv, op->d_diag, n, st));
    s = afm_matmult_bc_device(op, V.q, d_x, st);
    if (s) return s;
    AFM_CUDA(launch_cg_init(d_b, V.q, V.dinv, V.r, V.z, V.p, n, sc, part, st));
    AFM_CUDA(cudaMemcpyAsync(op->h_scalars, sc, sizeof(double) * kScalarSlots, cudaMemcpyDeviceToHost, st));
    AFM_CUDA(cudaStreamSynchronize(st));
    const double bn = std::sqrt(op->h_scalars[S_BB]);
    const double ref = (norm_type == AFM_CG_NORM_UNPRECONDITIONED) ? bn : std::sqrt(op->h_scalars[S_DB]);
    const double tol = std::max(rtol * ref, atol);
    int it = 0, status = AFM_ERR_MAXIT;
    s = run_cg_iterations<double>(op, op->cg64, V, tol, maxit, norm_type, &it, &status);
    if (s) return s;
    cudaEventRecord(e1, st);
    // true residual in FP64
    s = afm_matmult_bc_device(op, V.q, d_x, st);
    if (s) return s;
    AFM_CUDA(launch_axpby(V.q, d_b, 1.0, -1.0, n, st));  // q = b - A x
    AFM_CUDA(launch_norm2(V.q, n, sc, part, st));
    AFM_CUDA(cudaMemcpyAsync(op->h_scalars, sc, sizeof(double) * kScalarSlots, cudaMemcpyDeviceToHost, st));
    AFM_CUDA(cudaStreamSynchronize(st));
    const double rr = op->h_scalars[S_PQ];
    const double rn = std::sqrt(norm_type == AFM_CG_NORM_UNPRECONDITIONED ? op->h_scalars[S_RR] : op->h_scalars[S_ZZ]);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    s = check_device_error(op);
    if (s) return s;
    if (stats) {
        stats->iterations = it;
        stats->status = status;
        stats->rel_residual = bn > 0 ? std::sqrt(rr) / bn : std::sqrt(rr);
        stats->residual_norm = rn;
        stats->seconds = ms * 1e-3;
        stats->refinements = 0;
    }
    if (status != AFM_SUCCESS)
        return fail(status, status == AFM_ERR_MAXIT ? "CG reached maxit=%d" : "CG breakdown after %d iterations", it);
    return ok();
}

int afm_solve_cg(afm_operator* op, const double* b, double* x, double rtol, double atol, int maxit, int norm_type,
                 afm_solve_stats* stats) {
    AFM_CHECK_OP(op);
    if (!op->finalized) return fail(AFM_ERR_STATE, "solve before finalize");
    if (!b || !x) return fail(AFM_ERR_INVALID_ARG, "null vector");
    DeviceGuard g(op->device);
    int s = ensure_work(op, 8);
    if (s) return s;
    double* db = op->d_work;
    double* dx = op->d_work + op->n_dofs;
    const size_t bytes = sizeof(double) * op->n_dofs;
    AFM_CUDA(cudaMemcpyAsync(db, b, bytes, cudaMemcpyHostToDevice, op->stream));
    AFM_CUDA(cudaMemcpyAsync(dx, x, bytes, cudaMemcpyHostToDevice, op->stream));
    const int st = afm_solve_cg_device(op, db, dx, rtol, atol, maxit, norm_type, stats);
    const std::string msg = g_last_error;
    AFM_CUDA(cudaMemcpyAsync(x, dx, bytes, cudaMemcpyDeviceToHost, op->stream));
    AFM_CUDA(cudaStreamSynchronize(op->stream));
    if (st != AFM_SUCCESS) return fail(st, "%s", msg.c_str());
    return ok();
}


int afm_solve_cg_mixed_device(afm_operator* op, const double* d_b, double* d_x, double rtol, double atol,
                              int max_outer, double inner_rtol, int max_inner, afm_solve_stats* stats) {
    MixedSolve m;
    m.op = op;
    m.d_b = d_b;
    m.d_x = d_x;
    m.rtol = rtol;
    m.atol = atol;
    m.max_outer = max_outer;
    m.inner_rtol = inner_rtol;
    m.max_inner = max_inner;
    int s = mixed_begin(m);
    while (s == AFM_SUCCESS && m.phase != MS_DONE) {
        if (cudaEventSynchronize(m.ev) != cudaSuccess) {
            s = fail(AFM_ERR_CUDA, "mixed solve: %s", cudaGetErrorString(cudaGetLastError()));
            break;
        }
        s = mixed_advance(m);
    }
    const int st = mixed_end(m, stats);
    return s != AFM_SUCCESS ? s : st;
}

int afm_debug_segment_geometry(int kind, uint32_t n, uint32_t* out) {
    if (!out || n <= kTpeMaxN || n > kMaxN || kind < 0 || kind > 6)
        return fail(AFM_ERR_INVALID_ARG, "kind %d (0..6), n %u (%u..%u)", kind, n, kTpeMaxN + 1, kMaxN);
    // the unit sizes of build_segments and layout_sym for one element of n DoFs
    const uint64_t plane = (uint64_t)(n * n + 3) / 4 * 4;
    const uint64_t S = (uint64_t)(n / 2 + 1) * n, P = (S + 3) / 4 * 4;
    uint64_t unit = 0, copy = 0;
    Segment s;
    s.n = n;
    s.regime = REG_WPE;
    s.units = s.count = 1u << 20;
    switch (kind) {
        case 0: unit = copy = round16((uint64_t)n * n * 8); segment_smem_fp64_geom(s, copy, unit, out); break;
        case 1: unit = copy = 2 * plane * 4; segment_smem_split_geom(s, copy, unit, out); break;
        case 2: unit = 2 * plane * 4; copy = plane * 4; segment_smem_fp32_geom(s, copy, unit, out); break;
        case 3: unit = copy = round16(S * 4); segment_smem_f32sym_geom(s, copy, unit, out); break;
        case 4: unit = copy = round16(P * 4 + S * 2); segment_smem_f32symx_geom(s, copy, unit, out); break;
        case 5: unit = copy = round16(P * 4 + S * 2); segment_smem_splitsymx_geom(s, copy, unit, out); break;
        default: unit = copy = round16(P * 4 + S * 2); segment_smem_f32symc_geom(s, copy, unit, out); break;
    }
    out[6] = (uint32_t)unit;
    out[7] = (uint32_t)copy;
    return ok();
}

int afm_get_solve_trace(afm_operator* op, uint32_t cap, int* inner_iterations, double* rel_residual, uint32_t* n) {
    AFM_CHECK_OP(op);
    if (!n || (cap && (!inner_iterations || !rel_residual))) return fail(AFM_ERR_INVALID_ARG, "null argument");
    *n = (uint32_t)op->trace_iters.size();
    const uint32_t k = std::min<uint32_t>(cap, *n);
    for (uint32_t i = 0; i < k; i++) {
        inner_iterations[i] = op->trace_iters[i];
        rel_residual[i] = op->trace_res[i];
    }
    return ok();
}

int afm_solve_cg_mixed(afm_operator* op, const double* b, double* x, double rtol, double atol, int max_outer,
                       double inner_rtol, int max_inner, afm_solve_stats* stats) {
    AFM_CHECK_OP(op);
    if (!op->finalized) return fail(AFM_ERR_STATE, "solve before finalize");
    if (!b || !x) return fail(AFM_ERR_INVALID_ARG, "null vector");
    DeviceGuard g(op->device);
    int s = ensure_work(op, 8);
    if (s) return s;
    double* db = op->d_work;
    double* dx = op->d_work + op->n_dofs;
    const size_t bytes = sizeof(double) * op->n_dofs;
    AFM_CUDA(cudaMemcpyAsync(db, b, bytes, cudaMemcpyHostToDevice, op->stream));
    AFM_CUDA(cudaMemcpyAsync(dx, x, bytes, cudaMemcpyHostToDevice, op->stream));
    const int st = afm_solve_cg_mixed_device(op, db, dx, rtol, atol, max_outer, inner_rtol, max_inner, stats);
    const std::string msg = g_last_error;
    AFM_CUDA(cudaMemcpyAsync(x, dx, bytes, cudaMemcpyDeviceToHost, op->stream));
    AFM_CUDA(cudaStreamSynchronize(op->stream));
    if (st != AFM_SUCCESS) return fail(st, "%s", msg.c_str());
    return ok();
}

int afm_matvec_batched_device(afm_operator* op, double* d_V, const double* d_U, uint32_t nrhs, uint32_t ld,
                              void* stream) {
    AFM_CHECK_OP(op);
    return batched_product<double>(op, d_V, d_U, nrhs, ld, 0, stream);
}

int afm_matvec_batched_device_f32(afm_operator* op, float* d_V, const float* d_U, uint32_t nrhs, uint32_t ld,
                                  void* stream) {
    AFM_CHECK_OP(op);
    return batched_product<float>(op, d_V, d_U, nrhs, ld, 0, stream);
}

int afm_matmult_bc_batched_device(afm_operator* op, double* d_V, const double* d_U, uint32_t nrhs, uint32_t ld,
                                  void* stream) {
    AFM_CHECK_OP(op);
    return batched_product<double>(op, d_V, d_U, nrhs, ld, 1, stream);
}

int afm_matmult_bc_batched_device_f32(afm_operator* op, float* d_V, const float* d_U, uint32_t nrhs, uint32_t ld,
                                      void* stream) {
    AFM_CHECK_OP(op);
    return batched_product<float>(op, d_V, d_U, nrhs, ld, 1, stream);
}

int afm_get_batch_tuning(afm_operator* op, uint32_t nrhs, uint32_t ld, int f32, int* cols_per_thread,
                         int* rows_per_thread, float* ms) {
    AFM_CHECK_OP(op);
    if (f32 < 0 || f32 > 2) return fail(AFM_ERR_INVALID_ARG, "f32 %d: 0, 1 or 2", f32);
    const int kprec = f32 ? AFM_PREC_FP32 : op->precision;
    const uint64_t key =
        ((uint64_t)nrhs << 40) | ((uint64_t)ld << 8) | (uint64_t)kprec | (f32 == 2 ? 0x80u : 0u);
    for (const auto& t : op->batch_tune)
        if (t.key == key) {
            if (cols_per_thread) *cols_per_thread = t.tr;
            if (rows_per_thread) *rows_per_thread = t.ng;
            if (ms) *ms = t.ms;
            return ok();
        }
    return fail(AFM_ERR_STATE, "no batched call with nrhs %u yet", nrhs);
}

int afm_set_batch_tuning(afm_operator* op, uint32_t nrhs, uint32_t ld, int f32, int cols_per_thread,
                         int rows_per_thread) {
    AFM_CHECK_OP(op);
    if (!op->finalized) return fail(AFM_ERR_STATE, "before finalize");
    const bool tc = cols_per_thread == 0 && rows_per_thread == 0;
    if (tc && !(f32 && batched_tc_all(op, nrhs)))
        return fail(AFM_ERR_INVALID_ARG, "the tensor-core kernel takes FP32 products with nrhs 32, 64 or 128");
    const bool tile_ok = tc || (cols_per_thread == 4 && rows_per_thread == 4) ||
                         (cols_per_thread == 8 && (rows_per_thread == 2 || rows_per_thread == 4 || rows_per_thread == 6));
    if (!tile_ok || (!tc && nrhs % (uint32_t)cols_per_thread))
        return fail(AFM_ERR_INVALID_ARG, "tile %d rows x %d columns for nrhs %u", rows_per_thread, cols_per_thread, nrhs);
    const int groups_per_cta = rows_per_thread;
    const int kprec = f32 ? AFM_PREC_FP32 : op->precision;
    const uint64_t key = ((uint64_t)nrhs << 40) | ((uint64_t)ld << 8) | (uint64_t)kprec;
    for (auto& t : op->batch_tune)
        if (t.key == key) {
            t.tr = cols_per_thread;
            t.ng = groups_per_cta;
            return ok();
        }
    op->batch_tune.push_back({key, cols_per_thread, groups_per_cta, 0.0f});
    return ok();
}

int afm_solve_cg_batched_device(afm_operator* op, const double* d_B, double* d_X, uint32_t nrhs, double rtol,
                                double atol, int maxit, afm_solve_stats* stats) {
    AFM_CHECK_OP(op);
    int s = check_batched(op, nrhs, nrhs);
    if (s) return s;
    if (op->precision == AFM_PREC_FP32) return fail(AFM_ERR_STATE, "FP32 operator");
    if (!d_B || !d_X) return fail(AFM_ERR_INVALID_ARG, "null block");
    if (((uintptr_t)d_B | (uintptr_t)d_X) % 16) return fail(AFM_ERR_INVALID_ARG, "blocks must be 16-byte aligned");
    DeviceGuard g(op->device);
    const size_t n = op->n_dofs, N = n * nrhs;
    s = ensure_bwork(op, 4 * N + n);
    if (s) return s;
    s = ensure_bscalars(op, nrhs);
    if (s) return s;
    BVectors<double> V{op->d_bwork, op->d_bwork + N, op->d_bwork + 2 * N, op->d_bwork + 3 * N, op->d_bwork + 4 * N,
                       d_X};
    cudaStream_t st = op->stream;
    int tr = 4, ng = 2;
    s = batch_tuning(op, V.q, d_X, nrhs, nrhs, false, st, &tr, &ng);
    if (s) return s;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, st);
    AFM_CUDA(launch_invert(V.dinv, op->d_diag, n, st));
    s = enqueue_matvec_batched(op, V.q, d_X, nrhs, nrhs, 1, st, false, tr, ng);
    if (s) return s;
    AFM_CUDA(launch_bset_constrained(V.q, d_X, op->d_bc_idx, op->n_bc, nrhs, nrhs, st));
    AFM_CUDA(launch_bcg_init(d_B, V.q, V.dinv, V.r, V.z, V.p, n, nrhs, nrhs, op->d_bsc,
                             op->d_bsc + (size_t)nrhs * kBSlots, rtol, atol, st));
    int it = 0;
    bool breakdown = false;
    s = run_bcg<double>(op, V, nrhs, (double)maxit, tr, ng, &it, &breakdown);
    if (s) return s;
    cudaEventRecord(e1, st);
    double worst = 0.0;
    s = batched_residual(op, d_B, d_X, nrhs, V.q, &worst, tr, ng);
    if (s) return s;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    s = check_device_error(op);
    if (s) return s;
    const int status = breakdown ? AFM_ERR_BREAKDOWN : (it < maxit || worst <= rtol) ? AFM_SUCCESS : AFM_ERR_MAXIT;
    if (stats) {
        stats->iterations = it;
        stats->status = status;
        stats->rel_residual = worst;
        stats->residual_norm = worst;
        stats->seconds = ms * 1e-3;
        stats->refinements = 0;
    }
    if (status != AFM_SUCCESS)
        return fail(status, status == AFM_ERR_MAXIT ? "batched CG reached maxit=%d" : "batched CG breakdown (maxit %d)",
                    maxit);
    return ok();
}

int afm_solve_cg_batched_mixed_device(afm_operator* op, const double* d_B, double* d_X, uint32_t nrhs, double rtol,
                                      double atol, int max_outer, double inner_rtol, int max_inner,
                                      afm_solve_stats* stats) {
    AFM_CHECK_OP(op);
    int s = check_batched(op, nrhs, nrhs);
    if (s) return s;
    if (op->precision != AFM_PREC_FP64_SPLIT && op->matfree_type != 2)
        return fail(AFM_ERR_STATE, "mixed-precision solve needs an FP64_SPLIT or matrix-free operator");
    if (!d_B || !d_X) return fail(AFM_ERR_INVALID_ARG, "null block");
    if (((uintptr_t)d_B | (uintptr_t)d_X) % 16) return fail(AFM_ERR_INVALID_ARG, "blocks must be 16-byte aligned");
    DeviceGuard g(op->device);
    const size_t n = op->n_dofs, N = n * nrhs;
    // FP64: residual block (and a spare); FP32: rhs, r, z, p, q, d and 1/diag
    s = ensure_bwork(op, 2 * N + (7 * N + n + 1) / 2 + 2);
    if (s) return s;
    s = ensure_bscalars(op, nrhs);
    if (s) return s;
    double* q64 = op->d_bwork + N;
    float* f = reinterpret_cast<float*>(op->d_bwork + 2 * N);
    float* b32 = f;
    BVectors<float> V{f + N, f + 2 * N, f + 3 * N, f + 4 * N, f + 6 * N, f + 5 * N};
    cudaStream_t st = op->stream;
    int tr64 = 4, ng64 = 2, tr32 = 4, ng32 = 2;
    s = batch_tuning(op, q64, d_X, nrhs, nrhs, false, st, &tr64, &ng64);
    if (s) return s;
    AFM_CUDA(launch_to_f32(b32, d_B, N, st));
    s = batch_tuning(op, V.q, b32, nrhs, nrhs, true, st, &tr32, &ng32, false);
    if (s) return s;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, st);
    AFM_CUDA(launch_invert(V.dinv, op->d_diag, n, st));
    AFM_CUDA(cudaMemsetAsync(V.x, 0, N * sizeof(float), st));
    double* sc = op->d_bsc;
    double* part = op->d_bsc + (size_t)nrhs * kBSlots;
    AFM_CUDA(launch_bstore_norm(d_B, n, nrhs, sc, part, st));
    std::vector<double> hs((size_t)nrhs * kBSlots);
    int outer = 0, inner_total = 0, status = AFM_ERR_MAXIT, stall = 0;
    double worst = 0.0, best = HUGE_VAL;
    for (;;) {
        // FP64 residual block R = B - A X and per-column convergence
        s = enqueue_matvec_batched(op, q64, d_X, nrhs, nrhs, 1, st, false, tr64, ng64);
        if (s) return s;
        AFM_CUDA(launch_bset_constrained(q64, d_X, op->d_bc_idx, op->n_bc, nrhs, nrhs, st));
        AFM_CUDA(launch_axpby(q64, d_B, 1.0, -1.0, N, st));  // q = b - A x
        AFM_CUDA(launch_bcheck(q64, n, nrhs, sc, part, rtol, atol, st));
        AFM_CUDA(cudaMemcpyAsync(hs.data(), sc, hs.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
        AFM_CUDA(cudaStreamSynchronize(st));
        bool all = true, nan = false;
        worst = 0.0;
        for (uint32_t j = 0; j < nrhs; j++) {
            const double* c = &hs[(size_t)j * kBSlots];
            const double rn = std::sqrt(c[B_TRR]);
            nan = nan || std::isnan(rn);
            all = all && c[B_CONV] != 0.0;
            worst = std::max(worst, c[B_BN] > 0 ? rn / c[B_BN] : rn);
        }
        if (nan) {
            status = AFM_ERR_BREAKDOWN;
            break;
        }
        if (all) {
            status = AFM_SUCCESS;
            break;
        }
        if (!ir_progress(worst, &best, &stall) || outer >= max_outer) break;  // MAXIT
        if (outer == 0) {
            // FP32 block Jacobi-PCG on A D = R from D = 0
            AFM_CUDA(launch_to_f32(b32, q64, N, st));
            AFM_CUDA(cudaMemsetAsync(V.q, 0, N * sizeof(float), st));
            AFM_CUDA(launch_bcg_init(b32, V.q, V.dinv, V.r, V.z, V.p, n, nrhs, nrhs, sc, part, inner_rtol, 0.0, st));
        } else {
            // reliable update: each column's recursion continues from its true residual
            AFM_CUDA(launch_breliable(q64, V.r, V.z, V.p, V.dinv, n, nrhs, sc, part, inner_rtol, st));
        }
        int it = 0;
        s = run_bcg<float>(op, V, nrhs, (double)max_inner, tr32, ng32, &it);
        if (s) return s;
        inner_total += it;
        AFM_CUDA(launch_add_f32(d_X, V.x, N, st));  // X += X_s, X_s = 0
        outer++;
    }
    cudaEventRecord(e1, st);
    AFM_CUDA(cudaStreamSynchronize(st));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    s = check_device_error(op);
    if (s) return s;
    if (stats) {
        stats->iterations = inner_total;
        stats->status = status;
        stats->rel_residual = worst;
        stats->residual_norm = worst;
        stats->seconds = ms * 1e-3;
        stats->refinements = outer;
    }
    if (status != AFM_SUCCESS) return fail(status, "batched refinement stopped after %d steps", outer);
    return ok();
}

int afm_patch_plan_host_matvec(uint32_t n_elem, uint32_t n_dofs, const uint32_t* offsets, const uint32_t* map,
                               const double* ke, const double* u, double* v, uint32_t* n_patches,
                               uint32_t* n_patch_colors) {
    if (!offsets || !map || !ke || !u || !v || n_elem == 0) return fail(AFM_ERR_INVALID_ARG, "bad arguments");
    afm_operator op;
    op.n_elem = n_elem;
    op.n_dofs = n_dofs;
    op.offsets.assign(offsets, offsets + n_elem + 1);
    op.map.assign(map, map + offsets[n_elem]);
    const uint32_t n = offsets[1] - offsets[0];
    for (uint32_t e = 0; e < n_elem; e++) {
        if (offsets[e + 1] - offsets[e] != n) return fail(AFM_NOT_IMPLEMENTED, "elements of different sizes");
        for (uint32_t i = offsets[e]; i < offsets[e + 1]; i++) {
            if (map[i] >= n_dofs) return fail(AFM_INDEX_OUT_OF_BOUNDS, "DoF %u", map[i]);
            for (uint32_t k = offsets[e]; k < i; k++)
                if (map[k] == map[i]) return fail(AFM_NOT_IMPLEMENTED, "element %u lists DoF %u twice", e, map[i]);
        }
    }
    if (n == 0 || n > kPatchMaxN) return fail(AFM_NOT_IMPLEMENTED, "n = %u", n);
    std::vector<PatchDesc> desc;
    std::vector<unsigned char> idx;
    if (!build_patch_plan(&op, n, AFM_PREC_FP64, desc, idx)) return fail(AFM_NOT_IMPLEMENTED, "no patch plan");
    const Segment& s = op.segs[0];
    // every element in exactly one slot; slots agree with the descriptors
    std::vector<uint32_t> seen(n_elem, 0);
    for (uint32_t e : op.perm)
        if (e != kNoElement) seen[e]++;
    for (uint32_t e = 0; e < n_elem; e++)
        if (seen[e] != 1) return fail(AFM_ERR_INTERNAL, "element %u in %u slots", e, seen[e]);
    std::fill(v, v + n_dofs, 0.0);
    std::vector<uint32_t> stamp(n_dofs, UINT32_MAX);
    std::vector<uint32_t> listed(n_dofs, 0);
    std::vector<uint8_t> shared(n_dofs, 0);
    for (uint32_t g : op.shared_dof) shared[g] = 1;
    std::vector<double> us, ve;
    const size_t ncol = op.patch_color_first.size() - 1;
    for (size_t c = 0; c < ncol; c++) {
        for (uint32_t x = op.patch_color_first[c]; x < op.patch_color_first[c + 1]; x++) {
            const PatchDesc& d = desc[x];
            if (d.idx_off % 16 || d.idx_bytes % 16 || d.ke_off % s.unit_bytes || d.idx_off + d.idx_bytes > idx.size() ||
                d.ndof > op.patch_geom.max_ndof || d.units * 32 > op.patch_geom.max_slots ||
                d.idx_bytes > op.patch_geom.max_idx || d.elems > d.units * 32 || d.ndof == 0)
                return fail(AFM_ERR_INTERNAL, "patch %u descriptor", x);
            const unsigned char* blk = idx.data() + d.idx_off;
            const uint32_t* glob = reinterpret_cast<const uint32_t*>(blk);
            const uint16_t* lmap = reinterpret_cast<const uint16_t*>(blk + patch_lmap_off(d.ndof));
            const uint16_t* coff = reinterpret_cast<const uint16_t*>(blk + patch_csr_off(d.ndof, d.units, n));
            const uint16_t* slot = reinterpret_cast<const uint16_t*>(blk + patch_slot_off(d.ndof, d.units, n));
            const uint32_t cap = d.units * 32;
            // patches of one colour share no DoF
            for (uint32_t k = 0; k < d.ndof; k++) {
                const uint32_t g = glob[k] & kPatchDofMask;
                if (g >= n_dofs || (k && g <= (glob[k - 1] & kPatchDofMask)))
                    return fail(AFM_ERR_INTERNAL, "patch %u DoF list", x);
                if (stamp[g] == c) return fail(AFM_ERR_INTERNAL, "colour %zu: DoF %u in two patches", c, g);
                stamp[g] = (uint32_t)c;
            }
            if (coff[0] != 0 || coff[d.ndof] != d.elems * n) return fail(AFM_ERR_INTERNAL, "patch %u offsets", x);
            us.assign(d.ndof, 0.0);
            for (uint32_t k = 0; k < d.ndof; k++) us[k] = u[glob[k] & kPatchDofMask];
            ve.assign((size_t)n * cap, -1.0);
            const uint64_t slot0 = d.ke_off / s.unit_bytes * kTpeWidth;
            for (uint32_t un = 0; un < d.units; un++)
                for (uint32_t lane = 0; lane < 32; lane++) {
                    const uint32_t el = un * 32 + lane;
                    const uint32_t e = op.perm[slot0 + el];
                    if ((el < d.elems) != (e != kNoElement)) return fail(AFM_ERR_INTERNAL, "patch %u slot %u", x, el);
                    for (uint32_t r = 0; r < n; r++) {
                        double acc = 0.0;
                        for (uint32_t cc = 0; cc < n; cc++) {
                            const uint32_t l = lmap[((size_t)un * n + cc) * 32 + lane];
                            if (l >= d.ndof) return fail(AFM_ERR_INTERNAL, "patch %u local index", x);
                            if (e != kNoElement) {
                                if ((glob[l] & kPatchDofMask) != map[offsets[e] + cc])
                                    return fail(AFM_ERR_INTERNAL, "patch %u element %u column %u", x, e, cc);
                                acc += ke[(size_t)e * n * n + (size_t)r * n + cc] * us[l];
                            }
                        }
                        ve[(size_t)r * cap + el] = acc;
                    }
                }
            for (uint32_t k = 0; k < d.ndof; k++) {
                double sum = 0.0;
                for (uint32_t q = coff[k]; q < coff[k + 1]; q++) {
                    if (slot[q] >= n * cap || (slot[q] % cap) >= d.elems)
                        return fail(AFM_ERR_INTERNAL, "patch %u contribution slot", x);
                    sum += ve[slot[q]];
                }
                v[glob[k] & kPatchDofMask] += sum;
                listed[glob[k] & kPatchDofMask]++;
                if (((glob[k] & kSharedFlag) != 0) != (shared[glob[k] & kPatchDofMask] != 0))
                    return fail(AFM_ERR_INTERNAL, "patch %u: shared flag of DoF %u", x, glob[k] & kPatchDofMask);
            }
        }
    }
    // shared flags and combine lists: a DoF is shared iff several patches list it, and its list holds
    // one entry per listing patch, in patch order, inside the combine buffer
    for (uint32_t g = 0; g < n_dofs; g++)
        if ((listed[g] > 1) != (shared[g] != 0)) return fail(AFM_ERR_INTERNAL, "DoF %u shared flag", g);
    if (op.shared_off.size() != op.shared_dof.size() + 1 || op.shared_off.back() != op.shared_idx.size())
        return fail(AFM_ERR_INTERNAL, "combine list offsets");
    for (size_t i = 0; i < op.shared_dof.size(); i++) {
        const uint32_t g = op.shared_dof[i];
        if (op.shared_off[i + 1] - op.shared_off[i] != listed[g]) return fail(AFM_ERR_INTERNAL, "DoF %u list", g);
        for (uint32_t k = op.shared_off[i]; k < op.shared_off[i + 1]; k++) {
            if (op.shared_idx[k] >= op.pv_count || (k > op.shared_off[i] && op.shared_idx[k] <= op.shared_idx[k - 1]))
                return fail(AFM_ERR_INTERNAL, "DoF %u list entry %u", g, k);
            // the entry is the local index of g in the patch whose range holds it
            const uint32_t e = op.shared_idx[k];
            const auto it = std::upper_bound(desc.begin(), desc.end(), e,
                                             [](uint32_t val, const PatchDesc& d) { return val < d.pv_off; });
            const size_t x = (size_t)(it - desc.begin()) - 1;
            const uint32_t* glob = reinterpret_cast<const uint32_t*>(idx.data() + desc[x].idx_off);
            if (e - desc[x].pv_off >= desc[x].ndof || (glob[e - desc[x].pv_off] & kPatchDofMask) != g)
                return fail(AFM_ERR_INTERNAL, "DoF %u list entry %u points elsewhere", g, k);
        }
    }
    if (n_patches) *n_patches = op.n_patches;
    if (n_patch_colors) *n_patch_colors = (uint32_t)ncol;
    return ok();
}

int afm_get_info(afm_operator* op, afm_info* info) {
    AFM_CHECK_OP(op);
    if (!info) return fail(AFM_ERR_INVALID_ARG, "null info");
    memset(info, 0, sizeof(*info));
    info->n_elements = op->n_elem;
    info->n_dofs = op->n_dofs;
    info->n_colors = op->n_colors;
    info->max_dofs_per_element = op->nmax;
    info->precision = op->finalized ? op->precision : op->precision_req;
    info->ke_bytes = op->ke_bytes;
    info->map_bytes = op->map_bytes;
    const size_t eb = entry_bytes(op->finalized ? op->precision : AFM_PREC_FP64);
    const size_t vb = (op->finalized && op->precision == AFM_PREC_FP32) ? 4 : 8;
    uint64_t alg = 0;
    double fl = 0;
    for (uint32_t e = 0; e < op->n_elem; e++) {
        const uint64_t n = op->offsets[e + 1] - op->offsets[e];
        alg += n * n * eb + 4 * n;
        fl += 2.0 * (double)(n * n);
    }
    info->algorithmic_bytes = alg + 2 * vb * (uint64_t)op->n_dofs;
    info->algorithmic_flops = fl;
    uint32_t launches = 1;  // the zero fill of v
    if (op->matfree_type == 2 && op->finalized) {
        // matrix-free: node coordinates and the map per element instead of Ke
        info->algorithmic_bytes = (uint64_t)op->n_elem * (op->elem_nodes * 3 * 8 + (uint64_t)op->nmax * 4) +
                                  16 * (uint64_t)op->n_dofs;
        launches += (uint32_t)op->free_color_first.size() - 1;
    } else if (op->use_patches) {
        launches += op->patch_one_launch ? 1u + (op->n_shared ? 1u : 0u) : (uint32_t)op->patch_color_first.size() - 1;
    } else {
        for (const Segment& s : op->segs)
            if (s.units) launches++;
    }
    info->n_launches = launches;
    info->n_patches = op->n_patches;
    info->n_patch_colors = op->use_patches ? (uint32_t)op->patch_color_first.size() - 1 : 0;
    info->patch_index_bytes = op->use_patches ? op->patch_idx_bytes : 0;
    info->ke_symmetric = op->ke_symmetric ? 1 : 0;
    info->sym_available = sym_format(op);
    info->sym_bytes = op->d_sym ? op->sym_bytes : 0;
    info->csr_nnz = op->csr_nnz;
    info->work_bytes = op->work_elems * sizeof(double) + op->work32_elems * sizeof(float) +
                       op->work64i_elems * sizeof(double) +
                       op->bwork_elems * sizeof(double) + op->bsc_elems * sizeof(double);
    info->device = op->device;
    return ok();
}

int afm_get_colors(afm_operator* op, uint32_t* colors) {
    AFM_CHECK_OP(op);
    if (!op->finalized) return fail(AFM_ERR_STATE, "colours before finalize");
    if (!colors) return fail(AFM_ERR_INVALID_ARG, "null colors");
    memcpy(colors, op->colors.data(), sizeof(uint32_t) * op->n_elem);
    return ok();
}

int afm_get_stream(afm_operator* op, void** stream) {
    AFM_CHECK_OP(op);
    if (!stream) return fail(AFM_ERR_INVALID_ARG, "null stream");
    *stream = (void*)op->stream;
    return ok();
}

int afm_synchronize(afm_operator* op) {
    AFM_CHECK_OP(op);
    DeviceGuard g(op->device);
    int s = check_device_error(op);
    return s == AFM_SUCCESS ? ok() : s;
}

}  // extern "C"
