// Internal types shared by the host runtime (afm_capi.cpp) and the CUDA
// kernels (afm_kernels.cu, afm_solver.cu) of the GB300 AFM operator.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/afm.h"

namespace afm {

// Kernel regimes, picked per element size n.
//   TPE (thread per element, n <= kTpeMaxN): 32 elements of one colour form a
//       unit; the unit's Ke is stored entry-major [k][32] so that lane l reads
//       entry k of element l; map [i][32].
//   WPE (warp per element, n > kTpeMaxN): one element per unit; its Ke is
//       stored column-major so lane r reads row r of column c; map [i].
enum Regime : int { REG_TPE = 0, REG_WPE = 1 };
constexpr uint32_t kTpeMaxN = 16;
constexpr uint32_t kTpeWidth = 32;
constexpr uint32_t kMaxN = 96;           // largest element supported (3 rows per lane)
constexpr uint32_t kBcFlag = 0x80000000u;  // map bit: DoF is constrained
constexpr uint32_t kDofMask = 0x7fffffffu;
// Patch index blocks also flag DoFs that more than one patch lists (their sums
// go through the combine pass), so their DoF ids keep 30 bits.
constexpr uint32_t kSharedFlag = 0x40000000u;
constexpr uint32_t kPatchDofMask = 0x3fffffffu;

// Device error flags (bit set in err[0]); err[1..6] record the first failed
// bounds check (kind, block, thread and three values); kErrWords ints in all.
constexpr int kErrTimeout = 1;
constexpr int kErrBounds = 2;
constexpr int kErrWords = 8;  // the last word is never written: the flag of afm_set_wait_probe

// One launch of the matvec: the elements of one colour that share n.
struct Segment {
    uint32_t color = 0;
    uint32_t n = 0;
    int regime = REG_WPE;
    uint64_t first_pos = 0;   // first element position (colour-sorted order)
    uint32_t count = 0;       // elements
    uint32_t units = 0;       // work units (TPE: ceil(count/32), WPE: count)
    uint64_t ke_offset = 0;   // byte offset of the first unit in the Ke arena
    uint64_t unit_bytes = 0;  // arena bytes per unit (16-byte multiple)
    uint64_t map_offset = 0;  // uint32 offset of the first unit in the map
    uint32_t plane = 0;       // FP64_SPLIT: entries per plane of a unit (the lo plane follows the hi plane)
    uint64_t sym_offset = 0;     // byte offset of the first unit in the symmetric inner arena
    uint64_t sym_unit_bytes = 0; // its bytes per unit (0: no symmetric form)
    uint32_t sym_plane = 0;      // entries of a unit's FP32 plane before its BF16 correction plane (0: none)
};

// Colours of one fused (cooperative) launch of the warp-group kernel, at most.
constexpr uint32_t kMaxFusedColours = 48;

// Arguments of one segment launch.
struct SegArgs {
    const unsigned char* ke;  // arena + segment offset
    const uint32_t* map;      // map + segment offset
    const void* u;            // double* or float*
    void* v;                  // double* or float*
    uint32_t units;
    uint32_t count;           // elements (TPE: last unit may be partial)
    uint64_t unit_bytes;      // stride between units in the arena
    uint32_t copy_bytes;      // bytes copied per unit (the hi plane only for FP32 on a split arena)
    uint32_t plane;           // entries per plane (split arena)
    int bc_mode;              // 1: constrained columns read as zero (MatMult_mf)
    int* err;
    const unsigned long long* umax;  // split arithmetic: max|u| (bits of a non-negative double)
    unsigned long long wait_ns;  // limit of each pipeline wait (afm_set_wait_limit)
    const int* probe;         // test hook: a flag nothing sets, or null (afm_set_wait_probe)
};

// Arguments of one batched (multi right-hand side) segment launch.
struct BatchArgs {
    const unsigned char* ke;
    const uint32_t* map;
    const void* u;  // n_dofs x ld, row-major
    void* v;
    uint32_t units, count;
    uint64_t unit_bytes;
    uint32_t copy_bytes, plane;
    uint32_t nrhs, ld;
    int bc_mode;
    int* err;
    uint32_t n_dofs;      // rows of U and V (bounds checks)
    uint32_t smem_total;  // dynamic shared memory of the launch (bounds checks)
    const unsigned long long* umax;  // split arithmetic: max|U(:, j)| per column j (double bits)
    unsigned long long wait_ns;  // limit of each pipeline wait
    const int* probe;         // test hook: a flag nothing sets, or null (afm_set_wait_probe)
};

// ---- patch path (small elements) -----------------------------------------
// Elements with at most kPatchMaxN DoFs (all of one size, no DoF listed twice
// in an element) run as patches: compact groups of up to kPatchElems elements,
// coloured so that patches of one colour share no DoF (see afm_patch.cuh).
constexpr uint32_t kPatchMaxN = 12;
constexpr uint32_t kPatchMaxDofs = 1024;  // local DoFs per patch (uint16 indices)

constexpr uint32_t kNoElement = 0xffffffffu;  // empty element slot

#ifdef __CUDACC__
#define AFM_HD __host__ __device__
#else
#define AFM_HD
#endif
// Byte offsets inside one patch index block (all 16-byte aligned): glob
// (uint32 x ndof), lmap (uint16 x units x n x 32), csr_off (uint16 x ndof+1),
// slot (uint16 x contributions).
AFM_HD inline uint32_t patch_r16(uint32_t x) { return (x + 15u) & ~15u; }
AFM_HD inline uint32_t patch_lmap_off(uint32_t ndof) { return patch_r16(ndof * 4u); }
AFM_HD inline uint32_t patch_csr_off(uint32_t ndof, uint32_t units, uint32_t n) {
    return patch_lmap_off(ndof) + units * n * 64u;
}
AFM_HD inline uint32_t patch_slot_off(uint32_t ndof, uint32_t units, uint32_t n) {
    return patch_csr_off(ndof, units, n) + patch_r16((ndof + 1u) * 2u);
}

// One patch: its Ke units and its index block (both 16-byte aligned).
struct PatchDesc {
    uint64_t ke_off;     // bytes into the Ke arena (unit0 x its unit size)
    uint64_t idx_off;    // bytes into the index arena
    uint32_t units;      // units of 32 element slots
    uint32_t ndof;       // local DoFs
    uint32_t idx_bytes;  // size of the index block (16-byte multiple)
    uint32_t elems;      // elements (the rest of the slots are empty)
    uint32_t unit0;      // first unit of the patch, in units of any arena
    uint32_t pv_off;     // first entry of the patch's local DoF sums in the combine buffer
};

// Arguments of one patch-colour launch.
struct PatchArgs {
    const PatchDesc* desc;    // the colour's first patch
    uint32_t count;           // patches of the colour
    const unsigned char* ke;  // Ke arena
    const unsigned char* idx; // index arena
    const void* u;
    void* v;
    uint64_t unit_bytes;      // stride between units
    uint32_t copy_bytes;      // bytes copied per unit (hi plane only for FP32 on a split arena)
    uint32_t plane;           // entries per plane (split arena)
    int bc_mode;
    int* err;
    void* pv;                 // one launch for every colour: sums of shared DoFs go here (VO), others to v;
                              // null: one launch per colour, every sum added to v
    const unsigned long long* umax;  // split arithmetic: max|u| (double bits)
    unsigned long long wait_ns;  // limit of each pipeline wait
    const int* probe;         // test hook: a flag nothing sets, or null (afm_set_wait_probe)
};

// Patch launch geometry shared by all colours of an operator.
struct PatchPlanGeom {
    uint32_t n = 0;           // DoFs per element
    uint32_t max_slots = 0;   // largest patch, in element slots (32 x units)
    uint32_t max_ndof = 0;    // largest local DoF count
    uint32_t max_idx = 0;     // largest index block, bytes
};

cudaError_t launch_patches(int prec, const PatchPlanGeom& pg, const PatchArgs& a, int sm_count, bool pdl,
                           cudaStream_t stream);
// The combine pass of one-launch patches: v[dof[i]] = sum over k in
// [off[i], off[i+1]) of pv[idx[k]], in order (vo_bytes 8: double, 4: float).
// Launched with programmatic dependence on the patch launch.
cudaError_t launch_patch_combine(int vo_bytes, void* v, const void* pv, const uint32_t* dof, const uint32_t* off,
                                 const uint32_t* idx, uint32_t nb, cudaStream_t st);
// Shared memory of a patch launch (0 if it does not fit).
size_t patch_smem_bytes(int prec, const PatchPlanGeom& pg, uint32_t copy_bytes);

// Arguments of one matrix-free (method 2) launch: the elements first ..
// first + count - 1 of the colour-sorted order (one colour).
struct FreeArgs {
    const void* xe;        // node coordinates, element-major (nodes x 3), double or float
    const uint32_t* map;   // n DoFs per element (kBcFlag on constrained DoFs)
    const void* ref;       // dN of every node at every quadrature point ([q][node][3]), then the q weights
    const void* u;
    void* v;
    uint32_t first, count, nq;
    int bc_mode;
    double lam, mu;        // Lame parameters (elasticity)
};
cudaError_t launch_free(int kind, bool f32, const FreeArgs& a, int sm_count, cudaStream_t st);

// Kernel arithmetic for FP32 products from the symmetric inner arena (an
// internal value beside the afm_precision codes).
constexpr int kPrecF32Sym = 16;
// ... and from the symmetric inner arena with its BF16 correction plane.
constexpr int kPrecF32SymX = 17;
// FP64 vectors, double-float products from that corrected arena (ArithSplitSymX).
constexpr int kPrecSplitSymX = 18;
// The corrected arena on FP32 u with FP32 row sums and FP64 v (ArithF32SymC).
constexpr int kPrecF32SymC = 19;

// Fills segment s's part of the symmetric inner arena from its split-arena
// units (afm_mv_f32sym.cu).
cudaError_t build_sym_segment(const Segment& s, const unsigned char* ke, unsigned char* sym, int sm_count,
                              cudaStream_t st);

// Launches one segment on stream. prec: afm_precision (FP64, FP64_SPLIT, FP32)
// or kPrecF32Sym.
// pdl: allow the launch to begin while the previous kernel on the stream
// drains (programmatic dependent launch; v is touched only after it ends).
cudaError_t launch_segment(const Segment& s, int prec, const SegArgs& a, int sm_count, bool dup_in_element, bool pdl,
                           cudaStream_t stream);
// Dynamic shared memory the launch of segment s uses (for reporting).
size_t segment_smem_bytes(const Segment& s, int prec);

// ---- serving lane (afm_lane.cu) ---------------------------------------------
// One launch advances the FP32 CG recursion of many served solves at once:
// every request is one thread-block cluster of kLaneCtas CTAs that runs whole
// CG iterations (colour-ordered FP32 products on the hi plane of the split
// arena, dot products, vector updates) with cluster barriers between phases.
constexpr uint32_t kLaneCtas = 8;
constexpr uint32_t kLaneThreads = 512;

// One colour-size segment of a request, as the lane reads it.
struct LaneSeg {
    const float* ke;        // hi plane of the segment's first unit
    const uint32_t* map;    // the segment's map (kBcFlag on constrained DoFs)
    uint64_t unit_floats;   // floats from one unit to the next
    uint32_t n, regime, units, count;
    uint32_t sync_after;    // 1: the last segment of its colour (a cluster barrier follows)
    uint32_t pad;
};

// One request's FP32 recursion: the vectors of its solve (float, n_dofs) and
// its solver scalars on the device.
struct LaneJob {
    float *x, *r, *z, *p, *q;
    const float* dinv;
    const uint8_t* bcmask;  // 1 on constrained DoFs (q = p there), or null
    const LaneSeg* segs;
    double* sc;
    int* err;
    uint32_t n_dofs, n_segs;
};

// Runs at most iters CG iterations of each of the n_jobs requests (a request
// whose S_DONE is set does nothing), then writes every request's scalars to
// its sc.
cudaError_t launch_lane(const LaneJob* d_jobs, uint32_t n_jobs, uint32_t iters, cudaStream_t st);

// Replaces the operator's stream by one of the given priority (lower numbers
// run first, cudaDeviceGetStreamPriorityRange), after the old stream's work
// has finished. Call before any solve has captured work on the stream.
int set_stream_priority(afm_operator* op, int priority);

// Records the calling thread's last error message (returned by
// afm_last_error) and returns status.
int set_error(int status, const char* fmt, ...);


}  // namespace afm

// The operator handle.
struct afm_operator {
    int device = 0;
    int bc_method = AFM_BC_IMATRIX;
    int matfree_type = 1;
    int precision_req = AFM_PREC_AUTO;
    int precision = AFM_PREC_FP64;
    cudaStream_t stream = nullptr;
    int sm_count = 0;

    // maps (single rank: local == global)
    bool have_map = false;
    uint32_t n_elem = 0, n_dofs = 0, nmax = 0;
    std::vector<uint32_t> offsets;  // n_elem + 1
    std::vector<uint32_t> map;      // global DoF ids
    bool dup_in_element = false;    // some element lists a DoF twice
    int patch_mode = 1;             // small elements: patches, 1 one launch + combine pass when the patch colours
                                    // are small, else one launch per colour; 2 always per colour; 3 always one
                                    // launch; 0 colour segments
    bool patch_one_launch = false;  // the choice made at finalize

    // boundary conditions
    std::vector<uint64_t> constrained;
    std::vector<double> values;
    std::vector<uint32_t> bc_unique;  // sorted unique constrained ids

    // element matrices, host copy (row-major, reference layout)
    std::vector<uint64_t> kofs;     // n_elem + 1, entries
    std::vector<double> ke;
    bool ke_dirty = true;

    // finalize products
    bool finalized = false;
    std::vector<uint32_t> colors;
    uint32_t n_colors = 0;
    std::vector<uint32_t> perm;     // position -> element id
    std::vector<afm::Segment> segs;
    double trace = 0.0;
    std::vector<double> diag_host;  // Jacobi diagonal with BC rows

    // device state
    unsigned char* d_ke = nullptr;
    size_t ke_bytes = 0;
    uint32_t* d_map = nullptr;       // DoF map, constrained DoFs carry kBcFlag
    size_t map_bytes = 0;
    double* d_diag = nullptr;
    uint32_t* d_bc_idx = nullptr;    // constrained ids in reference order
    double* d_bc_val = nullptr;
    uint32_t n_bc = 0;
    int* d_err = nullptr;
    unsigned long long wait_ns = 4000000000ull;  // limit of each kernel pipeline wait (afm_set_wait_limit)
    bool wait_probe = false;         // afm_set_wait_probe
    unsigned long long* d_usc = nullptr;  // u-scale words of the split products (kUscWords, afm_solver.hpp)
    uint8_t* d_bcmask = nullptr;     // 1 per constrained DoF (null without constraints)
    // one cooperative launch for every colour of a split product (segment plans of one element size)
    bool fused_ok = false;           // the plan allows it (decided at finalize)
    bool fused = false;              // afm_set_fused_colours (off: measured slower than the colour launches)
    unsigned* d_gbar = nullptr;      // grid-barrier counters of the fused launch
    std::vector<int> trace_iters;    // the last mixed solve: inner iterations at each FP64 residual
    std::vector<double> trace_res;   // ... and that residual over ||b||
    double* d_work = nullptr;        // host-API staging and solver vectors
    size_t work_elems = 0;
    double* d_scalars = nullptr;     // solver scalars / reduction partials
    double* h_scalars = nullptr;     // pinned mirror
    float* d_work32 = nullptr;       // mixed-precision inner vectors
    size_t work32_elems = 0;
    double* d_work64i = nullptr;     // inner vectors of the FP64-vector mixed solve (symmetric inner format 3)
    size_t work64i_elems = 0;

    // captured CG iteration graphs (FP64 and FP32 inner), keyed by buffers
    struct CgGraph {
        cudaGraphExec_t exec = nullptr;
        const void* key[6] = {};
        int batch = 0;
        uint64_t gen = 0;
    };
    CgGraph cg64, cg32, cg64i, bcg64, bcg32;
    uint64_t generation = 0;  // bumped whenever device buffers are released

    // symmetric inner arena: FP32 element matrices with each symmetric pair of
    // entries stored once, built from the split arena on the first FP32 product
    bool ke_symmetric = false;      // every Ke symmetric to 1e-6 of its largest diagonal entry
    bool sym_ok = false;            // symmetric, split arena, and a layout the symmetric kernels cover
    int sym_mode = 1;               // afm_set_symmetric_inner: 0 off, 1 FP32, 2 FP32 + BF16 correction
    int sym_built = 0;              // format of d_sym (1 or 2; 0: not built)
    unsigned char* d_sym = nullptr;
    size_t sym_bytes = 0;
    double* d_vx = nullptr;         // format 2: FP64 product before its rounding to FP32 (n_dofs)

    // matrix-free operator (method 2, MATFREE_TYPE::FREE): element kind, material, quadrature and
    // node coordinates; on the device, coordinates and maps in colour order and the reference tables
    int elem_kind = -1;
    double elem_E = 1.0, elem_nu = 0.3;
    uint32_t elem_ngt = 2, elem_nodes = 0;
    std::vector<double> xe;         // n_elem x nodes x 3
    std::vector<uint32_t> free_color_first;  // colour offsets into the colour-sorted elements
    uint32_t free_nq = 0;
    double* d_free_xe64 = nullptr;
    float* d_free_xe32 = nullptr;
    double* d_free_ref64 = nullptr;
    float* d_free_ref32 = nullptr;

    // assembled operator (afm_assembled.cpp): CSR on the device
    uint64_t* d_csr_rp = nullptr;
    uint32_t* d_csr_cols = nullptr;
    double* d_csr_vals = nullptr;
    uint64_t csr_nnz = 0;
    int csr_width = 32;             // threads per row of the SpMV

    // patch path (small elements): patches in colour order
    bool use_patches = false;
    afm::PatchPlanGeom patch_geom;
    std::vector<uint32_t> patch_color_first;  // n_patch_colors + 1 offsets into the patch list
    uint32_t n_patches = 0;
    afm::PatchDesc* d_patch_desc = nullptr;
    unsigned char* d_patch_idx = nullptr;
    size_t patch_idx_bytes = 0;
    // one-launch patches: local sums of shared DoFs (pv_count entries of 8 bytes) and, per shared DoF,
    // the list of its entries in patch order
    size_t pv_count = 0;
    uint32_t n_shared = 0;
    std::vector<uint32_t> shared_dof, shared_off, shared_idx;  // host copies (finalize)
    double* d_pv = nullptr;
    uint32_t* d_shared_dof = nullptr;
    uint32_t* d_shared_off = nullptr;
    uint32_t* d_shared_idx = nullptr;

    // batched (multi right-hand side) state
    double* d_bwork = nullptr;
    size_t bwork_elems = 0;
    double* d_bsc = nullptr;        // per-column scalars and column partials
    size_t bsc_elems = 0;
    unsigned int* d_bremain = nullptr;
    unsigned int* h_bremain = nullptr;
    struct BatchTune {
        uint64_t key;
        int tr, ng;  // lane tile: columns, rows
        float ms;
    };
    std::vector<BatchTune> batch_tune;  // autotuner choices
};
