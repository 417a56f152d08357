/* afm.h - C ABI of the GB300 assembly-free (AFM) finite-element operator.
 *
 * Drop-in for the single-rank, stored-element-matrix path of paralab/aMat:
 * the operator v = sum_e P_e^T Ke P_e u of par::aMatFree with
 * MATFREE_TYPE::QUASI_FREE (include/enums.hpp:56), plus the calls a solver
 * makes around it. Each entry point below names the reference interface it
 * replaces (paths relative to the aMat checkout).
 *
 * Conventions
 *  - Every function returns an int status (afm_status). Values 0..12 are the
 *    reference's par::Error codes (include/enums.hpp:24-36); codes >= 100 are
 *    new. afm_last_error() gives a message for the calling thread.
 *  - Indices: local DoF ids are uint32 (the reference's LI), global ids
 *    uint64 (GI). One rank: global == local after set_map, no ghosts.
 *  - Host pointers are copied; nothing passed in is retained after the call
 *    returns (unlike Maps::set_map, which keeps dofs_per_element,
 *    include/maps.hpp:423).
 *  - All work for one operator is serialised on that operator's CUDA stream.
 *    Calls on one operator are not re-entrant (same as aMatFree,
 *    include/aMatFree.hpp:75-84); different operators may be used from
 *    different threads.
 *  - The device path has no CPU fallback: without a usable GB300 (sm_103)
 *    afm_create fails with AFM_ERR_CUDA.
 */
#ifndef AFM_GB300_AFM_H
#define AFM_GB300_AFM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum afm_status {
    AFM_SUCCESS = 0,                 /* par::Error::SUCCESS */
    AFM_INDEX_OUT_OF_BOUNDS = 1,     /* par::Error::INDEX_OUT_OF_BOUNDS */
    AFM_UNKNOWN_ELEMENT_TYPE = 2,
    AFM_UNKNOWN_ELEMENT_STATUS = 3,
    AFM_NULL_L2G_MAP = 4,
    AFM_GHOST_NODE_NOT_FOUND = 5,
    AFM_UNKNOWN_MAT_TYPE = 6,        /* unsupported MATFREE_TYPE */
    AFM_WRONG_COMMUNICATION = 7,     /* maps that need ghost exchange (more than one rank) */
    AFM_UNKNOWN_DOF_TYPE = 8,
    AFM_UNKNOWN_CONSTRAINT = 9,
    AFM_UNKNOWN_BC_METH = 10,
    AFM_NOT_IMPLEMENTED = 11,
    AFM_GLOBAL_DOF_ID_NOT_FOUND = 12,
    AFM_ERR_CUDA = 100,              /* CUDA runtime error or no sm_103 device */
    AFM_ERR_OOM = 101,               /* device or host allocation failed */
    AFM_ERR_TIMEOUT = 102,           /* a bounded device wait gave up */
    AFM_ERR_BREAKDOWN = 103,         /* CG breakdown: p.Ap <= 0, r.z < 0 or NaN */
    AFM_ERR_STATE = 104,             /* call out of order (e.g. matvec before finalize) */
    AFM_ERR_INVALID_ARG = 105,       /* null pointer, bad size, unsupported option */
    AFM_ERR_MAXIT = 106,             /* CG stopped at maxit without converging */
    AFM_ERR_INTERNAL = 107           /* an internal consistency check failed */
} afm_status;

/* par::BC_METH (include/enums.hpp:20-21) */
typedef enum afm_bc_method { AFM_BC_IMATRIX = 0, AFM_BC_PENALTY = 1 } afm_bc_method;

/* Arithmetic of the stored element matrices and of the matvec.
 *  AFM_PREC_FP64        Ke stored as double, native FP64 multiply-add.
 *  AFM_PREC_FP64_SPLIT  Ke stored as an unevaluated pair of floats (hi, lo)
 *                       taking the same 8 bytes per entry; the product runs
 *                       in double-float arithmetic (error-free TwoProduct and
 *                       TwoSum, Ogita, Rump & Oishi 2005) with FP64 gather and
 *                       scatter. About 2^-48 relative per entry; for
 *                       element matrices whose largest |entry| lies within
 *                       1e-30..1e30 (smaller entries of the element are fine).
 *  AFM_PREC_FP32        Ke stored as float, FP32 multiply and accumulate, on
 *                       float vectors (afm_matvec_device_f32).
 * AFM_PREC_AUTO picks FP64_SPLIT when every element matrix is in its range,
 * FP64 otherwise. */
typedef enum afm_precision {
    AFM_PREC_FP64 = 0,
    AFM_PREC_FP64_SPLIT = 1,
    AFM_PREC_FP32 = 2,
    AFM_PREC_AUTO = 3
} afm_precision;

/* CG stopping norm (afm_solve_cg) */
typedef enum afm_cg_norm {
    AFM_CG_NORM_UNPRECONDITIONED = 0, /* ||b - A x||_2 <= max(rtol ||b||_2, atol) */
    AFM_CG_NORM_PRECONDITIONED = 1    /* ||D^-1 r||_2 <= max(rtol ||D^-1 b||_2, atol): PETSc KSPCG default */
} afm_cg_norm;

typedef struct afm_operator afm_operator;

typedef struct afm_info {
    uint32_t n_elements;
    uint32_t n_dofs;
    uint32_t n_colors;          /* colours of the element conflict graph */
    uint32_t max_dofs_per_element;
    int precision;              /* effective afm_precision after finalize */
    uint64_t ke_bytes;          /* device bytes of the element-matrix arena */
    uint64_t map_bytes;         /* device bytes of the DoF map */
    uint64_t algorithmic_bytes; /* per matvec: sum_e (n_e^2 * entry + 4 n_e) + 16 n_dofs (matrix-free:
                                   sum_e (24 nodes_e + 4 n_e) + 16 n_dofs) */
    double algorithmic_flops;   /* per matvec: sum_e 2 n_e^2 */
    uint32_t n_launches;        /* kernel launches per matvec */
    int device;
    uint32_t n_patches;         /* small-element patches (0: colour segments) */
    uint32_t n_patch_colors;    /* colours of the patch conflict graph */
    uint64_t patch_index_bytes; /* device bytes of the patch index blocks */
    int ke_symmetric;           /* every Ke symmetric (FP64_SPLIT operators; 0 otherwise) */
    int sym_available;          /* format of the symmetric inner arena FP32 products use (0: none) */
    uint64_t sym_bytes;         /* device bytes of that arena once built (0: not built) */
    uint64_t csr_nnz;           /* entries of the assembled matrix (0: afm_assemble not called) */
    uint64_t work_bytes;        /* device bytes of the solver and staging work space allocated so far */
} afm_info;

typedef struct afm_solve_stats {
    int iterations;
    int status;                 /* afm_status of the solve */
    double rel_residual;        /* ||b - A x||_2 / ||b||_2 at exit, computed in FP64 */
    double residual_norm;       /* the monitored norm at exit */
    double seconds;             /* device time of the solve */
    int refinements;            /* outer FP64 steps (mixed-precision solve only) */
} afm_solve_stats;

/* ---- lifetime ---------------------------------------------------------- */

/* aMatFree(Maps&, BC_METH) (include/aMatFree.hpp:113, 406-442). device < 0
 * means the current device. */
int afm_create(afm_operator** out, int bc_method, int device);
/* ~aMatFree */
int afm_destroy(afm_operator* op);

/* aMat::set_matfree_type (include/aMat.hpp:184-187). QUASI_FREE (1) and
 * GPU_PURE (3) select the stored-Ke device operator; FREE (2) the matrix-free
 * one (afm_set_element_kind, afm_set_element_coords). */
int afm_set_matfree_type(afm_operator* op, int matfree_type);
/* Element kernels of the matrix-free operator (method 2): the device
 * counterpart of aMat::set_element_matrix_function (include/aMat.hpp:114-116)
 * for the element kinds of the reference's examples (afm_element_kind, the
 * kernels of examples/src/ke_matrix.cpp: Gauss-Legendre rules of ngt points
 * per direction, 1 to 3; E and nu for elasticity). */
typedef enum afm_element_kind {
    AFM_ELEM_HEX8_POISSON = 0,
    AFM_ELEM_HEX8_ELASTIC = 1,
    AFM_ELEM_HEX20_ELASTIC = 2,
    AFM_ELEM_TET10_POISSON = 3,
    AFM_ELEM_TET10_ELASTIC = 4
} afm_element_kind;
int afm_set_element_kind(afm_operator* op, int kind, double E, double nu, uint32_t ngt);
/* Node coordinates of elements first .. first + count - 1: count x nodes x 3
 * doubles, node order of the kind (what the reference's callback gathers
 * into xe, e.g. examples/src/example07a.cpp:54-71). With
 * afm_set_matfree_type(op, 2) (MATFREE_TYPE::FREE, include/aMatFree.hpp:
 * 2241-2745) every product integrates each element's stiffness from these
 * coordinates on the device instead of reading stored Ke: one warp per
 * element, one launch per colour, FP64 for afm_matvec(_device), FP32 for the
 * _f32 products and the inner CG of afm_solve_cg_mixed; the Jacobi diagonal
 * and trace come from the same kernels on the host at afm_finalize. */
int afm_set_element_coords(afm_operator* op, uint32_t first, uint32_t count, const double* xe);
/* Arithmetic of the stored Ke; call before afm_finalize. Default AUTO. */
int afm_set_precision(afm_operator* op, int precision);
/* Execution of small elements (no counterpart in the reference). When every
 * element has the same size n <= 12 and lists no DoF twice, the matvec can
 * run over patches, compact groups of 32 to 128 elements whose vector entries
 * are staged in shared memory. Patches run either in one launch over every
 * patch, which writes each DoF sum straight to v when one patch lists the DoF
 * and to a combine buffer otherwise, followed by a pass that adds the buffered
 * sums in patch order; or in one launch per patch colour (patches of one
 * colour share no DoF), each adding its sums to v. Both add every DoF's sums
 * in the same order, so they give the same bits. mode = 1 (default): one
 * launch when a patch colour holds fewer than 16 patches per SM, else one
 * per colour; 2: always one per colour; 3: always one launch; 0: no patches,
 * one launch per element colour, as for larger elements. All modes are
 * deterministic and agree within rounding. Takes effect at the next
 * afm_finalize. */
int afm_set_patch_mode(afm_operator* op, int mode);
/* FP32 products of an FP64_SPLIT operator (no counterpart in the reference),
 * which the mixed-precision solves use: when every Ke is symmetric (to 1e-6
 * of its largest diagonal entry; the copy holds the symmetric part) and the
 * elements run as patches or have more than 16 DoFs, they can stream a
 * symmetric copy of the element matrices that stores each pair K(i, j),
 * K(j, i) once. format = 1 (default): the pairs in FP32, about 55% of the
 * bytes of the hi plane, FP32 sums. format = 2: FP32 plus a BF16 correction
 * plane (about 83% of the hi plane's bytes), which represents Ke to about
 * 2^-32, with compensated sums in FP32 arithmetic and the element rows summed
 * in FP64 before v is rounded to FP32. FP32 rounding of Ke or of the sums
 * perturbs the product by ~2^-24 |K| |u|, which costs the inner CG of
 * ill-conditioned systems (elasticity under rough loads) up to ~1.9x the
 * iterations of FP64 CG; format 2 brings that to ~1.1-1.2x, at a higher cost
 * per product. format = 3: the arena of format 2, and the mixed-precision
 * solve's inner recursion in FP64 vectors with double-float products from it
 * (about 40% of the split arena's bytes per product, no FP32 rounding of the
 * vectors), for large ill-conditioned systems whose FP32 recursion stalls.
 * format = 4: as 3, but the products are those of format 2 on u rounded to
 * FP32 (summed into v in FP64): cheaper products, u perturbed by 2^-24.
 * format = 5: as 4 with each element row summed in plain FP32 ((hi + lo) u as
 * two FMAs; the rows summed into v in FP64): the cheapest FP64-vector product.
 * format = 0: FP32 products read the hi plane. The copy is
 * built on the device from the split arena by the first FP32 product or
 * mixed-precision solve after a change (outside any stream capture). FP64
 * products never use it. */
int afm_set_symmetric_inner(afm_operator* op, int format);
/* 1: the FP64-split product of a segment plan whose elements share one size
 * (warp-group regime, up to 48 colours) runs every colour in one cooperative
 * launch, a grid barrier between colours, outside stream capture (captured
 * solve iterations keep one launch per colour); same results bit for bit.
 * 0 (default): one launch per colour, which measured faster (hex20 elasticity
 * 64^3: 1.359 against 1.438 ms; the grid barriers cost more than the launch
 * boundaries they replace). */
int afm_set_fused_colours(afm_operator* op, int enable);
/* Limit of each wait inside the operator's element kernels (no counterpart
 * in the reference, which ends the process on a device error:
 * include/aMatGpu.hpp:303-306). The kernels' producer and consumer warps meet
 * on shared-memory barriers; a wait that outlasts the limit makes the launch
 * stop early and the call report AFM_ERR_TIMEOUT, after which the operator
 * stays usable. seconds in [1e-9, 600]; the default is 4 s. Takes effect at
 * the next call (captured CG iterations are captured again). */
int afm_set_wait_limit(afm_operator* op, double seconds);
/* Test hook of that failure path (no counterpart in the reference). While
 * enabled (1), one consumer warp of the first block of every element-kernel
 * launch first waits for a device flag that nothing sets; its wait runs out
 * after the wait limit, the launch stops early and the call reports
 * AFM_ERR_TIMEOUT. Nothing faults: every wait is bounded and the operator
 * gives correct results again once the hook is off (0). Set a short limit
 * (milliseconds) with it. */
int afm_set_wait_probe(afm_operator* op, int enable);

/* ---- maps (par::Maps) --------------------------------------------------- */

/* Maps::set_map (include/maps.hpp:279-286, 399-451), flattened:
 * element e owns DoFs element_to_rank_map[dof_offsets[e] .. dof_offsets[e+1])
 * (dof_offsets NULL: every element has dofs_per_element DoFs). Local ids are
 * mapped through rank_to_global_map (NULL: identity). owned_global_dof_end is
 * inclusive, as in the reference. One rank owns everything:
 * owned range [0, n_global_dofs-1] and n_all_dofs_on_rank == n_global_dofs,
 * else AFM_WRONG_COMMUNICATION. */
int afm_set_map(afm_operator* op, uint32_t n_elements, const uint32_t* dof_offsets, uint32_t dofs_per_element,
                const uint32_t* element_to_rank_map, uint32_t n_all_dofs_on_rank, const uint64_t* rank_to_global_map,
                uint64_t owned_global_dof_begin, uint64_t owned_global_dof_end, uint64_t n_global_dofs);

/* Maps::set_bdr_map (include/maps.hpp:829-880): constrained global DoFs and
 * their prescribed values. */
int afm_set_bdr_map(afm_operator* op, const uint64_t* constrained_dofs, const double* prescribed_values,
                    uint32_t n_constraints);

/* ---- element matrices --------------------------------------------------- */

/* aMatFree::set_element_matrix(eid, e_mat, block_i, block_j, blocks_dim)
 * (include/aMat.hpp:134-141, include/aMatFree.hpp:856-953): e_mat is the
 * (n/blocks_dim)^2 block (block_i, block_j) of element eid's matrix,
 * row-major. Blocks never set are zero (the reference's nullptr blocks). */
int afm_set_element_matrix(afm_operator* op, uint32_t eid, const double* e_mat, uint32_t block_i, uint32_t block_j,
                           uint32_t blocks_dim);
/* Bulk form: count whole element matrices, row-major, back to back, for
 * elements first_eid .. first_eid+count-1. */
int afm_set_element_matrices(afm_operator* op, uint32_t first_eid, uint32_t count, const double* ke);

/* aMatFree::finalize (include/aMatFree.hpp:151-155, 657-785): colours the
 * elements, lays out and uploads the DoF map and element matrices, builds the
 * Jacobi diagonal and tr(K). */
int afm_finalize(afm_operator* op);

/* ---- operator ----------------------------------------------------------- */

/* aMatFree::matvec(v, u, isGhosted) (include/aMatFree.hpp:226, 1682-1775):
 * v = K u on host arrays of n_dofs doubles; copies in, runs, copies out,
 * returns when v is written. is_ghosted is accepted for signature parity
 * (one rank: ghosted and local layouts coincide). */
int afm_matvec(afm_operator* op, double* v, const double* u, int is_ghosted);
/* v = K u on device arrays, enqueued on stream (NULL: the operator's stream)
 * and returned without waiting. */
int afm_matvec_device(afm_operator* op, double* d_v, const double* d_u, void* stream);
/* FP32 product on float device vectors: from an AFM_PREC_FP32 arena; from an
 * AFM_PREC_FP64_SPLIT arena's symmetric FP32 copy (afm_set_symmetric_inner)
 * or its hi plane (the FP32-rounded Ke); or, for the matrix-free operator,
 * by the element kernels in FP32. */
int afm_matvec_device_f32(afm_operator* op, float* d_v, const float* d_u, void* stream);
/* The inner product of symmetric inner formats 3 to 5 on double device
 * vectors (what the FP64-vector mixed solve iterates on): from the corrected
 * symmetric arena (K to about 2^-32), double-float products of u (3) or of u
 * rounded to FP32 (4), or FP32 row sums of u rounded to FP32 (5). FP64_SPLIT
 * operators with symmetric element matrices, after afm_set_symmetric_inner. */
int afm_matvec_inner_device(afm_operator* op, double* d_v, const double* d_u, void* stream);

/* aMatFree::MatMult_mf (include/aMatFree.hpp:3894-3941): u_c taken as zero
 * in the product, then v_c = u_c. Host arrays. */
int afm_matmult_bc(afm_operator* op, double* v, const double* u);
int afm_matmult_bc_device(afm_operator* op, double* d_v, const double* d_u, void* stream);

/* MatGetDiagonal_mf (include/aMatFree.hpp:3945-3975): sum of element
 * diagonals, constrained rows 1 (identity) or 100 tr(K) (penalty,
 * apply_bc_diagonal 4310-4338). Host array of n_dofs. */
int afm_get_diagonal(afm_operator* op, double* diag);

/* aMatFree::apply_bc (include/aMatFree.hpp:957-969, apply_bc_rhs 4537-4700):
 * identity: rhs_f -= K_fc U_c, rhs_c = U_c; penalty: rhs_c = 100 tr(K) U_c.
 * Host array of n_dofs, updated in place. */
int afm_apply_bc_rhs(afm_operator* op, double* rhs);

/* tr(K) as computed by finalize_end (include/aMatFree.hpp:749-785). */
int afm_get_trace(afm_operator* op, double* trace);

/* ---- solver --------------------------------------------------------------- */

/* par::solve (examples/include/solve.hpp:75-127): Jacobi-preconditioned CG on
 * the MatMult_mf operator, entirely on the device in FP64. b and x are host
 * arrays of n_dofs; x holds the initial guess on entry and the solution on
 * return. stats may be NULL. */
int afm_solve_cg(afm_operator* op, const double* b, double* x, double rtol, double atol, int maxit, int norm_type,
                 afm_solve_stats* stats);
/* Same on device arrays (synchronous; returns when x is written). */
int afm_solve_cg_device(afm_operator* op, const double* d_b, double* d_x, double rtol, double atol, int maxit,
                        int norm_type, afm_solve_stats* stats);

/* Diagnostic, host only: the launch geometry the warp-group kernel takes for
 * elements of n DoFs (16 < n <= 96) in arithmetic `kind` (0 FP64, 1 split,
 * 2 FP32 from the split arena's hi plane, 3 symmetric FP32 copy, 4 corrected
 * copy with FP32 u, 5 corrected copy with double-float u, 6 corrected copy with
 * FP32 row sums): out[0..7] = element units per ring slot, ring stages,
 * consumer warps, element groups, column groups, dynamic shared memory bytes,
 * unit bytes, bytes copied per unit. */
int afm_debug_segment_geometry(int kind, uint32_t n, uint32_t* out);
/* The last mixed-precision solve of the operator (afm_solve_cg_mixed*): at
 * each FP64 residual, the inner iterations done so far and ||b - A x|| / ||b||.
 * *n = the count; up to cap entries are written. */
int afm_get_solve_trace(afm_operator* op, uint32_t cap, int* inner_iterations, double* rel_residual, uint32_t* n);
/* Mixed-precision solve of the same system (no counterpart in the
 * reference): Jacobi-PCG whose recursion runs in FP32 (the FP32 products of
 * afm_matvec_device_f32: the symmetric FP32 copy of the element matrices at
 * ~28% of the split arena's bytes, or the hi plane, or the matrix-free
 * kernels; FP32 vectors; dot products in compensated FP32 reduced in FP64;
 * FP64 step scalars) with reliable updates in FP64: once the FP32
 * residual has dropped by inner_rtol (or after max_inner iterations), the FP32
 * increment is added to x in FP64, the true residual r = b - A x is computed
 * in FP64 (MatMult_mf semantics) and replaces
 * the FP32 residual, and the recursion continues with its search direction.
 * The solve stops at ||b - A x|| <= max(rtol ||b||, atol), after max_outer
 * updates, or after ten updates in a row without a new smallest residual.
 * Needs an FP64_SPLIT operator (AFM_PREC_AUTO with in-range Ke) or the
 * matrix-free operator. stats:
 * iterations = FP32 iterations, refinements = FP64 residual updates. */
int afm_solve_cg_mixed(afm_operator* op, const double* b, double* x, double rtol, double atol, int max_outer,
                       double inner_rtol, int max_inner, afm_solve_stats* stats);
int afm_solve_cg_mixed_device(afm_operator* op, const double* d_b, double* d_x, double rtol, double atol,
                              int max_outer, double inner_rtol, int max_inner, afm_solve_stats* stats);
/* MatMult_mf in FP32 on float device vectors (FP32 or FP64_SPLIT operator). */
int afm_matmult_bc_device_f32(afm_operator* op, float* d_v, const float* d_u, void* stream);

/* ---- batched: many right-hand sides at once -------------------------------
 * Blocks are n_dofs x ld row-major device arrays (the nrhs values of one DoF
 * are contiguous), 16-byte aligned; nrhs is a multiple of 4, at most 256, ld
 * >= nrhs a multiple of 4; every element must have more than 16 DoFs. Each
 * element matrix is streamed once per call and applied to all columns (for
 * example hex8 elasticity with 64 right-hand sides): a warp per element, a
 * register tile of V_e per lane. The first call for a given (nrhs, ld,
 * arithmetic) runs the autotuner, which times the lane tile shapes on the
 * caller's data and keeps the fastest for the operator. No counterpart in
 * the reference, whose matvec takes one vector. */
int afm_matvec_batched_device(afm_operator* op, double* d_V, const double* d_U, uint32_t nrhs, uint32_t ld,
                              void* stream);
int afm_matvec_batched_device_f32(afm_operator* op, float* d_V, const float* d_U, uint32_t nrhs, uint32_t ld,
                                  void* stream);
/* MatMult_mf semantics column by column. */
int afm_matmult_bc_batched_device(afm_operator* op, double* d_V, const double* d_U, uint32_t nrhs, uint32_t ld,
                                  void* stream);
int afm_matmult_bc_batched_device_f32(afm_operator* op, float* d_V, const float* d_U, uint32_t nrhs, uint32_t ld,
                                      void* stream);
/* The autotuner's choice for (nrhs, ld, f32): columns and rows of the lane
 * tile, and the time of one product in ms. f32 = 0: FP64 (or split) products;
 * 1: FP32 products; 2: the FP32 products of the batched mixed solve. */
int afm_get_batch_tuning(afm_operator* op, uint32_t nrhs, uint32_t ld, int f32, int* cols_per_thread,
                         int* rows_per_thread, float* ms);
/* Pins the lane tile for (nrhs, ld, f32) instead of the autotuner's choice:
 * (columns, rows) one of (8, 2), (8, 4), (8, 6), (4, 4); or (0, 0), the
 * tensor-core kernel (FP32 products, nrhs 32, 64 or 128, elements of 17 to 96
 * DoFs: 3xTF32 products on tcgen05, ~2^-21 of |K||u|), which the autotuner
 * also times when it applies. The batched mixed solve's FP32 recursion tunes
 * among the CUDA-core tiles only (IEEE FP32 products) and keeps its choice
 * apart from these. */
int afm_set_batch_tuning(afm_operator* op, uint32_t nrhs, uint32_t ld, int f32, int cols_per_thread,
                         int rows_per_thread);
/* Batched Jacobi-PCG: one CG per column (own scalars and stopping test
 * ||b_j - A x_j|| <= max(rtol ||b_j||, atol)), all advanced together, the
 * iterations captured in CUDA graphs. FP64 arithmetic of the operator. ld =
 * nrhs. stats->rel_residual: worst column. */
int afm_solve_cg_batched_device(afm_operator* op, const double* d_B, double* d_X, uint32_t nrhs, double rtol,
                                double atol, int maxit, afm_solve_stats* stats);
/* Batched mixed-precision solve: one FP32 block Jacobi-PCG recursion (FP64
 * scalars) on the hi plane of the split arena, with FP64 reliable updates of
 * every column from the FP64 residual block (as afm_solve_cg_mixed). A segment
 * ends once every running column's FP32 residual fell by inner_rtol or after
 * max_inner iterations; columns wait for the slowest, so a short max_inner
 * (tens of iterations) keeps all columns busy. Columns that meet rtol are
 * frozen. */
int afm_solve_cg_batched_mixed_device(afm_operator* op, const double* d_B, double* d_X, uint32_t nrhs, double rtol,
                                      double atol, int max_outer, double inner_rtol, int max_inner,
                                      afm_solve_stats* stats);

/* Host-side check of the small-element patch plan (no device work, no
 * counterpart in the reference): builds the patch plan afm_finalize would
 * build for this map (same-size elements, n <= 12, no DoF twice in an
 * element) and evaluates v = K u on the CPU by walking the plan's index
 * blocks the way the patch kernel does (FP64, ke row-major n x n per
 * element). Checks every structural invariant on the way and returns
 * AFM_ERR_INTERNAL with a message when one fails. */
int afm_patch_plan_host_matvec(uint32_t n_elem, uint32_t n_dofs, const uint32_t* offsets, const uint32_t* map,
                               const double* ke, const double* u, double* v, uint32_t* n_patches,
                               uint32_t* n_patch_colors);

/* ---- assembled operator (par::aMatBased) ----------------------------------
 * The matrix aMatBased assembles through PETSc, as CSR (row_ptr[n_dofs + 1],
 * cols ascending per row, FP64 values): set_element_matrix with ADD_VALUES in
 * element order (include/aMatBased.hpp:214-258), so every entry is summed in
 * the reference's order and matches its matrix bit for bit; apply_bc = 1 also
 * applies apply_bc_mat (294-352): identity method, constrained rows become
 * unit rows and constrained columns zero; penalty method, constrained
 * diagonals become 100 tr(K). The sparsity pattern is the union of the
 * element patterns (entries set to zero are kept, as in the reference). */
/* Host-only assembly (no device needed); ke holds the element matrices row
 * by row, one after another (offsets as afm_set_map). Call with row_ptr,
 * cols and vals NULL to get *nnz, then with arrays of that size (*nnz in:
 * their capacity). */
int afm_assemble_csr_host(uint32_t n_elem, uint32_t n_dofs, const uint32_t* offsets, const uint32_t* map,
                          const double* ke, const uint64_t* constrained, uint32_t n_constrained, int bc_method,
                          int apply_bc, uint64_t* nnz, uint64_t* row_ptr, uint32_t* cols, double* vals);
/* Assembles the finalized operator's matrix (its element matrices, boundary
 * conditions and method) and keeps it on the device. */
int afm_assemble(afm_operator* op, int apply_bc);
/* aMatBased::matmult (include/aMatBased.hpp:458-460) on device vectors: a
 * hand-written CSR SpMV, bit-reproducible. */
int afm_matvec_assembled_device(afm_operator* op, double* d_v, const double* d_u, void* stream);
/* dump_mat (include/aMatBased.hpp:262-292): the assembled matrix as CSR
 * (same calling convention as afm_assemble_csr_host). */
int afm_get_assembled_csr(afm_operator* op, uint64_t* nnz, uint64_t* row_ptr, uint32_t* cols, double* vals);

/* ---- serving: many CG solves on different operators ----------------------
 * No counterpart in the reference. A request is an operator whose maps and
 * element matrices are set on the host (finalize not needed) and a load b
 * (host, n_dofs, boundary conditions applied). Requests wait in a queue and
 * are admitted (requests small enough for the serving lane first, the rest in
 * arrival order) while the HBM budget, the device's free memory and the slot
 * limit allow; admission finalises the operator on a worker thread. An
 * admitted request keeps Ke, maps, b, x and its Krylov vectors on the device
 * and is solved by the mixed-precision solve (afm_solve_cg_mixed, to rtol,
 * FP64-checked). A progress thread of the server's own keeps admitting and
 * taking the next step of every request whose previous step has finished on
 * the GPU, so progress never waits for the caller. Each request runs on its
 * own stream, so the work of all running requests overlaps on the device, and
 * requests arriving meanwhile join as slots and memory free up; the FP32
 * iterations of small requests share one launch (afm_server_set_lane). A request's
 * result does not depend on the others: it is the same, bit for bit, alone
 * and in any mix. The calls below are thread-safe. */
typedef struct afm_server afm_server;
/* hbm_budget_bytes 0: 85% of the device memory free now; max_active 0: 64. */
int afm_server_create(afm_server** out, int device, uint64_t hbm_budget_bytes, uint32_t max_active);
/* Takes ownership of op (destroyed when the request finishes). inner_rtol:
 * FP32 residual reduction between FP64 updates (0 < inner_rtol < 1). */
int afm_server_submit(afm_server* s, afm_operator* op, const double* b, double rtol, double inner_rtol,
                      uint64_t* id);
/* Non-blocking: one more round of progress, and the counts of queued and
 * admitted requests (optional). */
int afm_server_poll(afm_server* s, uint32_t* n_queued, uint32_t* n_active);
/* *finished = 0 (and AFM_SUCCESS) while the request is queued or running.
 * Once it has finished: *finished = 1, x (host, n_dofs), stats and times[4]
 * (submit, admit, start of the solve, done; steady-clock seconds) are filled,
 * the request is forgotten, and the solve's status is returned. */
int afm_server_take(afm_server* s, uint64_t id, int* finished, double* x, afm_solve_stats* stats, double* times);
/* Waits for running work and releases everything. */
int afm_server_destroy(afm_server* s);
/* Serving lane: requests whose FP32 element matrices take at most
 * max_ke_bytes (n^2 x 4 bytes per element; 8 MB by default, 0 turns the lane
 * off) run their FP32 iterations in one launch shared by all such requests
 * (one thread-block cluster per request, at most iters_per_launch iterations,
 * 32 by default, per launch); larger requests run on their own streams. Takes
 * effect for requests admitted afterwards. */
int afm_server_set_lane(afm_server* s, uint64_t max_ke_bytes, uint32_t iters_per_launch);
/* 1 (default): each request's stream gets a priority by its size (the lane
 * and small requests first); 0: every request at the default priority. Takes
 * effect for requests started afterwards. */
int afm_server_set_priorities(afm_server* s, int enable);
/* Symmetric inner format (afm_set_symmetric_inner) of the requests with at
 * least 2^20 DoFs that run on their own streams: 4 by default (FP64 inner
 * vectors on the corrected symmetric arena), 0 to 5 as afm_set_symmetric_inner;
 * smaller ones use format 1. Takes effect for requests started afterwards. */
int afm_server_set_inner_format(afm_server* s, int format);
typedef struct {
    uint64_t lane_launches;       /* serving-lane launches */
    uint64_t lane_solve_launches; /* requests carried, summed over those launches */
    uint32_t lane_max_batch;      /* most requests carried by one launch */
    uint32_t reserved;
    uint64_t lane_requests;       /* requests whose FP32 iterations ran in the lane */
    uint64_t stream_requests;     /* requests whose FP32 iterations ran on their own streams */
} afm_server_info;
int afm_server_get_info(afm_server* s, afm_server_info* info);

/* Largest operator (DoFs) afm_solve_cg_device_noalloc accepts. */
#define AFM_NOALLOC_MAX_DOFS 262144u

/* Jacobi-PCG like afm_solve_cg_device, for callers that cannot allocate
 * device memory while they run. No counterpart in the reference.
 * Who needs it: code embedded in an application that has already reserved the
 * GPU's memory (a framework's caching allocator sized to the device, a fixed
 * per-process budget under MPS), or a loop that must not stall, since
 * cudaMalloc and cudaFree can synchronise the whole device. The call allocates
 * nothing: its CG vectors and reduction partials live in one array compiled
 * into the library (5 x AFM_NOALLOC_MAX_DOFS doubles plus 2.6k doubles of
 * partials, about 10.5 MB), which every GPU that loads the library holds until
 * the process exits. Operators with more DoFs fail with AFM_ERR_INVALID_ARG.
 * Every call looks up the array's device address (cudaGetSymbolAddress) with
 * the operator's device current; the first lookup on a device loads the
 * module that holds the array, so make the first call before any stream
 * capture. All calls on a device share the array and the call clears the
 * solver state it needs at its start, so calls whose work overlaps on the GPU
 * race: run them one at a time. Synchronous, like afm_solve_cg_device;
 * stats->seconds is host wall time here (each iteration's host round trip
 * included), not device time. */
int afm_solve_cg_device_noalloc(afm_operator* op, const double* d_b, double* d_x, double rtol, double atol,
                                int maxit, int norm_type, afm_solve_stats* stats);

/* ---- introspection ------------------------------------------------------ */

int afm_get_info(afm_operator* op, afm_info* info);
/* Colour of each element (n_elements entries), for checking determinism. */
int afm_get_colors(afm_operator* op, uint32_t* colors);
/* The operator's CUDA stream (cudaStream_t). */
int afm_get_stream(afm_operator* op, void** stream);
/* Waits for the operator's stream and reports a device-side error flag. */
int afm_synchronize(afm_operator* op);
const char* afm_status_string(int status);
/* Message of the last failing call on this thread ("" if none). */
const char* afm_last_error(void);

#ifdef __cplusplus
}
#endif
#endif
