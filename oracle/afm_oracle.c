/* CPU oracle for the assembly-free (AFM) element-by-element operator of
 * paralab/aMat. TEST INFRASTRUCTURE: only tests/, the smoke check and the
 * CPU-baseline / reference arms of bench.py load this library, always as the
 * checker or as the timed CPU baseline, never as the thing measured or
 * shipped. The product (amat_gb300/) never links it.
 *
 * It restates the reference's single-rank method-1 (QUASI_FREE) path in plain
 * C. Each function cites the reference lines it follows (paths relative to
 * the aMat checkout). Parity of this restatement with the reference itself is
 * pinned by tests/test_oracle.py against golden vectors written from the
 * reference compiled in place (oracle/build_ref.sh, tests/golden/make_golden.py).
 *
 * Storage conventions shared with the product's C ABI:
 *   element e has n_e = offsets[e+1]-offsets[e] DoFs, local ids
 *   map[offsets[e] .. offsets[e+1]), and its element matrix Ke is n_e x n_e
 *   row-major at ke + kofs[e], kofs[e] = sum_{f<e} n_f^2 (the reference's
 *   default row-major store, include/aMatFree.hpp:945-949).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORACLE_PENALTY_FACTOR 100.0 /* include/aMat.hpp:68 */

static uint64_t* ke_offsets(uint32_t n_elem, const uint32_t* offsets) {
    uint64_t* k = (uint64_t*)malloc(sizeof(uint64_t) * ((size_t)n_elem + 1));
    k[0] = 0;
    for (uint32_t e = 0; e < n_elem; e++) {
        uint64_t n = offsets[e + 1] - offsets[e];
        k[e + 1] = k[e] + n * n;
    }
    return k;
}

/* One element: ve = Ke * ue with the row-major scalar loop of the reference
 * (include/aMatFree.hpp:1858-1862 gather, 1994-1999 GEMV). */
static void element_product(uint32_t n, const uint32_t* emap, const double* ke, const double* u, double* ue,
                            double* ve) {
    for (uint32_t c = 0; c < n; c++) {
        ue[c] = u[emap[c]];
        ve[c] = 0.0;
    }
    for (uint32_t r = 0; r < n; r++)
        for (uint32_t c = 0; c < n; c++) ve[r] += ke[(size_t)r * n + c] * ue[c];
}

/* v = sum_e P_e^T Ke P_e u, elements in index order, sequential (deterministic).
 * matvec_ghosted_OMP (include/aMatFree.hpp:1778-2238) with one thread: zero v
 * (1789-1792), then per element gather, GEMV, scatter-add (2004-2008). */
void oracle_matvec(uint32_t n_elem, uint32_t n_dofs, const uint32_t* offsets, const uint32_t* map, const double* ke,
                   const double* u, double* v) {
    uint32_t nmax = 0;
    for (uint32_t e = 0; e < n_elem; e++) {
        uint32_t n = offsets[e + 1] - offsets[e];
        if (n > nmax) nmax = n;
    }
    double* ue = (double*)malloc(sizeof(double) * (nmax + 1));
    double* ve = (double*)malloc(sizeof(double) * (nmax + 1));
    memset(v, 0, sizeof(double) * n_dofs);
    uint64_t kofs = 0;
    for (uint32_t e = 0; e < n_elem; e++) {
        uint32_t n = offsets[e + 1] - offsets[e];
        const uint32_t* emap = map + offsets[e];
        element_product(n, emap, ke + kofs, u, ue, ve);
        for (uint32_t r = 0; r < n; r++) v[emap[r]] += ve[r];
        kofs += (uint64_t)n * n;
    }
    free(ue);
    free(ve);
}

/* The same product with the reference's OpenMP structure: parallel for over
 * elements with private ue/ve and an atomic scatter (1799-2013). The order of
 * additions into v depends on thread timing, exactly as in the reference.
 * This is the CPU baseline that bench.py times. Returns threads used. */
int oracle_matvec_omp(uint32_t n_elem, uint32_t n_dofs, const uint32_t* offsets, const uint32_t* map,
                      const double* ke, const uint64_t* kofs_in, const double* u, double* v) {
    uint64_t* kofs = kofs_in ? (uint64_t*)kofs_in : ke_offsets(n_elem, offsets);
    int threads = 1;
    for (uint32_t i = 0; i < n_dofs; i++) v[i] = 0.0;
#pragma omp parallel
    {
        double ue[128], ve[128]; /* n <= 128 asserted by the caller */
#ifdef _OPENMP
#pragma omp single
        threads = omp_get_num_threads();
#endif
#pragma omp for schedule(static)
        for (int64_t e = 0; e < (int64_t)n_elem; e++) {
            uint32_t n = offsets[e + 1] - offsets[e];
            const uint32_t* emap = map + offsets[e];
            element_product(n, emap, ke + kofs[e], u, ue, ve);
            for (uint32_t r = 0; r < n; r++) {
#pragma omp atomic
                v[emap[r]] += ve[r];
            }
        }
    }
    if (!kofs_in) free(kofs);
    return threads;
}

/* The same loop with a thread count (nthreads > 0: at most that many; 0:
 * the default) and, with simd = 1, the element product of the reference's
 * VECTORIZED_OPENMP build (include/aMatFree.hpp:1965-1973): the element
 * matrix stored column-major (the transposed copy that build keeps,
 * 931-937), v_e accumulated column by column, v_e += u_c * Ke(:, c), with the
 * row loop under omp simd. ke_cm holds every element matrix column-major
 * (null unless simd). Returns the threads used. */
int oracle_matvec_omp_cfg(uint32_t n_elem, uint32_t n_dofs, const uint32_t* offsets, const uint32_t* map,
                          const double* ke, const double* ke_cm, const double* u, double* v, int nthreads, int simd) {
    uint64_t* kofs = ke_offsets(n_elem, offsets);
    int threads = 1;
    for (uint32_t i = 0; i < n_dofs; i++) v[i] = 0.0;
#ifdef _OPENMP
    const int nt = nthreads > 0 ? nthreads : omp_get_max_threads();
#pragma omp parallel num_threads(nt)
#endif
    {
        double ue[128], ve[128]; /* n <= 128 asserted by the caller */
#ifdef _OPENMP
#pragma omp single
        threads = omp_get_num_threads();
#endif
#pragma omp for schedule(static)
        for (int64_t e = 0; e < (int64_t)n_elem; e++) {
            const uint32_t n = offsets[e + 1] - offsets[e];
            const uint32_t* emap = map + offsets[e];
            if (simd) {
                const double* kc = ke_cm + kofs[e];
                for (uint32_t r = 0; r < n; r++) {
                    ue[r] = u[emap[r]];
                    ve[r] = 0.0;
                }
                for (uint32_t c = 0; c < n; c++) {
                    const double alpha = ue[c];
                    const double* x = kc + (size_t)c * n;
#pragma omp simd
                    for (uint32_t r = 0; r < n; r++) ve[r] += alpha * x[r];
                }
            } else {
                element_product(n, emap, ke + kofs[e], u, ue, ve);
            }
            for (uint32_t r = 0; r < n; r++) {
#pragma omp atomic
                v[emap[r]] += ve[r];
            }
        }
    }
    free(kofs);
    return threads;
}

/* Greedy first-fit colouring of the element conflict graph, elements visited
 * in index order: restates meshGraph::mesh2Graph (include/meshGraph.hpp:132-155:
 * two elements are adjacent when they share a DoF) and greedyColoring (59-109:
 * element 0 gets colour 0, each later element the smallest colour not used by
 * an already-coloured neighbour). Returns the number of colours. */
uint32_t oracle_coloring(uint32_t n_dofs, uint32_t n_elem, const uint32_t* offsets, const uint32_t* map,
                         uint32_t* colors) {
    /* dof -> elements (CSR) */
    uint32_t* cnt = (uint32_t*)calloc((size_t)n_dofs + 1, sizeof(uint32_t));
    for (uint32_t e = 0; e < n_elem; e++)
        for (uint32_t k = offsets[e]; k < offsets[e + 1]; k++) cnt[map[k] + 1]++;
    for (uint32_t d = 0; d < n_dofs; d++) cnt[d + 1] += cnt[d];
    uint32_t* fill = (uint32_t*)malloc(sizeof(uint32_t) * ((size_t)n_dofs + 1));
    memcpy(fill, cnt, sizeof(uint32_t) * ((size_t)n_dofs + 1));
    uint32_t* d2e = (uint32_t*)malloc(sizeof(uint32_t) * ((size_t)offsets[n_elem] + 1));
    for (uint32_t e = 0; e < n_elem; e++)
        for (uint32_t k = offsets[e]; k < offsets[e + 1]; k++) d2e[fill[map[k]]++] = e;
    /* used[c] == e+1 marks colour c as taken by a neighbour of element e */
    uint32_t* used = (uint32_t*)calloc((size_t)n_elem + 1, sizeof(uint32_t));
    uint32_t ncol = n_elem ? 1 : 0;
    for (uint32_t e = 0; e < n_elem; e++) colors[e] = UINT32_MAX;
    for (uint32_t e = 0; e < n_elem; e++) {
        for (uint32_t k = offsets[e]; k < offsets[e + 1]; k++) {
            uint32_t d = map[k];
            for (uint32_t j = cnt[d]; j < cnt[d + 1]; j++) {
                uint32_t f = d2e[j];
                if (f != e && colors[f] != UINT32_MAX) used[colors[f]] = e + 1;
            }
        }
        uint32_t c = 0;
        while (used[c] == e + 1) c++;
        colors[e] = c;
        if (c + 1 > ncol) ncol = c + 1;
    }
    free(cnt);
    free(fill);
    free(d2e);
    free(used);
    return ncol;
}

/* tr(K) = sum_e sum_r Ke[r][r] (finalize_end, include/aMatFree.hpp:749-785). */
double oracle_trace(uint32_t n_elem, const uint32_t* offsets, const double* ke) {
    double t = 0.0;
    uint64_t kofs = 0;
    for (uint32_t e = 0; e < n_elem; e++) {
        uint32_t n = offsets[e + 1] - offsets[e];
        for (uint32_t r = 0; r < n; r++) t += ke[kofs + (size_t)r * n + r];
        kofs += (uint64_t)n * n;
    }
    return t;
}

/* constrained flag per DoF (Maps::set_bdr_map, include/maps.hpp:829-880) */
static unsigned char* bc_flags(uint32_t n_dofs, const uint64_t* constrained, uint32_t n_constraints) {
    unsigned char* f = (unsigned char*)calloc(n_dofs ? n_dofs : 1, 1);
    for (uint32_t i = 0; i < n_constraints; i++)
        if (constrained[i] < n_dofs) f[constrained[i]] = 1;
    return f;
}

/* Jacobi diagonal with boundary rows: mat_get_diagonal_ghosted
 * (include/aMatFree.hpp:998-1056) then apply_bc_diagonal (4310-4338): rows of
 * constrained DoFs become 1 (identity method) or 100*tr(K) (penalty). */
void oracle_get_diagonal(uint32_t n_elem, uint32_t n_dofs, const uint32_t* offsets, const uint32_t* map,
                         const double* ke, const uint64_t* constrained, uint32_t n_constraints, int bc_method,
                         double* diag) {
    memset(diag, 0, sizeof(double) * n_dofs);
    uint64_t kofs = 0;
    for (uint32_t e = 0; e < n_elem; e++) {
        uint32_t n = offsets[e + 1] - offsets[e];
        for (uint32_t r = 0; r < n; r++) diag[map[offsets[e] + r]] += ke[kofs + (size_t)r * n + r];
        kofs += (uint64_t)n * n;
    }
    /* apply_bc_diagonal visits constrained DoFs through the elements' boundary
     * maps, so a constrained DoF that belongs to no element keeps its sum (0) */
    double pen = (bc_method == 1) ? ORACLE_PENALTY_FACTOR * oracle_trace(n_elem, offsets, ke) : 1.0;
    unsigned char* flag = bc_flags(n_dofs, constrained, n_constraints);
    for (uint32_t k = 0; k < offsets[n_elem]; k++)
        if (flag[map[k]]) diag[map[k]] = pen;
    free(flag);
}

/* MatMult_mf (include/aMatFree.hpp:3894-3941): save U_c, zero it, v = K u,
 * then v_c = U_c. Applied identically for both BC methods, as the reference
 * does. */
void oracle_matmult_bc(uint32_t n_elem, uint32_t n_dofs, const uint32_t* offsets, const uint32_t* map,
                       const double* ke, const uint64_t* constrained, uint32_t n_constraints, const double* u,
                       double* v) {
    double* uu = (double*)malloc(sizeof(double) * (n_dofs ? n_dofs : 1));
    memcpy(uu, u, sizeof(double) * n_dofs);
    for (uint32_t i = 0; i < n_constraints; i++) uu[constrained[i]] = 0.0;
    oracle_matvec(n_elem, n_dofs, offsets, map, ke, uu, v);
    for (uint32_t i = 0; i < n_constraints; i++) v[constrained[i]] = u[constrained[i]];
    free(uu);
}

/* apply_bc_rhs (include/aMatFree.hpp:4537-4700), rhs updated in place.
 * Identity method: for every element row r of a free DoF, accumulate
 * -sum_{constrained columns c} Ke[r][c]*g_c into KfcUc[row]; then
 * rhs_c = g_c and rhs_f += KfcUc_f. Penalty: rhs_c = 100*tr(K)*g_c only. */
void oracle_apply_bc_rhs(uint32_t n_elem, uint32_t n_dofs, const uint32_t* offsets, const uint32_t* map,
                         const double* ke, const uint64_t* constrained, const double* values,
                         uint32_t n_constraints, int bc_method, double* rhs) {
    unsigned char* flag = bc_flags(n_dofs, constrained, n_constraints);
    double* g = (double*)calloc(n_dofs ? n_dofs : 1, sizeof(double));
    for (uint32_t i = 0; i < n_constraints; i++) g[constrained[i]] = values[i];
    if (bc_method == 0) {
        double* kfc = (double*)calloc(n_dofs ? n_dofs : 1, sizeof(double));
        uint64_t kofs = 0;
        for (uint32_t e = 0; e < n_elem; e++) {
            uint32_t n = offsets[e + 1] - offsets[e];
            const uint32_t* emap = map + offsets[e];
            for (uint32_t r = 0; r < n; r++) {
                if (flag[emap[r]]) continue;
                double t = 0.0;
                int any = 0;
                for (uint32_t c = 0; c < n; c++)
                    if (flag[emap[c]]) {
                        t += ke[kofs + (size_t)r * n + c] * g[emap[c]];
                        any = 1;
                    }
                if (any) kfc[emap[r]] += -1.0 * t;
            }
            kofs += (uint64_t)n * n;
        }
        for (uint32_t i = 0; i < n_constraints; i++) rhs[constrained[i]] = values[i];
        for (uint32_t d = 0; d < n_dofs; d++)
            if (!flag[d]) rhs[d] = kfc[d] + rhs[d];
        free(kfc);
    } else {
        double pen = ORACLE_PENALTY_FACTOR * oracle_trace(n_elem, offsets, ke);
        for (uint32_t i = 0; i < n_constraints; i++) rhs[constrained[i]] = pen * values[i];
    }
    free(g);
    free(flag);
}

static double dot(uint32_t n, const double* a, const double* b) {
    double s = 0.0;
    for (uint32_t i = 0; i < n; i++) s += a[i] * b[i];
    return s;
}

/* Jacobi-preconditioned CG on the boundary-wrapped operator: the solve of
 * examples/include/solve.hpp:75-127 (KSPCG + PCJACOBI, shell MULT =
 * MatMult_mf, GET_DIAGONAL = MatGetDiagonal_mf), restated (PETSc is not part
 * of the reference). Initial guess x (in/out). Stops when
 *   norm_type 0: ||b - A x||_2 <= max(rtol*||b||_2, atol)   (true residual)
 *   norm_type 1: ||D^-1 r||_2 <= max(rtol*||D^-1 b||_2, atol) (PETSc default)
 * Returns iterations (>= 0), -1 on breakdown (p.Ap <= 0 or r.z < 0), -2 when
 * maxit is reached. res_out: final relative true residual. */
int oracle_pcg(uint32_t n_elem, uint32_t n_dofs, const uint32_t* offsets, const uint32_t* map, const double* ke,
               const uint64_t* constrained, uint32_t n_constraints, int bc_method, const double* b, double* x,
               double rtol, double atol, int maxit, int norm_type, double* res_out) {
    size_t bytes = sizeof(double) * (n_dofs ? n_dofs : 1);
    double *d = (double*)malloc(bytes), *r = (double*)malloc(bytes), *z = (double*)malloc(bytes);
    double *p = (double*)malloc(bytes), *q = (double*)malloc(bytes);
    oracle_get_diagonal(n_elem, n_dofs, offsets, map, ke, constrained, n_constraints, bc_method, d);
    oracle_matmult_bc(n_elem, n_dofs, offsets, map, ke, constrained, n_constraints, x, q);
    for (uint32_t i = 0; i < n_dofs; i++) {
        r[i] = b[i] - q[i];
        z[i] = r[i] / d[i];
        p[i] = z[i];
    }
    double bn = sqrt(dot(n_dofs, b, b));
    double bz = 0.0;
    for (uint32_t i = 0; i < n_dofs; i++) bz += (b[i] / d[i]) * (b[i] / d[i]);
    bz = sqrt(bz);
    double ref = (norm_type == 0) ? bn : bz;
    double tol = rtol * ref > atol ? rtol * ref : atol;
    double rz = dot(n_dofs, r, z);
    int it = 0, status = -2;
    for (;;) {
        double rn = (norm_type == 0) ? sqrt(dot(n_dofs, r, r)) : sqrt(dot(n_dofs, z, z));
        if (rn <= tol) {
            status = it;
            break;
        }
        if (it >= maxit) break;
        if (rz < 0.0 || isnan(rz)) {
            status = -1;
            break;
        }
        oracle_matmult_bc(n_elem, n_dofs, offsets, map, ke, constrained, n_constraints, p, q);
        double pq = dot(n_dofs, p, q);
        if (!(pq > 0.0)) {
            status = -1;
            break;
        }
        double alpha = rz / pq;
        for (uint32_t i = 0; i < n_dofs; i++) {
            x[i] += alpha * p[i];
            r[i] -= alpha * q[i];
            z[i] = r[i] / d[i];
        }
        double rz_new = dot(n_dofs, r, z);
        double beta = rz_new / rz;
        rz = rz_new;
        for (uint32_t i = 0; i < n_dofs; i++) p[i] = z[i] + beta * p[i];
        it++;
    }
    if (res_out) {
        oracle_matmult_bc(n_elem, n_dofs, offsets, map, ke, constrained, n_constraints, x, q);
        double s = 0.0;
        for (uint32_t i = 0; i < n_dofs; i++) s += (b[i] - q[i]) * (b[i] - q[i]);
        *res_out = bn > 0 ? sqrt(s) / bn : sqrt(s);
    }
    free(d);
    free(r);
    free(z);
    free(p);
    free(q);
    return status;
}
