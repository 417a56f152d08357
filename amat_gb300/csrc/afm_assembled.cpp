// Assembled operator: the matrix par::aMatBased builds through PETSc
// (include/aMatBased.hpp), as CSR on the device, with a hand-written SpMV
// (afm_spmv.cu). A second baseline beside the assembly-free product and the
// source of a full-matrix equality check against the reference's own
// assembled matrix (dump_mat, include/aMatBased.hpp:262-292).
//
// Assembly follows the reference's arithmetic exactly: set_element_matrix adds
// every element matrix with ADD_VALUES in element order, row by row, columns
// in element order (include/aMatBased.hpp:214-258), so entry (i, j) is the sum
// over elements in ascending id, then element rows, then element columns; the
// identity method then INSERTs 1 on a constrained row's diagonal and 0 on the
// rest of the row and on constrained columns, the penalty method INSERTs
// 100 tr(K) on constrained diagonals (apply_bc_mat, 294-352). The sparsity
// pattern is the union of the element patterns (entries set to zero stay).
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

#include "afm_internal.hpp"

namespace afm {

cudaError_t launch_csr_spmv(const uint64_t* rp, const uint32_t* cols, const double* vals, const double* x, double* y,
                            uint32_t n_rows, int width, int sm_count, cudaStream_t st);

namespace {

struct CsrHost {
    std::vector<uint64_t> rp;
    std::vector<uint32_t> cols;
    std::vector<double> vals;
};

// Builds the CSR of sum_e P_e^T Ke P_e (and its boundary-condition edits).
// ke_of(e) returns element e's row-major matrix. Rows are independent, so
// they are filled in parallel; every entry's sum order is the reference's.
template <typename KeOf>
int assemble(uint32_t n_elem, uint32_t n_dofs, const uint32_t* off, const uint32_t* map, KeOf ke_of,
             const std::vector<uint8_t>& is_bc, int bc_method, double trace, int apply_bc, CsrHost& out) {
    // DoF -> elements containing it (ascending, one entry per element)
    std::vector<uint64_t> dptr((size_t)n_dofs + 1, 0);
    for (uint32_t e = 0; e < n_elem; e++)
        for (uint32_t k = off[e]; k < off[e + 1]; k++) {
            if (map[k] >= n_dofs) return set_error(AFM_INDEX_OUT_OF_BOUNDS, "element %u lists DoF %u", e, map[k]);
            bool first = true;
            for (uint32_t k2 = off[e]; k2 < k; k2++) first = first && map[k2] != map[k];
            if (first) dptr[map[k] + 1]++;
        }
    for (uint32_t d = 0; d < n_dofs; d++) dptr[d + 1] += dptr[d];
    std::vector<uint32_t> delem(dptr[n_dofs]);
    {
        std::vector<uint64_t> fill(dptr.begin(), dptr.end() - 1);
        for (uint32_t e = 0; e < n_elem; e++)
            for (uint32_t k = off[e]; k < off[e + 1]; k++) {
                bool first = true;
                for (uint32_t k2 = off[e]; k2 < k; k2++) first = first && map[k2] != map[k];
                if (first) delem[fill[map[k]]++] = e;
            }
    }
    // row patterns: the sorted union of the DoFs of the row's elements
    out.rp.assign((size_t)n_dofs + 1, 0);
#pragma omp parallel
    {
        std::vector<uint32_t> buf;
#pragma omp for schedule(dynamic, 256)
        for (int64_t i = 0; i < (int64_t)n_dofs; i++) {
            buf.clear();
            for (uint64_t q = dptr[i]; q < dptr[i + 1]; q++) {
                const uint32_t e = delem[q];
                buf.insert(buf.end(), map + off[e], map + off[e + 1]);
            }
            std::sort(buf.begin(), buf.end());
            out.rp[i + 1] = (uint64_t)(std::unique(buf.begin(), buf.end()) - buf.begin());
        }
    }
    for (uint32_t i = 0; i < n_dofs; i++) out.rp[i + 1] += out.rp[i];
    const uint64_t nnz = out.rp[n_dofs];
    out.cols.resize(nnz);
    out.vals.assign(nnz, 0.0);
    const double pen = 100.0 * trace;  // PENALTY_FACTOR * m_dtTraceK (include/aMat.hpp:68)
#pragma omp parallel
    {
        std::vector<uint32_t> buf;
#pragma omp for schedule(dynamic, 256)
        for (int64_t i = 0; i < (int64_t)n_dofs; i++) {
            buf.clear();
            for (uint64_t q = dptr[i]; q < dptr[i + 1]; q++) {
                const uint32_t e = delem[q];
                buf.insert(buf.end(), map + off[e], map + off[e + 1]);
            }
            std::sort(buf.begin(), buf.end());
            buf.erase(std::unique(buf.begin(), buf.end()), buf.end());
            uint32_t* c = out.cols.data() + out.rp[i];
            double* v = out.vals.data() + out.rp[i];
            std::copy(buf.begin(), buf.end(), c);
            const uint32_t len = (uint32_t)buf.size();
            auto at = [&](uint32_t col) { return (uint32_t)(std::lower_bound(c, c + len, col) - c); };
            // ADD_VALUES in element order, element rows, element columns
            for (uint64_t q = dptr[i]; q < dptr[i + 1]; q++) {
                const uint32_t e = delem[q], n = off[e + 1] - off[e];
                const double* k = ke_of(e);
                for (uint32_t r = 0; r < n; r++) {
                    if (map[off[e] + r] != (uint32_t)i) continue;
                    for (uint32_t cc = 0; cc < n; cc++) v[at(map[off[e] + cc])] += k[(size_t)r * n + cc];
                }
            }
            if (!apply_bc) continue;
            // apply_bc_mat: every pattern entry of a row comes from an element containing the row
            if (bc_method == AFM_BC_IMATRIX) {
                if (is_bc[i]) {
                    for (uint32_t t = 0; t < len; t++) v[t] = (c[t] == (uint32_t)i) ? 1.0 : 0.0;
                } else {
                    for (uint32_t t = 0; t < len; t++)
                        if (is_bc[c[t]]) v[t] = 0.0;
                }
            } else if (is_bc[i]) {
                // a constrained DoF of no element has an empty row, which apply_bc_mat never reaches
                const uint32_t t = at((uint32_t)i);
                if (t < len && c[t] == (uint32_t)i) v[t] = pen;
            }
        }
    }
    return AFM_SUCCESS;
}

int check_maps(uint32_t n_elem, const uint32_t* offsets) {
    for (uint32_t e = 0; e < n_elem; e++)
        if (offsets[e + 1] < offsets[e]) return set_error(AFM_ERR_INVALID_ARG, "offsets not monotone at %u", e);
    return AFM_SUCCESS;
}

}  // namespace
}  // namespace afm

using namespace afm;

extern "C" {

int afm_assemble_csr_host(uint32_t n_elem, uint32_t n_dofs, const uint32_t* offsets, const uint32_t* map,
                          const double* ke, const uint64_t* constrained, uint32_t n_constrained, int bc_method,
                          int apply_bc, uint64_t* nnz, uint64_t* row_ptr, uint32_t* cols, double* vals) {
    if (!offsets || !map || !ke || !nnz || (n_constrained && !constrained))
        return set_error(AFM_ERR_INVALID_ARG, "null argument");
    if (bc_method != AFM_BC_IMATRIX && bc_method != AFM_BC_PENALTY)
        return set_error(AFM_UNKNOWN_BC_METH, "bc method %d", bc_method);
    int s = check_maps(n_elem, offsets);
    if (s) return s;
    std::vector<uint64_t> kofs((size_t)n_elem + 1, 0);
    double trace = 0.0;
    for (uint32_t e = 0; e < n_elem; e++) {
        const uint64_t n = offsets[e + 1] - offsets[e];
        kofs[e + 1] = kofs[e] + n * n;
        for (uint64_t r = 0; r < n; r++) trace += ke[kofs[e] + r * n + r];  // element order (aMatBased.hpp:247-250)
    }
    std::vector<uint8_t> is_bc(n_dofs, 0);
    for (uint32_t k = 0; k < n_constrained; k++) {
        if (constrained[k] >= n_dofs) return set_error(AFM_INDEX_OUT_OF_BOUNDS, "constrained DoF %llu",
                                                       (unsigned long long)constrained[k]);
        is_bc[constrained[k]] = 1;
    }
    CsrHost csr;
    s = assemble(n_elem, n_dofs, offsets, map, [&](uint32_t e) { return ke + kofs[e]; }, is_bc, bc_method, trace,
                 apply_bc, csr);
    if (s) return s;
    const uint64_t have = *nnz;
    *nnz = csr.rp[n_dofs];
    if (row_ptr) memcpy(row_ptr, csr.rp.data(), sizeof(uint64_t) * (n_dofs + 1));
    if (cols || vals) {
        if (have < *nnz) return set_error(AFM_ERR_INVALID_ARG, "arrays hold %llu entries, %llu needed",
                                          (unsigned long long)have, (unsigned long long)*nnz);
        if (cols) memcpy(cols, csr.cols.data(), sizeof(uint32_t) * *nnz);
        if (vals) memcpy(vals, csr.vals.data(), sizeof(double) * *nnz);
    }
    return set_error(AFM_SUCCESS, "");
}

int afm_assemble(afm_operator* op, int apply_bc) {
    if (!op) return set_error(AFM_ERR_INVALID_ARG, "null operator");
    if (!op->finalized) return set_error(AFM_ERR_STATE, "assemble before finalize");
    if (op->ke.size() != op->kofs[op->n_elem])
        return set_error(AFM_ERR_STATE, "assembly needs the element matrices (set_element_matrix)");
    int prev = -1;
    cudaGetDevice(&prev);
    cudaSetDevice(op->device);
    std::vector<uint8_t> is_bc(op->n_dofs, 0);
    for (uint32_t d : op->bc_unique) is_bc[d] = 1;
    CsrHost csr;
    int s = assemble(op->n_elem, op->n_dofs, op->offsets.data(), op->map.data(),
                     [&](uint32_t e) { return op->ke.data() + op->kofs[e]; }, is_bc, op->bc_method, op->trace,
                     apply_bc, csr);
    if (s == AFM_SUCCESS) {
        cudaStream_t st = op->stream;
        if (op->d_csr_rp) cudaFreeAsync(op->d_csr_rp, st);
        if (op->d_csr_cols) cudaFreeAsync(op->d_csr_cols, st);
        if (op->d_csr_vals) cudaFreeAsync(op->d_csr_vals, st);
        op->d_csr_rp = nullptr, op->d_csr_cols = nullptr, op->d_csr_vals = nullptr;
        const uint64_t nnz = csr.rp[op->n_dofs];
        cudaError_t e = cudaMallocAsync((void**)&op->d_csr_rp, sizeof(uint64_t) * (op->n_dofs + 1), st);
        if (e == cudaSuccess) e = cudaMallocAsync((void**)&op->d_csr_cols, sizeof(uint32_t) * std::max<uint64_t>(nnz, 1), st);
        if (e == cudaSuccess) e = cudaMallocAsync((void**)&op->d_csr_vals, sizeof(double) * std::max<uint64_t>(nnz, 1), st);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(op->d_csr_rp, csr.rp.data(), sizeof(uint64_t) * (op->n_dofs + 1),
                                cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess && nnz)
            e = cudaMemcpyAsync(op->d_csr_cols, csr.cols.data(), sizeof(uint32_t) * nnz, cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess && nnz)
            e = cudaMemcpyAsync(op->d_csr_vals, csr.vals.data(), sizeof(double) * nnz, cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);  // the host arrays go out of scope
        if (e != cudaSuccess) {
            s = set_error(e == cudaErrorMemoryAllocation ? AFM_ERR_OOM : AFM_ERR_CUDA, "assembled upload: %s",
                          cudaGetErrorString(e));
        } else {
            op->csr_nnz = nnz;
            // threads per row: about a quarter of the mean row length, 4 to 32
            const double mean = op->n_dofs ? (double)nnz / op->n_dofs : 0.0;
            op->csr_width = mean <= 32.0 ? 4 : mean <= 64.0 ? 8 : mean <= 128.0 ? 16 : 32;
            s = set_error(AFM_SUCCESS, "");
        }
    }
    if (prev >= 0) cudaSetDevice(prev);
    return s;
}

int afm_matvec_assembled_device(afm_operator* op, double* d_v, const double* d_u, void* stream) {
    if (!op) return set_error(AFM_ERR_INVALID_ARG, "null operator");
    if (!op->d_csr_rp) return set_error(AFM_ERR_STATE, "assembled product before afm_assemble");
    if (!d_v || !d_u || (const double*)d_v == d_u) return set_error(AFM_ERR_INVALID_ARG, "bad vectors");
    int prev = -1;
    cudaGetDevice(&prev);
    cudaSetDevice(op->device);
    cudaStream_t st = stream ? (cudaStream_t)stream : op->stream;
    const cudaError_t e = launch_csr_spmv(op->d_csr_rp, op->d_csr_cols, op->d_csr_vals, d_u, d_v, op->n_dofs,
                                          op->csr_width, op->sm_count, st);
    if (prev >= 0) cudaSetDevice(prev);
    if (e != cudaSuccess) return set_error(AFM_ERR_CUDA, "assembled product: %s", cudaGetErrorString(e));
    return set_error(AFM_SUCCESS, "");
}

int afm_get_assembled_csr(afm_operator* op, uint64_t* nnz, uint64_t* row_ptr, uint32_t* cols, double* vals) {
    if (!op || !nnz) return set_error(AFM_ERR_INVALID_ARG, "null argument");
    if (!op->d_csr_rp) return set_error(AFM_ERR_STATE, "no assembled matrix (afm_assemble)");
    const uint64_t have = *nnz;
    *nnz = op->csr_nnz;
    int prev = -1;
    cudaGetDevice(&prev);
    cudaSetDevice(op->device);
    cudaError_t e = cudaSuccess;
    if (row_ptr)
        e = cudaMemcpyAsync(row_ptr, op->d_csr_rp, sizeof(uint64_t) * (op->n_dofs + 1), cudaMemcpyDeviceToHost,
                            op->stream);
    if ((cols || vals) && have < op->csr_nnz) {
        if (prev >= 0) cudaSetDevice(prev);
        return set_error(AFM_ERR_INVALID_ARG, "arrays hold %llu entries, %llu needed", (unsigned long long)have,
                         (unsigned long long)op->csr_nnz);
    }
    if (e == cudaSuccess && cols && op->csr_nnz)
        e = cudaMemcpyAsync(cols, op->d_csr_cols, sizeof(uint32_t) * op->csr_nnz, cudaMemcpyDeviceToHost, op->stream);
    if (e == cudaSuccess && vals && op->csr_nnz)
        e = cudaMemcpyAsync(vals, op->d_csr_vals, sizeof(double) * op->csr_nnz, cudaMemcpyDeviceToHost, op->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(op->stream);
    if (prev >= 0) cudaSetDevice(prev);
    if (e != cudaSuccess) return set_error(AFM_ERR_CUDA, "assembled copy: %s", cudaGetErrorString(e));
    return set_error(AFM_SUCCESS, "");
}

}  // extern "C"
