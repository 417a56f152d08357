// C entry points over the UNMODIFIED reference aMat code, compiled in place
// from the reference tree by oracle/build_ref.sh into oracle/_ref/libamat_ref.so.
// Test infrastructure only: the tests use it to pin the oracle restatement
// (oracle/afm_oracle.c) and to write the golden fixtures under tests/golden/.
// Nothing in the product links or loads it.
//
// Each function builds the reference objects exactly as the example drivers do
// (examples/src/example03a.cpp:411-483): Maps::set_map with an identity
// local-to-global map on one rank, Maps::set_bdr_map, aMatFree with
// MATFREE_TYPE::QUASI_FREE (method 1), set_element_matrix per element (split
// into blocks_dim x blocks_dim blocks; all-zero off-diagonal blocks are left
// unset, i.e. nullptr, as the reference's XFEM use does), finalize.
#include "aMatFree.hpp"
#include "aMatBased.hpp"
#include "meshGraph.hpp"
#include "integration.hpp"
#include "ke_matrix.hpp"

#include <cstdint>
#include <memory>
#include <vector>

namespace {

using LI = unsigned int;
using GI = unsigned long;
using Maps = par::Maps<double, GI, LI>;
using Free = par::aMatFree<double, GI, LI>;
using Based = par::aMatBased<double, GI, LI>;
using EMat = Eigen::Matrix<double, Eigen::Dynamic, Eigen::Dynamic>;

struct RefProblem {
    LI n_elem = 0, n_dofs = 0;
    std::vector<LI> dofs_per_elem;             // must outlive Maps (include/maps.hpp:423)
    std::vector<std::vector<LI>> local_map;    // jagged element -> local dof
    std::vector<LI*> local_map_ptrs;
    std::vector<GI> l2g;
    std::vector<GI> constrained;
    std::vector<double> values;
    std::unique_ptr<Maps> maps;
};

void build_maps(RefProblem& p, uint32_t n_elem, uint32_t n_dofs, const uint32_t* offsets, const uint32_t* map,
                const uint64_t* constrained, const double* values, uint32_t n_constraints) {
    p.n_elem = n_elem;
    p.n_dofs = n_dofs;
    p.dofs_per_elem.resize(n_elem);
    p.local_map.resize(n_elem);
    p.local_map_ptrs.resize(n_elem);
    for (uint32_t e = 0; e < n_elem; e++) {
        p.dofs_per_elem[e] = offsets[e + 1] - offsets[e];
        p.local_map[e].assign(map + offsets[e], map + offsets[e + 1]);
        p.local_map_ptrs[e] = p.local_map[e].data();
    }
    p.l2g.resize(n_dofs);
    for (uint32_t i = 0; i < n_dofs; i++) p.l2g[i] = i;
    p.constrained.assign(constrained, constrained + n_constraints);
    p.values.assign(values, values + n_constraints);
    p.maps.reset(new Maps(MPI_COMM_WORLD));
    p.maps->set_map(n_elem, p.local_map_ptrs.data(), p.dofs_per_elem.data(), n_dofs, p.l2g.data(), 0,
                    (GI)n_dofs - 1, n_dofs);
    p.maps->set_bdr_map(p.constrained.data(), p.values.data(), n_constraints);
}

// Splits a row-major n x n element matrix into blocks and hands every block
// that is not entirely zero (diagonal blocks always) to set_element_matrix.
template <typename Op>
void set_elements(Op& A, const RefProblem& p, const uint32_t* offsets, const double* ke, uint32_t blocks_dim) {
    size_t off = 0;
    for (LI e = 0; e < p.n_elem; e++) {
        const LI n = offsets[e + 1] - offsets[e];
        const LI nb = n / blocks_dim;
        for (LI bi = 0; bi < blocks_dim; bi++)
            for (LI bj = 0; bj < blocks_dim; bj++) {
                EMat blk(nb, nb);
                bool nz = (bi == bj);
                for (LI r = 0; r < nb; r++)
                    for (LI c = 0; c < nb; c++) {
                        blk(r, c) = ke[off + (size_t)(bi * nb + r) * n + (bj * nb + c)];
                        nz = nz || blk(r, c) != 0.0;
                    }
                if (nz) A.set_element_matrix(e, blk, bi, bj, blocks_dim);
            }
        off += (size_t)n * n;
    }
}

struct RefFree {
    RefProblem p;
    std::unique_ptr<Free> A;
    Mat shell = nullptr;
};

struct RefBased {
    RefProblem p;
    std::unique_ptr<Based> A;
};

Vec make_vec(LI n, const double* x) {
    Vec v;
    VecCreate(MPI_COMM_WORLD, &v);
    VecSetSizes(v, n, PETSC_DECIDE);
    if (x)
        for (LI i = 0; i < n; i++) v->a[i] = x[i];
    return v;
}

}  // namespace

extern "C" {

void* ref_afm_create(uint32_t n_elem, uint32_t n_dofs, const uint32_t* offsets, const uint32_t* map,
                     const double* ke, uint32_t blocks_dim, const uint64_t* constrained, const double* values,
                     uint32_t n_constraints, int bc_method) {
    auto* r = new RefFree();
    build_maps(r->p, n_elem, n_dofs, offsets, map, constrained, values, n_constraints);
    r->A.reset(new Free(*r->p.maps, (par::BC_METH)bc_method));
    r->A->set_matfree_type(par::MATFREE_TYPE::QUASI_FREE);
    set_elements(*r->A, r->p, offsets, ke, blocks_dim);
    r->A->finalize();
    r->shell = r->A->get_matrix();
    return r;
}

// aMatFree::matvec(v, u, true) (include/aMatFree.hpp:1682-1775 -> matvec_ghosted_OMP 1778-2238)
int ref_afm_matvec(void* h, double* v, const double* u) {
    auto* r = (RefFree*)h;
    return (int)r->A->matvec(v, u, true);
}

// PETSc MatMult on the shell -> aMatFree::MatMult_mf (include/aMatFree.hpp:3894-3941).
// apply_bc must have run first: it allocates the saved-U_c buffer (957-969).
int ref_afm_matmult_bc(void* h, double* v, const double* u) {
    auto* r = (RefFree*)h;
    Vec uv = make_vec(r->p.n_dofs, u), vv = make_vec(r->p.n_dofs, nullptr);
    MatMult(r->shell, uv, vv);
    for (LI i = 0; i < r->p.n_dofs; i++) v[i] = vv->a[i];
    VecDestroy(&uv);
    VecDestroy(&vv);
    return 0;
}

// PETSc MatGetDiagonal on the shell -> MatGetDiagonal_mf (3945-3975) + apply_bc_diagonal (4310-4338)
int ref_afm_get_diagonal(void* h, double* d) {
    auto* r = (RefFree*)h;
    Vec dv = make_vec(r->p.n_dofs, nullptr);
    MatGetDiagonal(r->shell, dv);
    for (LI i = 0; i < r->p.n_dofs; i++) d[i] = dv->a[i];
    VecDestroy(&dv);
    return 0;
}

// aMatFree::apply_bc (957-969) -> apply_bc_rhs (4537-4700), rhs updated in place
int ref_afm_apply_bc_rhs(void* h, double* rhs) {
    auto* r = (RefFree*)h;
    Vec b = make_vec(r->p.n_dofs, rhs);
    r->A->apply_bc(b);
    for (LI i = 0; i < r->p.n_dofs; i++) rhs[i] = b->a[i];
    VecDestroy(&b);
    return 0;
}

void ref_afm_destroy(void* h) {
    auto* r = (RefFree*)h;
    delete r;
}

// Assembled operator (include/aMatBased.hpp): set_element_matrix with
// ADD_VALUES (214-258), finalize, then apply_bc = apply_bc_rhs + apply_bc_mat
// (80-85, 294-352, 356-440), MatMult (458-460).
void* ref_based_create(uint32_t n_elem, uint32_t n_dofs, const uint32_t* offsets, const uint32_t* map,
                       const double* ke, uint32_t blocks_dim, const uint64_t* constrained, const double* values,
                       uint32_t n_constraints, int bc_method) {
    auto* r = new RefBased();
    build_maps(r->p, n_elem, n_dofs, offsets, map, constrained, values, n_constraints);
    r->A.reset(new Based(*r->p.maps, (par::BC_METH)bc_method));
    set_elements(*r->A, r->p, offsets, ke, blocks_dim);
    r->A->finalize();
    return r;
}

int ref_based_matmult(void* h, double* v, const double* u) {
    auto* r = (RefBased*)h;
    Vec uv = make_vec(r->p.n_dofs, u), vv = make_vec(r->p.n_dofs, nullptr);
    r->A->matmult(vv, uv);
    for (LI i = 0; i < r->p.n_dofs; i++) v[i] = vv->a[i];
    VecDestroy(&uv);
    VecDestroy(&vv);
    return 0;
}

int ref_based_apply_bc(void* h, double* rhs) {
    auto* r = (RefBased*)h;
    Vec b = make_vec(r->p.n_dofs, rhs);
    r->A->apply_bc(b);
    for (LI i = 0; i < r->p.n_dofs; i++) rhs[i] = b->a[i];
    VecDestroy(&b);
    return 0;
}

// The assembled matrix as CSR, rows in order, columns ascending (the shim's
// row maps; PETSc's MatView of dump_mat, include/aMatBased.hpp:262-292, lists
// the same entries). Returns the entry count; fills the arrays when given.
uint64_t ref_based_csr(void* h, uint64_t* row_ptr, uint32_t* cols, double* vals) {
    auto* r = (RefBased*)h;
    Mat A = r->A->get_matrix();
    uint64_t k = 0;
    for (size_t i = 0; i < A->rows.size(); i++) {
        if (row_ptr) row_ptr[i] = k;
        for (const auto& e : A->rows[i]) {
            if (cols) cols[k] = (uint32_t)e.first;
            if (vals) vals[k] = e.second;
            k++;
        }
    }
    if (row_ptr) row_ptr[A->rows.size()] = k;
    return k;
}

void ref_based_destroy(void* h) { delete (RefBased*)h; }

// meshGraph::mesh2Graph + greedyColoring (include/meshGraph.hpp:132-155, 59-109)
int ref_mesh_coloring(uint32_t n_dofs, uint32_t n_elem, const uint32_t* offsets, const uint32_t* map,
                      uint32_t* colors, uint32_t* n_colors) {
    std::vector<unsigned int> dpe(n_elem);
    std::vector<unsigned int*> mesh(n_elem);
    std::vector<std::vector<unsigned int>> rows(n_elem);
    for (uint32_t e = 0; e < n_elem; e++) {
        dpe[e] = offsets[e + 1] - offsets[e];
        rows[e].assign(map + offsets[e], map + offsets[e + 1]);
        mesh[e] = rows[e].data();
    }
    meshGraph g(n_elem);
    g.mesh2Graph(n_dofs, n_elem, dpe.data(), mesh.data());
    g.greedyColoring();
    std::vector<std::vector<unsigned int>> per_color(n_elem > 0 ? n_elem : 1);
    g.computeVerticesPerColor(per_color.data());
    for (uint32_t c = 0; c < g.nColors; c++)
        for (unsigned int e : per_color[c]) colors[e] = c;
    *n_colors = g.nColors;
    return 0;
}

// 1D Gauss-Legendre rule of the examples (examples/include/integration.hpp:82-113)
void ref_gauss(uint32_t ngt, double* pts_n_wts) {
    integration<double> ig(ngt);
    for (uint32_t i = 0; i < 2 * ngt; i++) pts_n_wts[i] = ig.Pts_n_Wts[i];
}

// Element matrices of the examples (examples/src/ke_matrix.cpp), row-major out.
void ref_ke_hex8(const double* xe, uint32_t ngt, double* ke) {
    integration<double> ig(ngt);
    ke_hex8(ke, xe, ig.Pts_n_Wts, ngt);
}
void ref_ke_tet10(const double* xe, uint32_t ngt, double* ke) {
    integration<double> ig(ngt);
    EMat k(10, 10);
    ke_tet10(k, xe, ig.Pts_n_Wts, ngt);
    for (int r = 0; r < 10; r++)
        for (int c = 0; c < 10; c++) ke[r * 10 + c] = k(r, c);
}
void ref_ke_hex8_iso(const double* xe, double E, double nu, uint32_t ngt, double* ke) {
    integration<double> ig(ngt);
    Eigen::Matrix<double, 24, 24> k;
    ke_hex8_iso(k, (double*)xe, E, nu, ig.Pts_n_Wts, ngt);
    for (int r = 0; r < 24; r++)
        for (int c = 0; c < 24; c++) ke[r * 24 + c] = k(r, c);
}
void ref_ke_hex20_iso(const double* xe, double E, double nu, uint32_t ngt, double* ke) {
    integration<double> ig(ngt);
    auto* k = new Eigen::Matrix<double, 60, 60>();
    ke_hex20_iso(*k, (double*)xe, E, nu, ig.Pts_n_Wts, ngt);
    for (int r = 0; r < 60; r++)
        for (int c = 0; c < 60; c++) ke[r * 60 + c] = (*k)(r, c);
    delete k;
}
void ref_ke_tet10_iso(const double* xe, double E, double nu, uint32_t ngt, double* ke) {
    integration<double> ig(ngt);
    auto* k = new Eigen::Matrix<double, 30, 30>();
    ke_tet10_iso(*k, (double*)xe, E, nu, ig.Pts_n_Wts, ngt);
    for (int r = 0; r < 30; r++)
        for (int c = 0; c < 30; c++) ke[r * 30 + c] = (*k)(r, c);
    delete k;
}

}  // extern "C"
