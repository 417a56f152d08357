/* afm_problems.h - finite-element problem generators for the AFM operator.
 *
 * The counterpart of the reference's example drivers and element kernels
 * (examples/src/example03a.cpp, example07a.cpp, example05a.cpp,
 * examples/src/ke_matrix.cpp, fe_vector.cpp, examples/include/shapeFunc.hpp,
 * integration.hpp): structured meshes with the examples' node numbering,
 * element stiffness matrices by isoparametric Gauss quadrature, load vectors.
 * Host-only (OpenMP); inputs for the operator of afm.h, not part of its hot
 * path. All randomness comes from a counter-based generator keyed by
 * (seed, node id), so results are identical on every host and thread count.
 */
#ifndef AFM_GB300_AFM_PROBLEMS_H
#define AFM_GB300_AFM_PROBLEMS_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct afm_mesh {
    uint32_t n_nodes;
    uint32_t n_elem;
    uint32_t nodes_per_elem;
    uint32_t nx, ny, nz;       /* elements per axis */
    double lx, ly, lz;         /* domain [0,lx] x [0,ly] x [0,lz] */
    double* coords;            /* n_nodes x 3 */
    uint32_t* elem_nodes;      /* n_elem x nodes_per_elem, element-local node order of the examples */
    uint32_t* lattice;         /* n_nodes x 3 integer lattice position (doubled lattice for quadratic meshes) */
} afm_mesh;

typedef enum afm_element_kind {
    AFM_KE_HEX8_POISSON = 0,   /* 8x8,   ke_hex8 (examples/src/ke_matrix.cpp:436-527) */
    AFM_KE_HEX8_ELASTIC = 1,   /* 24x24, ke_hex8_iso (1234-1400) */
    AFM_KE_HEX20_ELASTIC = 2,  /* 60x60, ke_hex20_iso (1403-1741) */
    AFM_KE_TET10_POISSON = 3,  /* 10x10, ke_tet10 (221-326) */
    AFM_KE_TET10_ELASTIC = 4   /* 30x30, ke_tet10_iso (2113-2296) */
} afm_element_kind;

/* Structured hex8 mesh, node id i + j(nx+1) + k(nx+1)(ny+1), element node
 * order of examples/src/example03a.cpp:240-255. Nodes not on the boundary are
 * moved by uniform(-jitter, jitter) * h per axis; boundary nodes only along
 * the faces they lie on. */
int afm_mesh_hex8(uint32_t nx, uint32_t ny, uint32_t nz, double lx, double ly, double lz, double jitter,
                  uint64_t seed, afm_mesh* out);
/* Structured 20-node serendipity hex mesh, node ids in the order of
 * examples/src/example07a.cpp:318-386 (lexicographic over the doubled
 * lattice, face and body centres skipped); element node order of the HEX20
 * shape functions (examples/include/shapeFunc.hpp:200-269). Vertex nodes are
 * jittered as for hex8; mid-edge nodes sit at the midpoints of their edges. */
int afm_mesh_hex20(uint32_t nx, uint32_t ny, uint32_t nz, double lx, double ly, double lz, double jitter,
                   uint64_t seed, afm_mesh* out);
/* Each cube of an nx x ny x nz grid split into 6 tetrahedra (Kuhn), with
 * mid-edge nodes: 10-node tetrahedra in the node order of
 * examples/include/shapeFunc.hpp:178-198, every tetrahedron positively
 * oriented. Node ids are lexicographic over the doubled lattice. */
int afm_mesh_tet10(uint32_t nx, uint32_t ny, uint32_t nz, double lx, double ly, double lz, double jitter,
                   uint64_t seed, afm_mesh* out);
void afm_mesh_free(afm_mesh* m);

/* DoFs per element and per node of a kind. */
uint32_t afm_element_dofs(int kind);
uint32_t afm_element_dofs_per_node(int kind);

/* Element matrices of elements first..first+count-1, row-major n x n each,
 * back to back. ngt: Gauss points per axis. E, nu: elasticity only. Returns
 * nonzero if an element has a non-positive Jacobian. */
int afm_element_matrices(int kind, const afm_mesh* m, uint32_t first, uint32_t count, double E, double nu,
                         uint32_t ngt, double* ke);
/* One element matrix from node coordinates xe (nodes x 3). */
int afm_element_matrix_xe(int kind, const double* xe, double E, double nu, uint32_t ngt, double* ke);
/* 1-D Gauss-Legendre points and weights on [-1,1], ascending, interleaved
 * (x0, w0, x1, w1, ...) as examples/include/integration.hpp:82-113. */
void afm_gauss_legendre(uint32_t n, double* pts_n_wts);

/* Element DoF map: dof = node * dofs_per_node + component (example07a.cpp:455-470). */
int afm_dof_map(const afm_mesh* m, uint32_t dofs_per_node, uint32_t* map);

/* Load vectors (length n_nodes * dofs_per_node), assembled in element order.
 * Poisson: f = sin(2 pi x/lx) sin(2 pi y/ly) sin(2 pi z/lz) (example03a.cpp:11).
 * Elastic bar: body force (0, 0, -rho_g) and traction (0, 0, rho_g * lz) on the
 * top face z = lz (example07a.cpp:590-700, 780-800). */
int afm_load_poisson_sine(int kind, const afm_mesh* m, uint32_t ngt, double* rhs);
int afm_load_elastic_bar(int kind, const afm_mesh* m, double rho_g, uint32_t ngt, double* rhs);

/* Boundary conditions of the examples, as (global DoF, value) lists sorted by
 * DoF (capacity: n_nodes * dofs_per_node). Returns the count.
 * Poisson: every boundary node, value 0 (example03a.cpp:344-367).
 * Elastic bar (example07a.cpp:515-560): node at the top-face centre fixed in
 * x, y, z; node at the bottom-face centre fixed in x, y; node at the centre of
 * the bottom face's x = lx edge fixed in y; values 0. */
uint32_t afm_bc_poisson_boundary(const afm_mesh* m, uint64_t* dofs, double* values);
uint32_t afm_bc_elastic_bar(const afm_mesh* m, uint64_t* dofs, double* values);

/* Counter-based uniform in [0, 1) of (seed, index), used for all jitter. */
double afm_uniform01(uint64_t seed, uint64_t index);

#ifdef __cplusplus
}
#endif
#endif
