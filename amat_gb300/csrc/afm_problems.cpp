// Finite-element problem generators (include/afm_problems.h): the meshes,
// element matrices, loads and boundary conditions of the reference's example
// drivers, written from the standard isoparametric formulation.
//
// Element matrices follow the reference's element kernels
// (examples/src/ke_matrix.cpp): Gauss-Legendre tensor rules on hexahedra,
// the collapsed-hexahedron rule with the Duffy weight on tetrahedra
// (ke_matrix.cpp:253-261), shape functions and node orders of
// examples/include/shapeFunc.hpp. Elastic stiffness is written per node pair,
//   K_ab(i,j) = sum_q w_q |J_q| (lam dNa_i dNb_j + mu dNa_j dNb_i + mu d_ij grad Na . grad Nb),
// which equals the reference's B^T C B product (lam = c2, mu = c3,
// lam + 2 mu = c1 of ke_hex20_iso, ke_matrix.cpp:1422-1448).
#include "afm_problems.h"

#include "afm_shape.hpp"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <vector>

namespace {

uint64_t splitmix64(uint64_t x) {
    x += 0x9e3779b97f4a7c15ull;
    x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
    x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
    return x ^ (x >> 31);
}

using afm_shape::Kind;
using afm_shape::kHex20Pos;
using afm_shape::kHex8Sign;
using afm_shape::kind_info;
using afm_shape::quadrature;

using afm_shape::gradients;

int element_matrix(int kind, const double* xe, double E, double nu, const std::vector<double>& q, double* ke) {
    Kind K;
    if (!kind_info(kind, &K)) return 1;
    const int nn = K.nodes, n = nn * K.dpn;
    memset(ke, 0, sizeof(double) * n * n);
    const double lam = E * nu / (1.0 + nu) / (1.0 - 2.0 * nu);
    const double mu = 0.5 * E / (1.0 + nu);
    double dNx[3 * 20], detJ;
    for (size_t t = 0; t < q.size(); t += 4) {
        if (!gradients(K, xe, &q[t], nullptr, dNx, &detJ)) return 2;
        const double w = detJ * q[t + 3];
        for (int a = 0; a < nn; a++)
            for (int b = 0; b < nn; b++) {
                const double* ga = dNx + 3 * a;
                const double* gb = dNx + 3 * b;
                const double gg = ga[0] * gb[0] + ga[1] * gb[1] + ga[2] * gb[2];
                if (K.dpn == 1) {
                    ke[a * n + b] += gg * w;
                } else {
                    for (int i = 0; i < 3; i++)
                        for (int j = 0; j < 3; j++) {
                            double v = lam * ga[i] * gb[j] + mu * ga[j] * gb[i];
                            if (i == j) v += mu * gg;
                            ke[(3 * a + i) * n + (3 * b + j)] += v * w;
                        }
                }
            }
    }
    return 0;
}

void gather_xe(const afm_mesh* m, uint32_t e, double* xe) {
    for (uint32_t a = 0; a < m->nodes_per_elem; a++) {
        const uint32_t nd = m->elem_nodes[(size_t)e * m->nodes_per_elem + a];
        for (int i = 0; i < 3; i++) xe[3 * a + i] = m->coords[3 * (size_t)nd + i];
    }
}

int alloc_mesh(afm_mesh* m, uint32_t nn, uint32_t ne, uint32_t npe) {
    m->n_nodes = nn;
    m->n_elem = ne;
    m->nodes_per_elem = npe;
    m->coords = (double*)malloc(sizeof(double) * 3 * (size_t)nn);
    m->lattice = (uint32_t*)malloc(sizeof(uint32_t) * 3 * (size_t)nn);
    m->elem_nodes = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)ne * npe);
    if (!m->coords || !m->lattice || !m->elem_nodes) {
        afm_mesh_free(m);
        return 1;
    }
    return 0;
}

// Jittered position of lattice point (X, Y, Z) of a lattice with spacing
// h[axis] and maximum index M[axis]; pure function of (seed, point).
void jitter_point(const uint32_t* P, const uint32_t* M, const double* h, double jitter, uint64_t seed,
                  uint64_t key, double* x) {
    for (int i = 0; i < 3; i++) {
        x[i] = P[i] * h[i];
        if (jitter > 0 && P[i] != 0 && P[i] != M[i])
            x[i] += (2.0 * afm_uniform01(seed, 3 * key + i) - 1.0) * jitter * h[i] * (M[i] > 0 ? 1.0 : 0.0);
    }
}

}  // namespace

extern "C" {

double afm_uniform01(uint64_t seed, uint64_t index) {
    const uint64_t r = splitmix64(seed * 0x632be59bd9b4e019ull ^ splitmix64(index));
    return (double)(r >> 11) * (1.0 / 9007199254740992.0);
}

void afm_gauss_legendre(uint32_t n, double* xw) { afm_shape::gauss_legendre(n, xw); }

void afm_mesh_free(afm_mesh* m) {
    if (!m) return;
    free(m->coords);
    free(m->lattice);
    free(m->elem_nodes);
    m->coords = nullptr;
    m->lattice = nullptr;
    m->elem_nodes = nullptr;
}

int afm_mesh_hex8(uint32_t nx, uint32_t ny, uint32_t nz, double lx, double ly, double lz, double jitter,
                  uint64_t seed, afm_mesh* m) {
    if (!m || nx == 0 || ny == 0 || nz == 0) return 1;
    memset(m, 0, sizeof(*m));
    const uint64_t nn = (uint64_t)(nx + 1) * (ny + 1) * (nz + 1);
    const uint64_t ne = (uint64_t)nx * ny * nz;
    if (nn > 0xffffffffull || ne * 8 > 0xffffffffull) return 1;
    if (alloc_mesh(m, (uint32_t)nn, (uint32_t)ne, 8)) return 2;
    m->nx = nx; m->ny = ny; m->nz = nz; m->lx = lx; m->ly = ly; m->lz = lz;
    const uint32_t M[3] = {nx, ny, nz};
    const double h[3] = {lx / nx, ly / ny, lz / nz};
#pragma omp parallel for schedule(static)
    for (int64_t id = 0; id < (int64_t)nn; id++) {
        const uint32_t P[3] = {(uint32_t)(id % (nx + 1)), (uint32_t)((id / (nx + 1)) % (ny + 1)),
                               (uint32_t)(id / ((uint64_t)(nx + 1) * (ny + 1)))};
        memcpy(m->lattice + 3 * id, P, sizeof(P));
        jitter_point(P, M, h, jitter, seed, (uint64_t)id, m->coords + 3 * id);
    }
    // element node order of example03a.cpp:244-253
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < (int64_t)ne; e++) {
        const uint32_t i = e % nx, j = (e / nx) % ny, k = (uint32_t)(e / ((uint64_t)nx * ny));
        uint32_t* en = m->elem_nodes + 8 * e;
        en[0] = i + j * (nx + 1) + k * (nx + 1) * (ny + 1);
        en[1] = en[0] + 1;
        en[3] = en[0] + (nx + 1);
        en[2] = en[3] + 1;
        en[4] = en[0] + (nx + 1) * (ny + 1);
        en[5] = en[4] + 1;
        en[7] = en[4] + (nx + 1);
        en[6] = en[7] + 1;
    }
    return 0;
}

int afm_mesh_hex20(uint32_t nx, uint32_t ny, uint32_t nz, double lx, double ly, double lz, double jitter,
                   uint64_t seed, afm_mesh* m) {
    if (!m || nx == 0 || ny == 0 || nz == 0) return 1;
    memset(m, 0, sizeof(*m));
    const uint64_t X = 2ull * nx + 1, Y = 2ull * ny + 1, Z = 2ull * nz + 1;
    // node index of each doubled-lattice point (UINT32_MAX: face/body centre)
    std::vector<uint32_t> id_of(X * Y * Z, UINT32_MAX);
    uint64_t nn = 0;
    for (uint64_t k = 0; k < Z; k++)
        for (uint64_t j = 0; j < Y; j++)
            for (uint64_t i = 0; i < X; i++) {
                const int odd = (int)(i & 1) + (int)(j & 1) + (int)(k & 1);
                if (odd <= 1) id_of[i + X * (j + Y * k)] = (uint32_t)nn++;
            }
    const uint64_t ne = (uint64_t)nx * ny * nz;
    if (nn > 0xffffffffull || ne * 20 > 0xffffffffull) return 1;
    if (alloc_mesh(m, (uint32_t)nn, (uint32_t)ne, 20)) return 2;
    m->nx = nx; m->ny = ny; m->nz = nz; m->lx = lx; m->ly = ly; m->lz = lz;
    const uint32_t M[3] = {(uint32_t)(X - 1), (uint32_t)(Y - 1), (uint32_t)(Z - 1)};
    const double h[3] = {lx / (2.0 * nx), ly / (2.0 * ny), lz / (2.0 * nz)};
    const double jv = 2.0 * jitter;  // jitter is relative to the element size 2h
#pragma omp parallel for schedule(dynamic, 4096)
    for (int64_t p = 0; p < (int64_t)(X * Y * Z); p++) {
        const uint32_t id = id_of[p];
        if (id == UINT32_MAX) continue;
        uint32_t P[3] = {(uint32_t)(p % X), (uint32_t)((p / X) % Y), (uint32_t)(p / (X * Y))};
        memcpy(m->lattice + 3 * (size_t)id, P, sizeof(P));
        double* x = m->coords + 3 * (size_t)id;
        int oddax = -1;
        for (int a = 0; a < 3; a++)
            if (P[a] & 1) oddax = a;
        if (oddax < 0) {
            jitter_point(P, M, h, jv, seed, (uint64_t)p, x);
        } else {
            // mid-edge node: midpoint of its two (jittered) end vertices
            uint32_t A[3] = {P[0], P[1], P[2]}, B[3] = {P[0], P[1], P[2]};
            A[oddax] -= 1;
            B[oddax] += 1;
            double xa[3], xb[3];
            jitter_point(A, M, h, jv, seed, A[0] + X * (A[1] + Y * (uint64_t)A[2]), xa);
            jitter_point(B, M, h, jv, seed, B[0] + X * (B[1] + Y * (uint64_t)B[2]), xb);
            for (int a = 0; a < 3; a++) x[a] = 0.5 * (xa[a] + xb[a]);
        }
    }
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < (int64_t)ne; e++) {
        const uint64_t i = e % nx, j = (e / nx) % ny, k = e / ((uint64_t)nx * ny);
        for (int a = 0; a < 20; a++) {
            const uint64_t pi = 2 * i + 1 + kHex20Pos[a][0], pj = 2 * j + 1 + kHex20Pos[a][1],
                           pk = 2 * k + 1 + kHex20Pos[a][2];
            m->elem_nodes[20 * e + a] = id_of[pi + X * (pj + Y * pk)];
        }
    }
    return 0;
}

int afm_mesh_tet10(uint32_t nx, uint32_t ny, uint32_t nz, double lx, double ly, double lz, double jitter,
                   uint64_t seed, afm_mesh* m) {
    if (!m || nx == 0 || ny == 0 || nz == 0) return 1;
    memset(m, 0, sizeof(*m));
    const uint64_t X = 2ull * nx + 1, Y = 2ull * ny + 1, Z = 2ull * nz + 1;
    const uint64_t nn = X * Y * Z, ne = 6ull * nx * ny * nz;
    if (nn > 0xffffffffull || ne * 10 > 0xffffffffull) return 1;
    if (alloc_mesh(m, (uint32_t)nn, (uint32_t)ne, 10)) return 2;
    m->nx = nx; m->ny = ny; m->nz = nz; m->lx = lx; m->ly = ly; m->lz = lz;
    const uint32_t M[3] = {(uint32_t)(X - 1), (uint32_t)(Y - 1), (uint32_t)(Z - 1)};
    const double h[3] = {lx / (2.0 * nx), ly / (2.0 * ny), lz / (2.0 * nz)};
    const double jv = 2.0 * jitter;
#pragma omp parallel for schedule(static)
    for (int64_t p = 0; p < (int64_t)nn; p++) {
        uint32_t P[3] = {(uint32_t)(p % X), (uint32_t)((p / X) % Y), (uint32_t)(p / (X * Y))};
        memcpy(m->lattice + 3 * p, P, sizeof(P));
        double* x = m->coords + 3 * p;
        if (!(P[0] & 1) && !(P[1] & 1) && !(P[2] & 1)) {
            jitter_point(P, M, h, jv, seed, (uint64_t)p, x);
        } else {
            // edge midpoint: the edge runs from A = P - odd axes to B = P + odd axes
            uint32_t A[3], B[3];
            for (int a = 0; a < 3; a++) {
                A[a] = P[a] - (P[a] & 1);
                B[a] = P[a] + (P[a] & 1);
            }
            double xa[3], xb[3];
            jitter_point(A, M, h, jv, seed, A[0] + X * (A[1] + Y * (uint64_t)A[2]), xa);
            jitter_point(B, M, h, jv, seed, B[0] + X * (B[1] + Y * (uint64_t)B[2]), xb);
            for (int a = 0; a < 3; a++) x[a] = 0.5 * (xa[a] + xb[a]);
        }
    }
    // Kuhn split: tetrahedron (a,b,c) = 0 -> e_a -> e_a+e_b -> (1,1,1)
    const int perms[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};
    const int parity[6] = {1, -1, -1, 1, 1, -1};
    const int edge[6][2] = {{0, 1}, {1, 2}, {2, 0}, {0, 3}, {1, 3}, {2, 3}};
#pragma omp parallel for schedule(static)
    for (int64_t c = 0; c < (int64_t)(ne / 6); c++) {
        const uint64_t i = c % nx, j = (c / nx) % ny, k = c / ((uint64_t)nx * ny);
        for (int t = 0; t < 6; t++) {
            int v[4][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {1, 1, 1}};
            v[1][perms[t][0]] = 1;
            v[2][perms[t][0]] = 1;
            v[2][perms[t][1]] = 1;
            if (parity[t] < 0)
                for (int a = 0; a < 3; a++) std::swap(v[1][a], v[2][a]);
            uint32_t* en = m->elem_nodes + 10 * (6 * c + t);
            auto node = [&](uint64_t px, uint64_t py, uint64_t pz) { return (uint32_t)(px + X * (py + Y * pz)); };
            for (int a = 0; a < 4; a++) en[a] = node(2 * (i + v[a][0]), 2 * (j + v[a][1]), 2 * (k + v[a][2]));
            for (int q = 0; q < 6; q++) {
                const int* A = v[edge[q][0]];
                const int* B = v[edge[q][1]];
                en[4 + q] = node(2 * i + A[0] + B[0], 2 * j + A[1] + B[1], 2 * k + A[2] + B[2]);
            }
        }
    }
    return 0;
}

uint32_t afm_element_dofs(int kind) {
    Kind K;
    return kind_info(kind, &K) ? (uint32_t)(K.nodes * K.dpn) : 0u;
}

uint32_t afm_element_dofs_per_node(int kind) {
    Kind K;
    return kind_info(kind, &K) ? (uint32_t)K.dpn : 0u;
}

int afm_element_matrix_xe(int kind, const double* xe, double E, double nu, uint32_t ngt, double* ke) {
    Kind K;
    if (!kind_info(kind, &K)) return 1;
    std::vector<double> q;
    quadrature(K.tet, ngt, q);
    return element_matrix(kind, xe, E, nu, q, ke);
}

int afm_element_matrices(int kind, const afm_mesh* m, uint32_t first, uint32_t count, double E, double nu,
                         uint32_t ngt, double* ke) {
    Kind K;
    if (!kind_info(kind, &K) || !m || (uint32_t)K.nodes != m->nodes_per_elem) return 1;
    if ((uint64_t)first + count > m->n_elem) return 1;
    std::vector<double> q;
    quadrature(K.tet, ngt, q);
    const size_t n = (size_t)K.nodes * K.dpn;
    int bad = 0;
#pragma omp parallel for schedule(static) reduction(| : bad)
    for (int64_t t = 0; t < (int64_t)count; t++) {
        double xe[3 * 20];
        gather_xe(m, first + (uint32_t)t, xe);
        if (element_matrix(kind, xe, E, nu, q, ke + (size_t)t * n * n)) bad |= 1;
    }
    return bad ? 2 : 0;
}

int afm_dof_map(const afm_mesh* m, uint32_t dpn, uint32_t* map) {
    if (!m || dpn == 0) return 1;
    const size_t npe = m->nodes_per_elem;
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < (int64_t)m->n_elem; e++)
        for (size_t a = 0; a < npe; a++)
            for (uint32_t d = 0; d < dpn; d++)
                map[((size_t)e * npe + a) * dpn + d] = m->elem_nodes[(size_t)e * npe + a] * dpn + d;
    return 0;
}

int afm_load_poisson_sine(int kind, const afm_mesh* m, uint32_t ngt, double* rhs) {
    Kind K;
    if (!kind_info(kind, &K) || K.dpn != 1 || !m) return 1;
    std::vector<double> q;
    quadrature(K.tet, ngt, q);
    memset(rhs, 0, sizeof(double) * m->n_nodes);
    const double tp = 2.0 * M_PI;
    double xe[3 * 20], N[20], dNx[60], detJ;
    for (uint32_t e = 0; e < m->n_elem; e++) {
        gather_xe(m, e, xe);
        double fe[20] = {0};
        for (size_t t = 0; t < q.size(); t += 4) {
            if (!gradients(K, xe, &q[t], N, dNx, &detJ)) return 2;
            double x[3] = {0, 0, 0};
            for (int a = 0; a < K.nodes; a++)
                for (int i = 0; i < 3; i++) x[i] += N[a] * xe[3 * a + i];
            const double f = sin(tp * x[0] / m->lx) * sin(tp * x[1] / m->ly) * sin(tp * x[2] / m->lz);
            for (int a = 0; a < K.nodes; a++) fe[a] += N[a] * f * detJ * q[t + 3];
        }
        for (int a = 0; a < K.nodes; a++) rhs[m->elem_nodes[(size_t)e * K.nodes + a]] += fe[a];
    }
    return 0;
}

int afm_load_elastic_bar(int kind, const afm_mesh* m, double rho_g, uint32_t ngt, double* rhs) {
    Kind K;
    if (!kind_info(kind, &K) || K.dpn != 3 || !m) return 1;
    std::vector<double> q;
    quadrature(K.tet, ngt, q);
    memset(rhs, 0, sizeof(double) * 3 * (size_t)m->n_nodes);
    std::vector<double> g(2 * ngt);
    afm_gauss_legendre(ngt, g.data());
    const uint32_t zmax = K.nodes == 8 ? m->nz : 2 * m->nz;
    double xe[3 * 20], N[20], dNx[60], detJ, dN[60];
    for (uint32_t e = 0; e < m->n_elem; e++) {
        gather_xe(m, e, xe);
        const uint32_t* en = m->elem_nodes + (size_t)e * K.nodes;
        double fe[60] = {0};
        for (size_t t = 0; t < q.size(); t += 4) {
            if (!gradients(K, xe, &q[t], N, dNx, &detJ)) return 2;
            for (int a = 0; a < K.nodes; a++) fe[3 * a + 2] += -rho_g * N[a] * detJ * q[t + 3];
        }
        // traction on the face zeta = +1 of hexahedra lying on z = lz
        if (!K.tet && m->lattice[3 * (size_t)en[4] + 2] == zmax && m->lattice[3 * (size_t)en[6] + 2] == zmax) {
            const double tz = rho_g * m->lz;
            for (uint32_t i = 0; i < ngt; i++)
                for (uint32_t j = 0; j < ngt; j++) {
                    const double x[3] = {g[2 * i], g[2 * j], 1.0};
                    K.shape(x, N, dN);
                    double a1[3] = {0, 0, 0}, a2[3] = {0, 0, 0};
                    for (int a = 0; a < K.nodes; a++)
                        for (int c = 0; c < 3; c++) {
                            a1[c] += xe[3 * a + c] * dN[3 * a + 0];
                            a2[c] += xe[3 * a + c] * dN[3 * a + 1];
                        }
                    const double nrm[3] = {a1[1] * a2[2] - a1[2] * a2[1], a1[2] * a2[0] - a1[0] * a2[2],
                                           a1[0] * a2[1] - a1[1] * a2[0]};
                    const double dA = sqrt(nrm[0] * nrm[0] + nrm[1] * nrm[1] + nrm[2] * nrm[2]);
                    for (int a = 0; a < K.nodes; a++) fe[3 * a + 2] += N[a] * tz * dA * g[2 * i + 1] * g[2 * j + 1];
                }
        }
        for (int a = 0; a < K.nodes; a++)
            for (int c = 0; c < 3; c++) rhs[3 * (size_t)en[a] + c] += fe[3 * a + c];
    }
    return 0;
}

uint32_t afm_bc_poisson_boundary(const afm_mesh* m, uint64_t* dofs, double* values) {
    const uint32_t f = (m->nodes_per_elem == 8) ? 1 : 2;
    const uint32_t M[3] = {f * m->nx, f * m->ny, f * m->nz};
    uint32_t c = 0;
    for (uint32_t id = 0; id < m->n_nodes; id++) {
        const uint32_t* P = m->lattice + 3 * (size_t)id;
        bool b = false;
        for (int a = 0; a < 3; a++) b = b || P[a] == 0 || P[a] == M[a];
        if (b) {
            dofs[c] = id;
            values[c] = 0.0;
            c++;
        }
    }
    return c;
}

uint32_t afm_bc_elastic_bar(const afm_mesh* m, uint64_t* dofs, double* values) {
    const uint32_t f = (m->nodes_per_elem == 8) ? 1 : 2;
    const uint32_t M[3] = {f * m->nx, f * m->ny, f * m->nz};
    std::vector<std::pair<uint64_t, double>> list;
    for (uint32_t id = 0; id < m->n_nodes; id++) {
        const uint32_t* P = m->lattice + 3 * (size_t)id;
        const bool cx = 2 * P[0] == M[0], cy = 2 * P[1] == M[1];
        if (cx && cy && P[2] == M[2])
            for (int d = 0; d < 3; d++) list.push_back({3ull * id + d, 0.0});
        if (cx && cy && P[2] == 0)
            for (int d = 0; d < 2; d++) list.push_back({3ull * id + d, 0.0});
        if (P[0] == M[0] && cy && P[2] == 0) list.push_back({3ull * id + 1, 0.0});
    }
    std::sort(list.begin(), list.end());
    list.erase(std::unique(list.begin(), list.end()), list.end());
    for (size_t i = 0; i < list.size(); i++) {
        dofs[i] = list[i].first;
        values[i] = list[i].second;
    }
    return (uint32_t)list.size();
}

}  // extern "C"
