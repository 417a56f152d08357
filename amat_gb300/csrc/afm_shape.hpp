// Reference-element data shared by the problem generators (afm_problems.cpp)
// and the matrix-free operator (afm_free.cpp): shape functions of hex8,
// hex20 and tet10 with the node orders of the reference's
// examples/include/shapeFunc.hpp, the Gauss-Legendre rule and the
// quadrature point lists of the reference's element kernels
// (examples/src/ke_matrix.cpp). Host code, double precision.
#pragma once

#include <math.h>
#include <stdint.h>

#include <vector>

namespace afm_shape {

// element kinds (include/afm_problems.h afm_ke_kind, include/afm.h afm_element_kind)
enum : int { HEX8_POISSON = 0, HEX8_ELASTIC = 1, HEX20_ELASTIC = 2, TET10_POISSON = 3, TET10_ELASTIC = 4 };

inline void gauss_legendre(uint32_t n, double* xw) {
    // roots of P_n by Newton iteration from the Tricomi estimate, weights
    // 2 / ((1 - x^2) P_n'(x)^2); ascending order
    const uint32_t m = (n + 1) / 2;
    for (uint32_t i = 1; i <= m; i++) {
        double z = cos(M_PI * (i - 0.25) / (n + 0.5)), pp = 0.0;
        for (int it = 0; it < 100; it++) {
            double p1 = 1.0, p2 = 0.0;
            for (uint32_t j = 1; j <= n; j++) {
                const double p3 = p2;
                p2 = p1;
                p1 = ((2.0 * j - 1.0) * z * p2 - (j - 1.0) * p3) / j;
            }
            pp = n * (z * p1 - p2) / (z * z - 1.0);
            const double z1 = z;
            z = z1 - p1 / pp;
            if (fabs(z - z1) < 1e-15) break;
        }
        const double w = 2.0 / ((1.0 - z * z) * pp * pp);
        xw[2 * (i - 1)] = -z;
        xw[2 * (i - 1) + 1] = w;
        xw[2 * (n - i)] = z;
        xw[2 * (n - i) + 1] = w;
    }
}

// ---- shape functions: N (nn) and dN (nn x 3) at reference point x ----------

constexpr int kHex8Sign[8][3] = {{-1, -1, -1}, {1, -1, -1}, {1, 1, -1}, {-1, 1, -1},
                             {-1, -1, 1},  {1, -1, 1},  {1, 1, 1},  {-1, 1, 1}};

// hex20: reference coordinates of the nodes (shapeFunc.hpp:200-269)
constexpr int kHex20Pos[20][3] = {{-1, -1, -1}, {1, -1, -1}, {1, 1, -1}, {-1, 1, -1}, {-1, -1, 1}, {1, -1, 1},
                              {1, 1, 1},    {-1, 1, 1},  {0, -1, -1}, {1, 0, -1},  {0, 1, -1},  {-1, 0, -1},
                              {0, -1, 1},   {1, 0, 1},   {0, 1, 1},   {-1, 0, 1},  {-1, -1, 0}, {1, -1, 0},
                              {1, 1, 0},    {-1, 1, 0}};

inline void shape_hex8(const double* x, double* N, double* dN) {
    for (int a = 0; a < 8; a++) {
        const double s0 = kHex8Sign[a][0], s1 = kHex8Sign[a][1], s2 = kHex8Sign[a][2];
        const double f0 = 1 + s0 * x[0], f1 = 1 + s1 * x[1], f2 = 1 + s2 * x[2];
        if (N) N[a] = f0 * f1 * f2 / 8.0;
        dN[3 * a + 0] = s0 * f1 * f2 / 8.0;
        dN[3 * a + 1] = f0 * s1 * f2 / 8.0;
        dN[3 * a + 2] = f0 * f1 * s2 / 8.0;
    }
}

inline void shape_hex20(const double* x, double* N, double* dN) {
    for (int a = 0; a < 20; a++) {
        const double p0 = kHex20Pos[a][0], p1 = kHex20Pos[a][1], p2 = kHex20Pos[a][2];
        if (a < 8) {
            const double f0 = 1 + p0 * x[0], f1 = 1 + p1 * x[1], f2 = 1 + p2 * x[2];
            const double g = p0 * x[0] + p1 * x[1] + p2 * x[2] - 2;
            if (N) N[a] = 0.125 * f0 * f1 * f2 * g;
            dN[3 * a + 0] = 0.125 * p0 * f1 * f2 * (g + f0);
            dN[3 * a + 1] = 0.125 * p1 * f0 * f2 * (g + f1);
            dN[3 * a + 2] = 0.125 * p2 * f0 * f1 * (g + f2);
        } else if (p0 == 0) {
            const double f1 = 1 + p1 * x[1], f2 = 1 + p2 * x[2], q = 1 - x[0] * x[0];
            if (N) N[a] = 0.25 * q * f1 * f2;
            dN[3 * a + 0] = -0.5 * x[0] * f1 * f2;
            dN[3 * a + 1] = 0.25 * q * p1 * f2;
            dN[3 * a + 2] = 0.25 * q * f1 * p2;
        } else if (p1 == 0) {
            const double f0 = 1 + p0 * x[0], f2 = 1 + p2 * x[2], q = 1 - x[1] * x[1];
            if (N) N[a] = 0.25 * q * f0 * f2;
            dN[3 * a + 0] = 0.25 * q * p0 * f2;
            dN[3 * a + 1] = -0.5 * x[1] * f0 * f2;
            dN[3 * a + 2] = 0.25 * q * f0 * p2;
        } else {
            const double f0 = 1 + p0 * x[0], f1 = 1 + p1 * x[1], q = 1 - x[2] * x[2];
            if (N) N[a] = 0.25 * q * f0 * f1;
            dN[3 * a + 0] = 0.25 * q * p0 * f1;
            dN[3 * a + 1] = 0.25 * q * f0 * p1;
            dN[3 * a + 2] = -0.5 * x[2] * f0 * f1;
        }
    }
}

// tet10 (shapeFunc.hpp:178-198): L0 = 1-x-y-z, L1 = x, L2 = y, L3 = z;
// corners 0..3, mid-edge 4:(0,1) 5:(1,2) 6:(2,0) 7:(0,3) 8:(1,3) 9:(2,3)
inline void shape_tet10(const double* x, double* N, double* dN) {
    const double L[4] = {1 - x[0] - x[1] - x[2], x[0], x[1], x[2]};
    // dL_i / dx_p
    const double dL[4][3] = {{-1, -1, -1}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    for (int a = 0; a < 4; a++) {
        if (N) N[a] = L[a] * (2 * L[a] - 1);
        for (int p = 0; p < 3; p++) dN[3 * a + p] = (4 * L[a] - 1) * dL[a][p];
    }
    const int edge[6][2] = {{0, 1}, {1, 2}, {2, 0}, {0, 3}, {1, 3}, {2, 3}};
    for (int m = 0; m < 6; m++) {
        const int i = edge[m][0], j = edge[m][1];
        if (N) N[4 + m] = 4 * L[i] * L[j];
        for (int p = 0; p < 3; p++) dN[3 * (4 + m) + p] = 4 * (dL[i][p] * L[j] + L[i] * dL[j][p]);
    }
}

struct Kind {
    int nodes, dpn;
    bool tet;
    void (*shape)(const double*, double*, double*);
};

inline bool kind_info(int kind, Kind* k) {
    switch (kind) {
        case HEX8_POISSON: *k = {8, 1, false, shape_hex8}; return true;
        case HEX8_ELASTIC: *k = {8, 3, false, shape_hex8}; return true;
        case HEX20_ELASTIC: *k = {20, 3, false, shape_hex20}; return true;
        case TET10_POISSON: *k = {10, 1, true, shape_tet10}; return true;
        case TET10_ELASTIC: *k = {10, 3, true, shape_tet10}; return true;
        default: return false;
    }
}

// Quadrature points (x, weight) in the order of the reference's triple loops.
inline void quadrature(bool tet, uint32_t ngt, std::vector<double>& q) {
    std::vector<double> g(2 * ngt);
    gauss_legendre(ngt, g.data());
    q.clear();
    for (uint32_t i = 0; i < ngt; i++)
        for (uint32_t j = 0; j < ngt; j++)
            for (uint32_t k = 0; k < ngt; k++) {
                const double xi = g[2 * i], eta = g[2 * j], zeta = g[2 * k];
                const double w = g[2 * i + 1] * g[2 * j + 1] * g[2 * k + 1];
                if (!tet) {
                    q.insert(q.end(), {xi, eta, zeta, w});
                } else {
                    // collapsed hexahedron -> unit tetrahedron (ke_matrix.cpp:253-261)
                    const double cm = (1 + xi) * (1 + xi) * (1 + eta) / 64.0 * w;
                    q.insert(q.end(), {(1 + xi) * (1 + eta) * (1 + zeta) / 8.0, (1 + xi) * (1 + eta) * (1 - zeta) / 8.0,
                                       (1 + xi) * (1 - eta) / 4.0, cm});
                }
            }
}

// Physical gradients dNx (nn x 3) and |J| at reference point x.
inline bool gradients(const Kind& K, const double* xe, const double* x, double* N, double* dNx, double* detJ) {
    double dN[3 * 20];
    K.shape(x, N, dN);
    double J[3][3] = {{0}};  // J[i][p] = d x_i / d xi_p
    for (int a = 0; a < K.nodes; a++)
        for (int i = 0; i < 3; i++)
            for (int p = 0; p < 3; p++) J[i][p] += xe[3 * a + i] * dN[3 * a + p];
    const double d = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) -
                     J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
                     J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
    if (!(d > 0.0)) return false;
    double Ji[3][3];  // Ji[p][i] = d xi_p / d x_i
    Ji[0][0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]) / d;
    Ji[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) / d;
    Ji[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) / d;
    Ji[1][0] = (J[1][2] * J[2][0] - J[1][0] * J[2][2]) / d;
    Ji[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) / d;
    Ji[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) / d;
    Ji[2][0] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) / d;
    Ji[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) / d;
    Ji[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) / d;
    for (int a = 0; a < K.nodes; a++)
        for (int i = 0; i < 3; i++)
            dNx[3 * a + i] = dN[3 * a + 0] * Ji[0][i] + dN[3 * a + 1] * Ji[1][i] + dN[3 * a + 2] * Ji[2][i];
    *detJ = d;
    return true;
}

}  // namespace afm_shape
