// Matrix-free product (method 2, par::aMatFree with MATFREE_TYPE::FREE,
// include/aMatFree.hpp:2241-2745): no element matrix is stored; every product
// integrates each element's stiffness action from its node coordinates,
//   v_e = sum_q w_q |J_q| B_q^T D B_q u_e,
// which is Ke u_e of the reference's element kernels (the callback
// m_eleMatFunc computes Ke from xe, include/aMat.hpp:104-116, then multiplies)
// up to the order of the sums. It trades the Ke bytes for arithmetic: in FP32
// it needs ~0.5 KB per hex20 element instead of 7-29 KB of stored Ke.
//
// G = 8, 16 or 32 lanes per element (32 / G elements per warp), elements of
// one colour per launch (they share no DoF, so v += v_e is a reduction at L2
// with no read of the old v, and bit-reproducible). Phase 1, lane =
// quadrature point: Jacobian J = sum_a xe_a (x) dN_a, its inverse, the
// gradient of u (Poisson: grad u; elasticity: H = du/dx), and the weighted
// flux / stress w |J| (lam tr(H) I + mu (H + H^T)), kept in shared memory with
// J^-1. Phase 2, lane = node: v_a = sum_q (J_q^-T dN_a(q)) . flux_q.
#include <cuda_runtime.h>
#include <stdint.h>

#include "afm_internal.hpp"

namespace afm {

namespace {

template <int KIND>
struct FreeKind;
// nodes, DoFs per node; the reference tables follow afm_shape.hpp
template <>
struct FreeKind<0> { static constexpr int NODES = 8, DPN = 1; };
template <>
struct FreeKind<1> { static constexpr int NODES = 8, DPN = 3; };
template <>
struct FreeKind<2> { static constexpr int NODES = 20, DPN = 3; };
template <>
struct FreeKind<3> { static constexpr int NODES = 10, DPN = 1; };
template <>
struct FreeKind<4> { static constexpr int NODES = 10, DPN = 3; };

constexpr int kFreeWarps = 8;
constexpr int kFreeMaxQ = 27;

// v[i] += x at L2, no load and no wait (round to nearest; the f32 form
// flushes subnormal values to zero). Elements of a launch share no DoF and
// launches are ordered, so each entry gets one add per colour, in colour order.
__device__ __forceinline__ void red_add(float* p, float x) {
    asm volatile("red.global.add.f32 [%0], %1;" ::"l"(p), "f"(x) : "memory");
}
__device__ __forceinline__ void red_add(double* p, double x) {
    asm volatile("red.global.add.f64 [%0], %1;" ::"l"(p), "d"(x) : "memory");
}

// G lanes per element (8, 16 or 32: at least the quadrature points and the
// nodes), 32 / G elements per warp side by side.
template <int KIND, typename T, int G>
__global__ void __launch_bounds__(kFreeWarps * 32) k_free(FreeArgs a) {
    constexpr int NN = FreeKind<KIND>::NODES, DPN = FreeKind<KIND>::DPN, N = NN * DPN;
    constexpr int QS = 9 + (DPN == 3 ? 6 : 3);  // per quadrature point: J^-1, weighted stress / flux
    constexpr int EPW = 32 / G, SLOTS = kFreeWarps * EPW, QM = G < kFreeMaxQ ? G : kFreeMaxQ;
    static_assert(NN <= G, "a lane per node");
    __shared__ T ref[QM * (NN * 3 + 1)];  // dN of every node at every point, then the weights
    __shared__ T ue[SLOTS][N];
    __shared__ T xs[SLOTS][NN * 3];
    __shared__ T qb[SLOTS][QM][QS];
    const int nq = (int)a.nq;
    const T* gref = static_cast<const T*>(a.ref);
    for (int i = threadIdx.x; i < nq * (NN * 3 + 1); i += blockDim.x) ref[i] = gref[i];
    __syncthreads();
    const T* dNref = ref;             // [q][a][p]
    const T* wq = ref + nq * NN * 3;  // [q]
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int slot = warp * EPW + lane / G, sl = lane % G;
    const T* __restrict__ u = static_cast<const T*>(a.u);
    T* __restrict__ v = static_cast<T*>(a.v);
    const T* __restrict__ xe = static_cast<const T*>(a.xe);
    const T lam = (T)a.lam, mu = (T)a.mu;
    const uint32_t stride = gridDim.x * SLOTS;
    // every lane of the warp runs the same number of rounds (the __syncwarp calls); a slot past the end idles
    // Gather pipeline: the element of the next round has its u entries and coordinates loaded (and the one
    // after it its map) while the current element is integrated, so a round waits on no load of its own.
    constexpr int CN = (N + G - 1) / G, CX = (NN * 3 + G - 1) / G;
    uint32_t mc[CN], mn[CN];  // maps of the next round and of the one after
    T uc[CN], xc[CX];         // u entries and coordinates of the next round
    auto load_map = [&](uint32_t base_r, uint32_t* out) {
        const uint32_t el_r = base_r + lane / G;
#pragma unroll
        for (int k = 0; k < CN; k++) {
            const int i = sl + k * G;
            out[k] = (el_r < a.count && i < N) ? a.map[(size_t)(a.first + el_r) * N + i] : 0u;
        }
    };
    auto load_ux = [&](uint32_t base_r, const uint32_t* mp) {
        const uint32_t el_r = base_r + lane / G;
        const bool ok = el_r < a.count;
#pragma unroll
        for (int k = 0; k < CN; k++) {
            const int i = sl + k * G;
            T x = (ok && i < N) ? u[mp[k] & kDofMask] : T(0);
            if (a.bc_mode && (mp[k] & kBcFlag)) x = T(0);
            uc[k] = x;
        }
#pragma unroll
        for (int k = 0; k < CX; k++) {
            const int i = sl + k * G;
            xc[k] = (ok && i < NN * 3) ? xe[(size_t)(a.first + el_r) * NN * 3 + i] : T(0);
        }
    };
    uint32_t base = blockIdx.x * SLOTS + warp * EPW;
    load_map(base, mc);
    load_ux(base, mc);
    load_map(base + stride, mn);
    for (; base < a.count; base += stride) {
        const uint32_t el = base + lane / G;
        const bool live = el < a.count;
        const uint32_t e = a.first + (live ? el : 0u);
        const uint32_t* m = a.map + (size_t)e * N;
        if (live) {
#pragma unroll
            for (int k = 0; k < CN; k++)
                if (sl + k * G < N) ue[slot][sl + k * G] = uc[k];
#pragma unroll
            for (int k = 0; k < CX; k++)
                if (sl + k * G < NN * 3) xs[slot][sl + k * G] = xc[k];
        }
        __syncwarp();
        // next round: its u and coordinates from the map loaded a round ago; the map of the round after
#pragma unroll
        for (int k = 0; k < CN; k++) mc[k] = mn[k];
        load_ux(base + stride, mc);
        load_map(base + 2 * stride, mn);
        if (live && sl < nq) {
            const int q = sl;
            const T* dN = dNref + q * NN * 3;
            T J[3][3] = {};  // J[i][p] = d x_i / d xi_p
#pragma unroll
            for (int b = 0; b < NN; b++)
#pragma unroll
                for (int i = 0; i < 3; i++)
#pragma unroll
                    for (int p = 0; p < 3; p++) J[i][p] += xs[slot][3 * b + i] * dN[3 * b + p];
            const T det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) -
                          J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
                          J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
            const T id = T(1) / det;
            T Ji[3][3];  // Ji[p][i] = d xi_p / d x_i
            Ji[0][0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]) * id;
            Ji[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) * id;
            Ji[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * id;
            Ji[1][0] = (J[1][2] * J[2][0] - J[1][0] * J[2][2]) * id;
            Ji[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * id;
            Ji[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) * id;
            Ji[2][0] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) * id;
            Ji[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) * id;
            Ji[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * id;
            T* o = qb[slot][q];
#pragma unroll
            for (int k = 0; k < 9; k++) o[k] = Ji[k / 3][k % 3];
            const T w = wq[q] * det;
            if constexpr (DPN == 1) {
                T gu[3] = {};
#pragma unroll
                for (int b = 0; b < NN; b++) {
                    const T ub = ue[slot][b];
#pragma unroll
                    for (int i = 0; i < 3; i++)
                        gu[i] += ub * (dN[3 * b] * Ji[0][i] + dN[3 * b + 1] * Ji[1][i] + dN[3 * b + 2] * Ji[2][i]);
                }
#pragma unroll
                for (int i = 0; i < 3; i++) o[9 + i] = w * gu[i];
            } else {
                T H[3][3] = {};  // H[i][j] = d u_i / d x_j
#pragma unroll
                for (int b = 0; b < NN; b++) {
                    T g[3];
#pragma unroll
                    for (int j = 0; j < 3; j++)
                        g[j] = dN[3 * b] * Ji[0][j] + dN[3 * b + 1] * Ji[1][j] + dN[3 * b + 2] * Ji[2][j];
#pragma unroll
                    for (int i = 0; i < 3; i++)
#pragma unroll
                        for (int j = 0; j < 3; j++) H[i][j] += ue[slot][3 * b + i] * g[j];
                }
                const T tr = lam * (H[0][0] + H[1][1] + H[2][2]);
                o[9] = w * (tr + mu * (H[0][0] + H[0][0]));   // s_xx
                o[10] = w * (tr + mu * (H[1][1] + H[1][1]));  // s_yy
                o[11] = w * (tr + mu * (H[2][2] + H[2][2]));  // s_zz
                o[12] = w * (mu * (H[0][1] + H[1][0]));       // s_xy
                o[13] = w * (mu * (H[1][2] + H[2][1]));       // s_yz
                o[14] = w * (mu * (H[0][2] + H[2][0]));       // s_xz
            }
        }
        __syncwarp();
        if (live && sl < NN) {
            const int b = sl;
            T acc[DPN] = {};
            for (int q = 0; q < nq; q++) {
                const T* o = qb[slot][q];
                const T* dN = dNref + (q * NN + b) * 3;
                T g[3];
#pragma unroll
                for (int i = 0; i < 3; i++) g[i] = dN[0] * o[i] + dN[1] * o[3 + i] + dN[2] * o[6 + i];
                if constexpr (DPN == 1) {
                    acc[0] += g[0] * o[9] + g[1] * o[10] + g[2] * o[11];
                } else {
                    acc[0] += g[0] * o[9] + g[1] * o[12] + g[2] * o[14];
                    acc[1] += g[0] * o[12] + g[1] * o[10] + g[2] * o[13];
                    acc[2] += g[0] * o[14] + g[1] * o[13] + g[2] * o[11];
                }
            }
#pragma unroll
            for (int i = 0; i < DPN; i++) red_add(v + (m[DPN * b + i] & kDofMask), acc[i]);
        }
        __syncwarp();
    }
}

template <int KIND, typename T>
void* free_kernel_g(int g) {
    constexpr int NN = FreeKind<KIND>::NODES;
    if constexpr (NN <= 8) {
        if (g == 8) return (void*)k_free<KIND, T, 8>;
    }
    if constexpr (NN <= 16) {
        if (g == 16) return (void*)k_free<KIND, T, 16>;
    }
    return g == 32 ? (void*)k_free<KIND, T, 32> : nullptr;
}

template <typename T>
void* free_kernel(int kind, int g) {
    switch (kind) {
        case 0: return free_kernel_g<0, T>(g);
        case 1: return free_kernel_g<1, T>(g);
        case 2: return free_kernel_g<2, T>(g);
        case 3: return free_kernel_g<3, T>(g);
        case 4: return free_kernel_g<4, T>(g);
        default: return nullptr;
    }
}

}  // namespace

cudaError_t launch_free(int kind, bool f32, const FreeArgs& a, int sm_count, cudaStream_t st) {
    if (a.count == 0) return cudaSuccess;
    if (a.nq == 0 || a.nq > (uint32_t)kFreeMaxQ) return cudaErrorInvalidValue;
    static const int nodes[5] = {8, 8, 20, 10, 10};
    if (kind < 0 || kind > 4) return cudaErrorInvalidValue;
    const uint32_t need = a.nq > (uint32_t)nodes[kind] ? a.nq : (uint32_t)nodes[kind];
    const int g = need <= 8 ? 8 : need <= 16 ? 16 : 32;
    void* fn = f32 ? free_kernel<float>(kind, g) : free_kernel<double>(kind, g);
    if (!fn) return cudaErrorInvalidValue;
    const uint32_t slots = kFreeWarps * (32 / g);
    const uint32_t want = (a.count + slots - 1) / slots;
    const uint32_t grid = want < (uint32_t)sm_count * 4 ? want : (uint32_t)sm_count * 4;
    FreeArgs args = a;
    void* params[] = {&args};
    return cudaLaunchKernel(fn, dim3(grid), dim3(kFreeWarps * 32), params, 0, st);
}

}  // namespace afm
