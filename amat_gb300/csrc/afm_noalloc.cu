// Allocation-free Jacobi-PCG (afm_solve_cg_device_noalloc in include/afm.h).
//
// Some callers must not allocate device memory once they are running: an
// application whose allocator has already reserved the GPU's memory (a
// framework's caching allocator sized to the device, a fixed budget under
// MPS), or a loop that must not stall, since cudaMalloc and cudaFree can
// synchronise the device. For them this solve takes its CG work vectors and
// reduction partials from one array compiled into the library,
// g_cg_scratch, instead of from the operator's cudaMalloc'd work space. The
// operator's own buffers (element matrices, map, diagonal) are allocated by
// afm_finalize beforehand, as for every other entry point.
//
// The array holds AFM_NOALLOC_MAX_DOFS DoFs; larger operators are rejected.
// It lives on every GPU that loads the library until the process exits.
// Every call on a device uses the same array, so calls whose work overlaps on
// the GPU (two operators' streams, two host threads) race; serialise them.
#include <cuda_runtime.h>
#include <stdint.h>

#include <chrono>
#include <cmath>

#include "afm_internal.hpp"
#include "afm_solver.hpp"

namespace {

constexpr size_t kVecs = 5;  // r, z, p, q, 1/diag
constexpr size_t kScratchDoubles = kVecs * (size_t)AFM_NOALLOC_MAX_DOFS + afm::kScalarSlots + afm::kPartialSlots;

static __device__ __align__(256) double g_cg_scratch[kScratchDoubles];

// Device address of g_cg_scratch on the current device. The symbol's
// host-side name is not a device address. The lookup is repeated on every call
// (it allocates nothing), so a context torn down and created again
// (cudaDeviceReset) never leaves a stale address behind; the first lookup on a
// device loads the module that holds the array.
int scratch_address(double** out) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_cg_scratch);
    if (e != cudaSuccess || !p)
        return afm::set_error(AFM_ERR_CUDA, "cudaGetSymbolAddress(g_cg_scratch): %s", cudaGetErrorString(e));
    *out = static_cast<double*>(p);
    return AFM_SUCCESS;
}

#define NA_CUDA(call)                                                                          \
    do {                                                                                       \
        cudaError_t e_ = (call);                                                               \
        if (e_ != cudaSuccess)                                                                 \
            return afm::set_error(AFM_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_));     \
    } while (0)

}  // namespace

extern "C" int afm_solve_cg_device_noalloc(afm_operator* op, const double* d_b, double* d_x, double rtol,
                                           double atol, int maxit, int norm_type, afm_solve_stats* stats) {
    using namespace afm;
    if (!op) return set_error(AFM_ERR_INVALID_ARG, "null operator");
    if (!op->finalized) return set_error(AFM_ERR_STATE, "solve before finalize");
    if (op->precision == AFM_PREC_FP32) return set_error(AFM_ERR_STATE, "FP32 operator");
    if (!d_b || !d_x) return set_error(AFM_ERR_INVALID_ARG, "null vector");
    if (norm_type != AFM_CG_NORM_UNPRECONDITIONED && norm_type != AFM_CG_NORM_PRECONDITIONED)
        return set_error(AFM_ERR_INVALID_ARG, "norm type %d", norm_type);
    if (op->n_dofs > AFM_NOALLOC_MAX_DOFS)
        return set_error(AFM_ERR_INVALID_ARG, "%u DoFs exceed the allocation-free limit of %u", op->n_dofs,
                         (unsigned)AFM_NOALLOC_MAX_DOFS);
    int prev = -1;
    cudaGetDevice(&prev);
    if (prev != op->device) NA_CUDA(cudaSetDevice(op->device));
    struct Restore {
        int dev;
        ~Restore() {
            if (dev >= 0) cudaSetDevice(dev);
        }
    } restore{prev != op->device ? prev : -1};

    double* base = nullptr;
    int s = scratch_address(&base);
    if (s) return s;
    const size_t n = op->n_dofs, N = AFM_NOALLOC_MAX_DOFS;
    double* r = base;
    double* z = base + N;
    double* p = base + 2 * N;
    double* q = base + 3 * N;
    double* dinv = base + 4 * N;
    double* sc = base + kVecs * N;
    double* part = sc + kScalarSlots;
    cudaStream_t st = op->stream;
    double* h = op->h_scalars;  // pinned, allocated by afm_create
    // stats->seconds: host wall time of the iterations (the allocating solve reports device time from
    // events; here each iteration's host round trip is included)
    const auto t0 = std::chrono::steady_clock::now();

    // the array keeps the previous call's contents: start the solver state from zero
    NA_CUDA(cudaMemsetAsync(sc, 0, sizeof(double) * (kScalarSlots + kPartialSlots), st));
    NA_CUDA(launch_invert(dinv, op->d_diag, n, st));
    s = afm_matmult_bc_device(op, q, d_x, st);
    if (s) return s;
    NA_CUDA(launch_cg_init(d_b, q, dinv, r, z, p, n, sc, part, st));
    NA_CUDA(cudaMemcpyAsync(h, sc, sizeof(double) * kScalarSlots, cudaMemcpyDeviceToHost, st));
    NA_CUDA(cudaStreamSynchronize(st));
    const double bn = std::sqrt(h[S_BB]);
    const double ref = (norm_type == AFM_CG_NORM_UNPRECONDITIONED) ? bn : std::sqrt(h[S_DB]);
    const double tol = std::max(rtol * ref, atol);
    int it = 0, status = AFM_ERR_MAXIT;
    double rn = 0.0;
    for (;;) {
        rn = std::sqrt(norm_type == AFM_CG_NORM_UNPRECONDITIONED ? h[S_RR] : h[S_ZZ]);
        if (h[S_FLAG] != 0.0 || std::isnan(rn)) {
            status = AFM_ERR_BREAKDOWN;
            break;
        }
        if (rn <= tol) {
            status = AFM_SUCCESS;
            break;
        }
        if (it >= maxit) break;
        s = afm_matmult_bc_device(op, q, p, st);
        if (s) return s;
        NA_CUDA(launch_cg_alpha(p, q, n, sc, part, st));
        NA_CUDA(launch_cg_update(d_x, r, z, p, q, dinv, n, sc, part, st));
        NA_CUDA(cudaMemcpyAsync(h, sc, sizeof(double) * kScalarSlots, cudaMemcpyDeviceToHost, st));
        NA_CUDA(cudaStreamSynchronize(st));
        it++;
    }
    const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    // true residual ||b - A x|| in FP64, reduced on the device into sc[S_PQ]
    s = afm_matmult_bc_device(op, q, d_x, st);
    if (s) return s;
    NA_CUDA(launch_axpby(q, d_b, 1.0, -1.0, n, st));
    NA_CUDA(launch_norm2(q, n, sc, part, st));
    NA_CUDA(cudaMemcpyAsync(h, sc, sizeof(double) * kScalarSlots, cudaMemcpyDeviceToHost, st));
    NA_CUDA(cudaStreamSynchronize(st));
    const double rr = h[S_PQ];
    s = afm_synchronize(op);
    if (s) return s;
    if (stats) {
        stats->iterations = it;
        stats->status = status;
        stats->rel_residual = bn > 0 ? std::sqrt(rr) / bn : std::sqrt(rr);
        stats->residual_norm = rn;
        stats->seconds = secs;
        stats->refinements = 0;
    }
    if (status != AFM_SUCCESS)
        return set_error(status, status == AFM_ERR_MAXIT ? "CG reached maxit=%d" : "CG breakdown after %d iterations",
                         it);
    return set_error(AFM_SUCCESS, "");
}
