// CSR SpMV of the assembled operator (afm_assembled.cpp): y = A x in FP64.
// W threads per row (4 to 32: about a quarter of the mean row length, so
// that each thread has four entries to load ahead); each thread sums the
// row's entries j = start + lane, start + lane + W, ... in order, then the W
// partial sums meet in a fixed shuffle tree, so y is
// bit-reproducible. Values and column indices are read once per product
// (streaming loads); x is gathered through the L1/L2 caches.
#include <cuda_runtime.h>
#include <stdint.h>

namespace afm {

namespace {

template <int W>
__global__ void __launch_bounds__(256) k_csr_spmv(const uint64_t* __restrict__ rp, const uint32_t* __restrict__ cols,
                                                  const double* __restrict__ vals, const double* __restrict__ x,
                                                  double* __restrict__ y, uint32_t n_rows) {
    const uint32_t lane = threadIdx.x % W;
    // the W lanes of a row group; the groups of a warp may leave the row loop at different times
    const unsigned mask = W == 32 ? 0xffffffffu : (((1u << W) - 1u) << ((threadIdx.x & 31u) & ~(uint32_t)(W - 1)));
    const uint64_t groups = (uint64_t)gridDim.x * blockDim.x / W;
    for (uint64_t row = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) / W; row < n_rows; row += groups) {
        const uint64_t b = rp[row], e = rp[row + 1];
        double s = 0.0;
        uint64_t j = b + lane;
        // four entries per step: their loads and gathers in flight together, the sum in index order
        for (; j + 3 * W < e; j += 4 * W) {
            uint32_t c[4];
            double a[4], xv[4];
#pragma unroll
            for (int q = 0; q < 4; q++) c[q] = __ldcs(cols + j + q * W), a[q] = __ldcs(vals + j + q * W);
#pragma unroll
            for (int q = 0; q < 4; q++) xv[q] = __ldg(x + c[q]);
#pragma unroll
            for (int q = 0; q < 4; q++) s = __fma_rn(a[q], xv[q], s);
        }
        for (; j < e; j += W) s = __fma_rn(__ldcs(vals + j), __ldg(x + __ldcs(cols + j)), s);
#pragma unroll
        for (int o = W / 2; o > 0; o >>= 1) s += __shfl_down_sync(mask, s, o, W);
        if (lane == 0) y[row] = s;
    }
}

}  // namespace

cudaError_t launch_csr_spmv(const uint64_t* rp, const uint32_t* cols, const double* vals, const double* x, double* y,
                            uint32_t n_rows, int width, int sm_count, cudaStream_t st) {
    if (n_rows == 0) return cudaSuccess;
    const uint64_t threads = (uint64_t)n_rows * width;
    const uint64_t want = (threads + 255) / 256;
    const uint32_t grid = (uint32_t)(want < (uint64_t)sm_count * 8 ? want : (uint64_t)sm_count * 8);
    switch (width) {
        case 4: k_csr_spmv<4><<<grid, 256, 0, st>>>(rp, cols, vals, x, y, n_rows); break;
        case 8: k_csr_spmv<8><<<grid, 256, 0, st>>>(rp, cols, vals, x, y, n_rows); break;
        case 16: k_csr_spmv<16><<<grid, 256, 0, st>>>(rp, cols, vals, x, y, n_rows); break;
        default: k_csr_spmv<32><<<grid, 256, 0, st>>>(rp, cols, vals, x, y, n_rows); break;
    }
    return cudaGetLastError();
}

}  // namespace afm
