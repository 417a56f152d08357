// Matvec kernels, ArithF32Sym instances (FP32 products from the symmetric
// inner arena), and the kernels that build that arena (with or without its
// BF16 correction plane) from a split arena.
#define ARITH ArithF32Sym
#define LAUNCH_FN launch_segment_f32sym
#define SMEM_FN segment_smem_f32sym
#define CONFIG_FN configure_kernels_f32sym
#define PATCH_FN launch_patches_f32sym
#define PATCH_SMEM_FN patch_smem_f32sym
#include "afm_mv_launch.inl"

#include <cuda_bf16.h>

namespace afm {

namespace {

// Symmetric part of an element pair from the split arena's hi + lo planes.
__device__ __forceinline__ double sym_entry(const float* h, uint32_t plane, size_t a, size_t b) {
    const double x = (double)h[a] + (double)h[a + plane];
    const double y = (double)h[b] + (double)h[b + plane];
    return 0.5 * (x + y);
}

// Writes entry q of a unit: hi = fl32(x); with a correction plane (lo_plane >
// 0 entries after the start of the unit, in floats), lo = bf16(x - hi).
__device__ __forceinline__ void put_sym(float* unit, uint64_t q, uint32_t lo_plane, double x) {
    const float h = __double2float_rn(x);
    unit[q] = h;
    if (lo_plane) {
        const __nv_bfloat16 l = __float2bfloat16_rn(__double2float_rn(x - (double)h));
        reinterpret_cast<unsigned short*>(unit + lo_plane)[q] = __bfloat16_as_ushort(l);
    }
}

// Patch units (32 element slots, entry (r, c) of slot l at (r n + c) 32 + l in
// each plane) -> packed upper triangle, entry k = j (j + 1) / 2 + i at k 32 + l.
__global__ void __launch_bounds__(256) k_sym_tpe(const unsigned char* __restrict__ src, uint64_t src_unit_bytes,
                                                 uint32_t plane, uint32_t n, uint64_t units, float* __restrict__ dst,
                                                 uint64_t dst_unit_floats, uint32_t lo_plane) {
    const uint32_t np = n * (n + 1) / 2;
    const uint64_t total = units * np * kTpeWidth;
    for (uint64_t x = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; x < total;
         x += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t l = (uint32_t)(x % kTpeWidth);
        const uint64_t rest = x / kTpeWidth;
        const uint32_t k = (uint32_t)(rest % np);
        const uint64_t u = rest / np;
        uint32_t j = 0;
        while ((j + 1) * (j + 2) / 2 <= k) j++;
        const uint32_t i = k - j * (j + 1) / 2;
        const float* h = reinterpret_cast<const float*>(src + u * src_unit_bytes);
        put_sym(dst + u * dst_unit_floats, (uint64_t)k * kTpeWidth + l, lo_plane,
                sym_entry(h, plane, ((size_t)i * n + j) * kTpeWidth + l, ((size_t)j * n + i) * kTpeWidth + l));
    }
}

// Element units (column-major planes, entry (r, c) at c n + r) -> wrapped
// diagonals, D[d][j] = K(j, (j + d) mod n) at d n + j, d = 0 .. n/2.
__global__ void __launch_bounds__(256) k_sym_wpe(const unsigned char* __restrict__ src, uint64_t src_unit_bytes,
                                                 uint32_t plane, uint32_t n, uint64_t units, float* __restrict__ dst,
                                                 uint64_t dst_unit_floats, uint32_t lo_plane) {
    const uint32_t per = (n / 2 + 1) * n;
    const uint64_t total = units * per;
    for (uint64_t x = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; x < total;
         x += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t q = (uint32_t)(x % per);
        const uint64_t u = x / per;
        const uint32_t d = q / n, j = q % n;
        const uint32_t c = j + d >= n ? j + d - n : j + d;
        const float* h = reinterpret_cast<const float*>(src + u * src_unit_bytes);
        put_sym(dst + u * dst_unit_floats, q, lo_plane, sym_entry(h, plane, (size_t)c * n + j, (size_t)j * n + c));
    }
}

}  // namespace

// Fills the symmetric inner arena of segment s (sym must be zeroed: unit
// padding stays zero) from its split-arena units; s.sym_plane > 0 adds the
// BF16 correction plane.
cudaError_t build_sym_segment(const Segment& s, const unsigned char* ke, unsigned char* sym, int sm_count,
                              cudaStream_t st) {
    if (s.units == 0 || s.sym_unit_bytes == 0) return cudaSuccess;
    const bool tpe = s.regime == REG_TPE;
    const uint64_t per = tpe ? (uint64_t)s.n * (s.n + 1) / 2 * kTpeWidth : (uint64_t)(s.n / 2 + 1) * s.n;
    const uint64_t total = per * s.units;
    const uint64_t want = (total + 255) / 256;
    const uint32_t grid = (uint32_t)std::min<uint64_t>(want, (uint64_t)sm_count * 8);
    float* dst = reinterpret_cast<float*>(sym + s.sym_offset);
    const unsigned char* src = ke + s.ke_offset;
    if (tpe)
        k_sym_tpe<<<grid, 256, 0, st>>>(src, s.unit_bytes, s.plane, s.n, s.units, dst, s.sym_unit_bytes / 4,
                                        s.sym_plane);
    else
        k_sym_wpe<<<grid, 256, 0, st>>>(src, s.unit_bytes, s.plane, s.n, s.units, dst, s.sym_unit_bytes / 4,
                                        s.sym_plane);
    return cudaGetLastError();
}

}  // namespace afm
