// Batched FP32 product V = K U on the tensor cores (tcgen05, kind::tf32).
//
// For a group of E = 128 / R elements of one colour (R right-hand sides, R in
// {32, 64, 128}), one accumulator D (128 TMEM lanes x N columns, FP32) holds
//   D[e R + j][e' n + r] = sum_c U[dof(e, c)][j] Ke_e'[r][c],
// i.e. the M = 128 rows stack the E elements' right-hand sides and the N = E n
// (rounded up to 16) columns the E elements' rows; the diagonal blocks e = e'
// are V_e^T, the rest is discarded (the tensor cores have throughput to spare:
// the product is bound by gathering U and updating V). Operands are staged in
// shared memory in the canonical K-major layout without swizzle (8-row x 16-byte
// core matrices) by the CUDA cores:
//   A (128 x Kp): A[e R + j][c] = U[dof(e, c)][j]      (0 for c >= n, and for
//                 constrained columns of a MatMult_mf product)
//   B (N x Kp):   B[e n + r][c] = Ke_e[r][c]            (0 in the padding)
// with Kp = n rounded up to 8 (one tf32 MMA is K = 8). FP32 accuracy from the
// 10-bit-mantissa tf32 inputs: each operand x is split into hi = x with its low
// 13 mantissa bits cleared and lo = x - hi (exact), and D accumulates
// A_lo B_hi + A_hi B_lo first and A_hi B_hi last (3xTF32: the dropped A_lo B_lo
// and the truncation of lo leave ~2^-21 of |K||u|).
//
// One thread issues the 3 Kp / 8 MMAs and commits them to an mbarrier; the
// epilogue warp w reads TMEM lanes 32 w .. 32 w + 31 (tcgen05.ld 32x32b): lane
// = one (element, right-hand side), registers = that element's n rows, and adds
// them into V rows (colour-exclusive, so a plain read-modify-write; lanes of a
// warp touch consecutive columns of a V row). 128 threads per CTA, several CTAs
// per SM overlap each other's gathers, MMAs and updates.
//
// Every wait is bounded; TMEM is always released before the CTA exits.
#include <mutex>
#include <vector>

#include "afm_matvec.cuh"

namespace afm {

namespace {

constexpr int kTcThreads = 128;

// Byte offset of element (row, k) of a K-major operand with kcores = Kp / 4
// core matrices per 8-row group: core matrices adjacent in K are 128 bytes
// apart (the leading byte offset), 8-row groups kcores * 128 bytes apart (the
// stride byte offset).
__host__ __device__ __forceinline__ uint32_t tc_off(uint32_t row, uint32_t k, uint32_t kcores) {
    return ((row >> 3) * kcores + (k >> 2)) * 128u + (row & 7u) * 16u + (k & 3u) * 4u;
}

// Shared-memory matrix descriptor of tcgen05 (no swizzle): start address,
// leading byte offset (K direction), stride byte offset (8-row groups), all
// in 16-byte units; bits 46-47 = 1 (the descriptor version of sm_100 family).
__device__ __forceinline__ uint64_t tc_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr >> 4) & 0x3fffu) | ((uint64_t)((lbo >> 4) & 0x3fffu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3fffu) << 32) | (1ull << 46);
}

// Instruction descriptor of kind::tf32: D in F32 (bits 4-5 = 1), A and B tf32
// (bits 7-9, 10-12 = 2), both K-major (bits 15, 16 = 0), N >> 3 at bits
// 17-22, M >> 4 at bits 24-28.
__host__ __device__ constexpr uint32_t tc_idesc(uint32_t m, uint32_t n) {
    return (1u << 4) | (2u << 7) | (2u << 10) | ((n >> 3) << 17) | ((m >> 4) << 24);
}

__device__ __forceinline__ void tc_mma(uint32_t tmem, uint64_t ad, uint64_t bd, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
        "l"(ad), "l"(bd), "r"(idesc), "r"(acc)
        : "memory");
}

__device__ __forceinline__ float tf32_hi(float x) { return __uint_as_float(__float_as_uint(x) & 0xffffe000u); }

// 8 consecutive TMEM columns of this warp's 32 lanes
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float* v) {
    uint32_t r[8];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                 : "r"(taddr));
#pragma unroll
    for (int i = 0; i < 8; i++) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void tmem_ld4(uint32_t taddr, float* v) {
    uint32_t r[4];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0,%1,%2,%3}, [%4];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(taddr));
#pragma unroll
    for (int i = 0; i < 4; i++) v[i] = __uint_as_float(r[i]);
}

}  // namespace

// Geometry of one launch (host-computed).
struct TcGeom {
    uint32_t R;        // right-hand sides (32, 64 or 128)
    uint32_t E;        // elements per group = 128 / R
    uint32_t Kp;       // n rounded up to 8
    uint32_t N;        // MMA N: E n rounded up to 16
    uint32_t cols;     // TMEM columns allocated (power of two >= max(32, N))
    uint32_t a_bytes;  // one plane of A: 128 Kp 4
    uint32_t b_bytes;  // one plane of B: N Kp 4
    uint32_t smem;     // dynamic shared memory
};

template <int NT>
__global__ void __launch_bounds__(kTcThreads, (NT != 0 && NT <= 32) ? 4 : 1) afm_batched_tc_kernel(BatchArgs a, TcGeom G, uint32_t n_rt) {
    const uint32_t n = NT ? NT : n_rt;
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned char* sA = smem;                           // hi plane, then lo plane
    unsigned char* sB = smem + 2 * G.a_bytes;           // hi plane, then lo plane
    const uint32_t mapw = (G.E * n + 1) & ~1u;
    uint32_t* mp0 = reinterpret_cast<uint32_t*>(sB + 2 * G.b_bytes);  // 2 x (E x n) map entries (double buffer)
    uint64_t* bar = reinterpret_cast<uint64_t*>(mp0 + 2 * mapw);
    uint32_t* tslot = reinterpret_cast<uint32_t*>(bar + 1);
    const uint32_t t = threadIdx.x, warp = t >> 5, lane = t & 31;
    const uint32_t kc = G.Kp / 4;
    const float* __restrict__ U = static_cast<const float*>(a.u);
    float* __restrict__ V = static_cast<float*>(a.v);
    const uint32_t groups = (a.count + G.E - 1) / G.E;

    if (t == 0) {
        mbar_init(bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(tslot)),
                     "r"(G.cols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tslot;
    wait_prior_grid();

    // epilogue role of this thread: row m = element em, right-hand side j
    const uint32_t m = t, em = m / G.R, j = m % G.R;
    const uint32_t idesc = tc_idesc(128, G.N);
    bool failed = false;
    uint32_t phase = 0;
    // map entry i (< E n <= 256) of the group starting at element e0 (0 past the segment's end)
    auto map_entry = [&](uint32_t e0, uint32_t i) -> uint32_t {
        const uint32_t e = e0 + i / n;
        return (i < G.E * n && e < a.count) ? __ldg(a.map + (size_t)e * n + i % n) : 0u;
    };
    if (blockIdx.x < groups) {
        const uint32_t e0 = blockIdx.x * G.E;
        if (t < mapw) mp0[t] = map_entry(e0, t);
        if (t + kTcThreads < mapw) mp0[t + kTcThreads] = map_entry(e0, t + kTcThreads);
    }
    __syncthreads();
    // A is gathered KA columns at a time, every load of a batch in flight before any is used
    constexpr uint32_t KA = (NT != 0 && NT <= 32) ? ((NT + 7) / 8) * 8 : 8;
    for (uint32_t grp = blockIdx.x, it = 0; grp < groups && !failed; grp += gridDim.x, phase ^= 1u, it++) {
        const uint32_t e0 = grp * G.E;
        uint32_t* mp = mp0 + (it & 1u) * mapw;
        uint32_t* mp_next = mp0 + ((it + 1u) & 1u) * mapw;
        const uint32_t e_next = (grp + gridDim.x) * G.E;
        uint32_t nm0 = 0, nm1 = 0;
        bool next_loaded = false;
        // A: this thread's row m, every column c (lanes read consecutive j of one U row), then 16-byte
        // stores of (hi, lo) into the core-matrix rows
        {
            const bool valid = e0 + em < a.count;
            for (uint32_t c0 = 0; c0 < G.Kp; c0 += KA) {
                float x[KA];
#pragma unroll
                for (uint32_t q = 0; q < KA; q++) {
                    const uint32_t c = c0 + q;
                    x[q] = 0.0f;
                    if (valid && c < n) {
                        const uint32_t d = mp[em * n + c];
                        const uint32_t row = d & kDofMask;
                        if (row >= a.n_dofs)
                            report_bad(a.err, 11, row, c, e0 + em);
                        else if (!(a.bc_mode && (d & kBcFlag)))
                            x[q] = __ldg(U + (size_t)row * a.ld + j);
                    }
                }
                if (!next_loaded) {
                    // the next group's map, in flight with this batch (stored after the conversion)
                    next_loaded = true;
                    if (grp + gridDim.x < groups) {
                        nm0 = map_entry(e_next, t);
                        nm1 = map_entry(e_next, t + kTcThreads);
                    }
                }
#pragma unroll
                for (uint32_t h4 = 0; h4 < KA / 4; h4++) {
                    float4 hi, lo;
                    hi.x = tf32_hi(x[4 * h4]), hi.y = tf32_hi(x[4 * h4 + 1]);
                    hi.z = tf32_hi(x[4 * h4 + 2]), hi.w = tf32_hi(x[4 * h4 + 3]);
                    lo.x = x[4 * h4] - hi.x, lo.y = x[4 * h4 + 1] - hi.y;
                    lo.z = x[4 * h4 + 2] - hi.z, lo.w = x[4 * h4 + 3] - hi.w;
                    const uint32_t off = tc_off(m, c0 + 4 * h4, kc);
                    *reinterpret_cast<float4*>(sA + off) = hi;
                    *reinterpret_cast<float4*>(sA + G.a_bytes + off) = lo;
                }
            }
        }
        // B: Ke of the group's elements (column-major in the arena: entry (r, c) at c n + r); thread
        // item = (row, 4 consecutive c), consecutive threads on consecutive rows
        {
            const uint32_t items = G.N * (G.Kp / 4);
            for (uint32_t i0 = 0; i0 < items; i0 += 4 * kTcThreads) {
                float x[4][4];
#pragma unroll
                for (int b = 0; b < 4; b++) {
                    const uint32_t i = i0 + b * kTcThreads + t;
                    const uint32_t row = i % G.N, c4 = (i / G.N) * 4;
                    const uint32_t e = row / n, r = row % n;
                    const bool ok = i < items && row < G.E * n && e0 + e < a.count;
                    const float* kp = reinterpret_cast<const float*>(a.ke + (size_t)(e0 + e) * a.unit_bytes);
#pragma unroll
                    for (int q = 0; q < 4; q++)
                        x[b][q] = (ok && c4 + q < n) ? __ldg(kp + (size_t)(c4 + q) * n + r) : 0.0f;
                }
#pragma unroll
                for (int b = 0; b < 4; b++) {
                    const uint32_t i = i0 + b * kTcThreads + t;
                    if (i >= items) continue;
                    const uint32_t row = i % G.N, c4 = (i / G.N) * 4;
                    float4 hi, lo;
                    hi.x = tf32_hi(x[b][0]), hi.y = tf32_hi(x[b][1]), hi.z = tf32_hi(x[b][2]), hi.w = tf32_hi(x[b][3]);
                    lo.x = x[b][0] - hi.x, lo.y = x[b][1] - hi.y, lo.z = x[b][2] - hi.z, lo.w = x[b][3] - hi.w;
                    const uint32_t off = tc_off(row, c4, kc);
                    *reinterpret_cast<float4*>(sB + off) = hi;
                    *reinterpret_cast<float4*>(sB + G.b_bytes + off) = lo;
                }
            }
        }
        // the next group's map into the other buffer (the epilogue below reads this group's)
        if (t < mapw) mp_next[t] = nm0;
        if (t + kTcThreads < mapw) mp_next[t + kTcThreads] = nm1;
        // generic-proxy stores -> async-proxy reads of the tensor cores
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncthreads();
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        if (t == 0) {
            const uint32_t a0 = smem_addr(sA), b0 = smem_addr(sB);
            const uint32_t sbo = kc * 128u;
            uint32_t acc = 0;
            // small cross terms first, the leading product last
            for (uint32_t pass = 0; pass < 3; pass++) {
                const uint32_t ap = pass == 1 ? G.a_bytes : 0u;  // pass 0: hi x lo, 1: lo x hi, 2: hi x hi
                const uint32_t bp = pass == 0 ? G.b_bytes : 0u;
                for (uint32_t ks = 0; ks < G.Kp / 8; ks++) {
                    tc_mma(tmem, tc_desc(a0 + ap + ks * 256u, 128u, sbo), tc_desc(b0 + bp + ks * 256u, 128u, sbo),
                           idesc, acc);
                    acc = 1;
                }
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                             smem_addr(bar))
                         : "memory");
        }
        // all threads: the MMAs' completion (bounded)
        if (!mbar_wait(bar, phase, a.wait_ns)) {
            atomicOr(a.err, kErrTimeout);
            failed = true;
        }
        failed = __syncthreads_or(failed);
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        if (!failed && e0 + em < a.count) {
            // this warp's lanes, the columns of element em
            const uint32_t tl = tmem + ((32u * warp) << 16) + em * n;
            float vals[NT ? ((NT + 7) / 8) * 8 : 96];
            const uint32_t n8 = n & ~7u;
            for (uint32_t c = 0; c < n8; c += 8) tmem_ld8(tl + c, vals + c);
            if (n & 7u) tmem_ld4(tl + n8, vals + n8);
            if ((n & 7u) > 4u) tmem_ld4(tl + n8 + 4, vals + n8 + 4);
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            // every old V entry in flight before the first update
            constexpr uint32_t NV = NT ? ((NT + 7) / 8) * 8 : 96;
            float old[NV];
#pragma unroll
            for (uint32_t r = 0; r < NV; r++) {
                old[r] = 0.0f;
                if (r < n) {
                    const uint32_t d = mp[em * n + r] & kDofMask;
                    if (d < a.n_dofs) old[r] = V[(size_t)d * a.ld + j];
                }
            }
#pragma unroll
            for (uint32_t r = 0; r < NV; r++) {
                if (r < n) {
                    const uint32_t d = mp[em * n + r] & kDofMask;
                    if (d < a.n_dofs)
                        V[(size_t)d * a.ld + j] = old[r] + vals[r];
                    else
                        report_bad(a.err, 12, d, r, e0 + em);
                }
            }
        }
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncthreads();  // smem operands and TMEM are reused by the next group
    }
    allow_dependent_launch();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(G.cols));
}

}  // namespace afm

namespace afm {

namespace {

void* tc_kernel_for(uint32_t n) {
    switch (n) {
        case 24: return (void*)afm_batched_tc_kernel<24>;
        case 30: return (void*)afm_batched_tc_kernel<30>;
        case 60: return (void*)afm_batched_tc_kernel<60>;
        default: return (void*)afm_batched_tc_kernel<0>;
    }
}

// Once per kernel and device: the largest dynamic shared memory, the whole
// carveout for shared memory, and the kernel's registers per thread (host
// calls kept out of every launch).
cudaError_t tc_configure(void* fn, int* regs) {
    struct Entry {
        void* fn;
        int device, regs;
    };
    static std::mutex mu;
    static std::vector<Entry> cache;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lk(mu);
    for (const Entry& c : cache)
        if (c.fn == fn && c.device == dev) {
            *regs = c.regs;
            return cudaSuccess;
        }
    e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemBudget);
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    if (e != cudaSuccess) return e;
    cudaFuncAttributes fa;
    e = cudaFuncGetAttributes(&fa, fn);
    if (e != cudaSuccess) return e;
    *regs = fa.numRegs > 0 ? fa.numRegs : 255;
    cache.push_back({fn, dev, *regs});
    return cudaSuccess;
}

bool tc_geom(uint32_t n, uint32_t nrhs, TcGeom* G) {
    if (nrhs != 32 && nrhs != 64 && nrhs != 128) return false;
    if (n <= kTpeMaxN || n > kMaxN) return false;
    G->R = nrhs;
    G->E = 128 / nrhs;
    G->Kp = (n + 7) / 8 * 8;
    G->N = (G->E * n + 15) / 16 * 16;
    if (G->N > 256) return false;
    G->cols = 32;
    while (G->cols < G->N) G->cols *= 2;
    // the epilogue reads whole groups of 4 columns past element (E - 1)'s first column
    if ((G->E - 1) * n + (n + 3) / 4 * 4 > G->cols) return false;
    G->a_bytes = 128 * G->Kp * 4;
    G->b_bytes = G->N * G->Kp * 4;
    const uint32_t map_words = (G->E * n + 1) & ~1u;
    if (G->E * n > 2 * kTcThreads) return false;  // each thread loads at most two map entries
    G->smem = 2 * G->a_bytes + 2 * G->b_bytes + 8 * map_words + 16;
    G->smem = (G->smem + 127) & ~127u;
    return G->smem <= kSmemBudget;
}

}  // namespace

bool batched_tc_supported(uint32_t n, uint32_t nrhs) {
    TcGeom G;
    return tc_geom(n, nrhs, &G);
}

// FP32 batched product of one segment on the tensor cores (a.u, a.v float,
// a.ke the FP32 Ke (the hi plane of a split arena), column-major per element).
cudaError_t launch_batched_tc(const Segment& s, const BatchArgs& a, int sm_count, bool pdl, cudaStream_t stream) {
    if (s.units == 0) return cudaSuccess;
    TcGeom G;
    if (s.regime != REG_WPE || !tc_geom(s.n, a.nrhs, &G)) return cudaErrorInvalidValue;
    void* fn = tc_kernel_for(s.n);
    // resident CTAs per SM from registers, shared memory (the whole carveout) and TMEM: the co-resident
    // CTAs must fit the SM's 512 TMEM columns, or an allocation would wait for another CTA to finish
    int regs = 0;
    cudaError_t e = tc_configure(fn, &regs);
    if (e != cudaSuccess) return e;
    int per_sm = 65536 / (regs * kTcThreads);
    const int by_smem = (int)((227u * 1024u) / (G.smem + 1024u));  // 1 KB reserved per CTA
    const int by_tmem = (int)(512 / G.cols);  // every resident CTA holds its TMEM columns
    if (per_sm > by_smem) per_sm = by_smem;
    if (per_sm > by_tmem) per_sm = by_tmem;
    if (per_sm > 8) per_sm = 8;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    const uint32_t groups = (s.count + G.E - 1) / G.E;
    const uint32_t cap = (uint32_t)(sm_count * per_sm);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(groups < cap ? groups : cap);
    cfg.blockDim = dim3(kTcThreads);
    cfg.dynamicSmemBytes = G.smem;
    cfg.stream = stream;
    // no programmatic overlap with the previous launch: its CTAs would hold TMEM columns that this
    // launch's allocations might wait for
    (void)pdl;
    BatchArgs args = a;
    args.smem_total = G.smem;
    uint32_t n_rt = s.n;
    void* params[] = {&args, &G, &n_rt};
    return cudaLaunchKernelExC(&cfg, fn, params);
}

}  // namespace afm
