// AFM matvec kernels for sm_103a: v += sum over the elements of one colour of
// P_e^T Ke P_e u, with Ke streamed from HBM by bulk TMA copies
// (cp.async.bulk) into a shared-memory ring.
//
// CTA = NW consumer warps + 1 producer warp, one persistent CTA per SM. The
// CTA owns a contiguous range of work units of the segment. The producer's
// elected lane copies unit i's Ke (one contiguous chunk of the arena) into
// ring slot i % S and signals full[slot] through the copy's transaction count;
// consumer warp i % NW waits on full[slot], multiplies, and releases the slot
// on empty[slot]. Gather of u_e and of the old v_e run two units ahead in
// registers so their L2 latency hides behind the product. Elements of one
// colour share no DoF, so the scatter is a plain v = v_old + ve store: no
// atomics, and each v entry receives its element contributions in colour
// order, independent of scheduling (bit-reproducible).
//
// Every mbarrier wait is bounded by wall time (globaltimer): the operator's
// wait limit (afm_set_wait_limit, 4 s by default) for the pipeline's waits;
// on expiry the warp sets kErrTimeout in *err and leaves its loop, and the
// host reports AFM_ERR_TIMEOUT. Before its CTA exits, the producer waits for
// every bulk copy it issued to land (drain_ring, bounded by kDrainLimitNs
// whatever the operator's limit), so that no copy writes into the shared
// memory of an exited CTA however short the limit.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "afm_internal.hpp"

namespace afm {

constexpr unsigned long long kDefaultWaitNs = 4000000000ull;  // 4 s per wait unless the operator sets another
constexpr unsigned long long kDrainLimitNs = 4000000000ull;   // copies in flight at exit: always 4 s
constexpr uint32_t kSmemBudget = 220 * 1024;
constexpr uint32_t kSlotAlign = 128;

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ unsigned long long globaltimer_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Non-blocking test of the phase with the given parity.
__device__ __forceinline__ bool mbar_test_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Limits below this are polled with non-blocking tests: try_wait may suspend
// the thread for a hardware-chosen while before it reports an incomplete
// phase, which would stretch a short limit.
constexpr unsigned long long kSpinBelowNs = 100000ull;

__device__ __forceinline__ bool mbar_poll(uint64_t* bar, uint32_t parity, bool spin) {
    return spin ? mbar_test_wait(bar, parity) : mbar_try_wait(bar, parity);
}

// Bounded wait for the phase with the given parity; false on timeout. The
// first test does not block; after it the timer is read after every poll.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, unsigned long long limit) {
    if (mbar_test_wait(bar, parity)) return true;
    const bool spin = limit < kSpinBelowNs;
    const unsigned long long t0 = globaltimer_ns();
    for (;;) {
        if (mbar_poll(bar, parity, spin)) return true;
        if (globaltimer_ns() - t0 > limit) return false;
    }
}

// The producer's last step: waits until each of the last min(issued, S) ring
// copies (the latest round of every slot) has landed, bounded by
// kDrainLimitNs. Consumers that gave up early leave copies in flight; the CTA
// must not exit before they land.
__device__ __forceinline__ void drain_ring(uint64_t* full, uint32_t S, uint32_t issued) {
    const unsigned long long t0 = globaltimer_ns();
    for (uint32_t i = issued > S ? issued - S : 0; i < issued; i++)
        while (!mbar_try_wait(&full[i % S], (i / S) & 1) && globaltimer_ns() - t0 < kDrainLimitNs) {
        }
}

// Test hook of the timeout path (afm_set_wait_probe): when `flag` is set in
// the launch arguments, one consumer warp of block 0 waits for *flag to
// become non-zero, which nothing ever makes it; the wait runs out after
// `limit` and the caller takes its timeout path. Returns false on expiry
// (the same verdict in every lane).
__device__ __forceinline__ bool probe_wait(const int* flag, unsigned long long limit) {
    const unsigned long long t0 = globaltimer_ns();
    bool set = false;
    while (!(set = (*(const volatile int*)flag != 0)) && globaltimer_ns() - t0 <= limit) __nanosleep(256);
    return __all_sync(0xffffffffu, set);
}

// Bounded wait that also gives up as soon as another warp of the CTA has set
// *abort (after a timeout), so that the whole CTA drains quickly and keeps
// meeting its named barriers.
__device__ __forceinline__ bool mbar_wait_abortable(uint64_t* bar, uint32_t parity, volatile int* abort,
                                                    unsigned long long limit) {
    if (mbar_test_wait(bar, parity)) return true;
    const bool spin = limit < kSpinBelowNs;
    const unsigned long long t0 = globaltimer_ns();
    for (;;) {
        if (mbar_poll(bar, parity, spin)) return true;
        if (*abort) return false;
        if (globaltimer_ns() - t0 > limit) {
            *abort = 1;
            return false;
        }
    }
}

__device__ __forceinline__ void named_barrier(uint32_t id, uint32_t threads) {
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(threads) : "memory");
}

__device__ __forceinline__ uint64_t l2_evict_first_policy() {
    uint64_t p;
    asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
    return p;
}

// 1-D bulk copy global -> shared, completion counted on bar. dst, src 16-byte
// aligned, bytes a multiple of 16 (guaranteed by the arena layout).
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar,
                                          uint64_t policy) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], %2, [%3], "
        "%4;" ::"r"(smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar)), "l"(policy)
        : "memory");
}

// Prefetch of bytes (16-byte aligned, a multiple of 16) from global memory
// into L2, no completion to wait for.
__device__ __forceinline__ void bulk_prefetch_l2(const void* src, uint32_t bytes) {
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(src), "r"(bytes) : "memory");
}

// Records a failed bounds check (the access is skipped by the caller): the
// first failure's kind, block, thread and three values in err[1..6], and
// kErrBounds in err[0]; the host reports AFM_ERR_INTERNAL.
__device__ __forceinline__ void report_bad(int* err, int kind, uint32_t a0, uint32_t a1, uint32_t a2) {
    if (atomicCAS(err + 1, 0, kind) == 0) {
        err[2] = (int)blockIdx.x;
        err[3] = (int)threadIdx.x;
        err[4] = (int)a0;
        err[5] = (int)a1;
        err[6] = (int)a2;
    }
    atomicOr(err, kErrBounds);
}

// ---- arithmetic policies ----------------------------------------------------
// KT: stored Ke entry, UT: staged u entry, VT: vector entry, Acc: accumulator.

struct ArithF64 {
    static constexpr bool kSym = false;
    static constexpr bool kScaled = false;  // u scaled by a power of two per launch (stage_s, finish_s)
    static constexpr uint32_t kWpgWarps = 16;  // consumer warps of the warp-group kernel
    using KT = double;
    using UT = double;
    using VT = double;
    using VO = double;  // the product vector v (VT but for ArithF32SymX)
    struct Acc { double s; };
    static __device__ __forceinline__ KT kload(const unsigned char* slot, size_t i, uint32_t) {
        return reinterpret_cast<const double*>(slot)[i];
    }
    static __device__ __forceinline__ Acc zero() { return {0.0}; }
    static __device__ __forceinline__ UT stage(VT x) { return x; }
    static __device__ __forceinline__ void fma(Acc& a, KT k, UT u) { a.s = __fma_rn(k, u, a.s); }
    static __device__ __forceinline__ VT finish(const Acc& a) { return a.s; }
    static __device__ __forceinline__ void combine(Acc& a, const Acc& b) { a.s += b.s; }
};

// Double-float product: Ke entry and u entry are unevaluated float pairs.
// p + e = kh*uh exactly (TwoProduct by FMA); the cross terms kh*ul + kl*uh
// are rounded once; s_hi collects the leading parts with the error of each
// addition recovered by TwoSum (Knuth), s_lo the rest (Ogita, Rump & Oishi,
// "Accurate sum and dot product", SIAM J. Sci. Comput. 26(6), 2005, Dot2).
// The _rn intrinsics keep the compiler from fusing the steps.
struct ArithSplit {
    static constexpr bool kSym = false;
    static constexpr bool kScaled = true;
    static constexpr uint32_t kWpgWarps = 16;
    using KT = float2;
    using UT = float2;
    using VT = double;
    using VO = double;
    struct Acc { float hi, lo; };
    // planar unit: hi plane, then the lo plane `plane` entries further on
    static __device__ __forceinline__ KT kload(const unsigned char* slot, size_t i, uint32_t plane) {
        const float* h = reinterpret_cast<const float*>(slot);
        return make_float2(h[i], h[i + plane]);
    }
    static __device__ __forceinline__ Acc zero() { return {0.0f, 0.0f}; }
    static __device__ __forceinline__ UT stage(VT x) {
        const float h = __double2float_rn(x);
        const float l = __double2float_rn(x - (double)h);
        return make_float2(h, l);
    }
    static __device__ __forceinline__ void fma(Acc& a, KT k, UT u) {
        const float p = __fmul_rn(k.x, u.x);
        const float e = __fmaf_rn(k.x, u.x, -p);
        const float t = __fmaf_rn(k.x, u.y, __fmaf_rn(k.y, u.x, e));
        const float s = __fadd_rn(a.hi, p);
        const float bp = __fsub_rn(s, a.hi);
        const float err = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bp)), __fsub_rn(p, bp));
        a.hi = s;
        a.lo = __fadd_rn(a.lo, __fadd_rn(err, t));
    }
    static __device__ __forceinline__ VT finish(const Acc& a) { return (double)a.hi + (double)a.lo; }
    // a += b, both double-float: TwoSum of the leading parts, the rest into lo
    static __device__ __forceinline__ void combine(Acc& a, const Acc& b) {
        const float s = __fadd_rn(a.hi, b.hi);
        const float bp = __fsub_rn(s, a.hi);
        const float err = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bp)), __fsub_rn(b.hi, bp));
        a.hi = s;
        a.lo = __fadd_rn(a.lo, __fadd_rn(b.lo, err));
    }
};

struct ArithF32 {
    static constexpr bool kSym = false;
    static constexpr bool kScaled = false;
    static constexpr uint32_t kWpgWarps = 24;  // more elements in flight: see wpg_gc
    using KT = float;
    using UT = float;
    using VT = float;
    using VO = float;
    struct Acc { float s; };
    static __device__ __forceinline__ KT kload(const unsigned char* slot, size_t i, uint32_t) {
        return reinterpret_cast<const float*>(slot)[i];
    }
    static __device__ __forceinline__ Acc zero() { return {0.0f}; }
    static __device__ __forceinline__ UT stage(VT x) { return x; }
    static __device__ __forceinline__ void fma(Acc& a, KT k, UT u) { a.s = __fmaf_rn(k, u, a.s); }
    static __device__ __forceinline__ VT finish(const Acc& a) { return a.s; }
    static __device__ __forceinline__ void combine(Acc& a, const Acc& b) { a.s += b.s; }
};

// FP32 products from the symmetric inner arena: each pair of entries K(i, j),
// K(j, i) of a symmetric element matrix is stored once, which cuts the bytes
// streamed per product to about 55%. Thread-per-element units (patches) hold
// the packed upper triangle, entry (i, j), i <= j, at j (j + 1) / 2 + i;
// element units (warp-group kernel) hold the n/2 + 1 wrapped diagonals,
// D[d][j] = K(j, (j + d) mod n) at d n + j, so that both the row and the
// transposed reads of a warp touch consecutive words.
struct ArithF32Sym : ArithF32 {
    static constexpr bool kSym = true;
};

// The symmetric inner arena with a correction plane: each stored entry is
// hi + lo, hi = fl32(K) in the first plane and lo = bf16(K - hi) in the
// plane `plane` entries further on (2 bytes each), which represents K to
// about 2^-32 instead of 2^-24 for 1.5x the bytes. Products are accumulated
// as double-float pairs in FP32 arithmetic (TwoProduct by FMA, TwoSum), and
// the element rows are summed into v in FP64 (VO = double), so that neither
// the correction nor the cancellation between element contributions is lost
// to FP32 rounding. Rounding the element matrices, or the sums, to FP32
// perturbs the product by about 2^-24 |K| |u|, far more than 2^-24 |K u| for
// smooth u, which slows the inner CG of ill-conditioned systems (elasticity)
// markedly; this arithmetic removes both.
struct ArithF32SymX {
    static constexpr bool kSym = true;
    static constexpr bool kScaled = false;
    static constexpr uint32_t kWpgWarps = 24;
    using KT = float2;  // (hi, lo)
    using UT = float;
    using VT = float;
    using VO = double;  // v sums the element products across colours without FP32 cancellation
    struct Acc { float hi, lo; };
    static __device__ __forceinline__ KT kload(const unsigned char* slot, size_t i, uint32_t plane) {
        const float h = reinterpret_cast<const float*>(slot)[i];
        const unsigned short b = reinterpret_cast<const unsigned short*>(slot + (size_t)plane * 4)[i];
        return make_float2(h, __uint_as_float((uint32_t)b << 16));
    }
    static __device__ __forceinline__ Acc zero() { return {0.0f, 0.0f}; }
    static __device__ __forceinline__ UT stage(VT x) { return x; }
    static __device__ __forceinline__ void fma(Acc& a, KT k, UT u) {
        const float p = __fmul_rn(k.x, u);
        const float e = __fmaf_rn(k.x, u, -p);
        const float t = __fmaf_rn(k.y, u, e);
        const float s = __fadd_rn(a.hi, p);
        const float bp = __fsub_rn(s, a.hi);
        const float err = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bp)), __fsub_rn(p, bp));
        a.hi = s;
        a.lo = __fadd_rn(a.lo, __fadd_rn(err, t));
    }
    static __device__ __forceinline__ VO finish(const Acc& a) { return (double)a.hi + (double)a.lo; }
    static __device__ __forceinline__ void combine(Acc& a, const Acc& b) {
        const float s = __fadd_rn(a.hi, b.hi);
        const float bp = __fsub_rn(s, a.hi);
        const float err = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bp)), __fsub_rn(b.hi, bp));
        a.hi = s;
        a.lo = __fadd_rn(a.lo, __fadd_rn(b.lo, err));
    }
};

// Products from the corrected symmetric arena on u rounded to FP32, each
// element row summed in plain FP32 ((hi + lo) u as two FMAs) and the rows
// summed into v in FP64: the inner product of symmetric inner format 5. Ke
// keeps its 2^-32 representation; the row sums are rounded to FP32, which
// perturbs the product far less than rounding Ke (emulated on hex20 12^3:
// FP32 Ke alone +50% CG iterations, FP32 sums on top of it +10%).
struct ArithF32SymC {
    static constexpr bool kSym = true;
    static constexpr bool kScaled = false;
    static constexpr uint32_t kWpgWarps = 24;
    using KT = float2;  // (hi, lo)
    using UT = float;
    using VT = float;
    using VO = double;
    struct Acc { float s; };
    static __device__ __forceinline__ KT kload(const unsigned char* slot, size_t i, uint32_t plane) {
        return ArithF32SymX::kload(slot, i, plane);
    }
    static __device__ __forceinline__ Acc zero() { return {0.0f}; }
    static __device__ __forceinline__ UT stage(VT x) { return x; }
    static __device__ __forceinline__ void fma(Acc& a, KT k, UT u) { a.s = __fmaf_rn(k.x, u, __fmaf_rn(k.y, u, a.s)); }
    static __device__ __forceinline__ VO finish(const Acc& a) { return (double)a.s; }
    static __device__ __forceinline__ void combine(Acc& a, const Acc& b) { a.s += b.s; }
};

// FP64 products from the corrected symmetric arena (the arena of ArithF32SymX:
// K to about 2^-32, each pair of entries once): u and v are FP64 vectors, u is
// staged as a scaled float pair like the split arithmetic, and each product
// is the double-float product of ArithSplit with the entry pair (hi, bf16 lo).
// The inner recursion of the FP64-vector mixed solve (symmetric inner format
// 3) runs on it: 40% of the split arena's bytes per product, and no FP32
// rounding of the vectors, whose loss of accuracy stalls the FP32 recursion on
// large ill-conditioned systems.
struct ArithSplitSymX {
    static constexpr bool kSym = true;
    static constexpr bool kScaled = true;
    static constexpr uint32_t kWpgWarps = 16;
    using KT = float2;  // (hi, lo)
    using UT = float2;
    using VT = double;
    using VO = double;
    struct Acc { float hi, lo; };
    static __device__ __forceinline__ KT kload(const unsigned char* slot, size_t i, uint32_t plane) {
        return ArithF32SymX::kload(slot, i, plane);
    }
    static __device__ __forceinline__ Acc zero() { return {0.0f, 0.0f}; }
    static __device__ __forceinline__ UT stage(VT x) { return ArithSplit::stage(x); }
    static __device__ __forceinline__ void fma(Acc& a, KT k, UT u) {
        ArithSplit::Acc b{a.hi, a.lo};
        ArithSplit::fma(b, k, u);
        a.hi = b.hi;
        a.lo = b.lo;
    }
    static __device__ __forceinline__ VT finish(const Acc& a) { return (double)a.hi + (double)a.lo; }
    static __device__ __forceinline__ void combine(Acc& a, const Acc& b) {
        ArithSplit::Acc x{a.hi, a.lo};
        ArithSplit::combine(x, ArithSplit::Acc{b.hi, b.lo});
        a.hi = x.hi;
        a.lo = x.lo;
    }
};

// Range guard of the double-float arithmetic. Its u pairs and products live in
// FP32's exponent range: unscaled, |u| above 3.4e38 would overflow and small
// entries would fall into FP32 subnormals and lose their low bits. So every
// launch scales u by 2^k with k = -eu, max|u| = f 2^eu (f in [0.5, 1)), over
// the DoFs the product reads: the largest scaled entry lies in [0.5, 1), and
// with each element's max|Ke| in [1e-30, 1e30] (checked at finalize) the
// products of a scaled u entry and the element's leading entries stay within
// FP32's normal range (smaller entries may reach FP32 subnormals, whose
// absolute rounding, below 2^-149, is far under the element's error bound). The element
// sums are scaled back by 2^-k in FP64. Both steps only move exponents, so
// they are exact, and they run on the integer pipe (GB300 issues FP64 at 1/64
// of the FP32 rate): the staged pair (hi, lo) of 2^k x is cut from the bits of
// x directly, hi = the leading 24 significant bits, lo = the next 29 rounded
// to FP32 (together 2^-47 of |x|). A scaled entry below 2^-126 becomes 0 and
// one below 2^-74 keeps only hi, i.e. changes of at most 2^-98 of max|u|:
// the norm-wise bound |v - K u| <= c 2^-44 |K| |u| holds for every finite u.
// A non-finite max|u| leaves k = 0 (the product is then non-finite, as in FP64).
__device__ __forceinline__ int uscale_of(unsigned long long mbits) {
    if (mbits == 0ull || mbits >= 0x7ff0000000000000ull) return 0;
    const int e = (int)(mbits >> 52);  // biased exponent of max|u| (0: subnormal)
    int eu = e - 1022;                 // frexp exponent of a normal max|u|
    if (e == 0) eu = -1022;            // a subnormal maximum: scale as the smallest normal
    return eu > 1000 ? -1000 : (eu < -1000 ? 1000 : -eu);
}

// u scale exponent k of a launch: from the max|u| word for a scaled
// arithmetic, 0 otherwise.
template <typename A>
__device__ __forceinline__ int load_uscale(const unsigned long long* umax) {
    if constexpr (A::kScaled) return uscale_of(*umax);
    return 0;
}

// (hi, lo) of 2^k x as above, with integer and FP32 operations only (the FP64
// pipe only for non-finite x).
__device__ __forceinline__ float2 split_scaled(double x, int k) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const int e = (int)((b >> 52) & 0x7ff);
    const unsigned sgn = (unsigned)(b >> 32) & 0x80000000u;
    if (e == 0x7ff) return make_float2(__double2float_rn(x), 0.0f);
    const int E = e - 1023 + k;  // unbiased exponent of 2^k x
    if (e == 0 || E < -126) return make_float2(__uint_as_float(sgn), 0.0f);
    if (E > 127) return make_float2(__uint_as_float(sgn | 0x7f800000u), 0.0f);
    const unsigned long long m = b & 0x000fffffffffffffull;
    const float h = __uint_as_float(sgn | ((unsigned)(E + 127) << 23) | (unsigned)(m >> 29));
    float l = 0.0f;
    const unsigned mlo = (unsigned)(m & 0x1fffffffu);
    if (mlo && E >= -74) {
        // mlo units of 2^(E - 52), a normal FP32 power of two for E >= -74
        const float unit = __uint_as_float((unsigned)(E - 52 + 127) << 23);
        l = __uint_as_float(__float_as_uint(__uint2float_rn(mlo) * unit) | sgn);
    }
    return make_float2(h, l);
}

// 2^k y through the exponent field (y normal and the result normal), else in FP64.
__device__ __forceinline__ double scale_pow2(double y, int k) {
    const long long b = __double_as_longlong(y);
    const int e = (int)((b >> 52) & 0x7ff);
    if (e != 0 && e != 0x7ff && e + k > 0 && e + k < 0x7ff) return __longlong_as_double(b + ((long long)k << 52));
    return y * __longlong_as_double((long long)(1023 + k) << 52);
}

template <typename A>
__device__ __forceinline__ typename A::UT stage_s(typename A::VT x, int k) {
    if constexpr (A::kScaled) return split_scaled(x, k);
    else return A::stage(x);
}

template <typename A>
__device__ __forceinline__ typename A::VO finish_s(const typename A::Acc& acc, int k) {
    if constexpr (A::kScaled) return scale_pow2(A::finish(acc), -k);
    else return A::finish(acc);
}

// Entry index of (r, c) in a thread-per-element unit.
template <typename A>
__host__ __device__ __forceinline__ uint32_t tpe_entry(uint32_t r, uint32_t c, uint32_t n) {
    if constexpr (A::kSym) {
        const uint32_t i = r < c ? r : c, j = r < c ? c : r;
        return j * (j + 1) / 2 + i;
    } else {
        return r * n + c;
    }
}

__device__ __forceinline__ uint64_t l2_evict_last_policy() {
    uint64_t p;
    asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
    return p;
}

// Vector accesses with an L2 policy: u and v are gathered by every colour
// pass and should stay in L2 while the element matrices stream past
// (evict_last); the DoF map is read once per matvec (evict_first).
__device__ __forceinline__ double ld_nc_hint(const double* p, uint64_t pol) {
    double x;
    asm volatile("ld.global.nc.L2::cache_hint.f64 %0, [%1], %2;" : "=d"(x) : "l"(p), "l"(pol));
    return x;
}
__device__ __forceinline__ float ld_nc_hint(const float* p, uint64_t pol) {
    float x;
    asm volatile("ld.global.nc.L2::cache_hint.f32 %0, [%1], %2;" : "=f"(x) : "l"(p), "l"(pol));
    return x;
}
__device__ __forceinline__ uint32_t ld_nc_hint(const uint32_t* p, uint64_t pol) {
    uint32_t x;
    asm volatile("ld.global.nc.L2::cache_hint.u32 %0, [%1], %2;" : "=r"(x) : "l"(p), "l"(pol));
    return x;
}
__device__ __forceinline__ double ld_hint(const double* p, uint64_t pol) {
    double x;
    asm volatile("ld.global.L2::cache_hint.f64 %0, [%1], %2;" : "=d"(x) : "l"(p), "l"(pol) : "memory");
    return x;
}
__device__ __forceinline__ float ld_hint(const float* p, uint64_t pol) {
    float x;
    asm volatile("ld.global.L2::cache_hint.f32 %0, [%1], %2;" : "=f"(x) : "l"(p), "l"(pol) : "memory");
    return x;
}
__device__ __forceinline__ void st_hint(double* p, double x, uint64_t pol) {
    asm volatile("st.global.L2::cache_hint.f64 [%0], %1, %2;" ::"l"(p), "d"(x), "l"(pol) : "memory");
}
__device__ __forceinline__ void st_hint(float* p, float x, uint64_t pol) {
    asm volatile("st.global.L2::cache_hint.f32 [%0], %1, %2;" ::"l"(p), "f"(x), "l"(pol) : "memory");
}

// Programmatic dependent launch: a colour launch may start (and prefetch its
// element matrices) while the previous colour drains; every access to v waits
// until the previous grid has completed and its writes are visible. Both are
// no-ops for a launch without the programmatic-serialisation attribute.
__device__ __forceinline__ void wait_prior_grid() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void allow_dependent_launch() { asm volatile("griddepcontrol.launch_dependents;"); }

template <typename VT>
__device__ __forceinline__ VT load_u(const VT* u, uint32_t m, int bc_mode) {
    const uint32_t d = m & kDofMask;
    VT x = __ldg(u + d);
    if (bc_mode && (m & kBcFlag)) x = VT(0);
    return x;
}

template <typename VT>
__device__ __forceinline__ VT load_u_hint(const VT* u, uint32_t m, int bc_mode, uint64_t pol) {
    VT x = ld_nc_hint(u + (m & kDofMask), pol);
    if (bc_mode && (m & kBcFlag)) x = VT(0);
    return x;
}

// Shared-memory layout of one CTA: S slots, then 2*S mbarriers and a 16-byte
// flag word, then extra_bytes of staging (per-warp u buffers of the WPE
// kernel; u double buffers and partial sums of the warp-group kernel).
// After the flag word come S uint32 slot tags (the ring index each slot was
// last loaded with; see ring_wait).
struct RingLayout {
    uint32_t slot_bytes, stages, warps, ubuf_bytes, extra_bytes;
    // warp-group kernel: consecutive element units per ring slot, copied by
    // one bulk copy (1 for the other kernels)
    uint32_t chunk = 1;
    __host__ __device__ uint32_t bars_offset() const { return slot_bytes * stages; }
    __host__ __device__ uint32_t tags_offset() const { return bars_offset() + 16 * stages + 16; }
    __host__ __device__ uint32_t ubuf_offset() const { return tags_offset() + ((4 * stages + 15) & ~15u); }
    __host__ __device__ uint32_t total() const { return ubuf_offset() + extra_bytes; }
};

// Waits until ring slot s holds ring index ii (parity = (ii / S) & 1). A
// parity test alone cannot tell round r of a slot from round r - 2 (a consumer
// that reaches a slot while its previous round is still loading would pass at
// once), so the producer writes the slot's tag = ring index before the arrive
// that completes the phase, and the consumer accepts the phase only with the
// matching tag. The polling loop is out of line: inlined, it costs the hot
// loops of the element kernels registers and spills. Bounded like
// mbar_wait_abortable.
static __device__ __noinline__ bool ring_wait_slow(uint64_t* bar, const volatile uint32_t* tag, uint32_t ii, uint32_t parity,
                                                   volatile int* abort, unsigned long long limit) {
    const bool spin = limit < kSpinBelowNs;
    const unsigned long long t0 = globaltimer_ns();
    for (;;) {
        if (mbar_poll(bar, parity, spin) && *tag == ii) return true;
        if (*abort) return false;
        if (globaltimer_ns() - t0 > limit) {
            *abort = 1;
            return false;
        }
    }
}

__device__ __forceinline__ bool ring_wait(uint64_t* bar, const volatile uint32_t* tag, uint32_t ii, uint32_t parity,
                                          volatile int* abort, unsigned long long limit) {
    if (mbar_test_wait(bar, parity) && *tag == ii) return true;
    return ring_wait_slow(bar, tag, ii, parity, abort, limit);
}

// ---- warp per element (n > 16) --------------------------------------------
// Ke of one element: column-major, entry (r, c) at c*n + r. Lane l owns rows
// l, l+32, l+64 (R = ceil(n/32) rows).
template <int NT, typename A, bool DUP>
__global__ void __launch_bounds__(9 * 32, 1) afm_wpe_kernel(SegArgs a, RingLayout L, uint32_t n_rt) {
    using KT = typename A::KT;
    using UT = typename A::UT;
    using VT = typename A::VT;
    constexpr int RMAX = NT ? (NT + 31) / 32 : 3;
    const uint32_t n = NT ? NT : n_rt;
    extern __shared__ __align__(128) unsigned char smem[];
    uint64_t* full = reinterpret_cast<uint64_t*>(smem + L.bars_offset());
    uint64_t* empty = full + L.stages;
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t NW = L.warps, S = L.stages;

    const uint32_t per = a.units / gridDim.x, rem = a.units % gridDim.x;
    const uint32_t begin = blockIdx.x * per + min(blockIdx.x, rem);
    const uint32_t cnt = per + (blockIdx.x < rem ? 1u : 0u);

    if (threadIdx.x == 0) {
        for (uint32_t s = 0; s < S; s++) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();

    if (warp == NW) {  // producer
        if (lane == 0) {
            const uint64_t pol = l2_evict_first_policy();
            uint32_t issued = 0;
            for (uint32_t i = 0; i < cnt; i++) {
                const uint32_t s = i % S;
                if (i >= S && !mbar_wait(&empty[s], ((i / S) - 1) & 1, a.wait_ns)) {
                    atomicOr(a.err, kErrTimeout);
                    break;
                }
                mbar_arrive_expect_tx(&full[s], a.copy_bytes);
                bulk_load(smem + (size_t)s * L.slot_bytes, a.ke + (size_t)(begin + i) * a.unit_bytes, a.copy_bytes,
                          &full[s], pol);
                issued = i + 1;
            }
            allow_dependent_launch();
            drain_ring(full, S, issued);
        }
        return;
    }
    wait_prior_grid();
    if (a.probe && blockIdx.x == 0 && warp == 0 && !probe_wait(a.probe, a.wait_ns)) {
        if (lane == 0) atomicOr(a.err, kErrTimeout);
        return;  // this warp's elements are left out; the producer's waits for their slots run out too
    }

    const int usk = load_uscale<A>(a.umax);
    const VT* __restrict__ u = static_cast<const VT*>(a.u);
    VT* __restrict__ v = static_cast<VT*>(a.v);
    UT* us = reinterpret_cast<UT*>(smem + L.ubuf_offset() + warp * L.ubuf_bytes);

    uint32_t dof_c[RMAX], dof_n[RMAX], dof_nn[RMAX];
    VT vold_c[RMAX], vold_n[RMAX], u_n[RMAX];
#pragma unroll
    for (int t = 0; t < RMAX; t++) {
        dof_c[t] = dof_n[t] = dof_nn[t] = 0u;
        vold_c[t] = vold_n[t] = u_n[t] = VT(0);
    }
    auto load_map = [&](uint32_t i, uint32_t* d) {
        const uint32_t* mp = a.map + (size_t)(begin + i) * n;
#pragma unroll
        for (int t = 0; t < RMAX; t++) {
            const uint32_t r = lane + 32 * t;
            d[t] = (r < n) ? __ldg(mp + r) : 0u;
        }
    };
    auto load_uv = [&](const uint32_t* d, VT* uu, VT* vv) {
#pragma unroll
        for (int t = 0; t < RMAX; t++) {
            const uint32_t r = lane + 32 * t;
            uu[t] = VT(0);
            vv[t] = VT(0);
            if (r < n) {
                uu[t] = load_u(u, d[t], a.bc_mode);
                if (!DUP) vv[t] = v[d[t] & kDofMask];
            }
        }
    };

    uint32_t i = warp;
    if (i < cnt) {
        VT u_c[RMAX];
        load_map(i, dof_c);
        load_uv(dof_c, u_c, vold_c);
#pragma unroll
        for (int t = 0; t < RMAX; t++)
            if (lane + 32 * t < n) us[lane + 32 * t] = stage_s<A>(u_c[t], usk);
        if (i + NW < cnt) load_map(i + NW, dof_n);
    }
    for (; i < cnt; i += NW) {
        if (i + NW < cnt) load_uv(dof_n, u_n, vold_n);
        if (i + 2 * NW < cnt) load_map(i + 2 * NW, dof_nn);
        __syncwarp();

        const uint32_t s = i % S;
        if (!__all_sync(0xffffffffu, mbar_wait(&full[s], (i / S) & 1, a.wait_ns))) {  // one verdict per warp
            if (lane == 0) atomicOr(a.err, kErrTimeout);
            break;
        }
        const unsigned char* ks = smem + (size_t)s * L.slot_bytes;
        typename A::Acc acc[RMAX];
#pragma unroll
        for (int t = 0; t < RMAX; t++) acc[t] = A::zero();
#pragma unroll(NT ? (NT < 64 ? NT : 16) : 4)
        for (uint32_t c = 0; c < n; c++) {
            const UT uc = us[c];
#pragma unroll
            for (int t = 0; t < RMAX; t++) {
                const uint32_t r = lane + 32 * t;
                if (r < n) A::fma(acc[t], A::kload(ks, (size_t)c * n + r, a.plane), uc);
            }
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[s]);

        if (!DUP) {
#pragma unroll
            for (int t = 0; t < RMAX; t++) {
                const uint32_t r = lane + 32 * t;
                if (r < n) v[dof_c[t] & kDofMask] = vold_c[t] + finish_s<A>(acc[t], usk);
            }
        } else {
            // an element lists a DoF more than once: add row by row in order
            for (uint32_t r = 0; r < n; r++) {
                if ((r & 31) == lane) {
                    const uint32_t d = dof_c[r >> 5] & kDofMask;
                    v[d] = v[d] + finish_s<A>(acc[r >> 5], usk);
                }
                __syncwarp();
            }
        }
        // rotate the pipeline
#pragma unroll
        for (int t = 0; t < RMAX; t++) {
            dof_c[t] = dof_n[t];
            vold_c[t] = vold_n[t];
            dof_n[t] = dof_nn[t];
        }
        if (i + NW < cnt) {
#pragma unroll
            for (int t = 0; t < RMAX; t++)
                if (lane + 32 * t < n) us[lane + 32 * t] = stage_s<A>(u_n[t], usk);
        }
    }
}


// ---- warp group per element (n > 16) ---------------------------------------
// Same Ke layout as the WPE kernel (column-major per element). An element is
// worked on by g = gr x gc warps: row group rg owns rows 32 rg + lane, column
// group cg owns columns [cg n / gc, (cg+1) n / gc). The cg > 0 warps leave
// their partial row sums in shared memory; after one named barrier per
// element the cg == 0 warps add them in column-group order (deterministic) and
// scatter. ng such groups run per CTA, group k of an element sequence taking
// elements k, k+ng, ... of the CTA's range. u_e is staged per group in a
// double buffer so that the next element's gather overlaps this one's product.
struct GroupGeom {
    uint32_t gr, gc, g, ng;
};

__host__ __device__ inline uint32_t wpg_ubuf_bytes(uint32_t n, uint32_t ut) { return (n * ut + 15) / 16 * 16; }

// Column groups of the warp-group kernel for gr row groups. Elements of two
// row groups (33..64 DoFs) with 8-byte staged u (FP64 and split arithmetic)
// take two column groups, so four warps share one element's long products;
// every other element takes one warp per row group: for short rows, splitting
// them across warps only adds the cross-warp sum, while more elements in
// flight per SM hide the gathers (hex8 elasticity, n = 24, at 48^3: split
// product 0.31 -> 0.19 ms, FP32 products 0.19-0.22 -> 0.18-0.20 ms).
__host__ __device__ constexpr uint32_t wpg_gc(uint32_t gr, uint32_t ut_bytes) {
    return gr == 2 && ut_bytes == 8 ? 2u : 1u;
}

// Terms [T0, T1) of row r of a symmetric element in the wrapped-diagonal
// layout (D[d][j] = K(j, (j + d) mod n) at d n + j): term t <= n/2 is
// D[t][r] u[r + t], term t > n/2 (d = t - n/2) is K(r, r - d) =
// D[d][(r - d) mod n] u[r - d]. kr = the unit + r, ur = the staged u + r,
// where u is staged twice in a row (u[j + n] = u[j]) so that no u index
// wraps. Every offset is a compile-time constant but the wrap of the
// transposed read (one select).
template <typename A, int NT, int T0, int T1>
__device__ __forceinline__ void sym_terms(typename A::Acc& acc, const unsigned char* ks, uint32_t plane,
                                          const typename A::UT* ur, uint32_t r) {
    constexpr int H = NT / 2;
#pragma unroll
    for (int t = T0; t < T1; t++) {
        if (t <= H) {
            A::fma(acc, A::kload(ks, r + t * NT, plane), ur[t]);
        } else {
            const int d = t - H;
            A::fma(acc, A::kload(ks, r + d * NT - d + ((int)r < d ? NT : 0), plane), ur[NT - d]);
        }
    }
}

// Synchronises an element group: a one-warp group with __syncwarp, a larger
// one with its named barrier (ids 1..15).
__device__ __forceinline__ void group_sync(uint32_t id, uint32_t threads) {
    if (threads == 32)
        __syncwarp();
    else
        named_barrier(id, threads);
}

// Colours of one fused launch (afm_wpg_fused_kernel): per colour the offset
// of its first unit in the arena (bytes) and in the map (entries), its units
// and elements; gbar[c - 1] counts the CTAs that finished colour c - 1.
struct ColourTable {
    uint32_t ncol;
    unsigned* gbar;
    uint64_t ke_off[kMaxFusedColours];
    uint64_t map_off[kMaxFusedColours];
    uint32_t units[kMaxFusedColours];
};

// ld.global.cg: an L2 load that bypasses L1, for v in a fused launch, whose
// earlier colours other CTAs have written since this SM may have cached it.
__device__ __forceinline__ double ld_cg_hint(const double* p, uint64_t pol) {
    double x;
    asm volatile("ld.global.cg.L2::cache_hint.f64 %0, [%1], %2;" : "=d"(x) : "l"(p), "l"(pol) : "memory");
    return x;
}
__device__ __forceinline__ float ld_cg_hint(const float* p, uint64_t pol) {
    float x;
    asm volatile("ld.global.cg.L2::cache_hint.f32 %0, [%1], %2;" : "=f"(x) : "l"(p), "l"(pol) : "memory");
    return x;
}

__device__ __forceinline__ unsigned ld_acquire_gpu(const unsigned* p) {
    unsigned x;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(x) : "l"(p) : "memory");
    return x;
}

// Grid barrier of a cooperative launch (all CTAs resident), between two
// colours: the CTA's consumer warps meet on named barrier 15, thread 0
// publishes the CTA's writes and counts it in, then waits (bounded by limit;
// on expiry it sets *abort) until every CTA has arrived.
__device__ __forceinline__ void grid_barrier(unsigned* ctr, uint32_t threads, volatile int* abort,
                                             unsigned long long limit) {
    named_barrier(15, threads);
    if (threadIdx.x == 0) {
        __threadfence();
        atomicAdd(ctr, 1u);
        const unsigned long long t0 = globaltimer_ns();
        while (ld_acquire_gpu(ctr) < gridDim.x) {
            if (*abort || globaltimer_ns() - t0 > limit) {
                *abort = 1;
                break;
            }
            __nanosleep(64);
        }
        __threadfence();
    }
    named_barrier(15, threads);
}

// CH: ring slots may hold several element units (L.chunk); without it the
// chunk is the constant 1 and the walk folds to one element per slot.
// FU: the colours of T in one cooperative launch, a grid barrier between
// them (every colour's CTA split as a colour launch of its own would have);
// without it one segment, a.units units from a.ke and a.map.
template <int NT, typename A, bool CH, bool FU>
__device__ __forceinline__ void wpg_run(const SegArgs& a, const RingLayout& L, const GroupGeom& G, uint32_t n_rt,
                                        const ColourTable* T) {
    using KT = typename A::KT;
    using UT = typename A::UT;
    using VT = typename A::VT;
    using VO = typename A::VO;
    using Acc = typename A::Acc;
    const uint32_t n = NT ? NT : n_rt;
    extern __shared__ __align__(128) unsigned char smem[];
    uint64_t* full = reinterpret_cast<uint64_t*>(smem + L.bars_offset());
    uint64_t* empty = full + L.stages;
    volatile int* abort = reinterpret_cast<volatile int*>(empty + L.stages);
    volatile uint32_t* tag = reinterpret_cast<volatile uint32_t*>(smem + L.tags_offset());
    const uint32_t ub = wpg_ubuf_bytes(A::kSym ? 2 * n : n, sizeof(UT));
    unsigned char* ubase = smem + L.ubuf_offset();                 // [ng][2] u buffers
    Acc* pbase = reinterpret_cast<Acc*>(ubase + (size_t)G.ng * 2 * ub);  // [ng][2][gc-1][n] partials
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t S = L.stages;

    const uint32_t ncol = FU ? T->ncol : 1u;
    // this CTA's units of colour col: [begin, begin + cnt), as a launch of that colour alone would split them
    auto share = [&](uint32_t col, uint32_t& begin, uint32_t& cnt) {
        const uint32_t units = FU ? T->units[col] : a.units;
        const uint32_t per = units / gridDim.x, rem = units % gridDim.x;
        begin = blockIdx.x * per + min(blockIdx.x, rem);
        cnt = per + (blockIdx.x < rem ? 1u : 0u);
    };

    if (threadIdx.x == 0) {
        for (uint32_t s = 0; s < S; s++) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], G.g);
            tag[s] = 0xffffffffu;
        }
        *abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();

    // ring slots hold chunks of E consecutive elements (one bulk copy each: the
    // copies of small element units are issue-bound one by one); chunk c goes
    // to group c % ng, which takes its elements in order
    const uint32_t E = CH ? L.chunk : 1u;
    if (warp == G.ng * G.g) {  // producer
        if (lane == 0) {
            const uint64_t pol = l2_evict_first_policy();
            // ring index g runs on across colours: the copies of a colour start while the previous one drains
            uint32_t issued = 0, gbase = 0;
            bool stop = false;
            for (uint32_t col = 0; col < ncol && !stop; col++) {
                uint32_t begin, cnt;
                share(col, begin, cnt);
                const unsigned char* ke = FU ? a.ke + T->ke_off[col] : a.ke;
                const uint32_t nch = (cnt + E - 1) / E;
                for (uint32_t c = 0; c < nch; c++) {
                    const uint32_t g = gbase + c, s = g % S;
                    if (g >= S && !mbar_wait_abortable(&empty[s], ((g / S) - 1) & 1, abort, a.wait_ns)) {
                        stop = true;
                        break;
                    }
                    const uint32_t e0 = c * E, ne = min(E, cnt - e0);
                    tag[s] = g;
                    // E > 1 only for whole units (copy_bytes == unit_bytes), so the chunk is contiguous
                    mbar_arrive_expect_tx(&full[s], ne * a.copy_bytes);
                    bulk_load(smem + (size_t)s * L.slot_bytes, ke + (size_t)(begin + e0) * a.unit_bytes,
                              ne * a.copy_bytes, &full[s], pol);
                    issued = g + 1;
                }
                gbase += nch;
            }
            allow_dependent_launch();
            if (*abort) atomicOr(a.err, kErrTimeout);
            // every issued copy lands before the CTA's shared memory is released
            drain_ring(full, S, issued);
        }
        return;
    }

    if (a.probe && blockIdx.x == 0 && warp == 0 && !probe_wait(a.probe, a.wait_ns)) *abort = 1;
    const uint32_t grp = warp / G.g, q = warp % G.g;
    const uint32_t rg = q / G.gc, cg = q % G.gc;
    const uint32_t r = 32 * rg + lane;
    const bool rvalid = r < n;
    const uint32_t cb = cg * n / G.gc, ce = (cg + 1) * n / G.gc;
    const bool gatherer = (cg == 0);
    const uint32_t bar_id = 1 + grp, bar_threads = G.g * 32;
    const VT* __restrict__ u = static_cast<const VT*>(a.u);
    VO* __restrict__ v = static_cast<VO*>(a.v);
    // the scale was written by a launch that completed before this segment's first launch
    const int usk = load_uscale<A>(a.umax);
    unsigned char* ubuf0 = ubase + (size_t)(grp * 2) * ub;
    const uint32_t pstride = (G.gc > 1 ? G.gc - 1 : 1) * n;
    Acc* pbuf0 = pbase + (size_t)(grp * 2) * pstride;
    auto ubuf = [&](uint32_t p) { return reinterpret_cast<UT*>(ubuf0 + (size_t)p * ub); };
    auto pbuf = [&](uint32_t p) { return pbuf0 + (size_t)p * pstride; };

    const uint64_t keep = l2_evict_last_policy(), stream_pol = l2_evict_first_policy();
    // v written by other CTAs in an earlier colour of a fused launch is read past L1
    auto v_load = [&](const VO* pv) { return FU ? ld_cg_hint(pv, keep) : ld_hint(pv, keep); };
    const uint32_t consumer_threads = G.ng * G.g * 32;
    uint32_t gbase = 0;  // ring index of the colour's first chunk
    for (uint32_t col = 0; col < ncol; col++) {
        uint32_t begin, cnt;
        share(col, begin, cnt);
        const uint32_t* __restrict__ mapc = FU ? a.map + T->map_off[col] : a.map;
        uint32_t dof_c = 0, dof_n = 0, dof_nn = 0;
        VO vold_c = VO(0), vold_n = VO(0);
        VT u_n = VT(0);
        auto map_at = [&](uint32_t i) {
            return rvalid ? ld_nc_hint(mapc + (size_t)(begin + i) * n + r, stream_pol) : 0u;
        };

        // The group's elements in order: element ch E + jc of chunk ch, the chunks
        // grp, grp + ng, ...; positions advance by increments (no division in
        // the loop but the slot of a new chunk).
        auto advance = [&](uint32_t& c, uint32_t& j) {
            if (++j == E) {
                j = 0;
                c += G.ng;
            }
        };
        uint32_t ch = grp, jc = 0, chn = grp, jn = 0;
        advance(chn, jn);
        uint32_t i = ch * E, inext = chn * E + jn;
        if (gatherer && i < cnt) {
            dof_c = map_at(i);
            if (rvalid) {
                const UT x = stage_s<A>(load_u_hint(u, dof_c, a.bc_mode, keep), usk);
                ubuf(0)[r] = x;
                if constexpr (A::kSym) ubuf(0)[r + n] = x;
            }
            if (inext < cnt) dof_n = map_at(inext);
        }
        if (!FU || col == 0)
            wait_prior_grid();
        else  // every CTA has written the previous colour's sums to v
            grid_barrier(T->gbar + (col - 1), consumer_threads, abort, a.wait_ns);
        if (gatherer && i < cnt && rvalid) vold_c = v_load(v + (dof_c & kDofMask));
        group_sync(bar_id, bar_threads);
        bool ok = false;  // the current chunk's slot has landed (one verdict per warp and chunk)
        uint32_t s = 0;   // the current chunk's ring slot
        for (uint32_t k = 0; i < cnt; k++) {
            const uint32_t par = k & 1;
            uint32_t chnn = chn, jnn = jn;
            advance(chnn, jnn);
            const uint32_t inn = chnn * E + jnn;
            if (gatherer && rvalid) {
                if (inext < cnt) {
                    u_n = load_u_hint(u, dof_n, a.bc_mode, keep);
                    vold_n = v_load(v + (dof_n & kDofMask));
                }
                if (inn < cnt) dof_nn = map_at(inn);
            }
            Acc acc = A::zero();
            // one verdict per warp and chunk: the block below synchronises the warp, so no lane may skip it alone
            if (jc == 0) {
                const uint32_t g = gbase + ch;
                s = g % S;
                ok = __all_sync(0xffffffffu, ring_wait(&full[s], &tag[s], g, (g / S) & 1, abort, a.wait_ns));
            }
            if (ok) {
                const unsigned char* ks = smem + (size_t)s * L.slot_bytes + (size_t)jc * a.unit_bytes;
                const UT* uu = ubuf(par);
                if (rvalid) {
                    if constexpr (A::kSym && NT != 0) {
                        // the column group's terms, with compile-time bounds
                        constexpr int GR = (NT + 31) / 32;
                        constexpr int GC = (int)wpg_gc(GR, sizeof(UT));
                        const UT* ur = uu + r;
                        const uint32_t pl = a.plane;
                        if constexpr (GC == 1) {
                            sym_terms<A, NT, 0, NT>(acc, ks, pl, ur, r);
                        } else if constexpr (GC == 2) {
                            if (cg == 0)
                                sym_terms<A, NT, 0, NT / 2>(acc, ks, pl, ur, r);
                            else
                                sym_terms<A, NT, NT / 2, NT>(acc, ks, pl, ur, r);
                        } else {
                            switch (cg) {
                                case 0: sym_terms<A, NT, 0, NT / 4>(acc, ks, pl, ur, r); break;
                                case 1: sym_terms<A, NT, NT / 4, 2 * NT / 4>(acc, ks, pl, ur, r); break;
                                case 2: sym_terms<A, NT, 2 * NT / 4, 3 * NT / 4>(acc, ks, pl, ur, r); break;
                                default: sym_terms<A, NT, 3 * NT / 4, NT>(acc, ks, pl, ur, r); break;
                            }
                        }
                    } else if constexpr (A::kSym) {
                        // run-time n: term t <= n/2: D[t][r] u[r + t]; term t > n/2, d = t - n/2:
                        // K(r, r - d) = D[d][(r - d) mod n] times u[r - d + n]
                        constexpr uint32_t NS = kMaxN;
                        constexpr uint32_t GR = (NS + 31) / 32;
                        constexpr uint32_t GC = wpg_gc(GR, sizeof(UT));
                        constexpr uint32_t TRIP = (NS + GC - 1) / GC;
                        const uint32_t h = n / 2;
    #pragma unroll 4
                        for (uint32_t j = 0; j < TRIP; j++) {
                            const uint32_t t = cb + j;
                            if (t < ce) {
                                uint32_t col, k;
                                if (t <= h) {
                                    col = r + t;
                                    k = t * n + r;
                                } else {
                                    const uint32_t d = t - h;
                                    col = r + n - d;
                                    k = d * n + (r >= d ? r - d : r + n - d);
                                }
                                A::fma(acc, A::kload(ks, k, a.plane), uu[col]);
                            }
                        }
                    } else if constexpr (NT != 0) {
                        constexpr uint32_t GR = (NT + 31) / 32;
                        constexpr uint32_t GC = wpg_gc(GR, sizeof(UT));
                        constexpr uint32_t TRIP = (NT + GC - 1) / GC;
    #pragma unroll
                        for (uint32_t j = 0; j < TRIP; j++) {
                            const uint32_t c = cb + j;
                            if (c < ce) A::fma(acc, A::kload(ks, (size_t)c * NT + r, a.plane), uu[c]);
                        }
                    } else {
    #pragma unroll 4
                        for (uint32_t c = cb; c < ce; c++) A::fma(acc, A::kload(ks, (size_t)c * n + r, a.plane), uu[c]);
                    }
                }
                __syncwarp();
                // the chunk's last element (a CTA's last chunk may be short) releases the slot
                if (lane == 0 && (jc + 1 == E || i + 1 == cnt)) mbar_arrive(&empty[s]);
            }
            if (!gatherer && rvalid) pbuf(par)[(cg - 1) * n + r] = acc;
            if (gatherer && rvalid && inext < cnt) {
                const UT x = stage_s<A>(u_n, usk);
                ubuf(par ^ 1)[r] = x;
                if constexpr (A::kSym) ubuf(par ^ 1)[r + n] = x;
            }
            group_sync(bar_id, bar_threads);
            if (gatherer) {
                for (uint32_t c2 = 1; c2 < G.gc; c2++) {
                    if (rvalid) A::combine(acc, pbuf(par)[(c2 - 1) * n + r]);
                }
                if (rvalid && !*abort) st_hint(v + (dof_c & kDofMask), vold_c + finish_s<A>(acc, usk), keep);
                dof_c = dof_n;
                vold_c = vold_n;
                dof_n = dof_nn;
            }
            ch = chn;
            jc = jn;
            i = inext;
            chn = chnn;
            jn = jnn;
            inext = inn;
        }
        gbase += (cnt + E - 1) / E;
    }
    if (lane == 0 && *abort) atomicOr(a.err, kErrTimeout);
}

template <int NT, typename A, bool CH>
__global__ void __launch_bounds__((A::kWpgWarps + 1) * 32, 1)
    afm_wpg_kernel(SegArgs a, RingLayout L, GroupGeom G, uint32_t n_rt) {
    wpg_run<NT, A, CH, false>(a, L, G, n_rt, nullptr);
}

// All colours of a segment plan with one element size in one cooperative
// launch (one CTA per SM, all resident), a grid barrier between colours.
template <int NT, typename A, bool CH>
__global__ void __launch_bounds__((A::kWpgWarps + 1) * 32, 1)
    afm_wpg_fused_kernel(SegArgs a, RingLayout L, GroupGeom G, uint32_t n_rt, const __grid_constant__ ColourTable T) {
    wpg_run<NT, A, CH, true>(a, L, G, n_rt, &T);
}

// ---- thread per element (n <= 16) ------------------------------------------
// A unit is 32 elements; its Ke is entry-major: entry k = r*n + c of element
// lane at k*32 + lane; its map entry i of element lane at i*32 + lane.
template <int NT, typename A, bool DUP>
__global__ void __launch_bounds__(9 * 32, 1) afm_tpe_kernel(SegArgs a, RingLayout L, uint32_t n_rt) {
    using KT = typename A::KT;
    using UT = typename A::UT;
    using VT = typename A::VT;
    constexpr int NM = NT ? NT : 16;
    const uint32_t n = NT ? NT : n_rt;
    extern __shared__ __align__(128) unsigned char smem[];
    uint64_t* full = reinterpret_cast<uint64_t*>(smem + L.bars_offset());
    uint64_t* empty = full + L.stages;
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t NW = L.warps, S = L.stages;

    const uint32_t per = a.units / gridDim.x, rem = a.units % gridDim.x;
    const uint32_t begin = blockIdx.x * per + min(blockIdx.x, rem);
    const uint32_t cnt = per + (blockIdx.x < rem ? 1u : 0u);

    if (threadIdx.x == 0) {
        for (uint32_t s = 0; s < S; s++) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();

    if (warp == NW) {
        if (lane == 0) {
            const uint64_t pol = l2_evict_first_policy();
            uint32_t issued = 0;
            for (uint32_t i = 0; i < cnt; i++) {
                const uint32_t s = i % S;
                if (i >= S && !mbar_wait(&empty[s], ((i / S) - 1) & 1, a.wait_ns)) {
                    atomicOr(a.err, kErrTimeout);
                    break;
                }
                mbar_arrive_expect_tx(&full[s], a.copy_bytes);
                bulk_load(smem + (size_t)s * L.slot_bytes, a.ke + (size_t)(begin + i) * a.unit_bytes, a.copy_bytes,
                          &full[s], pol);
                issued = i + 1;
            }
            allow_dependent_launch();
            drain_ring(full, S, issued);
        }
        return;
    }
    wait_prior_grid();
    if (a.probe && blockIdx.x == 0 && warp == 0 && !probe_wait(a.probe, a.wait_ns)) {
        if (lane == 0) atomicOr(a.err, kErrTimeout);
        return;  // this warp's elements are left out; the producer's waits for their slots run out too
    }

    const int usk = load_uscale<A>(a.umax);
    const VT* __restrict__ u = static_cast<const VT*>(a.u);
    VT* __restrict__ v = static_cast<VT*>(a.v);
    uint32_t dof_c[NM], dof_n[NM];
    VT u_c[NM], vold_c[NM];

    auto valid = [&](uint32_t i) { return (size_t)(begin + i) * kTpeWidth + lane < a.count; };
    auto load_map = [&](uint32_t i, uint32_t* d) {
        const uint32_t* mp = a.map + (size_t)(begin + i) * n * kTpeWidth + lane;
#pragma unroll
        for (int c = 0; c < NM; c++) d[c] = (c < (int)n) ? __ldg(mp + (size_t)c * kTpeWidth) : 0u;
    };
    auto load_uv = [&](const uint32_t* d, VT* uu, VT* vv, bool ok) {
#pragma unroll
        for (int c = 0; c < NM; c++) {
            uu[c] = VT(0);
            vv[c] = VT(0);
            if (c < (int)n && ok) {
                uu[c] = load_u(u, d[c], a.bc_mode);
                if (!DUP) vv[c] = v[d[c] & kDofMask];
            }
        }
    };

    uint32_t i = warp;
    if (i < cnt) {
        load_map(i, dof_c);
        load_uv(dof_c, u_c, vold_c, valid(i));
        if (i + NW < cnt) load_map(i + NW, dof_n);
    }
    for (; i < cnt; i += NW) {
        const bool ok = valid(i);
        VT u_n[NM], vold_n[NM];
        uint32_t dof_nn[NM];
#pragma unroll
        for (int c = 0; c < NM; c++) dof_nn[c] = 0u;
        const bool has_n = i + NW < cnt;
        if (has_n) load_uv(dof_n, u_n, vold_n, valid(i + NW));
        if (i + 2 * NW < cnt) load_map(i + 2 * NW, dof_nn);

        const uint32_t s = i % S;
        if (!__all_sync(0xffffffffu, mbar_wait(&full[s], (i / S) & 1, a.wait_ns))) {  // one verdict per warp
            if (lane == 0) atomicOr(a.err, kErrTimeout);
            break;
        }
        const unsigned char* ks = smem + (size_t)s * L.slot_bytes;
        UT us[NM];
#pragma unroll
        for (int c = 0; c < NM; c++) us[c] = stage_s<A>(u_c[c], usk);
        typename A::Acc acc[NM];
#pragma unroll
        for (int r = 0; r < NM; r++) {
            acc[r] = A::zero();
            if (r < (int)n) {
#pragma unroll
                for (int c = 0; c < NM; c++)
                    if (c < (int)n) A::fma(acc[r], A::kload(ks, (size_t)(r * n + c) * kTpeWidth + lane, a.plane), us[c]);
            }
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[s]);

        if (ok) {
#pragma unroll
            for (int r = 0; r < NM; r++) {
                if (r < (int)n) {
                    const uint32_t d = dof_c[r] & kDofMask;
                    if (!DUP)
                        v[d] = vold_c[r] + finish_s<A>(acc[r], usk);
                    else
                        v[d] = v[d] + finish_s<A>(acc[r], usk);
                }
            }
        }
#pragma unroll
        for (int c = 0; c < NM; c++) {
            dof_c[c] = dof_n[c];
            dof_n[c] = dof_nn[c];
            if (has_n) {
                u_c[c] = u_n[c];
                vold_c[c] = vold_n[c];
            }
        }
    }
}

}  // namespace afm
