// tg_device.cuh -- device-side building blocks shared by the pairwise kernels.
//
//  * exact IEEE double helpers (no FMA contraction) so the FP64 kernels keep
//    the reference's per-operation rounding (tupan/lib/src/*_kernel_common.h);
//  * packed f32x2 arithmetic (Blackwell FADD2/FMUL2/FFMA2) for the split-FP32
//    kernels, which evaluate two j-particles per instruction;
//  * mbarrier + cp.async.bulk (TMA bulk copy, no multicast) wrappers with
//    bounded waits for staging j-tiles into shared memory.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace tg {

// ---------------------------------------------------------------------------
// Status bits written by kernels into the per-call device status word.
// ---------------------------------------------------------------------------
enum : unsigned {
    ST_MBAR_TIMEOUT = 1u << 0,   // a bounded mbarrier wait gave up
    ST_KEPLER_CAP = 1u << 1,     // Sakura: Kepler retry cap reached
};

// ---------------------------------------------------------------------------
// Exact double arithmetic: every operation rounds once, never contracted.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double ddiv(double a, double b) { return __ddiv_rn(a, b); }
__device__ __forceinline__ double dsqrt(double a) { return __dsqrt_rn(a); }
// a*a + b*b + c*c evaluated left to right, as `rx * rx + ry * ry + rz * rz`
__device__ __forceinline__ double ddot3(double a0, double a1, double a2,
                                        double b0, double b1, double b2) {
    return dadd(dadd(dmul(a0, b0), dmul(a1, b1)), dmul(a2, b2));
}

// ---------------------------------------------------------------------------
// Packed float pairs.  Lane .x holds an even j, lane .y the next odd j.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float2 f2(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) {
    return __fadd2_rn(a, make_float2(-b.x, -b.y));
}
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
// c - a*b
__device__ __forceinline__ float2 fnma2(float2 a, float2 b, float2 c) {
    return __ffma2_rn(make_float2(-a.x, -a.y), b, c);
}

// Hardware reciprocal square root (MUFU.RSQ, ~2 ulp); the kernels may add
// one Newton step y <- y + y*(1/2 - (s/2) y^2) for ~1 ulp.
__device__ __forceinline__ float rsqrt_hw(float s) {
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(s));
    return y;
}

// Hardware reciprocal (MUFU.RCP, ~1 ulp): 1/s from the XU pipe instead of
// y*y on the FMA pipe.
__device__ __forceinline__ float rcp_hw(float s) {
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(s));
    return y;
}

// Pair exclusion: lane is kept when r != 0, i.e. any of dx, dy, dz is
// nonzero.  The split-FP32 kernels store every coordinate with -0 turned
// into +0, so the difference of two equal coordinates is +0 (all bits zero)
// and a nonzero difference is never -0; one 3-input OR then decides.
// Equivalent to the reference's `r2 > 0` except for |dr| below 1e-19, where
// the FP32 square underflows.
__device__ __forceinline__ bool nonzero3(float a, float b, float c) {
    return (__float_as_uint(a) | __float_as_uint(b) | __float_as_uint(c)) != 0u;
}

// ---------------------------------------------------------------------------
// Compensated accumulator: value = hi + lo, updated once per j-block with
// Kahan/Neumaier-free TwoSum-lite (Fast2Sum needs |hi| >= |x|; plain Kahan is
// used instead, which holds regardless of magnitudes).
// ---------------------------------------------------------------------------
struct Comp {
    float s, c;   // running sum and (negated) lost low part
};
__device__ __forceinline__ void comp_add(Comp &k, float x) {
    float y = __fsub_rn(x, k.c);
    float t = __fadd_rn(k.s, y);
    k.c = __fsub_rn(__fsub_rn(t, k.s), y);
    k.s = t;
}
__device__ __forceinline__ double comp_value(const Comp &k) {
    return (double)k.s - (double)k.c;
}

// ---------------------------------------------------------------------------
// Double-single ("float-float") arithmetic: a value is hi + lo with
// |lo| <= ulp(hi)/2, about 48 significant bits.  Built from the error-free
// transformations of Knuth (TwoSum), Dekker (Fast2Sum) and the FMA form of
// TwoProduct; every operation is an explicit round-to-nearest intrinsic so
// the compiler cannot contract or reassociate them.
// ---------------------------------------------------------------------------
struct DS {
    float hi, lo;
};
__device__ __forceinline__ DS ds_from(double x) {
    DS r;
    r.hi = __double2float_rn(x);
    r.lo = __double2float_rn(x - (double)r.hi);
    return r;
}
// s + e = a + b exactly (any magnitudes)
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
// s + e = a + b exactly, given |a| >= |b| (or a == 0)
__device__ __forceinline__ void fast_two_sum(float a, float b, float &s, float &e) {
    s = __fadd_rn(a, b);
    e = __fsub_rn(b, __fsub_rn(s, a));
}
__device__ __forceinline__ DS ds_add(DS a, DS b) {
    float s, e;
    two_sum(a.hi, b.hi, s, e);
    e = __fadd_rn(e, __fadd_rn(a.lo, b.lo));
    DS r;
    fast_two_sum(s, e, r.hi, r.lo);
    return r;
}
__device__ __forceinline__ DS ds_neg(DS a) { return DS{-a.hi, -a.lo}; }
__device__ __forceinline__ DS ds_mul(DS a, DS b) {
    const float p = __fmul_rn(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.hi, -p);
    e = __fmaf_rn(a.hi, b.lo, e);
    e = __fmaf_rn(a.lo, b.hi, e);
    DS r;
    fast_two_sum(p, e, r.hi, r.lo);
    return r;
}
// 1/sqrt(s) for s > 0: the hardware estimate refined by one Newton step
// whose residual 1 - s y0^2 is formed in double-single (error ~2^-43).
__device__ __forceinline__ DS ds_rsqrt(DS s) {
    float y0;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y0) : "f"(s.hi));
    DS y2;
    y2.hi = __fmul_rn(y0, y0);
    y2.lo = __fmaf_rn(y0, y0, -y2.hi);
    const DS q = ds_mul(s, y2);
    const DS r = ds_add(DS{1.0f, 0.0f}, ds_neg(q));
    const float corr = __fmul_rn(__fmul_rn(y0, r.hi), 0.5f);
    DS y;
    fast_two_sum(y0, corr, y.hi, y.lo);
    return y;
}
__device__ __forceinline__ double ds_value(DS a) { return (double)a.hi + (double)a.lo; }

// The same operations on two independent values per instruction (packed
// f32x2): lane .x and lane .y are separate double-single numbers.
struct DS2 {
    float2 hi, lo;
};
__device__ __forceinline__ float2 neg2(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ void two_sum2(float2 a, float2 b, float2 &s, float2 &e) {
    s = __fadd2_rn(a, b);
    const float2 bb = __fadd2_rn(s, neg2(a));
    e = __fadd2_rn(__fadd2_rn(a, neg2(__fadd2_rn(s, neg2(bb)))), __fadd2_rn(b, neg2(bb)));
}
__device__ __forceinline__ void fast_two_sum2(float2 a, float2 b, float2 &s, float2 &e) {
    s = __fadd2_rn(a, b);
    e = __fadd2_rn(b, neg2(__fadd2_rn(s, neg2(a))));
}
__device__ __forceinline__ DS2 ds2_add(DS2 a, DS2 b) {
    float2 s, e;
    two_sum2(a.hi, b.hi, s, e);
    e = __fadd2_rn(e, __fadd2_rn(a.lo, b.lo));
    DS2 r;
    fast_two_sum2(s, e, r.hi, r.lo);
    return r;
}
__device__ __forceinline__ DS2 ds2_neg(DS2 a) { return DS2{neg2(a.hi), neg2(a.lo)}; }
__device__ __forceinline__ DS2 ds2_mul(DS2 a, DS2 b) {
    const float2 p = __fmul2_rn(a.hi, b.hi);
    float2 e = __ffma2_rn(a.hi, b.hi, neg2(p));
    e = __ffma2_rn(a.hi, b.lo, e);
    e = __ffma2_rn(a.lo, b.hi, e);
    DS2 r;
    fast_two_sum2(p, e, r.hi, r.lo);
    return r;
}
__device__ __forceinline__ DS2 ds2_rsqrt(DS2 s) {
    float2 y0;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y0.x) : "f"(s.hi.x));
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y0.y) : "f"(s.hi.y));
    DS2 y2;
    y2.hi = __fmul2_rn(y0, y0);
    y2.lo = __ffma2_rn(y0, y0, neg2(y2.hi));
    const DS2 q = ds2_mul(s, y2);
    const DS2 r = ds2_add(DS2{make_float2(1.0f, 1.0f), make_float2(0.0f, 0.0f)}, ds2_neg(q));
    const float2 corr = __fmul2_rn(__fmul2_rn(y0, r.hi), make_float2(0.5f, 0.5f));
    DS2 y;
    fast_two_sum2(y0, corr, y.hi, y.lo);
    return y;
}

// ---------------------------------------------------------------------------
// mbarrier / bulk-copy PTX (sm_90+ forms, valid on sm_103a).
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_addr(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;"
                 ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
}
// Global -> shared bulk copy completing on `bar`.  dst, src 16-byte aligned,
// bytes a multiple of 16.
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
        ::"r"(smem_addr(dst)), "l"(src), "r"(bytes), "r"(smem_addr(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok) : "r"(smem_addr(bar)), "r"(parity) : "memory");
    return ok != 0;
}
// Bounded wait: gives up after `limit` polls and reports false.  A poll of
// a phase that has not completed suspends the thread for ~3.8 us on GB300
// (measured), so the default 2^18 polls give up after about one second; a
// j-tile copy normally lands within microseconds.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, uint32_t limit = (1u << 18)) {
    for (uint32_t it = 0; it < limit; ++it) {
        if (mbar_try_wait(bar, parity)) return true;
    }
    return false;
}

}  // namespace tg
