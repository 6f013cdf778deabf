// tg_ds32.cu -- split-FP32 ("double-single") pairwise kernels.
//
// Three families:
//   * the unordered stream-K kernels below (Phi below 2^31 pairs,
//     SnapCrackle, Tstep, PNAcc; Acc and AccJerk of the segmented ensembles
//     and of the no-allocation entry point);
//   * the ordered kernels (ds32_ord: Acc and AccJerk from 2^24 pairs, Phi
//     from 2^31): spatially sorted sets, single-float separations on far
//     blocks, cost-weighted stream-K, recompute of strongly cancelling
//     particles (Acc, AccJerk);
//   * the double-single kernel ds32_exact: Acc and AccJerk below 2^24 pairs
//     and at TG_PREC_DS32X, the Acc adjoint, and that recompute.
//
// Data layout in HBM (workspace, written by ds32_prepare once per call):
//   the j-set as pair-interleaved float records.  Record p holds j = 2p and
//   j = 2p+1; field f occupies floats [2f, 2f+1] of the record, so one
//   16-byte shared-memory load returns two fields for both j.  Positions are
//   stored as hi/lo float pairs (x = hi + lo to ~48 bits), so the difference
//   of two close positions, (xi_hi - xj_hi) + (xi_lo - xj_lo), keeps its
//   relative accuracy; velocities, accelerations, masses and softenings are
//   single floats.  The set is padded to whole tiles with massless particles
//   (and, for Tstep, an explicit valid flag).
//
// Work decomposition (stream-K): the (i-tile x j-tile) grid of units is cut
// into gridDim.x contiguous ranges of equal length, one per CTA, with
// gridDim.x = SMs x resident CTAs per SM, so every SM gets the same number of
// interactions for any N.  An i-tile covered by several CTAs is finished by
// the last of them to arrive (atomic ticket, no waiting), which adds the
// FP64 partials of all contributors in CTA order: the result is
// deterministic.
//
// Pipeline: one thread issues cp.async.bulk (TMA bulk copy, no multicast)
// of each j-tile into a 3-stage shared-memory ring completing on an mbarrier;
// all threads wait with a bounded poll and raise a status bit on timeout.
//
// Arithmetic: two i-particles per thread (one for small problems and for
// SnapCrackle and PNAcc), two j-particles per packed f32x2 instruction
// (FADD2/FMUL2/FFMA2); 1/sqrt from MUFU.RSQ and, where used, 1/s from
// MUFU.RCP (a Newton step on rsqrt is a compile-time option,
// TG_DS32_REFINE); per-thread sums run in FP32 over 64 j and are then folded
// into Kahan-compensated accumulators.  The roofline is the FP32 pipe (FFMA2
// issue).
#include <atomic>
#include <mutex>
#include <type_traits>
#include <vector>

#include "tg_device.cuh"
#include "tg_internal.h"
#include "tg_pn_terms.cuh"

namespace tg {

#ifndef TG_DS32_THREADS
#define TG_DS32_THREADS 256
#endif
constexpr int DS_THREADS = TG_DS32_THREADS;   // threads per CTA
#ifndef TG_DS32_TILE
#define TG_DS32_TILE 512
#endif
#ifndef TG_DS32_STAGES
#define TG_DS32_STAGES 3
#endif
#ifndef TG_DS32_FOLD
#define TG_DS32_FOLD 64
#endif
#ifndef TG_DS32_UNROLL
#define TG_DS32_UNROLL 4   // j-records per unrolled block (kernels may override)
#endif
constexpr int DS_TILE = TG_DS32_TILE;     // j-particles per tile
constexpr int DS_PAIRS = DS_TILE / 2;
constexpr int DS_STAGES = TG_DS32_STAGES;
constexpr int DS_FOLD = TG_DS32_FOLD;     // j per compensated fold
constexpr int DS_FOLD_PAIRS = DS_FOLD / 2;

// ---------------------------------------------------------------------------
// Record formats (floats per j, even).
// ---------------------------------------------------------------------------
enum RecField {
    R_XH = 0, R_YH, R_ZH, R_XL, R_YL, R_ZL,   // positions hi / lo
};

struct DsArgs {
    PairArgs p;
    const float4 *rec;   // packed j-records
    double *part;        // [gridDim.x][2][IPT][NP][DS_THREADS]
    int *ticket;         // [NIT]
    const float *tile_e2;  // [NJT] common j softening per tile or NaN; may be null
    long long nit, njt;  // i-tiles, j-tiles
};

__device__ __forceinline__ float fzero_norm(float x) { return x + 0.0f; }  // -0 -> +0

__device__ __forceinline__ void split_ds(double x, float &hi, float &lo) {
    hi = __double2float_rn(x);
    lo = __double2float_rn(x - (double)hi);
    hi = fzero_norm(hi);
    lo = fzero_norm(lo);
}

// ---------------------------------------------------------------------------
// Pack kernel: one thread per (record, lane); JF floats per j.
//   fields: 0..5 position hi/lo, then the kernel's list of extra fields.
// ---------------------------------------------------------------------------
struct PackSpec {
    int jf;            // floats per j in the record (even)
    int nextra;        // extra fields after the 6 position floats
    int extra[12];     // tg::Field of each extra field, or -1 = valid flag, -2 = pad
};

__global__ void ds32_pack(PSet J, size_t nj, size_t npairs, PackSpec ps, float *rec) {
    const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= npairs * 2) return;
    const size_t p = t >> 1;
    const int lane = (int)(t & 1);
    const size_t j = 2 * p + lane;
    const bool valid = j < nj;
    float *r = rec + p * (size_t)(2 * ps.jf);
    float h, l;
    for (int c = 0; c < 3; ++c) {
        split_ds(valid ? J.f[F_RX + c][j] : 0.0, h, l);
        r[2 * (R_XH + c) + lane] = h;
        r[2 * (R_XL + c) + lane] = l;
    }
    for (int q = 0; q < ps.nextra; ++q) {
        const int f = ps.extra[q];
        float v;
        if (f == -1) v = valid ? 1.0f : 0.0f;
        else if (f == -2) v = 0.0f;
        else if (f == F_E2) v = valid ? __double2float_rn(J.f[f][j]) : 1.0f;
        else v = valid ? __double2float_rn(J.f[f][j]) : 0.0f;
        r[2 * (6 + q) + lane] = v;
    }
}

// Fused per-call preparation, one CTA of DS_TILE threads per j-tile, one j
// per thread: the tile's records (as ds32_pack), its softening flag
// (tile_e2[t]: the common float e2 of its valid particles or NaN; skipped if
// tile_e2 is null), and, grid-stride, the zeroed stream-K tickets.  Every
// thread issues its loads at once, so the launch costs about one memory
// round trip.
struct PrepArgs {
    int *ticket; long long nticket;
};
__global__ void __launch_bounds__(DS_TILE) ds32_prepare(PSet J, size_t nj, PackSpec ps, float *rec, float *tile_e2,
                                                        PrepArgs z) {
    const size_t tile = blockIdx.x;
    const int q = threadIdx.x;
    const size_t p = tile * DS_PAIRS + (q >> 1);
    const int lane = q & 1;
    const size_t j = 2 * p + lane;
    const bool valid = j < nj;
    float *r = rec + p * (size_t)(2 * ps.jf);
    float h, l;
    for (int c = 0; c < 3; ++c) {
        split_ds(valid ? J.f[F_RX + c][j] : 0.0, h, l);
        r[2 * (R_XH + c) + lane] = h;
        r[2 * (R_XL + c) + lane] = l;
    }
    for (int e = 0; e < ps.nextra; ++e) {
        const int f = ps.extra[e];
        float v;
        if (f == -1) v = valid ? 1.0f : 0.0f;
        else if (f == -2) v = 0.0f;
        else if (f == F_E2) v = valid ? __double2float_rn(J.f[f][j]) : 1.0f;
        else v = valid ? __double2float_rn(J.f[f][j]) : 0.0f;
        r[2 * (6 + e) + lane] = v;
    }
    if (tile_e2 != nullptr) {   // uniform softening of the tile (block-uniform branch)
        // the tile's first particle, j = tile * DS_TILE, is always valid
        __shared__ unsigned first;
        const unsigned mine = valid ? __float_as_uint(__double2float_rn(J.f[F_E2][j])) : 0u;
        if (q == 0) first = mine;
        __syncthreads();
        const bool same = __syncthreads_and(!valid || mine == first);
        if (q == 0) {
            const float v = __uint_as_float(first);
            tile_e2[tile] = (same && v == v) ? v : __uint_as_float(0x7fc00000u);
        }
    }
    const size_t g = (size_t)blockIdx.x * blockDim.x + threadIdx.x, stride = (size_t)gridDim.x * blockDim.x;
    for (size_t x = g; x < (size_t)z.nticket; x += stride) z.ticket[x] = 0;
}

// ---------------------------------------------------------------------------
// i-side state helpers
// ---------------------------------------------------------------------------
struct IPos {
    float2 xh, yh, zh, xl, yl, zl;
};
__device__ __forceinline__ void load_pos(const PairArgs &a, size_t i, IPos &q) {
    float h, l;
    split_ds(a.I.f[F_RX][i], h, l); q.xh = f2(h); q.xl = f2(l);
    split_ds(a.I.f[F_RY][i], h, l); q.yh = f2(h); q.yl = f2(l);
    split_ds(a.I.f[F_RZ][i], h, l); q.zh = f2(h); q.zl = f2(l);
}
// dr = (i_hi - j_hi) + (i_lo - j_lo) for both lanes.
__device__ __forceinline__ void pair_dr(const IPos &q, float2 jxh, float2 jyh, float2 jzh,
                                        float2 jxl, float2 jyl, float2 jzl,
                                        float2 &dx, float2 &dy, float2 &dz) {
    dx = add2(sub2(q.xh, jxh), sub2(q.xl, jxl));
    dy = add2(sub2(q.yh, jyh), sub2(q.yl, jyl));
    dz = add2(sub2(q.zh, jzh), sub2(q.zl, jzl));
}
// Masked 1/sqrt(s) per lane (Newton-refined if REFINE); zero where dr == 0.
// 1/sqrt(s) and 1/s per lane from the XU pipe; both zero where dr == 0
// (the excluded lane gets s = +inf, whose reciprocal and rsqrt are 0).
__device__ __forceinline__ void inv_r_r2(float2 s, float2 dx, float2 dy, float2 dz, float2 &y, float2 &y2) {
    const float inf = __int_as_float(0x7f800000);
    const float sx = nonzero3(dx.x, dy.x, dz.x) ? s.x : inf;
    const float sy = nonzero3(dx.y, dy.y, dz.y) ? s.y : inf;
    y = make_float2(rsqrt_hw(sx), rsqrt_hw(sy));
    y2 = make_float2(rcp_hw(sx), rcp_hw(sy));
}

template <bool REFINE>
__device__ __forceinline__ float2 inv_r(float2 s, float2 dx, float2 dy, float2 dz) {
    float2 y;
    y.x = nonzero3(dx.x, dy.x, dz.x) ? rsqrt_hw(s.x) : 0.0f;
    y.y = nonzero3(dx.y, dy.y, dz.y) ? rsqrt_hw(s.y) : 0.0f;
    if (REFINE) {
        const float2 hs = mul2(s, f2(0.5f));
        const float2 t = mul2(hs, y);
        const float2 c = fnma2(t, y, f2(0.5f));
        y = fma2(y, c, y);
    }
    return y;
}

__device__ __forceinline__ float2 lo2(float4 q) { return make_float2(q.x, q.y); }
__device__ __forceinline__ float2 hi2(float4 q) { return make_float2(q.z, q.w); }

// ---------------------------------------------------------------------------
// Kernels.  Each provides, for IPT i-particles per thread:
//   IPT, JF (floats per j), NQ (float4 per record), NP (FP64 partials per i)
//   IS                          per-i state (position, sums)
//   load(IS&, args, i)          read and split one i-particle, clear sums
//   step(IS (&)[IPT], rec)      one record (two j) against the IPT i-particles
//   fold(IS&)                   fold the FP32 lane sums into compensated sums
//   partials(const IS&, double*), combine(double*, const double*)
//   store(const double*, args, i)   final outputs from the FP64 partials
//   pack()                      j-record field list
// ---------------------------------------------------------------------------
template <int IPT_, bool REFINE>
struct AccDS {
    static constexpr int IPT = IPT_, JF = 8, NQ = 4, NP = 3;
    static constexpr bool UE2 = true;
    struct IS { IPos q; float2 e; float2 a[3]; Comp c[3]; };
    __device__ static void load(IS &s, const PairArgs &a, size_t i) {
        load_pos(a, i, s.q);
        s.e = f2(__double2float_rn(a.I.f[F_E2][i]));
        for (int k = 0; k < 3; ++k) { s.a[k] = f2(0.f); s.c[k] = Comp{0.f, 0.f}; }
    }
    // record: {xh,yh} {zh,xl} {yl,zl} {m,e2}.  UE: every pair of the tile
    // has the softening E (= ie2 + je2 for all pairs), so the add is hoisted.
    template <bool UE>
    __device__ __forceinline__ static void step(IS (&S)[IPT], const float4 *R, float2 E) {
        const float4 q0 = R[0], q1 = R[1], q2 = R[2], q3 = R[3];
#pragma unroll
        for (int u = 0; u < IPT; ++u) {
            IS &s = S[u];
            float2 dx, dy, dz;
            pair_dr(s.q, lo2(q0), hi2(q0), lo2(q1), hi2(q1), lo2(q2), hi2(q2), dx, dy, dz);
            const float2 e2 = UE ? E : add2(s.e, hi2(q3));
            const float2 ss = fma2(dx, dx, fma2(dy, dy, fma2(dz, dz, e2)));
            // 1/r^2 from y*y here: with one more MUFU per pair Acc would be
            // XU-bound (18 packed FP32 ops vs 4 MUFU per two pairs).  With a
            // uniform softening E > 1e-20 no mask is needed: a pair at r = 0
            // has dr = +0, so its finite m y^3 adds exactly nothing, as the
            // masked form does.
            const float2 y = UE ? make_float2(rsqrt_hw(ss.x), rsqrt_hw(ss.y)) : inv_r<REFINE>(ss, dx, dy, dz);
            const float2 y2 = mul2(y, y);
            const float2 mr3 = mul2(mul2(lo2(q3), y), y2);
            s.a[0] = fnma2(mr3, dx, s.a[0]);
            s.a[1] = fnma2(mr3, dy, s.a[1]);
            s.a[2] = fnma2(mr3, dz, s.a[2]);
        }
    }
    __device__ static void fold(IS &s) {
        for (int k = 0; k < 3; ++k) { comp_add(s.c[k], __fadd_rn(s.a[k].x, s.a[k].y)); s.a[k] = f2(0.f); }
    }
    __device__ static void partials(const IS &s, double *p) { for (int k = 0; k < 3; ++k) p[k] = comp_value(s.c[k]); }
    __device__ static void combine(double *acc, const double *p) { for (int k = 0; k < 3; ++k) acc[k] += p[k]; }
    __device__ static void store(const double *p, const PairArgs &a, size_t i) {
        for (int k = 0; k < 3; ++k) a.out[k][i] = p[k];
    }
    static PackSpec pack() { return PackSpec{8, 2, {F_M, F_E2}}; }
};

template <int IPT_, bool REFINE>
struct PhiDS {
    static constexpr int IPT = IPT_, JF = 8, NQ = 4, NP = 1;
    static constexpr bool UE2 = true;
    struct IS { IPos q; float2 e; float2 p; Comp c; };
    __device__ static void load(IS &s, const PairArgs &a, size_t i) {
        load_pos(a, i, s.q);
        s.e = f2(__double2float_rn(a.I.f[F_E2][i]));
        s.p = f2(0.f); s.c = Comp{0.f, 0.f};
    }
    template <bool UE>
    __device__ __forceinline__ static void step(IS (&S)[IPT], const float4 *R, float2 E) {
        const float4 q0 = R[0], q1 = R[1], q2 = R[2], q3 = R[3];
#pragma unroll
        for (int u = 0; u < IPT; ++u) {
            IS &s = S[u];
            float2 dx, dy, dz;
            pair_dr(s.q, lo2(q0), hi2(q0), lo2(q1), hi2(q1), lo2(q2), hi2(q2), dx, dy, dz);
            const float2 e2 = UE ? E : add2(s.e, hi2(q3));
            const float2 ss = fma2(dx, dx, fma2(dy, dy, fma2(dz, dz, e2)));
            const float2 y = inv_r<REFINE>(ss, dx, dy, dz);
            s.p = fnma2(lo2(q3), y, s.p);
        }
    }
    __device__ static void fold(IS &s) { comp_add(s.c, __fadd_rn(s.p.x, s.p.y)); s.p = f2(0.f); }
    __device__ static void partials(const IS &s, double *p) { p[0] = comp_value(s.c); }
    __device__ static void combine(double *acc, const double *p) { acc[0] += p[0]; }
    __device__ static void store(const double *p, const PairArgs &a, size_t i) { a.out[0][i] = p[0]; }
    static PackSpec pack() { return PackSpec{8, 2, {F_M, F_E2}}; }
};

// The unordered split-FP32 AccJerk (ensembles and the no-allocation entry
// point).  Compensated sums stay in registers (shared-memory sums measured
// 0.3% slower); eight records per unrolled block (0.8% faster than four).
template <int IPT_, bool REFINE>
struct AccJerkDS {
    static constexpr int IPT = IPT_, JF = 12, NQ = 6, NP = 6;
    static constexpr bool UE2 = false;
    static constexpr int UNROLL = 8;
    struct IS { IPos q; float2 u, v, w, e; float2 a[6]; Comp c[6]; };
    __device__ static void load(IS &s, const PairArgs &a, size_t i) {
        load_pos(a, i, s.q);
        s.u = f2(__double2float_rn(a.I.f[F_VX][i]));
        s.v = f2(__double2float_rn(a.I.f[F_VY][i]));
        s.w = f2(__double2float_rn(a.I.f[F_VZ][i]));
        s.e = f2(__double2float_rn(a.I.f[F_E2][i]));
        for (int k = 0; k < 6; ++k) { s.a[k] = f2(0.f); s.c[k] = Comp{0.f, 0.f}; }
    }
    __device__ __forceinline__ static void step(IS (&S)[IPT], const float4 *R) {
        step<false>(S, R, f2(0.f));
    }
    // record: {xh,yh} {zh,xl} {yl,zl} {vx,vy} {vz,m} {e2,pad}
    template <bool UE>
    __device__ __forceinline__ static void step(IS (&S)[IPT], const float4 *R, float2 E) {
        const float4 q0 = R[0], q1 = R[1], q2 = R[2], q3 = R[3], q4 = R[4];
        const float4 q5 = UE ? q4 : R[5];
#pragma unroll
        for (int u = 0; u < IPT; ++u) {
            IS &s = S[u];
            float2 dx, dy, dz;
            pair_dr(s.q, lo2(q0), hi2(q0), lo2(q1), hi2(q1), lo2(q2), hi2(q2), dx, dy, dz);
            const float2 du = sub2(s.u, lo2(q3)), dv = sub2(s.v, hi2(q3)), dw = sub2(s.w, lo2(q4));
            const float2 e2 = UE ? E : add2(s.e, lo2(q5));
            const float2 ss = fma2(dx, dx, fma2(dy, dy, fma2(dz, dz, e2)));
            float2 y, y2;
            if (REFINE) {
                y = inv_r<true>(ss, dx, dy, dz);
                y2 = mul2(y, y);
            } else {
                inv_r_r2(ss, dx, dy, dz, y, y2);
            }
            const float2 mr3 = mul2(mul2(hi2(q4), y), y2);
            const float2 rv = fma2(dx, du, fma2(dy, dv, mul2(dz, dw)));
            const float2 al = mul2(mul2(rv, y2), f2(3.0f));
            const float2 tu = fnma2(al, dx, du), tv = fnma2(al, dy, dv), tw = fnma2(al, dz, dw);
            s.a[0] = fnma2(mr3, dx, s.a[0]);
            s.a[1] = fnma2(mr3, dy, s.a[1]);
            s.a[2] = fnma2(mr3, dz, s.a[2]);
            s.a[3] = fnma2(mr3, tu, s.a[3]);
            s.a[4] = fnma2(mr3, tv, s.a[4]);
            s.a[5] = fnma2(mr3, tw, s.a[5]);
        }
    }
    __device__ static void fold(IS &s) {
        for (int k = 0; k < 6; ++k) { comp_add(s.c[k], __fadd_rn(s.a[k].x, s.a[k].y)); s.a[k] = f2(0.f); }
    }
    __device__ static void partials(const IS &s, double *p) { for (int k = 0; k < 6; ++k) p[k] = comp_value(s.c[k]); }
    __device__ static void combine(double *acc, const double *p) { for (int k = 0; k < 6; ++k) acc[k] += p[k]; }
    __device__ static void store(const double *p, const PairArgs &a, size_t i) {
        for (int k = 0; k < 6; ++k) a.out[k][i] = p[k];
    }
    static PackSpec pack() { return PackSpec{12, 6, {F_VX, F_VY, F_VZ, F_M, F_E2, -2}}; }
};

template <int IPT_, bool REFINE>
struct TstepDS {
    static constexpr int IPT = IPT_, JF = 12, NQ = 6, NP = 2;
    static constexpr bool UE2 = false;
    struct IS { IPos q; float2 u, v, w, e, m; float eta; float2 ws; float wmax; Comp c; };
    __device__ static void load(IS &s, const PairArgs &a, size_t i) {
        load_pos(a, i, s.q);
        s.u = f2(__double2float_rn(a.I.f[F_VX][i]));
        s.v = f2(__double2float_rn(a.I.f[F_VY][i]));
        s.w = f2(__double2float_rn(a.I.f[F_VZ][i]));
        s.e = f2(__double2float_rn(a.I.f[F_E2][i]));
        s.m = f2(__double2float_rn(a.I.f[F_M][i]));
        s.eta = __double2float_rn(a.eta);
        s.ws = f2(0.f); s.c = Comp{0.f, 0.f}; s.wmax = 0.f;
    }
    // record: {xh,yh} {zh,xl} {yl,zl} {vx,vy} {vz,m} {e2,valid}
    __device__ __forceinline__ static void step(IS (&S)[IPT], const float4 *R) {
        const float4 q0 = R[0], q1 = R[1], q2 = R[2], q3 = R[3], q4 = R[4], q5 = R[5];
#pragma unroll
        for (int u = 0; u < IPT; ++u) {
            IS &s = S[u];
            float2 dx, dy, dz;
            pair_dr(s.q, lo2(q0), hi2(q0), lo2(q1), hi2(q1), lo2(q2), hi2(q2), dx, dy, dz);
            const float2 du = sub2(s.u, lo2(q3)), dv = sub2(s.v, hi2(q3)), dw = sub2(s.w, lo2(q4));
            const float2 e2 = add2(s.e, lo2(q5));
            const float2 m = add2(s.m, hi2(q4));
            const float2 ss = fma2(dx, dx, fma2(dy, dy, fma2(dz, dz, e2)));
            const float2 rv = fma2(dx, du, fma2(dy, dv, mul2(dz, dw)));
            const float2 v2 = fma2(du, du, fma2(dv, dv, mul2(dw, dw)));
            const float2 y = inv_r<REFINE>(ss, dx, dy, dz);
            const float2 q2v = mul2(y, y);
            const float2 phi = mul2(m, y);
            float2 w2 = mul2(q2v, fma2(f2(2.0f), phi, v2));
            float2 gam = mul2(q2v, fma2(mul2(f2(2.0f), q2v), phi, w2));
            float2 rw;
            rw.x = rsqrt_hw(w2.x);
            rw.y = rsqrt_hw(w2.y);
            gam = mul2(gam, mul2(f2(s.eta), rw));
            w2 = fnma2(gam, rv, w2);
            w2.x = (nonzero3(dx.x, dy.x, dz.x) && q5.z != 0.f) ? w2.x : 0.f;
            w2.y = (nonzero3(dx.y, dy.y, dz.y) && q5.w != 0.f) ? w2.y : 0.f;
            s.ws = add2(s.ws, w2);
            s.wmax = fmaxf(fmaxf(w2.x, w2.y), s.wmax);
        }
    }
    __device__ static void fold(IS &s) { comp_add(s.c, __fadd_rn(s.ws.x, s.ws.y)); s.ws = f2(0.f); }
    __device__ static void partials(const IS &s, double *p) { p[0] = comp_value(s.c); p[1] = (double)s.wmax; }
    __device__ static void combine(double *acc, const double *p) { acc[0] += p[0]; acc[1] = fmax(p[1], acc[1]); }
    __device__ static void store(const double *p, const PairArgs &a, size_t i) {
        a.out[0][i] = a.eta / sqrt(1.0 + p[0]);
        a.out[1][i] = a.eta / sqrt(1.0 + p[1]);
    }
    static PackSpec pack() { return PackSpec{12, 6, {F_VX, F_VY, F_VZ, F_M, F_E2, -1}}; }
};

template <int IPT_, bool REFINE>
struct SnapCrackleDS {
    static constexpr int IPT = IPT_, JF = 18, NQ = 9, NP = 6;
    static constexpr bool UE2 = false;
    struct IS { IPos q; float2 v[3], A[3], J[3], e; float2 o[6]; Comp c[6]; };
    __device__ static void load(IS &s, const PairArgs &a, size_t i) {
        load_pos(a, i, s.q);
        for (int k = 0; k < 3; ++k) {
            s.v[k] = f2(__double2float_rn(a.I.f[F_VX + k][i]));
            s.A[k] = f2(__double2float_rn(a.I.f[F_AX + k][i]));
            s.J[k] = f2(__double2float_rn(a.I.f[F_JX + k][i]));
        }
        s.e = f2(__double2float_rn(a.I.f[F_E2][i]));
        for (int k = 0; k < 6; ++k) { s.o[k] = f2(0.f); s.c[k] = Comp{0.f, 0.f}; }
    }
    // record: {xh,yh} {zh,xl} {yl,zl} {vx,vy} {vz,ax} {ay,az} {jx,jy} {jz,m} {e2,pad}
    __device__ __forceinline__ static void step(IS (&S)[IPT], const float4 *R) {
        const float4 q0 = R[0], q1 = R[1], q2 = R[2], q3 = R[3], q4 = R[4];
        const float4 q5 = R[5], q6 = R[6], q7 = R[7], q8 = R[8];
#pragma unroll
        for (int u = 0; u < IPT; ++u) {
            IS &s = S[u];
            float2 r[3];
            pair_dr(s.q, lo2(q0), hi2(q0), lo2(q1), hi2(q1), lo2(q2), hi2(q2), r[0], r[1], r[2]);
            float2 v[3] = {sub2(s.v[0], lo2(q3)), sub2(s.v[1], hi2(q3)), sub2(s.v[2], lo2(q4))};
            float2 A[3] = {sub2(s.A[0], hi2(q4)), sub2(s.A[1], lo2(q5)), sub2(s.A[2], hi2(q5))};
            float2 J[3] = {sub2(s.J[0], lo2(q6)), sub2(s.J[1], hi2(q6)), sub2(s.J[2], lo2(q7))};
            const float2 e2 = add2(s.e, lo2(q8));
            const float2 ss = fma2(r[0], r[0], fma2(r[1], r[1], fma2(r[2], r[2], e2)));
            const float2 rv = fma2(r[0], v[0], fma2(r[1], v[1], mul2(r[2], v[2])));
            const float2 v2 = fma2(v[0], v[0], fma2(v[1], v[1], mul2(v[2], v[2])));
            const float2 rJ = fma2(r[0], J[0], fma2(r[1], J[1], mul2(r[2], J[2])));
            const float2 rA = fma2(r[0], A[0], fma2(r[1], A[1], mul2(r[2], A[2])));
            const float2 vA = fma2(v[0], A[0], fma2(v[1], A[1], mul2(v[2], A[2])));
            const float2 y = inv_r<REFINE>(ss, r[0], r[1], r[2]);
            const float2 q2v = mul2(y, y);
            float2 al = mul2(rv, q2v);
            const float2 al2 = mul2(al, al);
            float2 be = mul2(f2(3.0f), fma2(add2(v2, rA), q2v, al2));
            float2 ga = fma2(fma2(f2(3.0f), vA, rJ), q2v, mul2(al, fnma2(f2(4.0f), al2, be)));
            al = mul2(al, f2(3.0f));
            ga = mul2(ga, f2(3.0f));
            // the reference's A - (2 al v + be r) and J - (al A + be v + ga r)
            // as chains of fused negated multiply-adds (two and three
            // operations per component instead of three and four)
            for (int k = 0; k < 3; ++k) v[k] = fnma2(al, r[k], v[k]);
            const float2 two_al = mul2(f2(2.0f), al);
            for (int k = 0; k < 3; ++k) A[k] = fnma2(two_al, v[k], fnma2(be, r[k], A[k]));
            al = mul2(al, f2(3.0f));
            be = mul2(be, f2(3.0f));
            for (int k = 0; k < 3; ++k) J[k] = fnma2(al, A[k], fnma2(be, v[k], fnma2(ga, r[k], J[k])));
            const float2 mr3 = mul2(mul2(hi2(q7), y), q2v);
            for (int k = 0; k < 3; ++k) {
                s.o[k] = fnma2(mr3, A[k], s.o[k]);
                s.o[3 + k] = fnma2(mr3, J[k], s.o[3 + k]);
            }
        }
    }
    __device__ static void fold(IS &s) {
        for (int k = 0; k < 6; ++k) { comp_add(s.c[k], __fadd_rn(s.o[k].x, s.o[k].y)); s.o[k] = f2(0.f); }
    }
    __device__ static void partials(const IS &s, double *p) { for (int k = 0; k < 6; ++k) p[k] = comp_value(s.c[k]); }
    __device__ static void combine(double *acc, const double *p) { for (int k = 0; k < 6; ++k) acc[k] += p[k]; }
    __device__ static void store(const double *p, const PairArgs &a, size_t i) {
        for (int k = 0; k < 6; ++k) a.out[k][i] = p[k];
    }
    static PackSpec pack() {
        return PackSpec{18, 12, {F_VX, F_VY, F_VZ, F_AX, F_AY, F_AZ, F_JX, F_JY, F_JZ, F_M, F_E2, -2}};
    }
};

template <int IPT_, bool REFINE>
struct PNAccDS {
    static constexpr int IPT = IPT_, JF = 12, NQ = 6, NP = 3;
    static constexpr bool UE2 = false;
    struct IS {
        IPos q; float iu, iv, iw; float2 u, v, w, e; float im, iv2; unsigned long order;
        float inv2, inv4, inv5, inv6, inv7; float2 a[3]; Comp c[3];
    };
    __device__ static void load(IS &s, const PairArgs &a, size_t i) {
        load_pos(a, i, s.q);
        const double u = a.I.f[F_VX][i], v = a.I.f[F_VY][i], w = a.I.f[F_VZ][i];
        s.iu = __double2float_rn(u); s.iv = __double2float_rn(v); s.iw = __double2float_rn(w);
        s.u = f2(s.iu); s.v = f2(s.iv); s.w = f2(s.iw);
        s.e = f2(__double2float_rn(a.I.f[F_E2][i]));
        s.im = __double2float_rn(a.I.f[F_M][i]);
        s.iv2 = __double2float_rn(u * u + v * v + w * w);
        s.order = a.order;
        s.inv2 = (float)a.inv[2]; s.inv4 = (float)a.inv[4]; s.inv5 = (float)a.inv[5];
        s.inv6 = (float)a.inv[6]; s.inv7 = (float)a.inv[7];
        for (int k = 0; k < 3; ++k) { s.a[k] = f2(0.f); s.c[k] = Comp{0.f, 0.f}; }
    }
    __device__ __forceinline__ static void lane(IS &s, float dx, float dy, float dz, float du, float dv,
                                                float dw, float y, float ju, float jv, float jw,
                                                float jm, float &ax, float &ay, float &az) {
        const float y2 = y * y;
        const float nx = dx * y, ny = dy * y, nz = dz * y;
        const float jv2 = ju * ju + jv * jv + jw * jw;
        const float ivjv = s.iu * ju + s.iv * jv + s.iw * jw;
        const float niv = nx * s.iu + ny * s.iv + nz * s.iw;
        const float njv = nx * ju + ny * jv + nz * jw;
        const float nv = nx * du + ny * dv + nz * dw;
        const float v2 = du * du + dv * dv + dw * dw;
        float A, B;
        pn_factors<float>(s.order, s.im, jm, y, s.iv2, jv2, ivjv, niv, njv, nv, v2,
                          s.inv2, s.inv4, s.inv5, s.inv6, s.inv7, A, B);
        A *= jm * y2 * y;
        B *= jm * y2;
        ax += A * dx + B * du;
        ay += A * dy + B * dv;
        az += A * dz + B * dw;
    }
    __device__ __forceinline__ static void step(IS (&S)[IPT], const float4 *R) {
        const float4 q0 = R[0], q1 = R[1], q2 = R[2], q3 = R[3], q4 = R[4], q5 = R[5];
#pragma unroll
        for (int u = 0; u < IPT; ++u) {
            IS &s = S[u];
            float2 dx, dy, dz;
            pair_dr(s.q, lo2(q0), hi2(q0), lo2(q1), hi2(q1), lo2(q2), hi2(q2), dx, dy, dz);
            const float2 du = sub2(s.u, lo2(q3)), dv = sub2(s.v, hi2(q3)), dw = sub2(s.w, lo2(q4));
            const float2 e2 = add2(s.e, lo2(q5));
            const float2 ss = fma2(dx, dx, fma2(dy, dy, fma2(dz, dz, e2)));
            const float2 y = inv_r<REFINE>(ss, dx, dy, dz);
            lane(s, dx.x, dy.x, dz.x, du.x, dv.x, dw.x, y.x, q3.x, q3.z, q4.x, q4.z,
                 s.a[0].x, s.a[1].x, s.a[2].x);
            lane(s, dx.y, dy.y, dz.y, du.y, dv.y, dw.y, y.y, q3.y, q3.w, q4.y, q4.w,
                 s.a[0].y, s.a[1].y, s.a[2].y);
        }
    }
    __device__ static void fold(IS &s) {
        for (int k = 0; k < 3; ++k) { comp_add(s.c[k], __fadd_rn(s.a[k].x, s.a[k].y)); s.a[k] = f2(0.f); }
    }
    __device__ static void partials(const IS &s, double *p) { for (int k = 0; k < 3; ++k) p[k] = comp_value(s.c[k]); }
    __device__ static void combine(double *acc, const double *p) { for (int k = 0; k < 3; ++k) acc[k] += p[k]; }
    __device__ static void store(const double *p, const PairArgs &a, size_t i) {
        for (int k = 0; k < 3; ++k) a.out[k][i] = p[k];
    }
    static PackSpec pack() { return PackSpec{12, 6, {F_VX, F_VY, F_VZ, F_M, F_E2, -2}}; }
};

// One packed step of kernel K over a j-record; UE selects the uniform-
// softening form for kernels that have it (E = the tile's common ie2 + je2).
template <class K, bool UE>
__device__ __forceinline__ void kstep(typename K::IS (&st)[K::IPT], const float4 *R, float2 E) {
    if constexpr (K::UE2) K::template step<UE>(st, R, E);
    else K::step(st, R);
}

// j-records per unrolled block: K::UNROLL if the kernel sets it, else
// TG_DS32_UNROLL.
template <class K, class = void>
struct kunroll : std::integral_constant<int, TG_DS32_UNROLL> {};
template <class K>
struct kunroll<K, decltype(void(K::UNROLL))> : std::integral_constant<int, K::UNROLL> {};



// ---------------------------------------------------------------------------
// Stream-K geometry helpers.
// ---------------------------------------------------------------------------
__device__ __forceinline__ long long unit_start(long long k, long long U, long long G) {
    return (k * U) / G;
}
__device__ __forceinline__ long long unit_owner(long long u, long long U, long long G) {
    return ((u + 1) * G - 1) / U;
}

#ifndef TG_DS32_MINB
#define TG_DS32_MINB 2
#endif

// i-tile t is finished for CTA k (units [u0, u1) of U, nju units per
// i-tile, G CTAs).  If the CTA covered all of the tile's units it stores the
// results; otherwise it hands its FP64 partials over (slot 0 for the tile it
// started in, 1 for the tile it ends in) and the last contributor to arrive,
// told by an atomic ticket (no waiting), sums every contributor's partials in
// CTA order -- a deterministic result.  store(q, p) writes the final values of
// the thread's q-th i-particle.
// CTA k owns units [k U / G, (k + 1) U / G).
struct EvenBounds {
    long long U, G;
    __device__ long long start(long long k) const { return unit_start(k, U, G); }
    __device__ long long owner(long long u) const { return unit_owner(u, U, G); }
};
// CTA k owns units [s[k], s[k + 1]); s strictly increasing, s[0] = 0, s[G] = U.
struct TableBounds {
    const long long *s;
    long long G;
    __device__ long long start(long long k) const { return s[k]; }
    __device__ long long owner(long long u) const {   // largest k with s[k] <= u
        long long lo = 0, hi = G;
        while (hi - lo > 1) {
            const long long mid = (lo + hi) >> 1;
            if (s[mid] <= u) lo = mid; else hi = mid;
        }
        return lo;
    }
};

template <class K, class B, class Store>
__device__ __forceinline__ void finish_itile(typename K::IS (&st)[K::IPT], long long t, long long nju, long long u0,
                                             long long u1, const B &bounds, long long k, double *part,
                                             int *ticket, int *s_last, Store store) {
    constexpr int IPT = K::IPT;
    const int tid = threadIdx.x;
    const long long ta = t * nju, tb = ta + nju;
    if (ta >= u0 && tb <= u1) {
#pragma unroll
        for (int q = 0; q < IPT; ++q) {
            double p[K::NP];
            K::partials(st[q], p);
            store(q, p);
        }
        return;
    }
    const int slot = (t == u0 / nju) ? 0 : 1;
    double *mine = part + ((k * 2 + slot) * IPT * K::NP) * DS_THREADS;
#pragma unroll
    for (int q = 0; q < IPT; ++q) {
        double p[K::NP];
        K::partials(st[q], p);
        for (int v = 0; v < K::NP; ++v) mine[(q * K::NP + v) * DS_THREADS + tid] = p[v];
    }
    __threadfence();
    __syncthreads();
    // contributors: the CTAs from the owner of the tile's first unit to the
    // owner of its last that own at least one unit (a cost-weighted split
    // may leave a CTA empty)
    const long long klo = bounds.owner(ta), khi = bounds.owner(tb - 1);
    auto nonempty = [&](long long kk) { return bounds.start(kk) < bounds.start(kk + 1); };
    int ncontrib = 0;
    for (long long kk = klo; kk <= khi; ++kk) ncontrib += nonempty(kk) ? 1 : 0;
    if (tid == 0) {
        const int prev = atomicAdd(&ticket[t], 1);
        *s_last = (prev == ncontrib - 1);
    }
    __syncthreads();
    if (!*s_last) return;
    // Sum the contributors' partials in CTA order; two contributors' loads
    // are in flight per step.
    __threadfence();
    auto slot_ptr = [&](long long kk) {
        const int sl = (t == bounds.start(kk) / nju) ? 0 : 1;
        return part + ((kk * 2 + sl) * IPT * K::NP) * DS_THREADS + tid;
    };
    auto next = [&](long long kk) {   // first contributor after kk, or khi + 1
        for (++kk; kk <= khi && !nonempty(kk); ++kk) {}
        return kk;
    };
    double acc[IPT][K::NP];
    {
        const double *s0 = slot_ptr(klo);
#pragma unroll
        for (int q = 0; q < IPT; ++q)
#pragma unroll
            for (int w = 0; w < K::NP; ++w) acc[q][w] = __ldcg(s0 + (q * K::NP + w) * DS_THREADS);
    }
    for (long long kk = next(klo); kk <= khi;) {
        const long long k2 = next(kk);
        const bool two = k2 <= khi;
        const double *s0 = slot_ptr(kk);
        const double *s1 = two ? slot_ptr(k2) : s0;
#pragma unroll
        for (int q = 0; q < IPT; ++q) {
            double v0[K::NP], v1[K::NP];
#pragma unroll
            for (int w = 0; w < K::NP; ++w) {
                v0[w] = __ldcg(s0 + (q * K::NP + w) * DS_THREADS);
                v1[w] = __ldcg(s1 + (q * K::NP + w) * DS_THREADS);
            }
            K::combine(acc[q], v0);
            if (two) K::combine(acc[q], v1);
        }
        kk = two ? next(k2) : k2;
    }
#pragma unroll
    for (int q = 0; q < IPT; ++q) store(q, acc[q]);
}
template <class K, int JSUB>
__global__ void __launch_bounds__(DS_THREADS, TG_DS32_MINB) ds32_streamk(DsArgs a) {
    extern __shared__ __align__(128) float4 ring[];   // [DS_STAGES][DS_PAIRS * NQ]
    __shared__ __align__(8) uint64_t full[DS_STAGES];
    __shared__ int s_last;
    constexpr int IPT = K::IPT;
    constexpr int TILE_Q = DS_PAIRS * K::NQ;
    constexpr int BI = DS_THREADS * IPT;   // i-particles per i-tile
    constexpr int UNR = kunroll<K>::value;
    // JSUB parts per j-tile (1 or 2): a unit is an i-tile x one part
    constexpr int PART_PAIRS = DS_PAIRS / JSUB;
    constexpr int PART_Q = PART_PAIRS * K::NQ;
    const long long nju = a.njt * JSUB;

    const long long U = a.nit * nju;
    const long long G = gridDim.x;
    const long long k = blockIdx.x;
    const long long u0 = unit_start(k, U, G), u1 = unit_start(k + 1, U, G);
    if (u0 >= u1) return;
    const int tid = threadIdx.x;

    if (tid == 0) {
        for (int s = 0; s < DS_STAGES; ++s) mbar_init(&full[s], 1);
        fence_mbar_init();
    }
    __syncthreads();
    auto issue = [&](long long u, int s) {
        const long long jp = u % nju;       // part jp % JSUB of j-tile jp / JSUB
        constexpr unsigned bytes = (unsigned)(PART_Q * sizeof(float4));
        mbar_expect_tx(&full[s], bytes);
        bulk_g2s(ring + s * TILE_Q, a.rec + jp * PART_Q, bytes, &full[s]);
    };
    if (tid == 0) {
        for (int s = 0; s < DS_STAGES && u0 + s < u1; ++s) issue(u0 + s, s);
    }

    const size_t last = a.p.ni - 1;
    long long t = u0 / nju;
    typename K::IS st[IPT];
#pragma unroll
    for (int q = 0; q < IPT; ++q) {
        const size_t i = (size_t)t * BI + q * DS_THREADS + tid;
        K::load(st[q], a.p, i < a.p.ni ? i : last);
    }
    // i-tile softening: the common float(ie2) of the tile, or NaN
    __shared__ unsigned s_ie2;
    auto tile_ie2 = [&]() -> float {
        if constexpr (K::UE2) {
            if (a.tile_e2 == nullptr) return __uint_as_float(0x7fc00000u);
            if (tid == 0) s_ie2 = __float_as_uint(st[0].e.x);
            __syncthreads();
            bool same = true;
#pragma unroll
            for (int q = 0; q < IPT; ++q) same &= __float_as_uint(st[q].e.x) == s_ie2;
            same = __syncthreads_and(same);
            return same ? __uint_as_float(s_ie2) : __uint_as_float(0x7fc00000u);
        } else {
            return __uint_as_float(0x7fc00000u);
        }
    };
    float ie2 = tile_ie2();
    bool aborted = false;
    long long abort_u = u1;                  // first unit whose tile never arrived
    long long issued_to = (u0 + DS_STAGES < u1) ? u0 + DS_STAGES : u1;   // tid 0 only

    for (long long u = u0, it = 0; u < u1; ++u, ++it) {
        const int s = (int)(it % DS_STAGES);
        const uint32_t parity = (uint32_t)((it / DS_STAGES) & 1);
        if (!mbar_wait(&full[s], parity)) aborted = true;
        if (__syncthreads_or(aborted)) {
            aborted = true;
            abort_u = u;
            break;
        }
        const float4 *R = ring + s * TILE_Q;
        // uniform softening for this unit: E = ie2 + je2, the value every
        // pair's own add would give (NaN, i.e. not uniform, propagates)
        float ue = __uint_as_float(0x7fc00000u);
        if constexpr (K::UE2)
            if (a.tile_e2) ue = __fadd_rn(ie2, __ldg(a.tile_e2 + (u % nju) / JSUB));
        if (K::UE2 && ue > 1e-20f) {   // NaN (not uniform) and tiny softening take the per-pair form
            const float2 E = f2(ue);
#pragma unroll 1
            for (int fb = 0; fb < PART_PAIRS; fb += DS_FOLD_PAIRS) {
#pragma unroll UNR
                for (int pp = 0; pp < DS_FOLD_PAIRS; ++pp) kstep<K, true>(st, R + (fb + pp) * K::NQ, E);
#pragma unroll
                for (int q = 0; q < IPT; ++q) K::fold(st[q]);
            }
        } else {
#pragma unroll 1
            for (int fb = 0; fb < PART_PAIRS; fb += DS_FOLD_PAIRS) {
#pragma unroll UNR
                for (int pp = 0; pp < DS_FOLD_PAIRS; ++pp) kstep<K, false>(st, R + (fb + pp) * K::NQ, f2(0.f));
#pragma unroll
                for (int q = 0; q < IPT; ++q) K::fold(st[q]);
            }
        }
        __syncthreads();   // stage s fully consumed
        if (tid == 0 && u + DS_STAGES < u1) {
            issue(u + DS_STAGES, s);
            issued_to = u + DS_STAGES + 1;
        }
        const long long tn = (u + 1 < u1) ? (u + 1) / nju : -1;
        if (tn == t) continue;

        // ---- i-tile t is done for this CTA: store or hand over partials ----
        finish_itile<K>(st, t, nju, u0, u1, EvenBounds{U, G}, k, a.part, a.ticket, &s_last,
                        [&](int q, const double *p) {
                            const size_t i = (size_t)t * BI + q * DS_THREADS + tid;
                            if (i < a.p.ni) K::store(p, a.p, i);
                        });
        if (tn >= 0) {
            t = tn;
#pragma unroll
            for (int q = 0; q < IPT; ++q) {
                const size_t i = (size_t)t * BI + q * DS_THREADS + tid;
                K::load(st[q], a.p, i < a.p.ni ? i : last);
            }
            ie2 = tile_ie2();
        }
    }

    if (aborted && tid == 0) {
        atomicOr(a.p.status, ST_MBAR_TIMEOUT);
        // Wait (bounded) for the copies still in flight, units abort_u ..
        // issued_to - 1, before the CTA's shared memory is released.
        for (long long u = abort_u; u < issued_to; ++u) {
            const long long it = u - u0;
            mbar_wait(&full[it % DS_STAGES], (uint32_t)((it / DS_STAGES) & 1));
        }
    }
}



// ===========================================================================
// Ordered split-FP32 Acc and AccJerk (calls of >= 2^24 pairs) and Phi
// (>= 2^31 pairs).
//
// Per call, tg_order.cu sorts the j-set (light particles in Hilbert order,
// then the heavy ones, mass > max(m) / 32 and > 16 min(m)) and the i-set
// (Hilbert order), and
// ds32_ord_prepare writes the j-records in that order with positions
// relative to the centre c_b of their 64-j block.  The pairwise kernel then
// decides per 64-j block, from the block's and the i-tile's bounding boxes:
//   * far (box distance >= ORD_THETA x the block's half-extent):
//     dx = fl(xi - c_b) - x'h, one subtraction per component; its error is
//     at most eps (|xi - c_b| + |xj - c_b|) <= (1 + 2 / ORD_THETA) eps |dx|
//     = 5 eps |dx|;
//   * near: the hi/lo difference (xi - c_b) - (xj - c_b), as accurate as
//     the global hi/lo form;
//   * heavy (the block holds heavy j): the near form with a Newton-refined
//     1/sqrt and the compensated sums folded after every record, so the
//     large terms of massive particles never sit in an FP32 lane sum.
// The acceleration's FP32 lane sums are folded into Kahan sums every
// 2 ORD_ACC_FOLD_PAIRS j (far blocks of Acc: every 2 K::FAR_FOLD_PAIRS j,
// 32; far terms are of one size within a block, and the longer fold left
// the errors unchanged while saving 2% of Acc), the jerk's every 64 j.  A
// per-i proxy of the sum of term magnitudes (the sum of |folded lane sums|;
// AccJerk: one for the jerk too) travels with the partials; particles whose
// proxy exceeds tau |a| (or 2.5 tau |j|: strong cancellation, ord_tau) are
// listed and recomputed in double-single arithmetic (ds32_exact), AccJerk
// particles with their jerk.
// ===========================================================================
constexpr int ORD_BLOCK = 64;                              // j per block
constexpr int ORD_BLOCK_PAIRS = ORD_BLOCK / 2;
constexpr int ORD_BLOCKS_PER_TILE = DS_TILE / ORD_BLOCK;
#ifndef TG_ORD_ACC_FOLD_PAIRS
#define TG_ORD_ACC_FOLD_PAIRS 8
#endif
constexpr int ORD_ACC_FOLD_PAIRS = TG_ORD_ACC_FOLD_PAIRS;  // records per acceleration fold
#ifndef TG_ORD_UNROLL
#define TG_ORD_UNROLL 8    // records per unrolled body of the far and near forms
#endif
#ifndef TG_ORD_FAR_RCP
#define TG_ORD_FAR_RCP 0   // far blocks take 1/s from MUFU.RCP (else y * y on the FMA pipe)
#endif
constexpr int ORD_UNROLL = TG_ORD_UNROLL;
#ifndef TG_ORD_THETA
#define TG_ORD_THETA 0.5f  // far: box distance >= TG_ORD_THETA x the block's half-extent
#endif
constexpr float ORD_THETA = TG_ORD_THETA;

struct OrdInfo {
    float4 c;    // block centre (x, y, z), half-extent
    float4 lo;   // box minimum (x, y, z), heavy flag (1 or 0)
    float4 hi;   // box maximum (x, y, z), unused
};

// x - c as a hi/lo pair from x = xh + xl (split_ds) and a float c: the same
// float operations on the i-side and on the j-side, so one particle's two
// relative positions are bit-identical and its self pair has dx = +0.
__device__ __forceinline__ void rel_split(float xh, float xl, float c, float &h, float &l) {
    float e;
    two_sum(xh, -c, h, e);
    l = __fadd_rn(e, xl);
    h = fzero_norm(h);
    l = fzero_norm(l);
}
// x - c rounded to one float (far blocks).
__device__ __forceinline__ float rel_single(float xh, float xl, float c) {
    return __fadd_rn(__fsub_rn(xh, c), xl);
}

// FORM of a 64-j block in the ordered kernels.
enum : int { ORD_FAR = 0, ORD_NEAR = 1, ORD_HEAVY = 2 };

template <int IPT_>
struct AccJerkOrd {
    static constexpr bool ORDERED = true;
    static constexpr int IPT = IPT_, JF = 12, NQ = 6, NP = 8, PX = 6, PJ = 7;   // PJ: jerk proxy
    static constexpr int KERNEL = K_ACC_JERK;
    static constexpr int W_FAR = 4, W_NEAR = 5, W_HEAVY = 9;   // relative cost of a 64-j block
    static constexpr int FAR_FOLD_PAIRS = 8;                   // 16 j (32-j far folds were 1% slower here)
    static constexpr bool UE2 = true;
    struct IS { float2 dh[3], dl[3]; float2 u, v, w, e; float2 a[3], j[3]; Comp ca[3], cj[3]; float px, pj; };
    __device__ static void load(IS &s, const PairArgs &a, size_t i) {
        s.u = f2(__double2float_rn(a.I.f[F_VX][i]));
        s.v = f2(__double2float_rn(a.I.f[F_VY][i]));
        s.w = f2(__double2float_rn(a.I.f[F_VZ][i]));
        s.e = f2(__double2float_rn(a.I.f[F_E2][i]));
        for (int k = 0; k < 3; ++k) {
            s.a[k] = f2(0.f); s.j[k] = f2(0.f);
            s.ca[k] = Comp{0.f, 0.f}; s.cj[k] = Comp{0.f, 0.f};
        }
        s.px = 0.f;
        s.pj = 0.f;
    }
    // record: {x'h,y'h} {z'h,m} {vx,vy} {vz,e2} {x'l,y'l} {z'l,pad}
    __device__ static void write_record(float *r, int lane, const float h[3], const float l[3], const PSet &J,
                                        size_t j, bool valid) {
        r[0 + lane] = h[0]; r[2 + lane] = h[1]; r[4 + lane] = h[2];
        r[6 + lane] = valid ? __double2float_rn(J.f[F_M][j]) : 0.f;
        r[8 + lane] = valid ? __double2float_rn(J.f[F_VX][j]) : 0.f;
        r[10 + lane] = valid ? __double2float_rn(J.f[F_VY][j]) : 0.f;
        r[12 + lane] = valid ? __double2float_rn(J.f[F_VZ][j]) : 0.f;
        r[14 + lane] = valid ? __double2float_rn(J.f[F_E2][j]) : 1.f;
        r[16 + lane] = l[0]; r[18 + lane] = l[1]; r[20 + lane] = l[2];
        r[22 + lane] = 0.f;
    }
    struct Rec { float4 q[NQ]; };
    // the floats of one record that FORM reads (far: positions' hi parts,
    // mass, velocities, softening)
    template <int FORM, bool UE>
    __device__ __forceinline__ static Rec load_rec(const float4 *R) {
        Rec c;
        c.q[0] = R[0]; c.q[1] = R[1]; c.q[2] = R[2]; c.q[3] = R[3];
        c.q[4] = c.q[0]; c.q[5] = c.q[0];
        if (FORM != ORD_FAR) { c.q[4] = R[4]; c.q[5] = R[5]; }
        return c;
    }
    template <int FORM, bool UE>
    __device__ __forceinline__ static void step(IS (&S)[IPT], const Rec &c, float2 E) {
        const float4 q0 = c.q[0], q1 = c.q[1], q2 = c.q[2], q3 = c.q[3], q4 = c.q[4], q5 = c.q[5];
#pragma unroll
        for (int u = 0; u < IPT; ++u) {
            IS &s = S[u];
            float2 dx, dy, dz;
            if (FORM == ORD_FAR) {
                dx = sub2(s.dh[0], lo2(q0)); dy = sub2(s.dh[1], hi2(q0)); dz = sub2(s.dh[2], lo2(q1));
            } else {
                dx = add2(sub2(s.dh[0], lo2(q0)), sub2(s.dl[0], lo2(q4)));
                dy = add2(sub2(s.dh[1], hi2(q0)), sub2(s.dl[1], hi2(q4)));
                dz = add2(sub2(s.dh[2], lo2(q1)), sub2(s.dl[2], lo2(q5)));
            }
            const float2 du = sub2(s.u, lo2(q2)), dv = sub2(s.v, hi2(q2)), dw = sub2(s.w, lo2(q3));
            const float2 e2 = UE ? E : add2(s.e, hi2(q3));
            const float2 ss = fma2(dx, dx, fma2(dy, dy, fma2(dz, dz, e2)));
            float2 y, y2;
            if (FORM == ORD_FAR) {   // far blocks hold no pair at r = 0
                y = make_float2(rsqrt_hw(ss.x), rsqrt_hw(ss.y));
#if TG_ORD_FAR_RCP
                y2 = make_float2(rcp_hw(ss.x), rcp_hw(ss.y));
#else
                y2 = mul2(y, y);
#endif
            } else if (FORM == ORD_NEAR) {
                inv_r_r2(ss, dx, dy, dz, y, y2);
            } else {
                y = inv_r<true>(ss, dx, dy, dz);
                y2 = mul2(y, y);
            }
            const float2 mr3 = mul2(mul2(hi2(q1), y), y2);
            const float2 rv = fma2(dx, du, fma2(dy, dv, mul2(dz, dw)));
            const float2 al = mul2(mul2(rv, y2), f2(3.0f));
            const float2 tu = fnma2(al, dx, du), tv = fnma2(al, dy, dv), tw = fnma2(al, dz, dw);
            s.a[0] = fnma2(mr3, dx, s.a[0]);
            s.a[1] = fnma2(mr3, dy, s.a[1]);
            s.a[2] = fnma2(mr3, dz, s.a[2]);
            s.j[0] = fnma2(mr3, tu, s.j[0]);
            s.j[1] = fnma2(mr3, tv, s.j[1]);
            s.j[2] = fnma2(mr3, tw, s.j[2]);
        }
    }
    __device__ static void fold_acc(IS &s) {
        for (int k = 0; k < 3; ++k) {
            const float x = __fadd_rn(s.a[k].x, s.a[k].y);
            comp_add(s.ca[k], x);
            s.px = __fadd_rn(s.px, fabsf(x));
            s.a[k] = f2(0.f);
        }
    }
    __device__ static void fold_jerk(IS &s) {
        for (int k = 0; k < 3; ++k) {
            const float x = __fadd_rn(s.j[k].x, s.j[k].y);
            comp_add(s.cj[k], x);
            s.pj = __fadd_rn(s.pj, fabsf(x));
            s.j[k] = f2(0.f);
        }
    }
    __device__ static void partials(const IS &s, double *p) {
        for (int k = 0; k < 3; ++k) { p[k] = comp_value(s.ca[k]); p[3 + k] = comp_value(s.cj[k]); }
        p[6] = (double)s.px;
        p[7] = (double)s.pj;
    }
    __device__ static void combine(double *acc, const double *p) { for (int k = 0; k < NP; ++k) acc[k] += p[k]; }
    __device__ static void store(const double *p, const PairArgs &a, size_t i) {
        for (int k = 0; k < 6; ++k) a.out[k][i] = p[k];
    }
};

template <int IPT_>
struct AccOrd {
    static constexpr bool ORDERED = true;
    static constexpr int IPT = IPT_, JF = 8, NQ = 4, NP = 4, PX = 3, PJ = -1;
    static constexpr int KERNEL = K_ACC;
    static constexpr int W_FAR = 2, W_NEAR = 3, W_HEAVY = 6;   // relative cost of a 64-j block
    static constexpr int FAR_FOLD_PAIRS = 16;                  // far blocks fold every 32 j
    static constexpr bool UE2 = true;
    struct IS { float2 dh[3], dl[3]; float2 e; float2 a[3]; Comp ca[3]; float px; };
    __device__ static void load(IS &s, const PairArgs &a, size_t i) {
        s.e = f2(__double2float_rn(a.I.f[F_E2][i]));
        for (int k = 0; k < 3; ++k) { s.a[k] = f2(0.f); s.ca[k] = Comp{0.f, 0.f}; }
        s.px = 0.f;
    }
    // record: {x'h,y'h} {z'h,m} {x'l,y'l} {z'l,e2}
    __device__ static void write_record(float *r, int lane, const float h[3], const float l[3], const PSet &J,
                                        size_t j, bool valid) {
        r[0 + lane] = h[0]; r[2 + lane] = h[1]; r[4 + lane] = h[2];
        r[6 + lane] = valid ? __double2float_rn(J.f[F_M][j]) : 0.f;
        r[8 + lane] = l[0]; r[10 + lane] = l[1]; r[12 + lane] = l[2];
        r[14 + lane] = valid ? __double2float_rn(J.f[F_E2][j]) : 1.f;
    }
    struct Rec { float4 q[NQ]; };
    template <int FORM, bool UE>
    __device__ __forceinline__ static Rec load_rec(const float4 *R) {
        Rec c;
        c.q[0] = R[0]; c.q[1] = R[1];
        c.q[2] = c.q[0]; c.q[3] = c.q[1];
        if (FORM != ORD_FAR || !UE) c.q[3] = R[3];
        if (FORM != ORD_FAR) c.q[2] = R[2];
        return c;
    }
    template <int FORM, bool UE>
    __device__ __forceinline__ static void step(IS (&S)[IPT], const Rec &c, float2 E) {
        const float4 q0 = c.q[0], q1 = c.q[1], q2 = c.q[2], q3 = c.q[3];
#pragma unroll
        for (int u = 0; u < IPT; ++u) {
            IS &s = S[u];
            float2 dx, dy, dz;
            if (FORM == ORD_FAR) {
                dx = sub2(s.dh[0], lo2(q0)); dy = sub2(s.dh[1], hi2(q0)); dz = sub2(s.dh[2], lo2(q1));
            } else {
                dx = add2(sub2(s.dh[0], lo2(q0)), sub2(s.dl[0], lo2(q2)));
                dy = add2(sub2(s.dh[1], hi2(q0)), sub2(s.dl[1], hi2(q2)));
                dz = add2(sub2(s.dh[2], lo2(q1)), sub2(s.dl[2], lo2(q3)));
            }
            const float2 e2 = UE ? E : add2(s.e, hi2(q3));
            const float2 ss = fma2(dx, dx, fma2(dy, dy, fma2(dz, dz, e2)));
            // far blocks hold no pair at r = 0; with a uniform softening
            // E > 1e-20 a pair at r = 0 has dx = +0 and adds exactly nothing
            float2 y;
            if (FORM == ORD_FAR || (FORM == ORD_NEAR && UE)) y = make_float2(rsqrt_hw(ss.x), rsqrt_hw(ss.y));
            else y = inv_r<FORM == ORD_HEAVY>(ss, dx, dy, dz);
            const float2 y2 = mul2(y, y);
            const float2 mr3 = mul2(mul2(hi2(q1), y), y2);
            s.a[0] = fnma2(mr3, dx, s.a[0]);
            s.a[1] = fnma2(mr3, dy, s.a[1]);
            s.a[2] = fnma2(mr3, dz, s.a[2]);
        }
    }
    __device__ static void fold_acc(IS &s) {
        for (int k = 0; k < 3; ++k) {
            const float x = __fadd_rn(s.a[k].x, s.a[k].y);
            comp_add(s.ca[k], x);
            s.px = __fadd_rn(s.px, fabsf(x));
            s.a[k] = f2(0.f);
        }
    }
    __device__ static void fold_jerk(IS &) {}
    __device__ static void partials(const IS &s, double *p) {
        for (int k = 0; k < 3; ++k) p[k] = comp_value(s.ca[k]);
        p[3] = (double)s.px;
    }
    __device__ static void combine(double *acc, const double *p) { for (int k = 0; k < NP; ++k) acc[k] += p[k]; }
    __device__ static void store(const double *p, const PairArgs &a, size_t i) {
        for (int k = 0; k < 3; ++k) a.out[k][i] = p[k];
    }
};

// Ordered split-FP32 Phi (phi_kernel_common.h:7-31): phi_i = -sum_j m_j / r,
// r masked to 0 where r2 > 0 fails.  Every term has the same sign, so the
// sums cannot cancel: no proxy and no recompute.  Far blocks need neither
// the lo words nor the mask (no pair there has r = 0); near and heavy blocks
// keep the mask even with a uniform softening, because a self pair's
// -m / sqrt(e2) is not zero.
template <int IPT_>
struct PhiOrd {
    static constexpr bool ORDERED = true;
    static constexpr int IPT = IPT_, JF = 8, NQ = 4, NP = 1, PX = -1, PJ = -1;
    static constexpr int KERNEL = K_PHI;
    static constexpr int W_FAR = 2, W_NEAR = 3, W_HEAVY = 6;   // relative cost of a 64-j block
    static constexpr int FAR_FOLD_PAIRS = 16;                  // far blocks fold every 32 j
    static constexpr bool UE2 = true;
    struct IS { float2 dh[3], dl[3]; float2 e; float2 p; Comp cp; };
    __device__ static void load(IS &s, const PairArgs &a, size_t i) {
        s.e = f2(__double2float_rn(a.I.f[F_E2][i]));
        s.p = f2(0.f);
        s.cp = Comp{0.f, 0.f};
    }
    // record: {x'h,y'h} {z'h,m} {x'l,y'l} {z'l,e2}
    __device__ static void write_record(float *r, int lane, const float h[3], const float l[3], const PSet &J,
                                        size_t j, bool valid) {
        AccOrd<IPT_>::write_record(r, lane, h, l, J, j, valid);
    }
    struct Rec { float4 q[NQ]; };
    template <int FORM, bool UE>
    __device__ __forceinline__ static Rec load_rec(const float4 *R) {
        Rec c;
        c.q[0] = R[0]; c.q[1] = R[1];
        c.q[2] = c.q[0]; c.q[3] = c.q[1];
        if (FORM != ORD_FAR || !UE) c.q[3] = R[3];
        if (FORM != ORD_FAR) c.q[2] = R[2];
        return c;
    }
    template <int FORM, bool UE>
    __device__ __forceinline__ static void step(IS (&S)[IPT], const Rec &c, float2 E) {
        const float4 q0 = c.q[0], q1 = c.q[1], q2 = c.q[2], q3 = c.q[3];
#pragma unroll
        for (int u = 0; u < IPT; ++u) {
            IS &s = S[u];
            float2 dx, dy, dz;
            if (FORM == ORD_FAR) {
                dx = sub2(s.dh[0], lo2(q0)); dy = sub2(s.dh[1], hi2(q0)); dz = sub2(s.dh[2], lo2(q1));
            } else {
                dx = add2(sub2(s.dh[0], lo2(q0)), sub2(s.dl[0], lo2(q2)));
                dy = add2(sub2(s.dh[1], hi2(q0)), sub2(s.dl[1], hi2(q2)));
                dz = add2(sub2(s.dh[2], lo2(q1)), sub2(s.dl[2], lo2(q3)));
            }
            const float2 e2 = UE ? E : add2(s.e, hi2(q3));
            const float2 ss = fma2(dx, dx, fma2(dy, dy, fma2(dz, dz, e2)));
            float2 y;
            if (FORM == ORD_FAR) y = make_float2(rsqrt_hw(ss.x), rsqrt_hw(ss.y));
            else y = inv_r<FORM == ORD_HEAVY>(ss, dx, dy, dz);
            s.p = fnma2(hi2(q1), y, s.p);
        }
    }
    __device__ static void fold_acc(IS &s) {
        comp_add(s.cp, __fadd_rn(s.p.x, s.p.y));
        s.p = f2(0.f);
    }
    __device__ static void fold_jerk(IS &) {}
    __device__ static void partials(const IS &s, double *p) { p[0] = comp_value(s.cp); }
    __device__ static void combine(double *acc, const double *p) { acc[0] += p[0]; }
    __device__ static void store(const double *p, const PairArgs &a, size_t i) { a.out[0][i] = p[0]; }
};

// Double-single j-data of the exact kernel (ds32_exact), EXACT_JQ float4
// per j: {xh, xl, yh, yl} {zh, zl, mh, ml} {e2h, e2l, uzh, uzl}
// {uxh, uxl, uyh, uyl}, where u is the vector field `ufield` (F_VX: the
// velocity, F_AX: the adjoint's upstream gradient) or zero (ufield < 0).
constexpr int EXACT_JQ = 4;
__device__ __forceinline__ void write_exact_record(float4 *r, const PSet &J, size_t j, int ufield) {
    float xh[3], xl[3], mh, ml, eh, el, vh[3] = {0.f, 0.f, 0.f}, vl[3] = {0.f, 0.f, 0.f};
    for (int c = 0; c < 3; ++c) split_ds(J.f[F_RX + c][j], xh[c], xl[c]);
    split_ds(J.f[F_M][j], mh, ml);
    split_ds(J.f[F_E2][j], eh, el);
    if (ufield >= 0)
        for (int c = 0; c < 3; ++c) split_ds(J.f[ufield + c][j], vh[c], vl[c]);
    r[0] = make_float4(xh[0], xl[0], xh[1], xl[1]);
    r[1] = make_float4(xh[2], xl[2], mh, ml);
    r[2] = make_float4(eh, el, vh[2], vl[2]);
    r[3] = make_float4(vh[0], vl[0], vh[1], vl[1]);
}

// Records, block table, uniform-softening flags, the double-single j-data of
// the recompute (write_exact_record, sorted order) and zeroed counters; one
// CTA of DS_TILE threads per j-tile, one sorted j per thread.
template <class K>
__global__ void __launch_bounds__(DS_TILE) ds32_ord_prepare(PSet J, size_t nj, const int *pj, const unsigned *nlight,
                                                            float *rec, OrdInfo *blk, float *tile_e2, int *ticket,
                                                            long long nticket, int *flag_count, float4 *jd,
                                                            int *ref_ticket, int nref_ticket) {
    __shared__ float s_box[DS_TILE / 32][6];
    __shared__ unsigned s_first;
    const size_t tile = blockIdx.x;
    const int q = threadIdx.x;
    const size_t p = tile * DS_TILE + q;
    const bool valid = p < nj;
    const size_t j = valid ? (size_t)pj[p] : 0;
    float xh[3], xl[3];
    for (int c = 0; c < 3; ++c) split_ds(valid ? J.f[F_RX + c][j] : 0.0, xh[c], xl[c]);
    // block box over the valid j (a block is two warps)
    float lo[3], hi[3];
    for (int c = 0; c < 3; ++c) {
        lo[c] = (valid && isfinite(xh[c])) ? xh[c] : INFINITY;
        hi[c] = (valid && isfinite(xh[c])) ? xh[c] : -INFINITY;
    }
    for (int o = 16; o > 0; o >>= 1)
        for (int c = 0; c < 3; ++c) {
            lo[c] = fminf(lo[c], __shfl_xor_sync(0xffffffffu, lo[c], o));
            hi[c] = fmaxf(hi[c], __shfl_xor_sync(0xffffffffu, hi[c], o));
        }
    if ((q & 31) == 0)
        for (int c = 0; c < 3; ++c) { s_box[q >> 5][c] = lo[c]; s_box[q >> 5][3 + c] = hi[c]; }
    __syncthreads();
    const int b = q / ORD_BLOCK, w0 = 2 * b;
    float cc[3], ext = 0.f;
    for (int c = 0; c < 3; ++c) {
        lo[c] = fminf(s_box[w0][c], s_box[w0 + 1][c]);
        hi[c] = fmaxf(s_box[w0][3 + c], s_box[w0 + 1][3 + c]);
        if (!(lo[c] <= hi[c])) lo[c] = hi[c] = 0.f;   // no valid, finite coordinate
        cc[c] = __fmul_rn(0.5f, __fadd_rn(lo[c], hi[c]));
        if (!isfinite(cc[c])) cc[c] = 0.f;
        ext = fmaxf(ext, fmaxf(__fsub_rn(hi[c], cc[c]), __fsub_rn(cc[c], lo[c])));
    }
    ext = __fmul_ru(ext, 1.0f + 0x1p-20f);
    const size_t gb = tile * ORD_BLOCKS_PER_TILE + b;
    if ((q % ORD_BLOCK) == 0) {
        const size_t start = gb * ORD_BLOCK;
        const bool heavy = start < nj && start + ORD_BLOCK > (size_t)*nlight;
        OrdInfo info;
        info.c = make_float4(cc[0], cc[1], cc[2], ext);
        info.lo = make_float4(lo[0], lo[1], lo[2], heavy ? 1.f : 0.f);
        info.hi = make_float4(hi[0], hi[1], hi[2], 0.f);
        blk[gb] = info;
    }
    // the record: positions relative to the block centre
    float h[3], l[3];
    for (int c = 0; c < 3; ++c) {
        if (valid) rel_split(xh[c], xl[c], cc[c], h[c], l[c]);
        else { h[c] = 0.f; l[c] = 0.f; }
    }
    K::write_record(rec + (p >> 1) * (size_t)(2 * K::JF), (int)(p & 1), h, l, J, j, valid);
    if (K::PX >= 0 && valid) write_exact_record(jd + EXACT_JQ * p, J, j, K::PJ >= 0 ? F_VX : -1);
    if (tile_e2 != nullptr) {   // the tile's common float softening, or NaN
        const unsigned mine = valid ? __float_as_uint(__double2float_rn(J.f[F_E2][j])) : 0u;
        if (q == 0) s_first = mine;   // the tile's first j is always valid
        __syncthreads();
        const bool same = __syncthreads_and(!valid || mine == s_first);
        if (q == 0) {
            const float v = __uint_as_float(s_first);
            tile_e2[tile] = (same && v == v) ? v : __uint_as_float(0x7fc00000u);
        }
    }
    const size_t g = (size_t)blockIdx.x * blockDim.x + threadIdx.x, stride = (size_t)gridDim.x * blockDim.x;
    for (size_t x = g; x < (size_t)nticket; x += stride) ticket[x] = 0;
    for (size_t x = g; x < (size_t)nref_ticket; x += stride) ref_ticket[x] = 0;
    if (g == 0) *flag_count = 0;
}

// Float bounding box of each i-tile of blockDim.x sorted i-particles.
__global__ void ds32_ord_ibox(PSet I, size_t ni, const int *pi, float4 *ibox) {
    __shared__ float s_box[32][6];
    const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    float lo[3], hi[3];
    for (int c = 0; c < 3; ++c) {
        const float x = p < ni ? __double2float_rn(I.f[F_RX + c][pi[p]]) : NAN;
        lo[c] = isfinite(x) ? x : INFINITY;
        hi[c] = isfinite(x) ? x : -INFINITY;
    }
    for (int o = 16; o > 0; o >>= 1)
        for (int c = 0; c < 3; ++c) {
            lo[c] = fminf(lo[c], __shfl_xor_sync(0xffffffffu, lo[c], o));
            hi[c] = fmaxf(hi[c], __shfl_xor_sync(0xffffffffu, hi[c], o));
        }
    const int w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if ((threadIdx.x & 31) == 0)
        for (int c = 0; c < 3; ++c) { s_box[w][c] = lo[c]; s_box[w][3 + c] = hi[c]; }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int v = 1; v < nw; ++v)
            for (int c = 0; c < 3; ++c) { lo[c] = fminf(lo[c], s_box[v][c]); hi[c] = fmaxf(hi[c], s_box[v][3 + c]); }
        ibox[2 * blockIdx.x] = make_float4(lo[0], lo[1], lo[2], 0.f);
        ibox[2 * blockIdx.x + 1] = make_float4(hi[0], hi[1], hi[2], 0.f);
    }
}

struct DsOrdArgs {
    DsArgs d;
    const int *pi;                // sorted i position -> i index
    const OrdInfo *blk;           // per 64-j block
    const unsigned char *form;    // [i-tile][64-j block]: ORD_FAR, ORD_NEAR or ORD_HEAVY
    const long long *start;       // CTA k owns units [start[k], start[k + 1])
    int *flag_count, *flag_list;
    float tau;                    // recompute when proxy > tau |a|
    float tau_jerk;               // or jerk proxy > tau_jerk |j| (AccJerk)
};

// Recompute threshold tau (process-wide, tg_set_recompute_threshold; 20 by
// default) at nj >= 65536, scaled with sqrt(nj) below (fewer terms average
// out less of their rounding), at least 4 (and at most tau).  The jerk's
// threshold is ORD_TAU_JERK_FACTOR times the acceleration's: its bound
// (1e-5) is ten times looser, its proxy coarser (folds every 64 j).
constexpr float ORD_TAU_JERK_FACTOR = 2.5f;
std::atomic<float> g_ord_tau{20.0f};
static float ord_tau(size_t nj) {
    const double tau = g_ord_tau.load(), t = tau * sqrt((double)nj / 65536.0);
    return (float)(t > tau ? tau : (t < 4.0 ? (tau < 4.0 ? tau : 4.0) : t));
}

double set_recompute_threshold(double tau) {
    if (!(tau >= 1.0 && tau <= 1e6)) return -1.0;
    return (double)g_ord_tau.exchange((float)tau);
}

// Form of 64-j block `b` for an i-tile with float bounding box [ilo, ihi]:
// heavy if it holds heavy j, far if the boxes are at least the block's
// half-extent apart (and clearly separated relative to the coordinates'
// magnitude), else near.
__device__ __forceinline__ int block_form(float4 ilo, float4 ihi, const OrdInfo &b) {
    if (b.lo.w != 0.f) return ORD_HEAVY;
    const float gx = fmaxf(0.f, fmaxf(ilo.x - b.hi.x, b.lo.x - ihi.x));
    const float gy = fmaxf(0.f, fmaxf(ilo.y - b.hi.y, b.lo.y - ihi.y));
    const float gz = fmaxf(0.f, fmaxf(ilo.z - b.hi.z, b.lo.z - ihi.z));
    const float d2 = gx * gx + gy * gy + gz * gz;
    const float cm = fmaxf(fabsf(b.c.x), fmaxf(fabsf(b.c.y), fabsf(b.c.z)));
    const float th = fmaxf(ORD_THETA * b.c.w, cm * 0x1p-16f);
    return (d2 > 0.f && d2 >= th * th) ? ORD_FAR : ORD_NEAR;
}

// Plan: the form of every (i-tile, 64-j block) and the cost of every unit
// (i-tile x one of the jsub parts of a j-tile), the sum of its blocks'
// weights w_far, w_near, w_heavy.  One CTA per i-tile.
__global__ void ds32_ord_plan(const float4 *ibox, const OrdInfo *blk, long long nblk, long long nju,
                              int part_blocks, int w_far, int w_near, int w_heavy, unsigned char *form,
                              int *ucost) {
    const long long t = blockIdx.x;
    const float4 ilo = ibox[2 * t], ihi = ibox[2 * t + 1];
    unsigned char *row = form + t * nblk;
    for (long long b = threadIdx.x; b < nblk; b += blockDim.x) row[b] = (unsigned char)block_form(ilo, ihi, blk[b]);
    __syncthreads();
    for (long long jp = threadIdx.x; jp < nju; jp += blockDim.x) {
        int c = 0;
        for (int q = 0; q < part_blocks; ++q) {
            const int f = row[jp * part_blocks + q];
            c += f == ORD_FAR ? w_far : (f == ORD_NEAR ? w_near : w_heavy);
        }
        ucost[t * nju + jp] = c;
    }
}

// CTA boundaries at equal cost, one thread per unit: with ucum the inclusive
// prefix sums of the unit costs (total C), CTA k starts at the unit that
// holds cost position floor(k C / G).  A unit costing more than C / G holds
// several positions, and the CTAs between get no unit.
__global__ void ds32_ord_bounds(const int *ucost, const int *ucum, long long U, long long G, long long *start) {
    const long long u = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (u == 0) start[G] = U;
    if (u >= U) return;
    const long long total = ucum[U - 1];
    const long long ce = ucum[u], cs = ce - ucost[u];
    const long long klo = (cs * G + total - 1) / total;
    long long khi = (ce * G + total - 1) / total - 1;
    if (khi > G - 1) khi = G - 1;
    for (long long k = klo; k <= khi; ++k) start[k] = u;
}

// One 64-j block of FORM against the thread's i-particles: acceleration
// folds every ORD_ACC_FOLD_PAIRS records (far blocks: K::FAR_FOLD_PAIRS),
// jerk fold at the end (heavy blocks: both after every record).
template <class K, int FORM, bool UE>
__device__ __forceinline__ void ord_block(typename K::IS (&st)[K::IPT], const float4 *R, float2 E) {
    if constexpr (FORM == ORD_HEAVY) {
#pragma unroll 1
        for (int r = 0; r < ORD_BLOCK_PAIRS; ++r) {
            K::template step<FORM, UE>(st, K::template load_rec<FORM, UE>(R + r * K::NQ), E);
#pragma unroll
            for (int q = 0; q < K::IPT; ++q) { K::fold_acc(st[q]); K::fold_jerk(st[q]); }
        }
    } else {
        constexpr int FOLD = FORM == ORD_FAR ? K::FAR_FOLD_PAIRS : ORD_ACC_FOLD_PAIRS;
        static_assert(ORD_BLOCK_PAIRS % FOLD == 0, "folds must tile a block");
        for (int r0 = 0; r0 < ORD_BLOCK_PAIRS; r0 += FOLD) {
#pragma unroll ORD_UNROLL
            for (int r = 0; r < FOLD; ++r)
                K::template step<FORM, UE>(st, K::template load_rec<FORM, UE>(R + (r0 + r) * K::NQ), E);
#pragma unroll
            for (int q = 0; q < K::IPT; ++q) K::fold_acc(st[q]);
        }
#pragma unroll
        for (int q = 0; q < K::IPT; ++q) K::fold_jerk(st[q]);
    }
}

template <class K, int JSUB>
__global__ void __launch_bounds__(DS_THREADS, TG_DS32_MINB) ds32_ord(DsOrdArgs oa) {
    extern __shared__ __align__(128) float4 ring[];   // [DS_STAGES][DS_PAIRS * NQ]
    __shared__ __align__(8) uint64_t full[DS_STAGES];
    __shared__ int s_last;
    __shared__ float s_xi[6][DS_THREADS * K::IPT];     // i-tile positions: hi x, y, z, lo x, y, z
    const DsArgs &a = oa.d;
    constexpr int IPT = K::IPT;
    constexpr int TILE_Q = DS_PAIRS * K::NQ;
    constexpr int BI = DS_THREADS * IPT;
    constexpr int PART_PAIRS = DS_PAIRS / JSUB;
    constexpr int PART_Q = PART_PAIRS * K::NQ;
    constexpr int PART_BLOCKS = PART_PAIRS / ORD_BLOCK_PAIRS;
    const long long nju = a.njt * JSUB;
    const long long G = gridDim.x;
    const long long k = blockIdx.x;
    const long long u0 = oa.start[k], u1 = oa.start[k + 1];
    if (u0 >= u1) return;
    const TableBounds bounds{oa.start, G};
    const long long nblk = a.njt * ORD_BLOCKS_PER_TILE;
    const int tid = threadIdx.x;

    if (tid == 0) {
        for (int s = 0; s < DS_STAGES; ++s) mbar_init(&full[s], 1);
        fence_mbar_init();
    }
    __syncthreads();
    auto issue = [&](long long u, int s) {
        const long long jp = u % nju;
        constexpr unsigned bytes = (unsigned)(PART_Q * sizeof(float4));
        mbar_expect_tx(&full[s], bytes);
        bulk_g2s(ring + s * TILE_Q, a.rec + jp * PART_Q, bytes, &full[s]);
    };
    if (tid == 0) {
        for (int s = 0; s < DS_STAGES && u0 + s < u1; ++s) issue(u0 + s, s);
    }

    const size_t ni = a.p.ni;
    long long t = u0 / nju;
    typename K::IS st[IPT];
    auto load_tile = [&](long long tt) {
#pragma unroll
        for (int q = 0; q < IPT; ++q) {
            const size_t ii = (size_t)tt * BI + q * DS_THREADS + tid;
            const size_t i = (size_t)oa.pi[ii < ni ? ii : ni - 1];
            K::load(st[q], a.p, i);
            for (int c = 0; c < 3; ++c) {
                float h, l;
                split_ds(a.p.I.f[F_RX + c][i], h, l);
                s_xi[c][q * DS_THREADS + tid] = h;
                s_xi[3 + c][q * DS_THREADS + tid] = l;
            }
        }
    };
    load_tile(t);
    __shared__ unsigned s_ie2;
    auto tile_ie2 = [&]() -> float {
        if (tid == 0) s_ie2 = __float_as_uint(st[0].e.x);
        __syncthreads();
        bool same = true;
#pragma unroll
        for (int q = 0; q < IPT; ++q) same &= __float_as_uint(st[q].e.x) == s_ie2;
        same = __syncthreads_and(same);
        return same ? __uint_as_float(s_ie2) : __uint_as_float(0x7fc00000u);
    };
    float ie2 = tile_ie2();
    bool aborted = false;
    long long abort_u = u1;
    long long issued_to = (u0 + DS_STAGES < u1) ? u0 + DS_STAGES : u1;

    for (long long u = u0, it = 0; u < u1; ++u, ++it) {
        const int s = (int)(it % DS_STAGES);
        const uint32_t parity = (uint32_t)((it / DS_STAGES) & 1);
        if (!mbar_wait(&full[s], parity)) aborted = true;
        if (__syncthreads_or(aborted)) {
            aborted = true;
            abort_u = u;
            break;
        }
        const float4 *R = ring + s * TILE_Q;
        const long long jp = u % nju, jt = jp / JSUB;
        const float ue = __fadd_rn(ie2, __ldg(a.tile_e2 + jt));
        // ue is NaN unless both tiles' softenings are uniform.  Far blocks
        // take the uniform value whenever there is one (zero included: no
        // pair there has r = 0); near blocks only above 1e-20, where a pair
        // at r = 0 adds exactly nothing without the mask
        const bool uniform = ue == ue;
        const bool UEok = ue > 1e-20f;
        const float2 E = f2(ue);
#pragma unroll 1
        for (int bl = 0; bl < PART_BLOCKS; ++bl) {
            const long long gb = jt * ORD_BLOCKS_PER_TILE + (jp % JSUB) * PART_BLOCKS + bl;
            const float4 bc = __ldg(&oa.blk[gb].c);
            const int form = __ldg(oa.form + t * nblk + gb);
            const bool far = form == ORD_FAR, heavy = form == ORD_HEAVY;
            const float cc[3] = {bc.x, bc.y, bc.z};
            const float4 *Rb = R + bl * ORD_BLOCK_PAIRS * K::NQ;
            if (far) {
#pragma unroll
                for (int q = 0; q < IPT; ++q)
                    for (int c = 0; c < 3; ++c) {
                        const int x = q * DS_THREADS + tid;
                        st[q].dh[c] = f2(rel_single(s_xi[c][x], s_xi[3 + c][x], cc[c]));
                    }
                if (uniform) ord_block<K, ORD_FAR, true>(st, Rb, E);
                else ord_block<K, ORD_FAR, false>(st, Rb, E);
            } else {
#pragma unroll
                for (int q = 0; q < IPT; ++q)
                    for (int c = 0; c < 3; ++c) {
                        const int x = q * DS_THREADS + tid;
                        float h, l;
                        rel_split(s_xi[c][x], s_xi[3 + c][x], cc[c], h, l);
                        st[q].dh[c] = f2(h);
                        st[q].dl[c] = f2(l);
                    }
                if (heavy) ord_block<K, ORD_HEAVY, false>(st, Rb, E);
                else if (UEok) ord_block<K, ORD_NEAR, true>(st, Rb, E);
                else ord_block<K, ORD_NEAR, false>(st, Rb, E);
            }
        }
        __syncthreads();   // stage s fully consumed
        if (tid == 0 && u + DS_STAGES < u1) {
            issue(u + DS_STAGES, s);
            issued_to = u + DS_STAGES + 1;
        }
        const long long tn = (u + 1 < u1) ? (u + 1) / nju : -1;
        if (tn == t) continue;
        finish_itile<K>(st, t, nju, u0, u1, bounds, k, a.part, a.ticket, &s_last,
                        [&](int q, const double *p) {
                            const size_t ii = (size_t)t * BI + q * DS_THREADS + tid;
                            if (ii >= ni) return;
                            const size_t i = (size_t)oa.pi[ii];
                            K::store(p, a.p, i);
                            if constexpr (K::PX >= 0) {
                                const double am = sqrt(p[0] * p[0] + p[1] * p[1] + p[2] * p[2]);
                                bool redo = !(p[K::PX] <= (double)oa.tau * am);
                                if constexpr (K::PJ >= 0) {
                                    const double jm = sqrt(p[3] * p[3] + p[4] * p[4] + p[5] * p[5]);
                                    redo = redo || !(p[K::PJ] <= (double)oa.tau_jerk * jm);
                                }
                                if (redo) {
                                    const int f = atomicAdd(oa.flag_count, 1);
                                    oa.flag_list[f] = (int)i;
                                }
                            }
                        });
        if (tn >= 0) {
            t = tn;
            load_tile(t);
            ie2 = tile_ie2();
        }
    }

    if (aborted && tid == 0) {
        atomicOr(a.p.status, ST_MBAR_TIMEOUT);
        for (long long u = abort_u; u < issued_to; ++u) {
            const long long it = u - u0;
            mbar_wait(&full[it % DS_STAGES], (uint32_t)((it / DS_STAGES) & 1));
        }
    }
}

// Double-single arithmetic, ~2^-43 per term, from the hi/lo floats of
// write_exact_record (no FP64 operation in the pair loop), for the
// i-particles listed in `list` (count *count) or, with list == nullptr, for
// all ni of them.  MODE: EX_ACC (acceleration), EX_ACC_JERK (and the jerk),
// EX_VJP (the adjoint of Acc: r-bar and m-bar, the pair formulas of the FP64
// AccVjp64).  It serves as the recompute of the particles the ordered kernels
// flag (acceleration only), as the whole split-FP32 Acc and AccJerk of calls
// below 2^24 pairs, and as the split-FP32 adjoint.
// One warp per work item: with F particles and GW warps in the grid each
// particle's j-range is cut into nch = clamp(GW / F, 1, EXACT_MAX_CHUNKS)
// chunks; a warp reduces its chunk by a double-single butterfly, and with
// nch > 1 the last chunk of a particle to finish (atomic ticket) adds the
// chunk sums in chunk order: the result is deterministic.  Pairs with r2 > 0 false get 1/r = 0 as in the reference
// (acc_kernel_common.h, acc_jerk_kernel_common.h; smoothing.h), so a NaN
// separation still reaches the sums as it does there.
constexpr int EXACT_THREADS = 256;                 // 8 warps per CTA
constexpr int EXACT_WARPS = EXACT_THREADS / 32;
constexpr int EXACT_MAX_CHUNKS = 16;
#ifndef TG_EXACT_MAX_SPLIT
#define TG_EXACT_MAX_SPLIT 4096
#endif
constexpr int EXACT_MAX_SPLIT = TG_EXACT_MAX_SPLIT;   // particles that may be split (ticket and partial slots)
enum : int { EX_ACC = 0, EX_ACC_JERK = 1, EX_VJP = 2 };
template <int MODE>
__global__ void __launch_bounds__(EXACT_THREADS) ds32_exact(PairArgs a, const float4 *jd, const int *count,
                                                             const int *list, double *partial, int *ticket) {
    constexpr bool JERK = MODE == EX_ACC_JERK, VJP = MODE == EX_VJP, UVEC = JERK || VJP;
    constexpr int NO = JERK ? 6 : (VJP ? 4 : 3);
    const long long F = list ? (long long)*count : (long long)a.ni;
    if (F == 0) return;
    const int lane = threadIdx.x & 31;
    const long long GW = (long long)gridDim.x * EXACT_WARPS;
    long long nch = GW / F;
    nch = nch < 1 ? 1 : (nch > EXACT_MAX_CHUNKS ? EXACT_MAX_CHUNKS : nch);
    if (F > EXACT_MAX_SPLIT) nch = 1;
    const long long W = F * nch;
    const size_t nj = a.nj;
    for (long long w = (long long)blockIdx.x * EXACT_WARPS + (threadIdx.x >> 5); w < W; w += GW) {
        const long long f = w / nch, ch = w % nch;
        const size_t i = list ? (size_t)list[f] : (size_t)f;
        const size_t j0 = nj * ch / nch, j1 = nj * (ch + 1) / nch;
        // the i-particle's double-single values: lane q converts field q
        // (x, y, z, e2, u (v or g) x, y, z, m), then every lane takes them
        DS own{0.f, 0.f};
        if (lane < 8) {
            const int ufld = VJP ? F_AX : F_VX;
            const int fld = lane < 3 ? F_RX + lane : (lane == 3 ? F_E2 : (lane < 7 ? ufld + lane - 4 : F_M));
            if (lane < 4 || UVEC) own = ds_from(a.I.f[fld][i]);
        }
        DS s_i[8];
        for (int q = 0; q < 8; ++q)
            s_i[q] = DS{__shfl_sync(0xffffffffu, own.hi, q), __shfl_sync(0xffffffffu, own.lo, q)};
        // two j per packed step: lane .x takes j, lane .y j + 32
        DS2 xi[3], vi[3], mi;
        for (int c = 0; c < 3; ++c) xi[c] = DS2{f2(s_i[c].hi), f2(s_i[c].lo)};
        if (UVEC)
            for (int c = 0; c < 3; ++c) vi[c] = DS2{f2(s_i[4 + c].hi), f2(s_i[4 + c].lo)};
        if (VJP) mi = DS2{f2(s_i[7].hi), f2(s_i[7].lo)};
        const DS2 ie2{f2(s_i[3].hi), f2(s_i[3].lo)};
        DS2 acc2[NO];
        for (int c = 0; c < NO; ++c) acc2[c] = DS2{f2(0.f), f2(0.f)};
        for (size_t p = j0 + lane; p < j1; p += 64) {
            const size_t p1 = p + 32;
            const bool has1 = p1 < j1;
            const float4 A0 = __ldg(jd + EXACT_JQ * p), B0 = __ldg(jd + EXACT_JQ * p + 1),
                         C0 = __ldg(jd + EXACT_JQ * p + 2);
            // a missing second j: massless, at the i-particle (adds 0)
            const float4 A1 = has1 ? __ldg(jd + EXACT_JQ * p1) : make_float4(xi[0].hi.x, xi[0].lo.x, xi[1].hi.x, xi[1].lo.x);
            const float4 B1 = has1 ? __ldg(jd + EXACT_JQ * p1 + 1) : make_float4(xi[2].hi.x, xi[2].lo.x, 0.f, 0.f);
            const float4 C1 = has1 ? __ldg(jd + EXACT_JQ * p1 + 2) : make_float4(1.f, 0.f, 0.f, 0.f);
            DS2 d[3];
            d[0] = ds2_add(xi[0], DS2{make_float2(-A0.x, -A1.x), make_float2(-A0.y, -A1.y)});
            d[1] = ds2_add(xi[1], DS2{make_float2(-A0.z, -A1.z), make_float2(-A0.w, -A1.w)});
            d[2] = ds2_add(xi[2], DS2{make_float2(-B0.x, -B1.x), make_float2(-B0.y, -B1.y)});
            const DS2 r2 = ds2_add(ds2_add(ds2_mul(d[0], d[0]), ds2_mul(d[1], d[1])), ds2_mul(d[2], d[2]));
            const DS2 s2 = ds2_add(r2, ds2_add(ie2, DS2{make_float2(C0.x, C1.x), make_float2(C0.y, C1.y)}));
            DS2 y = ds2_rsqrt(s2);
            // excluded pairs (r2 > 0 false) get 1/r = 0, as in the reference,
            // whose terms then still carry a NaN separation into the sums
            if (!(r2.hi.x > 0.f)) { y.hi.x = 0.f; y.lo.x = 0.f; }
            if (!(r2.hi.y > 0.f)) { y.hi.y = 0.f; y.lo.y = 0.f; }
            const DS2 y2 = ds2_mul(y, y);
            const DS2 mj{make_float2(B0.z, B1.z), make_float2(B0.w, B1.w)};
            if (VJP) {
                // w = m_i g_j - m_j g_i; r-bar += q3 w - 3 q3 q2 (r.w) r;
                // m-bar += (g_j . r) q3  (q2 = y^2, q3 = y^3)
                const float4 D0 = __ldg(jd + EXACT_JQ * p + 3);
                const float4 D1 = has1 ? __ldg(jd + EXACT_JQ * p1 + 3) : make_float4(0.f, 0.f, 0.f, 0.f);
                const float gzh1 = has1 ? C1.z : 0.f, gzl1 = has1 ? C1.w : 0.f;
                const DS2 gj[3] = {DS2{make_float2(D0.x, D1.x), make_float2(D0.y, D1.y)},
                                   DS2{make_float2(D0.z, D1.z), make_float2(D0.w, D1.w)},
                                   DS2{make_float2(C0.z, gzh1), make_float2(C0.w, gzl1)}};
                const DS2 q3 = ds2_mul(y2, y);
                DS2 w[3];
                for (int c = 0; c < 3; ++c) w[c] = ds2_add(ds2_mul(mi, gj[c]), ds2_neg(ds2_mul(mj, vi[c])));
                const DS2 rw = ds2_add(ds2_add(ds2_mul(d[0], w[0]), ds2_mul(d[1], w[1])), ds2_mul(d[2], w[2]));
                const DS2 cc = ds2_mul(DS2{f2(3.0f), f2(0.0f)}, ds2_mul(ds2_mul(q3, y2), rw));
                for (int c = 0; c < 3; ++c)
                    acc2[c] = ds2_add(acc2[c], ds2_add(ds2_mul(q3, w[c]), ds2_neg(ds2_mul(cc, d[c]))));
                const DS2 gr = ds2_add(ds2_add(ds2_mul(gj[0], d[0]), ds2_mul(gj[1], d[1])), ds2_mul(gj[2], d[2]));
                acc2[3] = ds2_add(acc2[3], ds2_mul(gr, q3));
                continue;
            }
            const DS2 mr3 = ds2_mul(mj, ds2_mul(y2, y));
            for (int c = 0; c < 3; ++c) acc2[c] = ds2_add(acc2[c], ds2_neg(ds2_mul(mr3, d[c])));
            if (JERK) {
                const float4 D0 = __ldg(jd + EXACT_JQ * p + 3);
                const float4 D1 = has1 ? __ldg(jd + EXACT_JQ * p1 + 3)
                                       : make_float4(vi[0].hi.x, vi[0].lo.x, vi[1].hi.x, vi[1].lo.x);
                const float vzh1 = has1 ? C1.z : vi[2].hi.x, vzl1 = has1 ? C1.w : vi[2].lo.x;
                DS2 v[3];
                v[0] = ds2_add(vi[0], DS2{make_float2(-D0.x, -D1.x), make_float2(-D0.y, -D1.y)});
                v[1] = ds2_add(vi[1], DS2{make_float2(-D0.z, -D1.z), make_float2(-D0.w, -D1.w)});
                v[2] = ds2_add(vi[2], DS2{make_float2(-C0.z, -vzh1), make_float2(-C0.w, -vzl1)});
                const DS2 rv = ds2_add(ds2_add(ds2_mul(d[0], v[0]), ds2_mul(d[1], v[1])), ds2_mul(d[2], v[2]));
                const DS2 al = ds2_mul(DS2{f2(3.0f), f2(0.0f)}, ds2_mul(rv, y2));
                for (int c = 0; c < 3; ++c) {
                    const DS2 t = ds2_add(v[c], ds2_neg(ds2_mul(al, d[c])));
                    acc2[3 + c] = ds2_add(acc2[3 + c], ds2_neg(ds2_mul(mr3, t)));
                }
            }
        }
        DS acc[NO];
        for (int c = 0; c < NO; ++c)
            acc[c] = ds_add(DS{acc2[c].hi.x, acc2[c].lo.x}, DS{acc2[c].hi.y, acc2[c].lo.y});
        // butterfly over the warp (ds_add is commutative: every lane ends
        // with the same, deterministic value)
        for (int o = 16; o > 0; o >>= 1)
            for (int c = 0; c < NO; ++c)
                acc[c] = ds_add(acc[c], DS{__shfl_xor_sync(0xffffffffu, acc[c].hi, o),
                                           __shfl_xor_sync(0xffffffffu, acc[c].lo, o)});
        if (nch == 1) {
            if (lane == 0)
                for (int c = 0; c < NO; ++c) a.out[c][i] = ds_value(acc[c]);
        } else if (lane == 0) {
            double *mine = partial + ((size_t)f * EXACT_MAX_CHUNKS + ch) * NO;
            for (int c = 0; c < NO; ++c) mine[c] = ds_value(acc[c]);
            __threadfence();
            if (atomicAdd(ticket + f, 1) == (int)nch - 1) {
                __threadfence();
                double v[NO];
                for (int c = 0; c < NO; ++c) v[c] = 0.0;
                for (long long r = 0; r < nch; ++r)
                    for (int c = 0; c < NO; ++c) v[c] += __ldcg(partial + ((size_t)f * EXACT_MAX_CHUNKS + r) * NO + c);
                for (int c = 0; c < NO; ++c) a.out[c][i] = v[c];
            }
        }
        __syncwarp();
    }
}

// j-data of ds32_exact in the caller's order, and zeroed chunk tickets.
__global__ void ds32_exact_prepare(PSet J, size_t nj, int ufield, float4 *jd, int *ticket, int nticket) {
    const size_t j = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j < nj) write_exact_record(jd + EXACT_JQ * j, J, j, ufield);
    if (j < (size_t)nticket) ticket[j] = 0;
}

// ---------------------------------------------------------------------------
// Segmented (ensemble) form: many independent clusters in one launch.
// Cluster c owns particles [seg_start[c], seg_start[c] + seg_n[c]) and
// interacts only with itself.  Its (i-tile x j-tile) units are numbered
// after those of the previous clusters (unit_off), so the stream-K split
// runs over all clusters at once; its j-records start at record tile
// rec_tile_off[c]; its i-tiles are numbered itile_off[c] + t for the
// tickets.  A CTA's unit range may span clusters.
// ---------------------------------------------------------------------------
struct DsSegArgs {
    PairArgs p;
    const float4 *rec;
    double *part;
    int *ticket;
    const long long *unit_off, *itile_off, *rec_tile_off, *seg_start, *seg_n;
    long long C, U;
};

// largest c in [0, C) with off[c] <= u (off nondecreasing, off[C] > u)
__device__ __forceinline__ long long seg_find(const long long *off, long long C, long long u) {
    long long lo = 0, hi = C;
    while (hi - lo > 1) {
        const long long mid = (lo + hi) >> 1;
        if (__ldg(off + mid) <= u) lo = mid; else hi = mid;
    }
    return lo;
}

__global__ void ds32_pack_seg(PSet J, const long long *rec_tile_off, const long long *seg_start,
                              const long long *seg_n, long long C, size_t npairs, PackSpec ps, float *rec) {
    const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= npairs * 2) return;
    const size_t p = t >> 1;
    const int lane = (int)(t & 1);
    const long long c = seg_find(rec_tile_off, C, (long long)(p / DS_PAIRS));
    const long long lj = 2 * ((long long)p - rec_tile_off[c] * DS_PAIRS) + lane;
    const bool valid = lj < seg_n[c];
    const size_t j = (size_t)(seg_start[c] + (valid ? lj : 0));
    float *r = rec + p * (size_t)(2 * ps.jf);
    float h, l;
    for (int q = 0; q < 3; ++q) {
        split_ds(valid ? J.f[F_RX + q][j] : 0.0, h, l);
        r[2 * (R_XH + q) + lane] = h;
        r[2 * (R_XL + q) + lane] = l;
    }
    for (int q = 0; q < ps.nextra; ++q) {
        const int f = ps.extra[q];
        float v;
        if (f == -1) v = valid ? 1.0f : 0.0f;
        else if (f == -2) v = 0.0f;
        else if (f == F_E2) v = valid ? __double2float_rn(J.f[f][j]) : 1.0f;
        else v = valid ? __double2float_rn(J.f[f][j]) : 0.0f;
        r[2 * (6 + q) + lane] = v;
    }
}

template <class K>
__global__ void __launch_bounds__(DS_THREADS, TG_DS32_MINB) ds32_streamk_seg(DsSegArgs a) {
    extern __shared__ __align__(128) float4 ring[];
    __shared__ __align__(8) uint64_t full[DS_STAGES];
    __shared__ int s_last;
    constexpr int IPT = K::IPT;
    constexpr int TILE_Q = DS_PAIRS * K::NQ;
    constexpr unsigned TILE_BYTES = TILE_Q * sizeof(float4);
    constexpr int BI = DS_THREADS * IPT;
    constexpr int UNR = kunroll<K>::value;

    const long long U = a.U;
    const long long G = gridDim.x;
    const long long k = blockIdx.x;
    const long long u0 = unit_start(k, U, G), u1 = unit_start(k + 1, U, G);
    if (u0 >= u1) return;
    const int tid = threadIdx.x;

    if (tid == 0) {
        for (int s = 0; s < DS_STAGES; ++s) mbar_init(&full[s], 1);
        fence_mbar_init();
    }
    __syncthreads();
    long long pc = seg_find(a.unit_off, a.C, u0);   // producer's cluster cursor (tid 0)
    auto issue = [&](long long u, int s) {
        while (a.unit_off[pc + 1] <= u) ++pc;
        const long long njt = a.rec_tile_off[pc + 1] - a.rec_tile_off[pc];
        const long long jt = (u - a.unit_off[pc]) % njt;
        mbar_expect_tx(&full[s], TILE_BYTES);
        bulk_g2s(ring + s * TILE_Q, a.rec + (a.rec_tile_off[pc] + jt) * TILE_Q, TILE_BYTES, &full[s]);
    };
    if (tid == 0) {
        for (int s = 0; s < DS_STAGES && u0 + s < u1; ++s) issue(u0 + s, s);
    }

    // the unit's cluster, local i-tile and global i-tile
    long long c = seg_find(a.unit_off, a.C, u0);
    auto tile_of = [&](long long cl, long long u) {
        const long long njt = a.rec_tile_off[cl + 1] - a.rec_tile_off[cl];
        return (u - a.unit_off[cl]) / njt;
    };
    long long t = tile_of(c, u0);
    const long long git_first = a.itile_off[c] + t;
    typename K::IS st[IPT];
    auto load_tile = [&](long long cl, long long tt) {
#pragma unroll
        for (int q = 0; q < IPT; ++q) {
            const long long li = tt * BI + q * DS_THREADS + tid;
            const size_t i = (size_t)(a.seg_start[cl] + (li < a.seg_n[cl] ? li : 0));
            K::load(st[q], a.p, i);
        }
    };
    load_tile(c, t);
    bool aborted = false;
    long long abort_u = u1;
    long long issued_to = (u0 + DS_STAGES < u1) ? u0 + DS_STAGES : u1;

    for (long long u = u0, it = 0; u < u1; ++u, ++it) {
        const int s = (int)(it % DS_STAGES);
        const uint32_t parity = (uint32_t)((it / DS_STAGES) & 1);
        if (!mbar_wait(&full[s], parity)) aborted = true;
        if (__syncthreads_or(aborted)) {
            aborted = true;
            abort_u = u;
            break;
        }
        const float4 *R = ring + s * TILE_Q;
#pragma unroll 1
        for (int fb = 0; fb < DS_PAIRS; fb += DS_FOLD_PAIRS) {
#pragma unroll UNR
            for (int pp = 0; pp < DS_FOLD_PAIRS; ++pp) kstep<K, false>(st, R + (fb + pp) * K::NQ, f2(0.f));
#pragma unroll
            for (int q = 0; q < IPT; ++q) K::fold(st[q]);
        }
        __syncthreads();
        if (tid == 0 && u + DS_STAGES < u1) {
            issue(u + DS_STAGES, s);
            issued_to = u + DS_STAGES + 1;
        }
        // next unit's cluster and tile
        long long cn = c, tn = -1;
        if (u + 1 < u1) {
            while (a.unit_off[cn + 1] <= u + 1) ++cn;
            tn = tile_of(cn, u + 1);
        }
        if (cn == c && tn == t) continue;

        const long long njt = a.rec_tile_off[c + 1] - a.rec_tile_off[c];
        const long long ta = a.unit_off[c] + t * njt, tb = ta + njt;
        const long long git = a.itile_off[c] + t;
        if (ta >= u0 && tb <= u1) {
#pragma unroll
            for (int q = 0; q < IPT; ++q) {
                const long long li = t * BI + q * DS_THREADS + tid;
                double p[K::NP];
                K::partials(st[q], p);
                if (li < a.seg_n[c]) K::store(p, a.p, (size_t)(a.seg_start[c] + li));
            }
        } else {
            const int slot = (git == git_first) ? 0 : 1;
            double *mine = a.part + ((k * 2 + slot) * IPT * K::NP) * DS_THREADS;
#pragma unroll
            for (int q = 0; q < IPT; ++q) {
                double p[K::NP];
                K::partials(st[q], p);
                for (int v = 0; v < K::NP; ++v) mine[(q * K::NP + v) * DS_THREADS + tid] = p[v];
            }
            __threadfence();
            __syncthreads();
            const long long klo = unit_owner(ta, U, G), khi = unit_owner(tb - 1, U, G);
            if (tid == 0) {
                const int prev = atomicAdd(&a.ticket[git], 1);
                s_last = (prev == (int)(khi - klo));
            }
            __syncthreads();
            if (s_last) {
                // contributors summed in CTA order; two in flight per step
                __threadfence();
                auto slot_ptr = [&](long long kk) {
                    const long long us = unit_start(kk, U, G);
                    const long long ck = seg_find(a.unit_off, a.C, us);
                    const int sl = (git == a.itile_off[ck] + tile_of(ck, us)) ? 0 : 1;
                    return a.part + ((kk * 2 + sl) * IPT * K::NP) * DS_THREADS + tid;
                };
                double acc[IPT][K::NP];
                {
                    const double *s0 = slot_ptr(klo);
#pragma unroll
                    for (int q = 0; q < IPT; ++q)
#pragma unroll
                        for (int w = 0; w < K::NP; ++w) acc[q][w] = __ldcg(s0 + (q * K::NP + w) * DS_THREADS);
                }
                for (long long kk = klo + 1; kk <= khi; kk += 2) {
                    const bool two = kk + 1 <= khi;
                    const double *s0 = slot_ptr(kk);
                    const double *s1 = two ? slot_ptr(kk + 1) : s0;
#pragma unroll
                    for (int q = 0; q < IPT; ++q) {
                        double v0[K::NP], v1[K::NP];
#pragma unroll
                        for (int w = 0; w < K::NP; ++w) {
                            v0[w] = __ldcg(s0 + (q * K::NP + w) * DS_THREADS);
                            v1[w] = __ldcg(s1 + (q * K::NP + w) * DS_THREADS);
                        }
                        K::combine(acc[q], v0);
                        if (two) K::combine(acc[q], v1);
                    }
                }
#pragma unroll
                for (int q = 0; q < IPT; ++q) {
                    const long long li = t * BI + q * DS_THREADS + tid;
                    if (li < a.seg_n[c]) K::store(acc[q], a.p, (size_t)(a.seg_start[c] + li));
                }
            }
        }
        if (tn >= 0) {
            c = cn;
            t = tn;
            load_tile(c, t);
        }
    }

    if (aborted && tid == 0) {
        atomicOr(a.p.status, ST_MBAR_TIMEOUT);
        for (long long u = abort_u; u < issued_to; ++u) {
            const long long it = u - u0;
            mbar_wait(&full[it % DS_STAGES], (uint32_t)((it / DS_STAGES) & 1));
        }
    }
}

// ---------------------------------------------------------------------------
// Host side.
// ---------------------------------------------------------------------------
#ifndef TG_ORD_PHI
#define TG_ORD_PHI 1   // Phi calls of 2^24 pairs and more take the ordered kernel
#endif
#ifndef TG_ORD_UNITS_PER_CTA
#define TG_ORD_UNITS_PER_CTA 8   // ordered kernel: j-tiles are split until units >= this x CTA slots
#endif
constexpr long long ORD_UNITS_PER_CTA = TG_ORD_UNITS_PER_CTA;
constexpr long long ORD_MAX_CONTRIB = 24;   // mean CTAs per i-tile the j-split may reach
#ifndef TG_DS32_MAX_JSUB
#define TG_DS32_MAX_JSUB 2   // parts a j-tile may be split into (1 or 2; 2 measured best at N = 4096)
#endif
struct Geometry {
    long long nit, njt, units, grid;
    int jsub;
    size_t rec_bytes, part_bytes, ticket_bytes, tile_bytes;
};

// Resident CTAs per SM of kernel K (computed once; concurrent first calls
// compute the same value, so the atomic only makes the publication safe).
template <class K>
static int ctas_per_sm() {
    static std::atomic<int> cached{-1};
    int c = cached.load(std::memory_order_acquire);
    if (c < 0) {
        const size_t smem = (size_t)DS_STAGES * DS_PAIRS * K::NQ * sizeof(float4);
        cudaFuncSetAttribute(ds32_streamk<K, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        cudaFuncSetAttribute(ds32_streamk<K, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        int n = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, ds32_streamk<K, 1>, DS_THREADS, smem) != cudaSuccess || n < 1)
            n = 1;
        cached.store(n, std::memory_order_release);
        c = n;
    }
    return c;
}

static size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

template <class K, class = void>
struct is_ordered : std::false_type {};
template <class K>
struct is_ordered<K, std::void_t<decltype(K::ORDERED)>> : std::true_type {};

// Resident CTAs per SM of the ordered kernel for K (as ctas_per_sm).
template <class K>
static int ctas_per_sm_ord() {
    static std::atomic<int> cached{-1};
    int c = cached.load(std::memory_order_acquire);
    if (c < 0) {
        const size_t smem = (size_t)DS_STAGES * DS_PAIRS * K::NQ * sizeof(float4);
        cudaFuncSetAttribute(ds32_ord<K, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        cudaFuncSetAttribute(ds32_ord<K, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        cudaFuncSetAttribute(ds32_ord<K, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        cudaFuncSetAttribute(ds32_ord<K, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        int n = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, ds32_ord<K, 1>, DS_THREADS, smem) != cudaSuccess || n < 1)
            n = 1;
        cached.store(n, std::memory_order_release);
        c = n;
    }
    return c;
}

template <class K>
static int ctas_for() {
    if constexpr (is_ordered<K>::value) return ctas_per_sm_ord<K>();
    else return ctas_per_sm<K>();
}

template <class K>
static Geometry geometry(size_t ni, size_t nj, int sms) {
    Geometry g;
    const size_t bi = (size_t)DS_THREADS * K::IPT;
    g.nit = (long long)((ni + bi - 1) / bi);
    g.njt = (long long)((nj + DS_TILE - 1) / DS_TILE);
    const long long slots = (long long)sms * ctas_for<K>();
    // Split j-tiles in two when there are fewer than two units per CTA slot,
    // or when halving the units evens out the CTAs' shares by 10% or more:
    // a CTA's time is its whole-unit count, ceil(U / slots) units of size
    // 1 / jsub (N = 16384, AccJerk: 4 whole units per CTA, or 7 halves).
    g.jsub = 1;
    if constexpr (is_ordered<K>::value) {
        // cost-weighted CTA ranges end on unit boundaries: split j-tiles
        // (up to 8 parts of 64 j) until there are ORD_UNITS_PER_CTA units
        // per CTA slot, so small calls fill the GPU and a CTA's share is
        // within about 1 / ORD_UNITS_PER_CTA of the mean -- but not so far
        // that an i-tile's partial sums come from more than ORD_MAX_CONTRIB
        // CTAs on average (its last CTA adds them all; N = 4096: 0.18 ms
        // with 8 parts, 0.16 ms with 2)
        while (g.jsub < 8 && g.nit * g.njt * g.jsub < ORD_UNITS_PER_CTA * slots) {
            const long long u2 = g.nit * g.njt * g.jsub * 2, grid2 = u2 < slots ? u2 : slots;
            if (grid2 > ORD_MAX_CONTRIB * g.nit) break;
            g.jsub *= 2;
        }
    } else if (TG_DS32_MAX_JSUB >= 2) {
        const long long u = g.nit * g.njt;
        const double t1 = (double)((u + slots - 1) / slots), t2 = 0.5 * (double)((2 * u + slots - 1) / slots);
        if (u < 2 * slots || t2 <= 0.9 * t1) g.jsub = 2;
    }
    g.units = g.nit * g.njt * g.jsub;
    g.grid = g.units < slots ? g.units : slots;
    g.rec_bytes = align_up((size_t)g.njt * DS_PAIRS * K::NQ * sizeof(float4), 256);
    g.part_bytes = align_up((size_t)g.grid * 2 * K::IPT * K::NP * DS_THREADS * sizeof(double), 256);
    g.ticket_bytes = align_up((size_t)g.nit * sizeof(int), 256);
    g.tile_bytes = K::UE2 ? align_up((size_t)g.njt * sizeof(float), 256) : 0;
    return g;
}

template <class K>
static size_t ws_bytes_for(size_t ni, size_t nj, int sms) {
    const Geometry g = geometry<K>(ni, nj, sms);
    return g.rec_bytes + g.part_bytes + g.ticket_bytes + g.tile_bytes;
}

template <class K>
static cudaError_t run_ds(const PairArgs &p, void *ws, size_t ws_bytes, int sms, cudaStream_t s) {
    const Geometry g = geometry<K>(p.ni, p.nj, sms);
    if (g.rec_bytes + g.part_bytes + g.ticket_bytes + g.tile_bytes > ws_bytes) return cudaErrorInvalidValue;
    char *base = static_cast<char *>(ws);
    DsArgs a;
    a.p = p;
    a.rec = reinterpret_cast<const float4 *>(base);
    a.part = reinterpret_cast<double *>(base + g.rec_bytes);
    a.ticket = reinterpret_cast<int *>(base + g.rec_bytes + g.part_bytes);
    float *tile_e2 = reinterpret_cast<float *>(base + g.rec_bytes + g.part_bytes + g.ticket_bytes);
    a.tile_e2 = K::UE2 ? tile_e2 : nullptr;
    a.nit = g.nit;
    a.njt = g.njt;
    const size_t smem = (size_t)DS_STAGES * DS_PAIRS * K::NQ * sizeof(float4);
    PrepArgs z{a.ticket, g.nit};
    ds32_prepare<<<(unsigned)g.njt, DS_TILE, 0, s>>>(p.J, p.nj, K::pack(), reinterpret_cast<float *>(base),
                                                 K::UE2 ? tile_e2 : nullptr, z);
    if (g.jsub == 2) ds32_streamk<K, 2><<<(unsigned)g.grid, DS_THREADS, smem, s>>>(a);
    else ds32_streamk<K, 1><<<(unsigned)g.grid, DS_THREADS, smem, s>>>(a);
    return cudaGetLastError();
}

// Same launch as run_ds with the grid limited to max_grid CTAs.
template <class K>
static Geometry geometry_capped(size_t ni, size_t nj, int sms, long long max_grid) {
    Geometry g = geometry<K>(ni, nj, sms);
    if (max_grid > 0 && g.grid > max_grid) {
        g.grid = max_grid;
        g.part_bytes = align_up((size_t)g.grid * 2 * K::IPT * K::NP * DS_THREADS * sizeof(double), 256);
    }
    return g;
}

template <class K>
static cudaError_t run_ds_capped(const PairArgs &p, void *ws, size_t ws_bytes, int sms,
                                 long long max_grid, cudaStream_t s) {
    const Geometry g = geometry_capped<K>(p.ni, p.nj, sms, max_grid);
    if (g.rec_bytes + g.part_bytes + g.ticket_bytes > ws_bytes) return cudaErrorInvalidValue;
    char *base = static_cast<char *>(ws);
    DsArgs a;
    a.p = p;
    a.rec = reinterpret_cast<const float4 *>(base);
    a.part = reinterpret_cast<double *>(base + g.rec_bytes);
    a.ticket = reinterpret_cast<int *>(base + g.rec_bytes + g.part_bytes);
    a.tile_e2 = nullptr;   // general path only: the scratch layout stays fixed
    a.nit = g.nit;
    a.njt = g.njt;

    const size_t npairs = (size_t)g.njt * DS_PAIRS;
    const PackSpec spec = K::pack();
    const unsigned pack_blocks = (unsigned)((npairs * 2 + 255) / 256);
    ds32_pack<<<pack_blocks, 256, 0, s>>>(p.J, p.nj, npairs, spec, reinterpret_cast<float *>(base));
    cudaError_t e = cudaMemsetAsync(a.ticket, 0, g.ticket_bytes, s);
    if (e != cudaSuccess) return e;
    const size_t smem = (size_t)DS_STAGES * DS_PAIRS * K::NQ * sizeof(float4);
    if (g.jsub == 2) ds32_streamk<K, 2><<<(unsigned)g.grid, DS_THREADS, smem, s>>>(a);
    else ds32_streamk<K, 1><<<(unsigned)g.grid, DS_THREADS, smem, s>>>(a);
    return cudaGetLastError();
}


// ---------------------------------------------------------------------------
// Ordered launch (Acc, AccJerk): spatial order, records with block-relative
// positions, block and i-tile boxes, the pairwise kernel, then the
// double-single recompute of the particles it flagged.
// ---------------------------------------------------------------------------
struct OrdLayout {
    Geometry g;
    size_t blk_bytes, ibox_bytes, flag_bytes, jd_bytes, ref_bytes, form_bytes, cost_bytes, scan_bytes, start_bytes,
        order_bytes;
    size_t total() const {
        return g.rec_bytes + g.part_bytes + g.ticket_bytes + g.tile_bytes + blk_bytes + ibox_bytes + flag_bytes +
               jd_bytes + ref_bytes + form_bytes + 2 * cost_bytes + scan_bytes + start_bytes + order_bytes;
    }
};

template <class K>
static OrdLayout ord_layout(size_t ni, size_t nj, int sms, bool same) {
    OrdLayout L;
    L.g = geometry<K>(ni, nj, sms);
    L.blk_bytes = align_up((size_t)L.g.njt * ORD_BLOCKS_PER_TILE * sizeof(OrdInfo), 256);
    L.ibox_bytes = align_up((size_t)L.g.nit * 2 * sizeof(float4), 256);
    L.flag_bytes = align_up((ni + 64) * sizeof(int), 256);
    L.jd_bytes = align_up(nj * EXACT_JQ * sizeof(float4), 256);
    L.ref_bytes = align_up((size_t)EXACT_MAX_SPLIT * (EXACT_MAX_CHUNKS * 6 * sizeof(double) + sizeof(int)), 256);
    L.form_bytes = align_up((size_t)L.g.nit * L.g.njt * ORD_BLOCKS_PER_TILE, 256);
    L.cost_bytes = align_up((size_t)L.g.units * sizeof(int), 256);
    L.scan_bytes = align_up(inclusive_sum_bytes((size_t)L.g.units), 256);
    L.start_bytes = align_up(((size_t)L.g.grid + 1) * sizeof(long long), 256);
    L.order_bytes = order_workspace_bytes(ni, nj, same);
    return L;
}

// Calls below the ordered path's size take the double-single kernel for
// every i-particle: j-data, chunk partials and tickets.
static size_t exact_ws_bytes(size_t nj) {
    return align_up(nj * EXACT_JQ * sizeof(float4), 256) +
           align_up((size_t)EXACT_MAX_SPLIT * (EXACT_MAX_CHUNKS * 6 * sizeof(double) + sizeof(int)), 256);
}
template <int MODE>
static cudaError_t run_exact(const PairArgs &p, void *ws, size_t ws_bytes, int sms, cudaStream_t s) {
    if (exact_ws_bytes(p.nj) > ws_bytes) return cudaErrorInvalidValue;
    char *q = static_cast<char *>(ws);
    float4 *jd = reinterpret_cast<float4 *>(q); q += align_up(p.nj * EXACT_JQ * sizeof(float4), 256);
    double *part = reinterpret_cast<double *>(q);
    int *ticket = reinterpret_cast<int *>(part + (size_t)EXACT_MAX_SPLIT * EXACT_MAX_CHUNKS * 6);
    const size_t n = p.nj > (size_t)EXACT_MAX_SPLIT ? p.nj : (size_t)EXACT_MAX_SPLIT;
    const int ufield = MODE == EX_ACC_JERK ? F_VX : (MODE == EX_VJP ? F_AX : -1);
    ds32_exact_prepare<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(p.J, p.nj, ufield, jd, ticket, EXACT_MAX_SPLIT);
    ds32_exact<MODE><<<(unsigned)(sms * 4), EXACT_THREADS, 0, s>>>(p, jd, nullptr, nullptr, part, ticket);
    return cudaGetLastError();
}

// The ordered path serves Acc and AccJerk calls of at least 2^24 pairs.
static bool ord_applies(size_t ni, size_t nj) {
    return ni >= 512 && nj >= 512 && (double)ni * (double)nj >= 16777216.0 && nj < ((size_t)1 << 30);
}
// Phi has no cancellation to guard against (every term has one sign), so it
// takes the ordered kernel for speed alone: from 2^31 pairs, where its
// cheaper far blocks outweigh the ordering's fixed cost (N = 65536: 1.63 ms
// against 2.02 ms unordered; N = 16384: 0.25 against 0.17 ms).
static bool phi_ord_applies(size_t ni, size_t nj) {
    return TG_ORD_PHI && ord_applies(ni, nj) && (double)ni * (double)nj >= 2147483648.0;
}

static bool same_sets(const PairArgs &p, int nfields) {
    if (p.ni != p.nj) return false;
    for (int f = 0; f < nfields; ++f)
        if (p.I.f[f] != p.J.f[f]) return false;
    return true;
}

// Optional timing of the ordered pairwise kernel (tg_time_pair_kernel):
// CUDA events recorded on the call's stream around its launch.
static std::atomic<int> g_prof{0};
static std::mutex g_prof_mu;
struct ProfRec {
    int kernel;
    cudaEvent_t e0, e1;
};
static std::vector<ProfRec> g_prof_rec;

int prof_enable(int on) { return g_prof.exchange(on ? 1 : 0); }

cudaError_t prof_read(int kernel, double *ms, long long *launches) {
    std::lock_guard<std::mutex> lk(g_prof_mu);
    *ms = 0.0;
    *launches = 0;
    cudaError_t err = cudaSuccess;
    std::vector<ProfRec> keep;
    for (const ProfRec &r : g_prof_rec) {
        if (r.kernel != kernel) { keep.push_back(r); continue; }
        float t = 0.f;
        cudaError_t e = cudaEventSynchronize(r.e1);
        if (e == cudaSuccess) e = cudaEventElapsedTime(&t, r.e0, r.e1);
        if (e != cudaSuccess && err == cudaSuccess) err = e;
        *ms += t;
        *launches += 1;
        cudaEventDestroy(r.e0);
        cudaEventDestroy(r.e1);
    }
    g_prof_rec.swap(keep);
    return err;
}

template <class K>
static cudaError_t run_ord(const PairArgs &p, int nfields, void *ws, size_t ws_bytes, int sms, cudaStream_t s) {
    const bool same = same_sets(p, nfields);
    const OrdLayout L = ord_layout<K>(p.ni, p.nj, sms, same);
    const Geometry &g = L.g;
    if (L.total() > ws_bytes) return cudaErrorInvalidValue;
    char *q = static_cast<char *>(ws);
    float *rec = reinterpret_cast<float *>(q); q += g.rec_bytes;
    double *part = reinterpret_cast<double *>(q); q += g.part_bytes;
    int *ticket = reinterpret_cast<int *>(q); q += g.ticket_bytes;
    float *tile_e2 = reinterpret_cast<float *>(q); q += g.tile_bytes;
    OrdInfo *blk = reinterpret_cast<OrdInfo *>(q); q += L.blk_bytes;
    float4 *ibox = reinterpret_cast<float4 *>(q); q += L.ibox_bytes;
    int *flags = reinterpret_cast<int *>(q); q += L.flag_bytes;   // [0] count, [64..] list
    float4 *jd = reinterpret_cast<float4 *>(q); q += L.jd_bytes;
    double *ref_part = reinterpret_cast<double *>(q);
    int *ref_ticket = reinterpret_cast<int *>(ref_part + (size_t)EXACT_MAX_SPLIT * EXACT_MAX_CHUNKS * 6);
    q += L.ref_bytes;
    unsigned char *form = reinterpret_cast<unsigned char *>(q); q += L.form_bytes;
    int *ucost = reinterpret_cast<int *>(q); q += L.cost_bytes;
    int *ucum = reinterpret_cast<int *>(q); q += L.cost_bytes;
    void *scan_ws = q; q += L.scan_bytes;
    long long *start = reinterpret_cast<long long *>(q); q += L.start_bytes;
    void *order_ws = q;

    OrderOut o;
    cudaError_t e = build_order(p.I, p.ni, p.J, p.nj, same, order_ws, L.order_bytes, o, s);
    if (e != cudaSuccess) return e;
    ds32_ord_prepare<K><<<(unsigned)g.njt, DS_TILE, 0, s>>>(p.J, p.nj, o.pj, o.nlight, rec, blk, tile_e2, ticket,
                                                          g.nit, flags, jd, ref_ticket, EXACT_MAX_SPLIT);
    constexpr int BI = DS_THREADS * K::IPT;
    ds32_ord_ibox<<<(unsigned)g.nit, BI, 0, s>>>(p.I, p.ni, o.pi, ibox);
    const long long nblk = g.njt * ORD_BLOCKS_PER_TILE, nju = g.njt * g.jsub;
    ds32_ord_plan<<<(unsigned)g.nit, 256, 0, s>>>(ibox, blk, nblk, nju, ORD_BLOCKS_PER_TILE / g.jsub, K::W_FAR,
                                                  K::W_NEAR, K::W_HEAVY, form, ucost);
    e = inclusive_sum(ucost, ucum, (size_t)g.units, scan_ws, L.scan_bytes, s);
    if (e != cudaSuccess) return e;
    ds32_ord_bounds<<<(unsigned)((g.units + 255) / 256), 256, 0, s>>>(ucost, ucum, g.units, g.grid, start);

    DsOrdArgs a;
    a.d.p = p;
    a.d.rec = reinterpret_cast<const float4 *>(rec);
    a.d.part = part;
    a.d.ticket = ticket;
    a.d.tile_e2 = tile_e2;
    a.d.nit = g.nit;
    a.d.njt = g.njt;
    a.pi = o.pi;
    a.blk = blk;
    a.form = form;
    a.start = start;
    a.flag_count = flags;
    a.flag_list = flags + 64;
    a.tau = ord_tau(p.nj);
    a.tau_jerk = ORD_TAU_JERK_FACTOR * a.tau;
    const size_t smem = (size_t)DS_STAGES * DS_PAIRS * K::NQ * sizeof(float4);
    ProfRec pr{K::KERNEL, nullptr, nullptr};
    const bool prof = (K::KERNEL == K_ACC || K::KERNEL == K_ACC_JERK) && g_prof.load() &&
                      cudaEventCreate(&pr.e0) == cudaSuccess &&
                      cudaEventCreate(&pr.e1) == cudaSuccess && cudaEventRecord(pr.e0, s) == cudaSuccess;
    switch (g.jsub) {
        case 8: ds32_ord<K, 8><<<(unsigned)g.grid, DS_THREADS, smem, s>>>(a); break;
        case 4: ds32_ord<K, 4><<<(unsigned)g.grid, DS_THREADS, smem, s>>>(a); break;
        case 2: ds32_ord<K, 2><<<(unsigned)g.grid, DS_THREADS, smem, s>>>(a); break;
        default: ds32_ord<K, 1><<<(unsigned)g.grid, DS_THREADS, smem, s>>>(a); break;
    }
    if (prof && cudaEventRecord(pr.e1, s) == cudaSuccess) {
        std::lock_guard<std::mutex> lk(g_prof_mu);
        g_prof_rec.push_back(pr);
    }
    // flagged AccJerk particles get both vectors recomputed (a second list
    // for the acceleration-only ones measured no faster); Phi has no recompute
    if constexpr (K::PX >= 0)
        ds32_exact<K::PJ >= 0 ? EX_ACC_JERK : EX_ACC><<<(unsigned)(sms * 4), EXACT_THREADS, 0, s>>>(
            p, jd, flags, flags + 64, ref_part, ref_ticket);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Segmented launch.  Host tables (per cluster, nondecreasing prefixes) are
// built by the caller for this kernel's i-tile size; `dev` points to the
// same tables on the device in the order unit_off[C+1], itile_off[C+1],
// rec_tile_off[C+1], seg_start[C], seg_n[C].
// ---------------------------------------------------------------------------
template <class K>
static int ds32_bi() { return DS_THREADS * K::IPT; }

template <class K>
static int ctas_per_sm_seg() {
    static std::atomic<int> cached{-1};
    int c = cached.load(std::memory_order_acquire);
    if (c < 0) {
        const size_t smem = (size_t)DS_STAGES * DS_PAIRS * K::NQ * sizeof(float4);
        cudaFuncSetAttribute(ds32_streamk_seg<K>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        int n = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, ds32_streamk_seg<K>, DS_THREADS, smem) != cudaSuccess || n < 1)
            n = 1;
        cached.store(n, std::memory_order_release);
        c = n;
    }
    return c;
}

template <class K>
static size_t seg_ws_bytes(long long U, long long NIT, long long NJT, int sms, int grid_mult) {
    const long long slots = (long long)sms * ctas_per_sm_seg<K>() * (grid_mult > 0 ? grid_mult : 1);
    const long long grid = U < slots ? U : slots;
    return align_up((size_t)NJT * DS_PAIRS * K::NQ * sizeof(float4), 256) +
           align_up((size_t)grid * 2 * K::IPT * K::NP * DS_THREADS * sizeof(double), 256) +
           align_up((size_t)NIT * sizeof(int), 256);
}

template <class K>
static cudaError_t run_ds_seg(const PairArgs &p, const SegGeometry &g, void *ws, size_t ws_bytes, int sms,
                              int grid_mult, cudaStream_t s) {
    if (g.U == 0) return cudaSuccess;
    const long long slots = (long long)sms * ctas_per_sm_seg<K>() * (grid_mult > 0 ? grid_mult : 1);
    const long long grid = g.U < slots ? g.U : slots;
    const size_t rec_bytes = align_up((size_t)g.NJT * DS_PAIRS * K::NQ * sizeof(float4), 256);
    const size_t part_bytes = align_up((size_t)grid * 2 * K::IPT * K::NP * DS_THREADS * sizeof(double), 256);
    const size_t ticket_bytes = align_up((size_t)g.NIT * sizeof(int), 256);
    if (rec_bytes + part_bytes + ticket_bytes > ws_bytes) return cudaErrorInvalidValue;
    char *base = static_cast<char *>(ws);
    DsSegArgs a;
    a.p = p;
    a.rec = reinterpret_cast<const float4 *>(base);
    a.part = reinterpret_cast<double *>(base + rec_bytes);
    a.ticket = reinterpret_cast<int *>(base + rec_bytes + part_bytes);
    a.C = g.C;
    a.U = g.U;
    a.unit_off = g.dev;
    a.itile_off = g.dev + (g.C + 1);
    a.rec_tile_off = g.dev + 2 * (g.C + 1);
    a.seg_start = g.dev + 3 * (g.C + 1);
    a.seg_n = g.dev + 3 * (g.C + 1) + g.C;
    const size_t npairs = (size_t)g.NJT * DS_PAIRS;
    const unsigned pack_blocks = (unsigned)((npairs * 2 + 255) / 256);
    ds32_pack_seg<<<pack_blocks, 256, 0, s>>>(p.J, a.rec_tile_off, a.seg_start, a.seg_n, g.C, npairs,
                                              K::pack(), reinterpret_cast<float *>(base));
    cudaError_t e = cudaMemsetAsync(a.ticket, 0, ticket_bytes, s);
    if (e != cudaSuccess) return e;
    const size_t smem = (size_t)DS_STAGES * DS_PAIRS * K::NQ * sizeof(float4);
    ds32_streamk_seg<K><<<(unsigned)grid, DS_THREADS, smem, s>>>(a);
    return cudaGetLastError();
}

#ifndef TG_DS32_REFINE
#define TG_DS32_REFINE 0
#endif
#ifndef TG_DS32_IPT
#define TG_DS32_IPT 2
#endif
constexpr bool REF = TG_DS32_REFINE != 0;
constexpr int IPT2 = TG_DS32_IPT;

// Small problems take the one-i-per-thread instance K1 (256-particle
// i-tiles) of a kernel whose default instance K2 holds two: when even
// half-size units leave CTA slots empty, smaller i-tiles give twice the
// units, each half as long (N = 4096: 256 units instead of 128).
template <class K2, class K1>
static bool small_pick(size_t ni, size_t nj, int sms) {
    if (K2::IPT == K1::IPT) return false;
    const Geometry g = geometry<K2>(ni, nj, sms);
    return g.units < (long long)sms * ctas_per_sm<K2>();
}
template <class K2, class K1>
static size_t ws_pick(size_t ni, size_t nj, int sms) {
    return small_pick<K2, K1>(ni, nj, sms) ? ws_bytes_for<K1>(ni, nj, sms) : ws_bytes_for<K2>(ni, nj, sms);
}
template <class K2, class K1>
static cudaError_t run_pick(const PairArgs &a, void *ws, size_t ws_bytes, int sms, cudaStream_t s) {
    return small_pick<K2, K1>(a.ni, a.nj, sms) ? run_ds<K1>(a, ws, ws_bytes, sms, s)
                                               : run_ds<K2>(a, ws, ws_bytes, sms, s);
}

bool ds32_supported(int kernel) { return kernel != K_SAKURA && kernel >= 0 && kernel < K_COUNT; }

size_t ds32_workspace_bytes(int kernel, size_t ni, size_t nj, int sms) {
    switch (kernel) {
        case K_PHI:
            if (phi_ord_applies(ni, nj)) return ord_layout<PhiOrd<2>>(ni, nj, sms, false).total();
            return ws_pick<PhiDS<IPT2, REF>, PhiDS<1, REF>>(ni, nj, sms);
        case K_ACC:
            if (ord_applies(ni, nj)) return ord_layout<AccOrd<2>>(ni, nj, sms, false).total();
            return exact_ws_bytes(nj);
        case K_ACC_JERK:
            if (ord_applies(ni, nj)) return ord_layout<AccJerkOrd<2>>(ni, nj, sms, false).total();
            return exact_ws_bytes(nj);
        case K_SNAP_CRACKLE: return ws_bytes_for<SnapCrackleDS<1, REF>>(ni, nj, sms);
        case K_TSTEP: return ws_pick<TstepDS<IPT2, REF>, TstepDS<1, REF>>(ni, nj, sms);
        case K_PNACC: return ws_bytes_for<PNAccDS<1, REF>>(ni, nj, sms);
        case K_ACC_VJP: return exact_ws_bytes(nj);
        default: return 0;
    }
}

cudaError_t launch_ds32(int kernel, const PairArgs &a, void *ws, size_t ws_bytes, int sms, cudaStream_t s) {
    switch (kernel) {
        case K_PHI:
            if (phi_ord_applies(a.ni, a.nj)) return run_ord<PhiOrd<2>>(a, 5, ws, ws_bytes, sms, s);
            return run_pick<PhiDS<IPT2, REF>, PhiDS<1, REF>>(a, ws, ws_bytes, sms, s);
        case K_ACC:
            if (ord_applies(a.ni, a.nj)) return run_ord<AccOrd<2>>(a, 5, ws, ws_bytes, sms, s);
            return run_exact<EX_ACC>(a, ws, ws_bytes, sms, s);
        case K_ACC_JERK:
            if (ord_applies(a.ni, a.nj)) return run_ord<AccJerkOrd<2>>(a, 8, ws, ws_bytes, sms, s);
            return run_exact<EX_ACC_JERK>(a, ws, ws_bytes, sms, s);
        case K_SNAP_CRACKLE: return run_ds<SnapCrackleDS<1, REF>>(a, ws, ws_bytes, sms, s);
        case K_TSTEP: return run_pick<TstepDS<IPT2, REF>, TstepDS<1, REF>>(a, ws, ws_bytes, sms, s);
        case K_PNACC: return run_ds<PNAccDS<1, REF>>(a, ws, ws_bytes, sms, s);
        case K_ACC_VJP: return run_exact<EX_VJP>(a, ws, ws_bytes, sms, s);
        default: return cudaErrorInvalidValue;
    }
}

bool ds32x_supported(int kernel) { return kernel == K_ACC || kernel == K_ACC_JERK || kernel == K_ACC_VJP; }

size_t ds32x_workspace_bytes(int kernel, size_t nj) { return ds32x_supported(kernel) ? exact_ws_bytes(nj) : 0; }

// TG_PREC_DS32X: the double-single kernel for every particle, whatever the size
cudaError_t launch_ds32x(int kernel, const PairArgs &a, void *ws, size_t ws_bytes, int sms, cudaStream_t s) {
    switch (kernel) {
        case K_ACC: return run_exact<EX_ACC>(a, ws, ws_bytes, sms, s);
        case K_ACC_JERK: return run_exact<EX_ACC_JERK>(a, ws, ws_bytes, sms, s);
        case K_ACC_VJP: return run_exact<EX_VJP>(a, ws, ws_bytes, sms, s);
        default: return cudaErrorInvalidValue;
    }
}

size_t ds32_workspace_bytes_capped(int kernel, size_t ni, size_t nj, int sms, long long max_grid) {
    if (kernel != K_ACC_JERK) return 0;
    const Geometry g = geometry_capped<AccJerkDS<IPT2, REF>>(ni, nj, sms, max_grid);
    return g.rec_bytes + g.part_bytes + g.ticket_bytes;
}

cudaError_t launch_ds32_capped(int kernel, const PairArgs &a, void *ws, size_t ws_bytes, int sms,
                               long long max_grid, cudaStream_t s) {
    if (kernel != K_ACC_JERK) return cudaErrorInvalidValue;
    return run_ds_capped<AccJerkDS<IPT2, REF>>(a, ws, ws_bytes, sms, max_grid, s);
}

// i-particles per thread of the segmented instances: 1 or 2 (2 is the
// default of the single-set kernels); SnapCrackle always uses 1.
int ds32_tile_i(int kernel, int ipt) {
    if (kernel == K_SNAP_CRACKLE) return ds32_bi<SnapCrackleDS<1, REF>>();
    return ipt == 1 ? DS_THREADS : DS_THREADS * 2;
}

int ds32_tile_j() { return DS_TILE; }

size_t ds32_seg_workspace_bytes(int kernel, int ipt, const SegGeometry &g, int sms, int grid_mult) {
    const bool one = ipt == 1;
    switch (kernel) {
        case K_PHI: return one ? seg_ws_bytes<PhiDS<1, REF>>(g.U, g.NIT, g.NJT, sms, grid_mult)
                               : seg_ws_bytes<PhiDS<2, REF>>(g.U, g.NIT, g.NJT, sms, grid_mult);
        case K_ACC: return one ? seg_ws_bytes<AccDS<1, REF>>(g.U, g.NIT, g.NJT, sms, grid_mult)
                               : seg_ws_bytes<AccDS<2, REF>>(g.U, g.NIT, g.NJT, sms, grid_mult);
        case K_ACC_JERK: return one ? seg_ws_bytes<AccJerkDS<1, REF>>(g.U, g.NIT, g.NJT, sms, grid_mult)
                                    : seg_ws_bytes<AccJerkDS<2, REF>>(g.U, g.NIT, g.NJT, sms, grid_mult);
        case K_SNAP_CRACKLE: return seg_ws_bytes<SnapCrackleDS<1, REF>>(g.U, g.NIT, g.NJT, sms, grid_mult);
        default: return 0;
    }
}

cudaError_t launch_ds32_seg(int kernel, int ipt, const PairArgs &a, const SegGeometry &g, void *ws,
                            size_t ws_bytes, int sms, int grid_mult, cudaStream_t s) {
    const bool one = ipt == 1;
    switch (kernel) {
        case K_PHI: return one ? run_ds_seg<PhiDS<1, REF>>(a, g, ws, ws_bytes, sms, grid_mult, s)
                               : run_ds_seg<PhiDS<2, REF>>(a, g, ws, ws_bytes, sms, grid_mult, s);
        case K_ACC: return one ? run_ds_seg<AccDS<1, REF>>(a, g, ws, ws_bytes, sms, grid_mult, s)
                               : run_ds_seg<AccDS<2, REF>>(a, g, ws, ws_bytes, sms, grid_mult, s);
        case K_ACC_JERK: return one ? run_ds_seg<AccJerkDS<1, REF>>(a, g, ws, ws_bytes, sms, grid_mult, s)
                                    : run_ds_seg<AccJerkDS<2, REF>>(a, g, ws, ws_bytes, sms, grid_mult, s);
        case K_SNAP_CRACKLE: return run_ds_seg<SnapCrackleDS<1, REF>>(a, g, ws, ws_bytes, sms, grid_mult, s);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace tg
