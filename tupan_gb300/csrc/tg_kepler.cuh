// tg_kepler.cuh -- FP64 two-body propagation for the Sakura kernel.
//
// Restates, for the GPU, the pair evolution of tupan/lib/src/
// sakura_kernel_common.h:8-191 (get_acc, leapfrog, twobody_solver,
// evolve_twobody) and the universal-variable Kepler solver of
// tupan/lib/src/universal_kepler_solver.h:17-614 (also behind the Kepler
// pair solver of kepler_solver_kernel_common.h:8-81): Stumpff functions in their
// closed forms, order-5 Laguerre iteration (tolerance 2^-42, 64 iterations),
// period folding for bound orbits, the hyperbolic first guess, the Lagrange
// f/g update with r1 = sqrt(r1^2 + e2), step halving when the solver fails and
// step doubling when the softened two-body energy drifts by more than
// 64 * 2^-42.
//
// The reference retries without bound and never returns for some inputs
// (radial orbits with v = 0; softened close pairs whose energy test cannot
// pass).  Here every retry loop is bounded: at most split_cap halvings,
// energy_cap doublings and solve_budget Kepler solves per pair (KepBudget;
// KEP_* for Sakura, KEP_PAIR_* for the pair solver).  When
// a bound is hit the last iterate is kept and a status bit is raised, which
// the host turns into a nonzero return code.  Arithmetic operations use the
// exact (uncontracted) helpers so that the leapfrog branch is bit-identical to
// the reference; cos/sin/cosh/sinh/log are CUDA's double routines.
#pragma once
#include "tg_device.cuh"

namespace tg {

constexpr double KEP_TOL = 2.2737367544323205948e-13;  // 2^-42
constexpr int KEP_MAXITER = 64;
// Bounds for Sakura's pairwise kernel (N^2 pair evolutions per call) ...
constexpr int KEP_SPLIT_CAP = 6;       // up to 64 sub-steps after solver failures
constexpr int KEP_ENERGY_CAP = 4;      // up to 16 sub-steps for the energy test
constexpr int KEP_SOLVE_BUDGET = 1024; // Kepler solves per pair evolution
// ... and for the Kepler pair solver (a few pairs per call): up to 1024
// sub-steps for either test and 65536 solves per pair.
constexpr int KEP_PAIR_SPLIT_CAP = 10;
constexpr int KEP_PAIR_ENERGY_CAP = 10;
constexpr int KEP_PAIR_SOLVE_BUDGET = 65536;
constexpr double KEP_PI = 3.141592653589793;

struct KepBudget {
    int solves = 0;
    unsigned flags = 0;
    int split_cap = KEP_SPLIT_CAP;
    int energy_cap = KEP_ENERGY_CAP;
    int solve_budget = KEP_SOLVE_BUDGET;
};

__device__ __forceinline__ int ksign(double x) { return (x > 0) - (x < 0); }

__device__ __forceinline__ double stumpff0(double z) {
    if (z < 0) return cos(dsqrt(-z));
    if (z > 0) return cosh(dsqrt(z));
    return 1.0;
}
__device__ __forceinline__ double stumpff1(double z) {
    if (z < 0) { double q = dsqrt(-z); return ddiv(sin(q), q); }
    if (z > 0) { double q = dsqrt(z); return ddiv(sinh(q), q); }
    return 1.0;
}
__device__ __forceinline__ double stumpff2(double z) {
    if (z < 0) { double q = dsqrt(-z); return ddiv(dsub(cos(q), 1.0), z); }
    if (z > 0) { double q = dsqrt(z); return ddiv(dsub(cosh(q), 1.0), z); }
    return 0.5;
}
__device__ __forceinline__ double stumpff3(double z) {
    if (z < 0) { double q = dsqrt(-z); return ddiv(dsub(ddiv(sin(q), q), 1.0), z); }
    if (z > 0) { double q = dsqrt(z); return ddiv(dsub(ddiv(sinh(q), q), 1.0), z); }
    return 1.0 / 6.0;
}

// G_k(s) = s^k c_k(alpha s^2)
__device__ __forceinline__ double gfun0(double s, double al) { return stumpff0(dmul(al, dmul(s, s))); }
__device__ __forceinline__ double gfun1(double s, double al) { return dmul(s, stumpff1(dmul(al, dmul(s, s)))); }
__device__ __forceinline__ double gfun2(double s, double al) { double s2 = dmul(s, s); return dmul(s2, stumpff2(dmul(al, s2))); }
__device__ __forceinline__ double gfun3(double s, double al) {
    double s2 = dmul(s, s);
    return dmul(dmul(s, s2), stumpff3(dmul(al, s2)));
}

struct KepEq { double dt, r0, rv, m, al; };

__device__ __forceinline__ double kep_f(double s, const KepEq &k) {
    double mu = dadd(k.m, dmul(k.al, k.r0));
    return dsub(dadd(dadd(dmul(k.r0, s), dmul(k.rv, gfun2(s, k.al))), dmul(mu, gfun3(s, k.al))), k.dt);
}
__device__ __forceinline__ double kep_df(double s, const KepEq &k) {
    double mu = dadd(k.m, dmul(k.al, k.r0));
    return dadd(dadd(k.r0, dmul(k.rv, gfun1(s, k.al))), dmul(mu, gfun2(s, k.al)));
}
__device__ __forceinline__ double kep_ddf(double s, const KepEq &k) {
    double mu = dadd(k.m, dmul(k.al, k.r0));
    return dadd(dmul(k.rv, gfun0(s, k.al)), dmul(mu, gfun1(s, k.al)));
}

// Order-5 Laguerre root finder for the universal Kepler equation.
__device__ int kep_laguerre(double s0, double &s, const KepEq &k, KepBudget &b) {
    double x = s0, step;
    int it = 0;
    do {
        double f0 = kep_f(x, k), f1 = kep_df(x, k), f2 = kep_ddf(x, k);
        double f1sq = dmul(f1, f1);
        double bb = dsub(f1sq, dmul(f0, f2));
        double g = dmul(5.0, f0);
        double h = dadd(f1, dmul((double)ksign(f1), dsqrt(fabs(dmul(4.0, dsub(dmul(5.0, bb), f1sq))))));
        if (h == 0) { s = x; return -1; }
        step = ddiv(-g, h);
        x = dadd(x, step);
        it += 1;
        if (it > KEP_MAXITER) { s = x; return -2; }   // caller halves the step
    } while (fabs(step) > KEP_TOL);
    s = x;
    if (ksign(x) != ksign(s0)) return -3;
    return 0;
}

// One solve over dt0; updates r, v only on success.
__device__ int kep_once(double dt0, double m, double e2, double r[3], double v[3], KepBudget &b) {
    b.solves += 1;
    double r2 = ddot3(r[0], r[1], r[2], r[0], r[1], r[2]);
    if (!(r2 > 0)) return 0;
    r2 = dadd(r2, e2);
    double rn = dsqrt(r2);
    double v2 = ddot3(v[0], v[1], v[2], v[0], v[1], v[2]);
    double rv = ddot3(r[0], r[1], r[2], v[0], v[1], v[2]);
    double beta = dsub(2.0, ddiv(e2, r2));
    double al = dsub(v2, ddiv(dmul(beta, m), rn));
    double dt = dt0;
    if (al < 0) {
        double a = ddiv(m, fabs(al));
        double T = dmul(dmul(dmul(2.0, KEP_PI), a), dsqrt(ddiv(a, m)));
        double ratio = ddiv(dt0, T);
        dt = dmul(dsub(ratio, (double)(long long)ratio), T);
    }
    double s0 = ddiv(dt, rn);
    if (al > 0) {
        double sal = dsqrt(al);
        double ss = fabs(ddiv(dmul(dmul(2.0, al), dt), dadd(rv, ddiv(dadd(m, dmul(al, rn)), sal))));
        if (ss > 1) s0 = ddiv(dmul((double)ksign(dt), log(ss)), sal);
    }
    KepEq k{dt, rn, rv, m, al};
    double s;
    int err = kep_laguerre(s0, s, k, b);
    if (err != 0) return err;
    double lf = dsub(1.0, ddiv(dmul(m, gfun2(s, al)), rn));
    double lg = dsub(dt, dmul(m, gfun3(s, al)));
    double r1[3];
    for (int q = 0; q < 3; ++q) r1[q] = dadd(dmul(r[q], lf), dmul(v[q], lg));
    double r1n = dsqrt(dadd(ddot3(r1[0], r1[1], r1[2], r1[0], r1[1], r1[2]), e2));
    double ldf = ddiv(dmul(-m, gfun1(s, al)), dmul(rn, r1n));
    double ldg = ddiv(dadd(1.0, dmul(lg, ldf)), lf);
    for (int q = 0; q < 3; ++q) {
        double vq = dadd(dmul(r[q], ldf), dmul(v[q], ldg));
        r[q] = r1[q];
        v[q] = vq;
    }
    return 0;
}

// dt split into n equal solves, n doubling after a failed solve.
__device__ void kep_split(double dt, double m, double e2, const double r0[3], const double v0[3],
                          double r[3], double v[3], KepBudget &b) {
    long long n = 1;
    for (int tries = 0;; ++tries) {
        for (int q = 0; q < 3; ++q) { r[q] = r0[q]; v[q] = v0[q]; }
        bool failed = false;
        for (long long i = 0; i < n; ++i) {
            if (b.solves >= b.solve_budget) { b.flags |= ST_KEPLER_CAP; return; }
            if (kep_once(ddiv(dt, (double)n), m, e2, r, v, b) != 0) { failed = true; break; }
        }
        if (!failed) return;
        if (tries >= b.split_cap) { b.flags |= ST_KEPLER_CAP; return; }
        n *= 2;
    }
}

__device__ __forceinline__ void kep_energy(double m, double e2, const double r[3], const double v[3],
                                           double &u, double &en) {
    double r2 = dadd(ddot3(r[0], r[1], r[2], r[0], r[1], r[2]), e2);
    double rn = dsqrt(r2);
    double v2 = ddot3(v[0], v[1], v[2], v[0], v[1], v[2]);
    u = ddiv(dmul(2.0, m), rn);
    en = dsub(v2, u);
}

__device__ void kep_solve(double dt, double m, double e2, const double r0[3], const double v0[3],
                          double r[3], double v[3], KepBudget &b) {
    kep_split(dt, m, e2, r0, v0, r, v, b);
    if (e2 == 0) return;
    double r2 = ddot3(r0[0], r0[1], r0[2], r0[0], r0[1], r0[2]);
    if (!(r2 > 0)) {
        for (int q = 0; q < 3; ++q) { r[q] = r0[q]; v[q] = v0[q]; }
        return;
    }
    double u0, en0, u1, en1;
    kep_energy(m, e2, r0, v0, u0, en0);
    kep_energy(m, e2, r, v, u1, en1);
    const double tol = dmul(64.0, KEP_TOL);
    if (dmul(2.0, fabs(dsub(en1, en0))) < dmul(tol, dadd(u1, u0))) return;
    long long n = 1;
    for (int tries = 0; tries < b.energy_cap; ++tries) {
        n *= 2;
        for (int q = 0; q < 3; ++q) { r[q] = r0[q]; v[q] = v0[q]; }
        bool bad = false;
        for (long long i = 0; i < n; ++i) {
            double rs[3] = {r[0], r[1], r[2]}, vs[3] = {v[0], v[1], v[2]};
            kep_split(ddiv(dt, (double)n), m, e2, rs, vs, r, v, b);
            kep_energy(m, e2, r, v, u1, en1);
            if (dmul(2.0, fabs(dsub(en1, en0))) > dmul(tol, dadd(u1, u0))) { bad = true; break; }
            if (b.flags & ST_KEPLER_CAP) return;
        }
        if (!bad) return;
    }
    b.flags |= ST_KEPLER_CAP;
}

__device__ __forceinline__ void rel_acc(double m, double e2, const double r[3], double a[3]) {
    double r2 = ddot3(r[0], r[1], r[2], r[0], r[1], r[2]);
    double q2 = ddiv(1.0, dadd(r2, e2));
    if (!(r2 > 0)) q2 = 0;
    double q3 = dmul(q2, dsqrt(q2));
    double mq = dmul(m, q3);
    for (int k = 0; k < 3; ++k) a[k] = dmul(-mq, r[k]);
}

// dt / 2 as dt * 0.5 here and below: both round the same exact value.
__device__ __forceinline__ void pair_leapfrog(double dt, double m, double e2, const double r0[3],
                                              const double v0[3], double r[3], double v[3]) {
    double h = dmul(dt, 0.5);
    double a[3];
    for (int k = 0; k < 3; ++k) r[k] = dadd(r0[k], dmul(v0[k], h));
    rel_acc(m, e2, r, a);
    for (int k = 0; k < 3; ++k) v[k] = dadd(v0[k], dmul(a[k], dt));
    for (int k = 0; k < 3; ++k) r[k] = dadd(r[k], dmul(v[k], h));
}

// twobody_solver's branch (sakura_kernel_common.h:111-122): the
// universal-variable solver unless r^2 > (64 m / v^2)^2.
__device__ __forceinline__ bool twobody_uses_kepler(double m, const double r0[3], const double v0[3]) {
    double r2 = ddot3(r0[0], r0[1], r0[2], r0[0], r0[1], r0[2]);
    double v2 = ddot3(v0[0], v0[1], v0[2], v0[0], v0[1], v0[2]);
    double R = dmul(64.0, ddiv(m, v2));
    return !(r2 > dmul(R, R));
}

__device__ __forceinline__ void pair_twobody(double dt, double m, double e2, const double r0[3],
                                             const double v0[3], double r[3], double v[3],
                                             KepBudget &b) {
    if (!twobody_uses_kepler(m, r0, v0)) pair_leapfrog(dt, m, e2, r0, v0, r, v);
    else kep_solve(dt, m, e2, r0, v0, r, v, b);
}

// Whether pair_evolve with flag -1 or +1 (one two-body step) takes the
// universal-variable solver; the test is pair_twobody's on the same state.
__device__ __forceinline__ bool sakura_uses_kepler(double dt, long long flag, double m, const double r0[3],
                                                   const double v0[3]) {
    if (flag == -1) {
        double r[3];
        for (int k = 0; k < 3; ++k) r[k] = dsub(r0[k], dmul(v0[k], dt));
        return twobody_uses_kepler(m, r, v0);
    }
    return twobody_uses_kepler(m, r0, v0);
}

// Sakura's four flags (sakura_kernel_common.h:126-191); others are a no-op.
__device__ void pair_evolve(double dt, long long flag, double m, double e2, const double r0[3],
                            const double v0[3], double r1[3], double v1[3], KepBudget &b) {
    double r[3] = {r0[0], r0[1], r0[2]}, v[3] = {v0[0], v0[1], v0[2]};
    double rt[3], vt[3];
    if (flag == -1) {
        for (int k = 0; k < 3; ++k) r[k] = dsub(r[k], dmul(v[k], dt));
        pair_twobody(dt, m, e2, r, v, rt, vt, b);
        for (int k = 0; k < 3; ++k) { r[k] = rt[k]; v[k] = vt[k]; }
    } else if (flag == 1) {
        pair_twobody(dt, m, e2, r, v, rt, vt, b);
        for (int k = 0; k < 3; ++k) { r[k] = rt[k]; v[k] = vt[k]; }
        for (int k = 0; k < 3; ++k) r[k] = dsub(r[k], dmul(v[k], dt));
    } else if (flag == -2) {
        for (int k = 0; k < 3; ++k) r[k] = dsub(r[k], dmul(dmul(v[k], dt), 0.5));
        pair_twobody(dt, m, e2, r, v, rt, vt, b);
        for (int k = 0; k < 3; ++k) { r[k] = rt[k]; v[k] = vt[k]; }
        for (int k = 0; k < 3; ++k) r[k] = dsub(r[k], dmul(dmul(v[k], dt), 0.5));
    } else if (flag == 2) {
        double h = dmul(dt, 0.5);
        pair_twobody(h, m, e2, r, v, rt, vt, b);
        for (int k = 0; k < 3; ++k) { r[k] = rt[k]; v[k] = vt[k]; }
        for (int k = 0; k < 3; ++k) r[k] = dsub(r[k], dmul(v[k], dt));
        pair_twobody(h, m, e2, r, v, rt, vt, b);
        for (int k = 0; k < 3; ++k) { r[k] = rt[k]; v[k] = vt[k]; }
    }
    for (int k = 0; k < 3; ++k) { r1[k] = r[k]; v1[k] = v[k]; }
}

// pair_evolve for flag -1 or +1 when the pair is known to take the
// leapfrog branch of its two-body step (sakura_uses_kepler is false): the
// same operations without the test.
__device__ __forceinline__ void pair_evolve_leapfrog(double dt, long long flag, double m, double e2,
                                                     const double r0[3], const double v0[3], double r1[3],
                                                     double v1[3]) {
    double r[3], rt[3], vt[3];
    if (flag == -1) {
        for (int k = 0; k < 3; ++k) r[k] = dsub(r0[k], dmul(v0[k], dt));
        pair_leapfrog(dt, m, e2, r, v0, r1, v1);
    } else {
        pair_leapfrog(dt, m, e2, r0, v0, rt, vt);
        for (int k = 0; k < 3; ++k) { r1[k] = dsub(rt[k], dmul(vt[k], dt)); v1[k] = vt[k]; }
    }
}

}  // namespace tg
