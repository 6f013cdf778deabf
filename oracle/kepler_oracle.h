/*
 * kepler_oracle.h -- CPU restatement of Sakura's two-body propagation.
 *
 * TEST INFRASTRUCTURE ONLY (included by tupan_oracle.c).
 *
 * Follows tupan/lib/src/sakura_kernel_common.h:8-191 (get_acc, leapfrog,
 * twobody_solver, evolve_twobody) and the universal-variable Kepler solver of
 * tupan/lib/src/universal_kepler_solver.h:17-614 (Stumpff functions c0..c3,
 * the universal Kepler equation and its two derivatives, order-5 Laguerre
 * iteration with tolerance 2^-42 and at most 64 steps, period folding of
 * bound orbits, the Bate-Mueller-White hyperbolic first guess, the Lagrange
 * f/g update with r1 = sqrt(r1^2 + e2), step halving on solver failure and
 * step doubling on an energy-error test).  The per-operation order is kept so
 * that results are bit-identical to the reference on the same machine.
 *
 * Deviation: the reference retries without bound (halving at :483-500,
 * doubling at :580-606).  Here the halving stops after orc_split_cap
 * doublings, the energy loop after orc_energy_cap, and a pair evolution
 * after orc_solve_budget Kepler solves, keeping the last iterate (the same
 * bounds as the GPU kernels: ORC_* for Sakura, ORC_PAIR_* for the Kepler
 * pair solver).  Within the bounds the steps are the reference's;
 * the bounds are reached only for inputs (radial free fall with v = 0, or
 * softened close pairs whose energy test never passes) on which the
 * reference itself never returns.
 */
#ifndef KEPLER_ORACLE_H
#define KEPLER_ORACLE_H

#include <math.h>

#define ORC_TOL 2.2737367544323205948e-13 /* 2^-42 */
#define ORC_MAXITER 64
/* Bounds for Sakura's pairwise kernel (many pairs per call)... */
#define ORC_SPLIT_CAP 6      /* up to 64 sub-steps after solver failures */
#define ORC_ENERGY_CAP 4     /* up to 16 sub-steps for the energy test */
#define ORC_SOLVE_BUDGET 1024
/* ...and for the Kepler pair solver (a few pairs per call). */
#ifndef ORC_PAIR_SPLIT_CAP
#define ORC_PAIR_SPLIT_CAP 10
#endif
#ifndef ORC_PAIR_ENERGY_CAP
#define ORC_PAIR_ENERGY_CAP 10
#endif
#ifndef ORC_PAIR_SOLVE_BUDGET
#define ORC_PAIR_SOLVE_BUDGET 65536
#endif
#define ORC_PI 3.141592653589793

static inline int orc_sign(double x) { return (x > 0) - (x < 0); }

/* Stumpff functions of zeta = alpha s^2, in the reference's closed forms. */
static inline double orc_c0(double z)
{
    if (z < 0) return cos(sqrt(-z));
    if (z > 0) return cosh(sqrt(z));
    return 1.0;
}
static inline double orc_c1(double z)
{
    if (z < 0) { double q = sqrt(-z); return sin(q) / q; }
    if (z > 0) { double q = sqrt(z); return sinh(q) / q; }
    return 1.0;
}
static inline double orc_c2(double z)
{
    if (z < 0) { double q = sqrt(-z); return (cos(q) - 1) / z; }
    if (z > 0) { double q = sqrt(z); return (cosh(q) - 1) / z; }
    return 1.0 / 2;
}
static inline double orc_c3(double z)
{
    if (z < 0) { double q = sqrt(-z); return (sin(q) / q - 1) / z; }
    if (z > 0) { double q = sqrt(z); return (sinh(q) / q - 1) / z; }
    return 1.0 / 6;
}

/* G-functions of the universal anomaly s. */
struct orc_g { double g0, g1, g2, g3; };

static inline double orc_G0(double s, double al) { double s2 = s * s; return orc_c0(al * s2); }
static inline double orc_G1(double s, double al) { double s2 = s * s; return s * orc_c1(al * s2); }
static inline double orc_G2(double s, double al) { double s2 = s * s; return s2 * orc_c2(al * s2); }
static inline double orc_G3(double s, double al) { double s2 = s * s; double s3 = s * s2; return s3 * orc_c3(al * s2); }

/* The Kepler equation t(s) - dt and its first two derivatives. */
struct orc_kep { double dt, r0, rv, m, al; };

static inline double orc_kf(double s, const struct orc_kep *k)
{
    double t = k->r0 * s + k->rv * orc_G2(s, k->al) + (k->m + k->al * k->r0) * orc_G3(s, k->al);
    return t - k->dt;
}
static inline double orc_kdf(double s, const struct orc_kep *k)
{
    return k->r0 + k->rv * orc_G1(s, k->al) + (k->m + k->al * k->r0) * orc_G2(s, k->al);
}
static inline double orc_kddf(double s, const struct orc_kep *k)
{
    return k->rv * orc_G0(s, k->al) + (k->m + k->al * k->r0) * orc_G1(s, k->al);
}

/* Laguerre's method of order 5; 0 on success, <0 on failure (reference codes). */
static int orc_laguerre(double s0, double *s, const struct orc_kep *k)
{
    const double n = 5;
    double x = s0, step;
    int it = 0;
    do {
        double f0 = orc_kf(x, k), f1 = orc_kdf(x, k), f2 = orc_kddf(x, k);
        double f1sq = f1 * f1;
        double b = f1sq - f0 * f2;
        double g = n * f0;
        double h = f1 + orc_sign(f1) * sqrt(fabs((n - 1) * (n * b - f1sq)));
        if (h == 0) { *s = x; return -1; }
        step = -g / h;
        x += step;
        it += 1;
        if (it > ORC_MAXITER) { *s = x; return -2; }
    } while (fabs(step) > ORC_TOL);
    *s = x;
    if (orc_sign(x) != orc_sign(s0)) return -3;
    return 0;
}

/* Kepler solves spent on the current pair evolution, and the bounds in
 * force (per thread; set by the caller before each pair). */
static __thread int orc_solves;
static __thread int orc_split_cap = ORC_SPLIT_CAP;
static __thread int orc_energy_cap = ORC_ENERGY_CAP;
static __thread int orc_solve_budget = ORC_SOLVE_BUDGET;
/* Set when a bound was reached during the current pair evolution. */
static __thread int orc_capped;

static inline void orc_set_caps(int split_cap, int energy_cap, int solve_budget)
{
    orc_split_cap = split_cap;
    orc_energy_cap = energy_cap;
    orc_solve_budget = solve_budget;
}

/* One Kepler solve over dt0; r,v updated in place only on success. */
static int orc_kepler_once(double dt0, double m, double e2, double r[3], double v[3])
{
    orc_solves += 1;
    double r2 = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
    if (!(r2 > 0)) return 0;
    r2 += e2;
    double rn = sqrt(r2);
    double v2 = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
    double rv = r[0] * v[0] + r[1] * v[1] + r[2] * v[2];
    double beta = 2 - (e2 / r2);
    double al = v2 - beta * m / rn;

    double dt = dt0;
    if (al < 0) {                      /* bound: fold dt into one period */
        double a = m / fabs(al);
        double T = 2 * ORC_PI * a * sqrt(a / m);
        double ratio = dt0 / T;
        dt = (ratio - (double)(long)(ratio)) * T;
    }
    double s0 = dt / rn;
    if (al > 0) {                      /* hyperbolic first guess */
        double sal = sqrt(al);
        double ss = fabs(2 * al * dt / (rv + (m + al * rn) / sal));
        if (ss > 1) s0 = orc_sign(dt) * log(ss) / sal;
    }
    struct orc_kep k = {dt, rn, rv, m, al};
    double s;
    int err = orc_laguerre(s0, &s, &k);
    if (err != 0) return err;

    /* Lagrange f, g and their rates */
    double lf = 1 - m * orc_G2(s, al) / rn;
    double lg = dt - m * orc_G3(s, al);
    double r1[3];
    for (int q = 0; q < 3; ++q) r1[q] = r[q] * lf + v[q] * lg;
    double r1sq = r1[0] * r1[0] + r1[1] * r1[1] + r1[2] * r1[2];
    double r1n = sqrt(r1sq + e2);
    double ldf = -m * orc_G1(s, al) / (rn * r1n);
    double ldg = (1 + lg * ldf) / lf;
    double v1[3];
    for (int q = 0; q < 3; ++q) v1[q] = r[q] * ldf + v[q] * ldg;
    for (int q = 0; q < 3; ++q) { r[q] = r1[q]; v[q] = v1[q]; }
    return 0;
}

/* dt split into n equal solves; n doubles whenever one solve fails. */
static void orc_kepler_split(double dt, double m, double e2,
                             const double r0[3], const double v0[3], double r[3], double v[3])
{
    long n = 1;
    for (int tries = 0; ; ++tries) {
        for (int q = 0; q < 3; ++q) { r[q] = r0[q]; v[q] = v0[q]; }
        int failed = 0;
        for (long i = 0; i < n; ++i) {
            if (orc_solves >= orc_solve_budget) { orc_capped = 1; return; }
            if (orc_kepler_once(dt / n, m, e2, r, v) != 0) { failed = 1; break; }
        }
        if (!failed) return;
        if (tries >= orc_split_cap) { orc_capped = 1; return; }
        n *= 2;
    }
}

static inline void orc_energy(double m, double e2, const double r[3], const double v[3],
                              double *u, double *en)
{
    double r2 = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
    r2 += e2;
    double rn = sqrt(r2);
    double v2 = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
    *u = 2 * m / rn;
    *en = v2 - *u;
}

/* Kepler propagation with the softened-energy consistency test. */
static void orc_kepler(double dt, double m, double e2,
                       const double r0[3], const double v0[3], double r[3], double v[3])
{
    orc_kepler_split(dt, m, e2, r0, v0, r, v);
    if (e2 == 0) return;
    double r2 = r0[0] * r0[0] + r0[1] * r0[1] + r0[2] * r0[2];
    if (!(r2 > 0)) {
        for (int q = 0; q < 3; ++q) { r[q] = r0[q]; v[q] = v0[q]; }
        return;
    }
    double u0, en0, u1, en1;
    orc_energy(m, e2, r0, v0, &u0, &en0);
    orc_energy(m, e2, r, v, &u1, &en1);
    const double tol = 64 * ORC_TOL;
    double err = fabs(en1 - en0);
    if (2 * err < tol * (u1 + u0)) return;

    long n = 1;
    for (int tries = 0; tries < orc_energy_cap; ++tries) {
        n *= 2;
        for (int q = 0; q < 3; ++q) { r[q] = r0[q]; v[q] = v0[q]; }
        int bad = 0;
        for (long i = 0; i < n; ++i) {
            double rs[3] = {r[0], r[1], r[2]}, vs[3] = {v[0], v[1], v[2]};
            orc_kepler_split(dt / n, m, e2, rs, vs, r, v);
            orc_energy(m, e2, r, v, &u1, &en1);
            err = fabs(en1 - en0);
            if (2 * err > tol * (u1 + u0)) { bad = 1; break; }
            if (orc_capped) return;
        }
        if (!bad) return;
    }
    orc_capped = 1;
}

/* Softened Newtonian acceleration of the relative orbit. */
static inline void orc_rel_acc(double m, double e2, const double r[3], double a[3])
{
    double r2 = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
    double q2 = 1 / (r2 + e2);
    if (!(r2 > 0)) q2 = 0;
    double q3 = q2 * sqrt(q2);
    double mq = m * q3;
    for (int k = 0; k < 3; ++k) a[k] = -mq * r[k];
}

/* Drift-kick-drift leapfrog for wide pairs. */
static void orc_leapfrog(double dt, double m, double e2,
                         const double r0[3], const double v0[3], double r[3], double v[3])
{
    double h = dt / 2;
    double a[3];
    for (int k = 0; k < 3; ++k) { r[k] = r0[k]; v[k] = v0[k]; }
    for (int k = 0; k < 3; ++k) r[k] += v[k] * h;
    orc_rel_acc(m, e2, r, a);
    for (int k = 0; k < 3; ++k) v[k] += a[k] * dt;
    for (int k = 0; k < 3; ++k) r[k] += v[k] * h;
}

/* Choose leapfrog when r > 64 m / v^2, else the Kepler solver. */
static void orc_twobody(double dt, double m, double e2,
                        const double r0[3], const double v0[3], double r[3], double v[3])
{
    double r2 = r0[0] * r0[0] + r0[1] * r0[1] + r0[2] * r0[2];
    double v2 = v0[0] * v0[0] + v0[1] * v0[1] + v0[2] * v0[2];
    double R = 64 * (m / v2);
    if (r2 > R * R) orc_leapfrog(dt, m, e2, r0, v0, r, v);
    else orc_kepler(dt, m, e2, r0, v0, r, v);
}

/* The four Sakura flags; any other flag leaves the pair unchanged. */
static void orc_twobody_evolve(double dt, long flag, double m, double e2,
                               const double r0[3], const double v0[3], double r1[3], double v1[3])
{
    double r[3] = {r0[0], r0[1], r0[2]}, v[3] = {v0[0], v0[1], v0[2]};
    double rt[3], vt[3];
    orc_solves = 0;
    if (flag == -1) {
        for (int k = 0; k < 3; ++k) r[k] -= v[k] * dt;
        orc_twobody(dt, m, e2, r, v, rt, vt);
        for (int k = 0; k < 3; ++k) { r[k] = rt[k]; v[k] = vt[k]; }
    }
    if (flag == 1) {
        orc_twobody(dt, m, e2, r, v, rt, vt);
        for (int k = 0; k < 3; ++k) { r[k] = rt[k]; v[k] = vt[k]; }
        for (int k = 0; k < 3; ++k) r[k] -= v[k] * dt;
    }
    if (flag == -2) {
        for (int k = 0; k < 3; ++k) r[k] -= v[k] * dt / 2;
        orc_twobody(dt, m, e2, r, v, rt, vt);
        for (int k = 0; k < 3; ++k) { r[k] = rt[k]; v[k] = vt[k]; }
        for (int k = 0; k < 3; ++k) r[k] -= v[k] * dt / 2;
    }
    if (flag == 2) {
        orc_twobody(dt / 2, m, e2, r, v, rt, vt);
        for (int k = 0; k < 3; ++k) { r[k] = rt[k]; v[k] = vt[k]; }
        for (int k = 0; k < 3; ++k) r[k] -= v[k] * dt;
        orc_twobody(dt / 2, m, e2, r, v, rt, vt);
        for (int k = 0; k < 3; ++k) { r[k] = rt[k]; v[k] = vt[k]; }
    }
    for (int k = 0; k < 3; ++k) { r1[k] = r[k]; v1[k] = v[k]; }
}

#endif
