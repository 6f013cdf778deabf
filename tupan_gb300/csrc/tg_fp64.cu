// tg_fp64.cu -- FP64 pairwise kernels.
//
// One thread owns one i-particle and walks the j-set in order, exactly like
// the reference loops (tupan/lib/src/<name>_kernel.c), staging j-tiles of
// the needed fields through shared memory.  Every per-pair operation uses
// the uncontracted IEEE helpers of tg_device.cuh in the reference's order
// (tupan/lib/src/<name>_kernel_common.h, smoothing.h), so Phi, Acc, AccJerk,
// SnapCrackle and Tstep return results bit-identical to the reference C
// backend.  PNAcc evaluates the post-Newtonian polynomial in its own order
// (tg_pn_terms.cuh); Sakura uses the bounded Kepler solver of tg_kepler.cuh.
//
// Roofline: FP64 issue.  GB300 executes FP64 at a small fraction of the FP32
// rate and each pair needs one IEEE divide and one square root, so these
// kernels are the accuracy reference on the GPU, not the fast path.
#include <type_traits>

#include "tg_device.cuh"
#include "tg_internal.h"
#include "tg_kepler.cuh"
#include "tg_pn_terms.cuh"

namespace tg {

constexpr int F64_THREADS = 128;
constexpr int F64_TILE = 64;

// Plummer-softened 1/(r2+e2), zero when r2 > 0 fails (smoothing.h:10-67).
__device__ __forceinline__ double soft_q2(double r2, double e2) {
    double q = ddiv(1.0, dadd(r2, e2));
    return (r2 > 0) ? q : 0.0;
}

// ---------------------------------------------------------------------------
// Per-kernel pair functors.  `sj[f][jj]` is the staged j-tile.
// ---------------------------------------------------------------------------
struct Phi64 {
    static constexpr int NF = 5, NO = 1, NT = 1;
    struct St { double x, y, z, e, acc[NT]; };
    __device__ static void init(St &s, const PairArgs &a, size_t i) {
        s = {a.I.f[F_RX][i], a.I.f[F_RY][i], a.I.f[F_RZ][i], a.I.f[F_E2][i], {0.0}};
    }
    __device__ static void terms(const St &s, const double (*sj)[F64_TILE], int jj, const PairArgs &, double *t) {
        double dx = dsub(s.x, sj[F_RX][jj]), dy = dsub(s.y, sj[F_RY][jj]), dz = dsub(s.z, sj[F_RZ][jj]);
        double e2 = dadd(s.e, sj[F_E2][jj]);
        double r2 = ddot3(dx, dy, dz, dx, dy, dz);
        double q1 = dsqrt(soft_q2(r2, e2));
        t[0] = dmul(sj[F_M][jj], q1);
    }
    __device__ static double accum(int, double acc, double t) { return dsub(acc, t); }
    __device__ static void store_acc(const double *acc, const St &, const PairArgs &a, size_t i) { a.out[0][i] = acc[0]; }
};

struct Acc64 {
    static constexpr int NF = 5, NO = 3, NT = 3;
    struct St { double x, y, z, e, acc[NT]; };
    __device__ static void init(St &s, const PairArgs &a, size_t i) {
        s = {a.I.f[F_RX][i], a.I.f[F_RY][i], a.I.f[F_RZ][i], a.I.f[F_E2][i], {0.0, 0.0, 0.0}};
    }
    __device__ static void terms(const St &s, const double (*sj)[F64_TILE], int jj, const PairArgs &, double *t) {
        double dx = dsub(s.x, sj[F_RX][jj]), dy = dsub(s.y, sj[F_RY][jj]), dz = dsub(s.z, sj[F_RZ][jj]);
        double e2 = dadd(s.e, sj[F_E2][jj]);
        double r2 = ddot3(dx, dy, dz, dx, dy, dz);
        double q2 = soft_q2(r2, e2);
        double q3 = dmul(dmul(q2, dsqrt(q2)), sj[F_M][jj]);
        t[0] = dmul(q3, dx);
        t[1] = dmul(q3, dy);
        t[2] = dmul(q3, dz);
    }
    __device__ static double accum(int, double acc, double t) { return dsub(acc, t); }
    __device__ static void store_acc(const double *acc, const St &, const PairArgs &a, size_t i) {
        a.out[0][i] = acc[0]; a.out[1][i] = acc[1]; a.out[2][i] = acc[2];
    }
};

struct AccJerk64 {
    static constexpr int NF = 8, NO = 6, NT = 6;
    struct St { double x, y, z, e, u, v, w, acc[NT]; };
    __device__ static void init(St &s, const PairArgs &a, size_t i) {
        s.x = a.I.f[F_RX][i]; s.y = a.I.f[F_RY][i]; s.z = a.I.f[F_RZ][i]; s.e = a.I.f[F_E2][i];
        s.u = a.I.f[F_VX][i]; s.v = a.I.f[F_VY][i]; s.w = a.I.f[F_VZ][i];
        for (int k = 0; k < NT; ++k) s.acc[k] = 0.0;
    }
    __device__ static void terms(const St &s, const double (*sj)[F64_TILE], int jj, const PairArgs &, double *t) {
        double dx = dsub(s.x, sj[F_RX][jj]), dy = dsub(s.y, sj[F_RY][jj]), dz = dsub(s.z, sj[F_RZ][jj]);
        double e2 = dadd(s.e, sj[F_E2][jj]);
        double du = dsub(s.u, sj[F_VX][jj]), dv = dsub(s.v, sj[F_VY][jj]), dw = dsub(s.w, sj[F_VZ][jj]);
        double r2 = ddot3(dx, dy, dz, dx, dy, dz);
        double rv = ddot3(dx, dy, dz, du, dv, dw);
        double q2 = soft_q2(r2, e2);
        double q3 = dmul(q2, dsqrt(q2));
        double al = dmul(dmul(3.0, rv), q2);
        du = dsub(du, dmul(al, dx));
        dv = dsub(dv, dmul(al, dy));
        dw = dsub(dw, dmul(al, dz));
        q3 = dmul(q3, sj[F_M][jj]);
        t[0] = dmul(q3, dx); t[1] = dmul(q3, dy); t[2] = dmul(q3, dz);
        t[3] = dmul(q3, du); t[4] = dmul(q3, dv); t[5] = dmul(q3, dw);
    }
    __device__ static double accum(int, double acc, double t) { return dsub(acc, t); }
    __device__ static void store_acc(const double *acc, const St &, const PairArgs &a, size_t i) {
        for (int k = 0; k < 6; ++k) a.out[k][i] = acc[k];
    }
};

struct SnapCrackle64 {
    static constexpr int NF = 14, NO = 6, NT = 6;
    struct St { double f[14]; double acc[NT]; };
    __device__ static void init(St &s, const PairArgs &a, size_t i) {
        for (int k = 0; k < 14; ++k) s.f[k] = a.I.f[k][i];
        for (int k = 0; k < NT; ++k) s.acc[k] = 0.0;
    }
    __device__ static void terms(const St &s, const double (*sj)[F64_TILE], int jj, const PairArgs &, double *t) {
        double r[3], v[3], A[3], J[3];
        for (int k = 0; k < 3; ++k) {
            r[k] = dsub(s.f[F_RX + k], sj[F_RX + k][jj]);
            v[k] = dsub(s.f[F_VX + k], sj[F_VX + k][jj]);
            A[k] = dsub(s.f[F_AX + k], sj[F_AX + k][jj]);
            J[k] = dsub(s.f[F_JX + k], sj[F_JX + k][jj]);
        }
        double e2 = dadd(s.f[F_E2], sj[F_E2][jj]);
        double r2 = ddot3(r[0], r[1], r[2], r[0], r[1], r[2]);
        double rv = ddot3(r[0], r[1], r[2], v[0], v[1], v[2]);
        double v2 = ddot3(v[0], v[1], v[2], v[0], v[1], v[2]);
        double rJ = ddot3(r[0], r[1], r[2], J[0], J[1], J[2]);
        double rA = ddot3(r[0], r[1], r[2], A[0], A[1], A[2]);
        double vA = ddot3(v[0], v[1], v[2], A[0], A[1], A[2]);
        double q2 = soft_q2(r2, e2);
        double q3 = dmul(q2, dsqrt(q2));
        double al = dmul(rv, q2);
        double al2 = dmul(al, al);
        double be = dmul(3.0, dadd(dmul(dadd(v2, rA), q2), al2));
        double ga = dadd(dmul(dadd(dmul(3.0, vA), rJ), q2), dmul(al, dsub(be, dmul(4.0, al2))));
        al = dmul(al, 3.0);
        ga = dmul(ga, 3.0);
        for (int k = 0; k < 3; ++k) v[k] = dsub(v[k], dmul(al, r[k]));
        double two_al = dmul(2.0, al);
        for (int k = 0; k < 3; ++k) A[k] = dsub(A[k], dadd(dmul(two_al, v[k]), dmul(be, r[k])));
        al = dmul(al, 3.0);
        be = dmul(be, 3.0);
        for (int k = 0; k < 3; ++k)
            J[k] = dsub(J[k], dadd(dadd(dmul(al, A[k]), dmul(be, v[k])), dmul(ga, r[k])));
        q3 = dmul(q3, sj[F_M][jj]);
        for (int k = 0; k < 3; ++k) {
            t[k] = dmul(q3, A[k]);
            t[3 + k] = dmul(q3, J[k]);
        }
    }
    __device__ static double accum(int, double acc, double t) { return dsub(acc, t); }
    __device__ static void store_acc(const double *acc, const St &, const PairArgs &a, size_t i) {
        for (int k = 0; k < 6; ++k) a.out[k][i] = acc[k];
    }
};

struct Tstep64 {
    static constexpr int NF = 8, NO = 2, NT = 2;
    struct St { double m, x, y, z, e, u, v, w, acc[NT]; };   // acc: sum w2, max w2
    __device__ static void init(St &s, const PairArgs &a, size_t i) {
        s.m = a.I.f[F_M][i]; s.x = a.I.f[F_RX][i]; s.y = a.I.f[F_RY][i]; s.z = a.I.f[F_RZ][i];
        s.e = a.I.f[F_E2][i]; s.u = a.I.f[F_VX][i]; s.v = a.I.f[F_VY][i]; s.w = a.I.f[F_VZ][i];
        s.acc[0] = 0.0; s.acc[1] = 0.0;
    }
    __device__ static void terms(const St &s, const double (*sj)[F64_TILE], int jj, const PairArgs &a, double *t) {
        double dx = dsub(s.x, sj[F_RX][jj]), dy = dsub(s.y, sj[F_RY][jj]), dz = dsub(s.z, sj[F_RZ][jj]);
        double e2 = dadd(s.e, sj[F_E2][jj]);
        double du = dsub(s.u, sj[F_VX][jj]), dv = dsub(s.v, sj[F_VY][jj]), dw = dsub(s.w, sj[F_VZ][jj]);
        double m = dadd(s.m, sj[F_M][jj]);
        double r2 = ddot3(dx, dy, dz, dx, dy, dz);
        double rv = ddot3(dx, dy, dz, du, dv, dw);
        double v2 = ddot3(du, dv, dw, du, dv, dw);
        double q2 = soft_q2(r2, e2);
        double q1 = dsqrt(q2);
        double b = dmul(2.0, q2);             // (1 + a/2) inv_r2 with a = 2
        double phi = dmul(m, q1);
        double w2 = dmul(q2, dadd(v2, dmul(2.0, phi)));
        double gam = dmul(q2, dadd(w2, dmul(b, phi)));
        gam = dmul(gam, ddiv(a.eta, dsqrt(w2)));
        w2 = dsub(w2, dmul(gam, rv));
        if (!(r2 > 0)) w2 = 0.0;
        t[0] = w2;
        t[1] = w2;
    }
    __device__ static double accum(int c, double acc, double t) { return c == 0 ? dadd(acc, t) : fmax(t, acc); }
    __device__ static void store_acc(const double *acc, const St &, const PairArgs &a, size_t i) {
        a.out[0][i] = ddiv(a.eta, dsqrt(dadd(1.0, acc[0])));
        a.out[1][i] = ddiv(a.eta, dsqrt(dadd(1.0, acc[1])));
    }
};

struct PNAcc64 {
    static constexpr int NF = 8, NO = 3, NT = 3;
    struct St { double m, x, y, z, e, u, v, w, iv2, acc[NT]; };
    __device__ static void init(St &s, const PairArgs &a, size_t i) {
        s.m = a.I.f[F_M][i]; s.x = a.I.f[F_RX][i]; s.y = a.I.f[F_RY][i]; s.z = a.I.f[F_RZ][i];
        s.e = a.I.f[F_E2][i]; s.u = a.I.f[F_VX][i]; s.v = a.I.f[F_VY][i]; s.w = a.I.f[F_VZ][i];
        s.iv2 = s.u * s.u + s.v * s.v + s.w * s.w;
        s.acc[0] = s.acc[1] = s.acc[2] = 0.0;
    }
    __device__ static void terms(const St &s, const double (*sj)[F64_TILE], int jj, const PairArgs &a, double *t) {
        double jm = sj[F_M][jj];
        double ju = sj[F_VX][jj], jv = sj[F_VY][jj], jw = sj[F_VZ][jj];
        double rx = s.x - sj[F_RX][jj], ry = s.y - sj[F_RY][jj], rz = s.z - sj[F_RZ][jj];
        double e2 = s.e + sj[F_E2][jj];
        double vx = s.u - ju, vy = s.v - jv, vz = s.w - jw;
        double r2 = rx * rx + ry * ry + rz * rz;
        double v2 = vx * vx + vy * vy + vz * vz;
        double q2 = soft_q2(r2, e2);
        double q1 = dsqrt(q2);
        double q3 = q2 * q1;
        double nx = rx * q1, ny = ry * q1, nz = rz * q1;
        double jv2 = ju * ju + jv * jv + jw * jw;
        double ivjv = s.u * ju + s.v * jv + s.w * jw;
        double niv = nx * s.u + ny * s.v + nz * s.w;
        double njv = nx * ju + ny * jv + nz * jw;
        double nv = nx * vx + ny * vy + nz * vz;
        double A, B;
        pn_factors<double>(a.order, s.m, jm, q1, s.iv2, jv2, ivjv, niv, njv, nv, v2,
                           a.inv[2], a.inv[4], a.inv[5], a.inv[6], a.inv[7], A, B);
        A *= jm * q3;
        B *= jm * q2;
        t[0] = A * rx + B * vx;
        t[1] = A * ry + B * vy;
        t[2] = A * rz + B * vz;
    }
    __device__ static double accum(int, double acc, double t) { return acc + t; }
    __device__ static void store_acc(const double *acc, const St &, const PairArgs &a, size_t i) {
        for (int k = 0; k < 3; ++k) a.out[k][i] = acc[k];
    }
};

struct Sakura64 {
    static constexpr int NF = 8, NO = 6, NT = 6;
    struct St { double f[8]; double acc[NT]; };
    __device__ static void init(St &s, const PairArgs &a, size_t i) {
        for (int k = 0; k < 8; ++k) s.f[k] = a.I.f[k][i];
        for (int k = 0; k < NT; ++k) s.acc[k] = 0.0;
    }
    // The pair state (i minus j) and the mass-weighted deltas of one pair;
    // a pair that reaches a retry bound raises its status bit (rare).
    __device__ static void state(const double *fi, const double *fj, double r0[3], double v0[3],
                                 double &e2, double &m) {
        for (int k = 0; k < 3; ++k) {
            r0[k] = dsub(fi[F_RX + k], fj[F_RX + k]);
            v0[k] = dsub(fi[F_VX + k], fj[F_VX + k]);
        }
        e2 = dadd(fi[F_E2], fj[F_E2]);
        m = dadd(fi[F_M], fj[F_M]);
    }
    __device__ static void pair_terms(const double *fi, const double *fj, const PairArgs &a, double *t) {
        double r0[3], v0[3], r1[3], v1[3], e2, m;
        state(fi, fj, r0, v0, e2, m);
        KepBudget b;
        pair_evolve(a.dt, a.flag, m, e2, r0, v0, r1, v1, b);
        if (b.flags) atomicOr(a.status, b.flags);
        double w = ddiv(fj[F_M], m);
        for (int k = 0; k < 3; ++k) {
            t[k] = dmul(w, dsub(r1[k], r0[k]));
            t[3 + k] = dmul(w, dsub(v1[k], v0[k]));
        }
    }
    __device__ static void terms(const St &s, const double (*sj)[F64_TILE], int jj, const PairArgs &a, double *t) {
        double fj[8];
        for (int k = 0; k < 8; ++k) fj[k] = sj[k][jj];
        pair_terms(s.f, fj, a, t);
    }
    // pair_terms of a pair known to take the leapfrog branch (flag -1 or +1)
    __device__ static void terms_leapfrog(const St &s, const double (*sj)[F64_TILE], int jj, const PairArgs &a,
                                          double *t) {
        double fj[8], r0[3], v0[3], r1[3], v1[3], e2, m;
        for (int k = 0; k < 8; ++k) fj[k] = sj[k][jj];
        state(s.f, fj, r0, v0, e2, m);
        pair_evolve_leapfrog(a.dt, a.flag, m, e2, r0, v0, r1, v1);
        double w = ddiv(fj[F_M], m);
        for (int k = 0; k < 3; ++k) {
            t[k] = dmul(w, dsub(r1[k], r0[k]));
            t[3 + k] = dmul(w, dsub(v1[k], v0[k]));
        }
    }
    __device__ static double accum(int, double acc, double t) { return dadd(acc, t); }
    __device__ static void store_acc(const double *acc, const St &, const PairArgs &a, size_t i) {
        for (int k = 0; k < 6; ++k) a.out[k][i] = acc[k];
    }
};

// Vector-Jacobian product of Acc for one particle set (i-set == j-set):
//   r-bar_k = sum_j T_kj (m_k g_j - m_j g_k),  T = s^-3/2 I - 3 s^-5/2 r r^T
//   m-bar_k = sum_j g_j . r_kj s^-3/2,          r = r_k - r_j, s = r^2 + e2
// with g the upstream gradient dL/da; pairs with r2 = 0 contribute nothing.
struct AccVjp64 {
    static constexpr int NF = 14, NO = 4;
    struct St { double m, x, y, z, e, g[3], rb[3], mb; };
    __device__ static void init(St &s, const PairArgs &a, size_t i) {
        s.m = a.I.f[F_M][i]; s.x = a.I.f[F_RX][i]; s.y = a.I.f[F_RY][i]; s.z = a.I.f[F_RZ][i];
        s.e = a.I.f[F_E2][i];
        for (int k = 0; k < 3; ++k) { s.g[k] = a.I.f[F_AX + k][i]; s.rb[k] = 0.0; }
        s.mb = 0.0;
    }
    __device__ static void pair(St &s, const double (*sj)[F64_TILE], int jj, const PairArgs &) {
        const double r[3] = {s.x - sj[F_RX][jj], s.y - sj[F_RY][jj], s.z - sj[F_RZ][jj]};
        const double r2 = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
        if (!(r2 > 0)) return;
        const double q2 = 1.0 / (r2 + s.e + sj[F_E2][jj]);
        const double q3 = q2 * sqrt(q2);
        const double mj = sj[F_M][jj];
        double w[3], gj[3];
        for (int k = 0; k < 3; ++k) {
            gj[k] = sj[F_AX + k][jj];
            w[k] = s.m * gj[k] - mj * s.g[k];
        }
        const double rw = r[0] * w[0] + r[1] * w[1] + r[2] * w[2];
        const double c = 3.0 * q3 * q2 * rw;
        for (int k = 0; k < 3; ++k) s.rb[k] += q3 * w[k] - c * r[k];
        s.mb += (gj[0] * r[0] + gj[1] * r[1] + gj[2] * r[2]) * q3;
    }
    __device__ static void store(const St &s, const PairArgs &a, size_t i) {
        for (int k = 0; k < 3; ++k) a.out[k][i] = s.rb[k];
        a.out[3][i] = s.mb;
    }
};

// NREG_X (nreg_kernels_common.h:7-60): the pair separation is drifted by dt
// with the relative velocity; sums m_j r_ij, the softened acceleration and
// m_i sum m_j / r_ij.
struct NregX64 {
    static constexpr int NF = 8, NO = 7, NT = 7;   // terms: m_j r (3), q3 r (3), m_j q1
    struct St { double m, x, y, z, e, u, v, w, acc[NT]; };
    __device__ static void init(St &s, const PairArgs &a, size_t i) {
        s.m = a.I.f[F_M][i]; s.x = a.I.f[F_RX][i]; s.y = a.I.f[F_RY][i]; s.z = a.I.f[F_RZ][i];
        s.e = a.I.f[F_E2][i]; s.u = a.I.f[F_VX][i]; s.v = a.I.f[F_VY][i]; s.w = a.I.f[F_VZ][i];
        for (int k = 0; k < NT; ++k) s.acc[k] = 0.0;
    }
    __device__ static void terms(const St &s, const double (*sj)[F64_TILE], int jj, const PairArgs &a, double *t) {
        double rx = dsub(s.x, sj[F_RX][jj]), ry = dsub(s.y, sj[F_RY][jj]), rz = dsub(s.z, sj[F_RZ][jj]);
        const double e2 = dadd(s.e, sj[F_E2][jj]);
        const double vx = dsub(s.u, sj[F_VX][jj]), vy = dsub(s.v, sj[F_VY][jj]), vz = dsub(s.w, sj[F_VZ][jj]);
        rx = dadd(rx, dmul(vx, a.dt));
        ry = dadd(ry, dmul(vy, a.dt));
        rz = dadd(rz, dmul(vz, a.dt));
        const double r2 = ddot3(rx, ry, rz, rx, ry, rz);
        const double q2 = soft_q2(r2, e2);
        const double q1 = dsqrt(q2);
        const double mj = sj[F_M][jj];
        const double q3 = dmul(dmul(q2, q1), mj);
        t[0] = dmul(mj, rx); t[1] = dmul(mj, ry); t[2] = dmul(mj, rz);
        t[3] = dmul(q3, rx); t[4] = dmul(q3, ry); t[5] = dmul(q3, rz);
        t[6] = dmul(mj, q1);
    }
    __device__ static double accum(int c, double acc, double t) {
        return (c >= 3 && c < 6) ? dsub(acc, t) : dadd(acc, t);
    }
    __device__ static void store_acc(const double *acc, const St &s, const PairArgs &a, size_t i) {
        for (int k = 0; k < 6; ++k) a.out[k][i] = acc[k];
        a.out[6][i] = dmul(s.m, acc[6]);
    }
};

// NREG_V (nreg_kernels_common.h:62-102): the relative velocity is kicked by
// dt with the relative acceleration; sums m_j v_ij and m_i sum m_j |v_ij|^2.
struct NregV64 {
    static constexpr int NF = 11, NO = 4, NT = 4;   // terms: m_j v (3), m_j |v|^2
    struct St { double m, u, v, w, ax, ay, az, acc[NT]; };
    __device__ static void init(St &s, const PairArgs &a, size_t i) {
        s.m = a.I.f[F_M][i]; s.u = a.I.f[F_VX][i]; s.v = a.I.f[F_VY][i]; s.w = a.I.f[F_VZ][i];
        s.ax = a.I.f[F_AX][i]; s.ay = a.I.f[F_AY][i]; s.az = a.I.f[F_AZ][i];
        for (int k = 0; k < NT; ++k) s.acc[k] = 0.0;
    }
    __device__ static void terms(const St &s, const double (*sj)[F64_TILE], int jj, const PairArgs &a, double *t) {
        double vx = dsub(s.u, sj[F_VX][jj]), vy = dsub(s.v, sj[F_VY][jj]), vz = dsub(s.w, sj[F_VZ][jj]);
        const double ax = dsub(s.ax, sj[F_AX][jj]), ay = dsub(s.ay, sj[F_AY][jj]), az = dsub(s.az, sj[F_AZ][jj]);
        vx = dadd(vx, dmul(ax, a.dt));
        vy = dadd(vy, dmul(ay, a.dt));
        vz = dadd(vz, dmul(az, a.dt));
        const double v2 = ddot3(vx, vy, vz, vx, vy, vz);
        const double mj = sj[F_M][jj];
        t[0] = dmul(mj, vx); t[1] = dmul(mj, vy); t[2] = dmul(mj, vz);
        t[3] = dmul(mj, v2);
    }
    __device__ static double accum(int, double acc, double t) { return dadd(acc, t); }
    __device__ static void store_acc(const double *acc, const St &s, const PairArgs &a, size_t i) {
        for (int k = 0; k < 3; ++k) a.out[k][i] = acc[k];
        a.out[3][i] = dmul(s.m, acc[3]);
    }
};

// Kepler pair solver (kepler_solver_kernel_common.h:8-81): one thread per
// pair (2p, 2p+1).  The centre of mass drifts freely; the relative orbit
// follows the bounded universal-variable solver with the pair bounds.  All
// inputs of a pair are read before any output is written, so the outputs
// may alias the inputs (the reference updates the particles in place).
__global__ void __launch_bounds__(64) kepler_pairs(size_t npairs, PSet in, double dt, double *o0,
                                                   double *o1, double *o2, double *o3, double *o4,
                                                   double *o5, unsigned *status) {
    const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npairs) return;
    const size_t ia = 2 * p, ib = 2 * p + 1;
    const double im = in.f[F_M][ia], jm = in.f[F_M][ib];
    double ir[3], jr[3], iv[3], jv[3];
    for (int q = 0; q < 3; ++q) {
        ir[q] = in.f[F_RX + q][ia]; jr[q] = in.f[F_RX + q][ib];
        iv[q] = in.f[F_VX + q][ia]; jv[q] = in.f[F_VX + q][ib];
    }
    const double e2 = dadd(in.f[F_E2][ia], in.f[F_E2][ib]);
    double r0[3], v0[3], rcm[3], vcm[3], r1[3], v1[3];
    for (int q = 0; q < 3; ++q) { r0[q] = dsub(ir[q], jr[q]); v0[q] = dsub(iv[q], jv[q]); }
    const double m = dadd(im, jm);
    const double imu = ddiv(im, m), jmu = ddiv(jm, m);
    for (int q = 0; q < 3; ++q) rcm[q] = dadd(dmul(imu, ir[q]), dmul(jmu, jr[q]));
    for (int q = 0; q < 3; ++q) vcm[q] = dadd(dmul(imu, iv[q]), dmul(jmu, jv[q]));
    for (int q = 0; q < 3; ++q) rcm[q] = dadd(rcm[q], dmul(vcm[q], dt));
    KepBudget b;
    b.split_cap = KEP_PAIR_SPLIT_CAP;
    b.energy_cap = KEP_PAIR_ENERGY_CAP;
    b.solve_budget = KEP_PAIR_SOLVE_BUDGET;
    kep_solve(dt, m, e2, r0, v0, r1, v1, b);
    double *o[6] = {o0, o1, o2, o3, o4, o5};
    for (int q = 0; q < 3; ++q) {
        o[q][ia] = dadd(rcm[q], dmul(jmu, r1[q]));
        o[3 + q][ia] = dadd(vcm[q], dmul(jmu, v1[q]));
        o[q][ib] = dsub(rcm[q], dmul(imu, r1[q]));
        o[3 + q][ib] = dsub(vcm[q], dmul(imu, v1[q]));
    }
    if (b.flags) atomicOr(status, b.flags);
}

cudaError_t launch_kepler_pairs(size_t npairs, const PSet &in, double dt, double *const out[6],
                                unsigned *status, cudaStream_t s) {
    if (npairs == 0) return cudaSuccess;
    const unsigned t = 64;
    kepler_pairs<<<(unsigned)((npairs + t - 1) / t), t, 0, s>>>(npairs, in, dt, out[0], out[1], out[2],
                                                                 out[3], out[4], out[5], status);
    return cudaGetLastError();
}

// Functors written as per-pair terms plus an ordered accumulation (Phi, Acc,
// AccJerk, SnapCrackle, Tstep): pair() and store() for the sequential
// engines are the terms folded into the accumulators one pair at a time,
// the same operations in the same order as the reference loop.
template <class K, class = void>
struct has_terms : std::false_type {};
template <class K>
struct has_terms<K, decltype(void(K::NT))> : std::true_type {};

template <class K>
struct Seq : K {
    __device__ static void pair(typename K::St &s, const double (*sj)[F64_TILE], int jj, const PairArgs &a) {
        double t[K::NT];
        K::terms(s, sj, jj, a, t);
#pragma unroll
        for (int c = 0; c < K::NT; ++c) s.acc[c] = K::accum(c, s.acc[c], t[c]);
    }
    __device__ static void store(const typename K::St &s, const PairArgs &a, size_t i) {
        K::store_acc(s.acc, s, a, i);
    }
};
template <class K, bool T = has_terms<K>::value>
struct SeqOf { using type = K; };
template <class K>
struct SeqOf<K, true> { using type = Seq<K>; };

// ---------------------------------------------------------------------------
// Generic sequential-j engine.
// ---------------------------------------------------------------------------
template <class K>
__global__ void __launch_bounds__(F64_THREADS) fp64_pairwise(PairArgs a) {
    __shared__ double sj[K::NF][F64_TILE];
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const bool live = i < a.ni;
    typename K::St st;
    K::init(st, a, live ? i : 0);
    for (size_t j0 = 0; j0 < a.nj; j0 += F64_TILE) {
        const int nt = (int)((a.nj - j0) < (size_t)F64_TILE ? (a.nj - j0) : F64_TILE);
        for (int q = threadIdx.x; q < K::NF * F64_TILE; q += blockDim.x) {
            const int f = q / F64_TILE, jj = q % F64_TILE;
            if (jj < nt) sj[f][jj] = a.J.f[f][j0 + jj];
        }
        __syncthreads();
        for (int jj = 0; jj < nt; ++jj) K::pair(st, sj, jj, a);
        __syncthreads();
    }
    if (live) K::store(st, a, i);
}

// The FP64 pipe, not occupancy, bounds these kernels, so a few warps per SM
// suffice; small i-sets use narrower CTAs to spread over more SMs.
static unsigned fp64_threads(size_t ni, int sms) {
    for (unsigned t = F64_THREADS; t > 32; t /= 2)
        if ((ni + t - 1) / t >= (size_t)(sms > 0 ? sms : 1)) return t;
    return 32;
}

// Segmented form: CTA b works on cluster c with block_off[c] <= b <
// block_off[c+1]; its threads walk that cluster's j-range in order, so each
// cluster's results are the single-set results bit for bit.
__device__ __forceinline__ long long seg_find64(const long long *off, long long C, long long u) {
    long long lo = 0, hi = C;
    while (hi - lo > 1) {
        const long long mid = (lo + hi) >> 1;
        if (off[mid] <= u) lo = mid; else hi = mid;
    }
    return lo;
}

template <class K>
__global__ void __launch_bounds__(F64_THREADS) fp64_pairwise_seg(PairArgs a, const long long *block_off,
                                                                 const long long *seg_start,
                                                                 const long long *seg_n, long long C) {
    __shared__ double sj[K::NF][F64_TILE];
    const long long c = seg_find64(block_off, C, (long long)blockIdx.x);
    const long long li = ((long long)blockIdx.x - block_off[c]) * blockDim.x + threadIdx.x;
    const long long n = seg_n[c], s0 = seg_start[c];
    const bool live = li < n;
    typename K::St st;
    K::init(st, a, (size_t)(s0 + (live ? li : 0)));
    for (long long j0 = 0; j0 < n; j0 += F64_TILE) {
        const int nt = (int)((n - j0) < F64_TILE ? (n - j0) : F64_TILE);
        for (int q = threadIdx.x; q < K::NF * F64_TILE; q += blockDim.x) {
            const int f = q / F64_TILE, jj = q % F64_TILE;
            if (jj < nt) sj[f][jj] = a.J.f[f][s0 + j0 + jj];
        }
        __syncthreads();
        for (int jj = 0; jj < nt; ++jj) K::pair(st, sj, jj, a);
        __syncthreads();
    }
    if (live) K::store(st, a, (size_t)(s0 + li));
}

template <class K0>
static cudaError_t run_seg(const PairArgs &a, long long C, long long nblocks, int threads,
                           const long long *block_off, const long long *seg_start, const long long *seg_n,
                           cudaStream_t s) {
    using K = typename SeqOf<K0>::type;
    if (nblocks == 0) return cudaSuccess;
    fp64_pairwise_seg<K><<<(unsigned)nblocks, threads, 0, s>>>(a, block_off, seg_start, seg_n, C);
    return cudaGetLastError();
}

cudaError_t launch_fp64_seg(int kernel, const PairArgs &a, long long C, long long nblocks, int threads,
                            const long long *block_off, const long long *seg_start, const long long *seg_n,
                            cudaStream_t s) {
    switch (kernel) {
        case K_PHI: return run_seg<Phi64>(a, C, nblocks, threads, block_off, seg_start, seg_n, s);
        case K_ACC: return run_seg<Acc64>(a, C, nblocks, threads, block_off, seg_start, seg_n, s);
        case K_ACC_JERK: return run_seg<AccJerk64>(a, C, nblocks, threads, block_off, seg_start, seg_n, s);
        case K_SNAP_CRACKLE: return run_seg<SnapCrackle64>(a, C, nblocks, threads, block_off, seg_start, seg_n, s);
        default: return cudaErrorInvalidValue;
    }
}

// ---------------------------------------------------------------------------
// Warp engine for small i-sets: IPW i-particles per warp, 32/IPW lanes per
// i.  In each round the lanes of an i-group compute the terms of 32/IPW
// consecutive j in parallel (the divide and square root dominate), write
// them to shared memory, and lane c of the group folds component c of the
// round's terms into its accumulator in j order -- the reference's
// sequence of operations, so results stay bit-identical, while the grid
// has 32/IPW times more threads than the thread-per-i engine.
// ---------------------------------------------------------------------------
constexpr int F64W_THREADS = 256;

template <class K, int IPW>
__global__ void __launch_bounds__(F64W_THREADS) fp64_warp(PairArgs a) {
    constexpr int LPI = 32 / IPW;
    constexpr int WARPS = F64W_THREADS / 32;
    static_assert(K::NT <= LPI, "one lane per accumulated component");
    __shared__ double sj[K::NF][F64_TILE];
    __shared__ double tt[WARPS][IPW][K::NT][LPI + 1];
    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    const int g = lane / LPI, l = lane % LPI;
    const size_t i = ((size_t)blockIdx.x * WARPS + warp) * IPW + g;
    const bool live = i < a.ni;
    typename K::St st;
    K::init(st, a, live ? i : 0);
    double acc = 0.0;   // every accumulator of these kernels starts at 0
    for (size_t j0 = 0; j0 < a.nj; j0 += F64_TILE) {
        const int nt = (int)((a.nj - j0) < (size_t)F64_TILE ? (a.nj - j0) : F64_TILE);
        for (int q = threadIdx.x; q < K::NF * F64_TILE; q += blockDim.x) {
            const int f = q / F64_TILE, jj = q % F64_TILE;
            if (jj < nt) sj[f][jj] = a.J.f[f][j0 + jj];
        }
        __syncthreads();
        for (int r = 0; r < nt; r += LPI) {
            if (r + l < nt) {
                double t[K::NT];
                K::terms(st, sj, r + l, a, t);
#pragma unroll
                for (int c = 0; c < K::NT; ++c) tt[warp][g][c][l] = t[c];
            }
            __syncwarp();
            const int m = (nt - r) < LPI ? (nt - r) : LPI;
            if (l < K::NT)
                for (int q = 0; q < m; ++q) acc = K::accum(l, acc, tt[warp][g][l][q]);
            __syncwarp();
        }
        __syncthreads();
    }
    double res[K::NT];
#pragma unroll
    for (int c = 0; c < K::NT; ++c) res[c] = __shfl_sync(0xffffffffu, acc, g * LPI + c);
    if (l == 0 && live) K::store_acc(res, st, a, i);
}

// i-sets below this size use the warp engine (the thread-per-i engine has
// fewer than ~14 warps per SM there, too few to keep the FP64 pipe busy).
constexpr size_t F64W_MAX_NI = 32768;

template <class K>
static cudaError_t run_warp(const PairArgs &a, int sms, cudaStream_t s) {
    constexpr int WARPS = F64W_THREADS / 32;
    // fewest i per warp that still gives ~16 warps per SM
    const size_t want = (size_t)16 * (sms > 0 ? sms : 1);
    int ipw = 1;
    if (K::NT <= 16 && a.ni / 2 >= want) ipw = 2;
    if (K::NT <= 8 && a.ni / 4 >= want) ipw = 4;
    const size_t warps = (a.ni + ipw - 1) / ipw;
    const unsigned blocks = (unsigned)((warps + WARPS - 1) / WARPS);
    if (ipw == 4) fp64_warp<K, 4><<<blocks, F64W_THREADS, 0, s>>>(a);
    else if (ipw == 2) fp64_warp<K, 2><<<blocks, F64W_THREADS, 0, s>>>(a);
    else fp64_warp<K, 1><<<blocks, F64W_THREADS, 0, s>>>(a);
    return cudaGetLastError();
}

template <class K0>
static cudaError_t run(const PairArgs &a, int sms, cudaStream_t s) {
    if constexpr (has_terms<K0>::value) {
        if (a.ni <= F64W_MAX_NI) return run_warp<K0>(a, sms, s);
    }
    using K = typename SeqOf<K0>::type;
    const unsigned t = fp64_threads(a.ni, sms);
    const size_t blocks = (a.ni + t - 1) / t;
    fp64_pairwise<K><<<(unsigned)blocks, t, 0, s>>>(a);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Sakura with its Kepler pairs solved apart (flags -1 and +1).
//
// The pairs whose two-body step takes the universal-variable solver (the
// branch of sakura_kernel_common.h:111-122) are a few percent of all pairs,
// but in the warp engine each one holds the 31 other lanes of its round for
// the whole solve.  Here
//   1. sakura_mark tests every pair (twobody_uses_kepler, the solver's own
//      test) and writes one bitmap row of j per i and the row's count;
//   2. sakura_scan turns the counts into row offsets;
//   3. sakura_solve evolves the marked pairs, one per thread, and stores
//      their six terms in row order;
//   4. sakura_fold walks j in order like the warp engine, evolving leapfrog
//      pairs inline and reading the marked pairs' terms back,
// so every output is the same sum, in the same order, of the same terms as
// the one-pass kernel: bit-identical.  Marked pairs beyond the term buffer's
// capacity are evolved inline in step 4.
// ---------------------------------------------------------------------------
constexpr int SAK_WARPS = F64W_THREADS / 32;

__global__ void __launch_bounds__(F64W_THREADS) sakura_mark(PairArgs a, unsigned *bits, size_t W,
                                                           long long *count) {
    const int warp = threadIdx.x / 32, l = threadIdx.x % 32;
    const size_t i = (size_t)blockIdx.x * SAK_WARPS + warp;
    if (i >= a.ni) return;   // warp-uniform
    double fi[8], fj[8];
    for (int k = 0; k < 8; ++k) fi[k] = a.I.f[k][i];
    long long cnt = 0;
    for (size_t w = 0; w < W; ++w) {
        const size_t j = w * 32 + l;
        bool kep = false;
        if (j < a.nj) {
            for (int k = 0; k < 8; ++k) fj[k] = a.J.f[k][j];
            double r0[3], v0[3], e2, m;
            Sakura64::state(fi, fj, r0, v0, e2, m);
            kep = sakura_uses_kepler(a.dt, a.flag, m, r0, v0);
        }
        const unsigned b = __ballot_sync(0xffffffffu, kep);
        if (l == 0) bits[i * W + w] = b;
        cnt += __popc(b);
    }
    if (l == 0) count[i] = cnt;
}

// Exclusive scan of count[0, n) into off[0, n]; one CTA, each thread a
// contiguous chunk.
__global__ void __launch_bounds__(1024) sakura_scan(const long long *count, size_t n, long long *off) {
    __shared__ long long part[1024];
    const size_t chunk = (n + blockDim.x - 1) / blockDim.x;
    const size_t a0 = threadIdx.x * chunk, a1 = (a0 + chunk < n) ? a0 + chunk : n;
    long long sum = 0;
    for (size_t q = a0; q < a1; ++q) sum += count[q];
    part[threadIdx.x] = sum;
    __syncthreads();
    for (int d = 1; d < (int)blockDim.x; d *= 2) {   // inclusive Hillis-Steele scan
        const long long v = threadIdx.x >= (unsigned)d ? part[threadIdx.x - d] : 0;
        __syncthreads();
        part[threadIdx.x] += v;
        __syncthreads();
    }
    long long run = part[threadIdx.x] - sum;
    for (size_t q = a0; q < a1; ++q) { off[q] = run; run += count[q]; }
    if (threadIdx.x == blockDim.x - 1) off[n] = part[threadIdx.x];
}

// Marked pair number e (row i, rank e - off[i] within the row), one per
// thread, grid-stride; entries from `cap` on are left to sakura_fold.
__global__ void sakura_solve(PairArgs a, const unsigned *bits, size_t W, const long long *off,
                             double *terms, long long cap) {
    const long long total = off[a.ni];
    const long long n = total < cap ? total : cap;
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n;
         e += (long long)gridDim.x * blockDim.x) {
        size_t lo = 0, hi = a.ni;   // last row with off[row] <= e
        while (hi - lo > 1) {
            const size_t mid = (lo + hi) / 2;
            if (off[mid] <= e) lo = mid; else hi = mid;
        }
        const size_t i = lo;
        long long rank = e - off[i];
        size_t j = 0;
        for (size_t w = 0; w < W; ++w) {
            unsigned b = bits[i * W + w];
            const int p = __popc(b);
            if (rank < p) {
                for (long long q = 0; q < rank; ++q) b &= b - 1u;   // drop the lower set bits
                j = w * 32 + (size_t)(__ffs(b) - 1);
                break;
            }
            rank -= p;
        }
        double fi[8], fj[8], t[6];
        for (int k = 0; k < 8; ++k) { fi[k] = a.I.f[k][i]; fj[k] = a.J.f[k][j]; }
        Sakura64::pair_terms(fi, fj, a, t);
        for (int k = 0; k < 6; ++k) terms[e * 6 + k] = t[k];
    }
}

// The warp engine with one i per warp (32 consecutive j per round, one
// bitmap word), the marked pairs' terms read back in row order.
#ifndef TG_SAKURA_FOLD_MINB
#define TG_SAKURA_FOLD_MINB 3
#endif
__global__ void __launch_bounds__(F64W_THREADS, TG_SAKURA_FOLD_MINB) sakura_fold(PairArgs a, const unsigned *bits, size_t W,
                                                           const long long *off, const double *terms,
                                                           long long cap) {
    using K = Sakura64;
    __shared__ double sj[K::NF][F64_TILE];
    __shared__ double tt[SAK_WARPS][K::NT][33];
    const int warp = threadIdx.x / 32, l = threadIdx.x % 32;
    const size_t i = (size_t)blockIdx.x * SAK_WARPS + warp;
    const bool live = i < a.ni;
    K::St st;
    K::init(st, a, live ? i : 0);
    double acc = 0.0;
    long long e = live ? off[i] : 0;   // the row's next marked pair
    for (size_t j0 = 0; j0 < a.nj; j0 += F64_TILE) {
        const int nt = (int)((a.nj - j0) < (size_t)F64_TILE ? (a.nj - j0) : F64_TILE);
        for (int q = threadIdx.x; q < K::NF * F64_TILE; q += blockDim.x) {
            const int f = q / F64_TILE, jj = q % F64_TILE;
            if (jj < nt) sj[f][jj] = a.J.f[f][j0 + jj];
        }
        __syncthreads();
        for (int r = 0; r < nt; r += 32) {
            const unsigned word = live ? bits[i * W + (j0 + r) / 32] : 0u;
            if (r + l < nt) {
                double t[K::NT];
                const long long mine = e + __popc(word & ((1u << l) - 1u));
                if (!((word >> l) & 1u)) {
                    K::terms_leapfrog(st, sj, r + l, a, t);
                } else if (mine < cap) {
#pragma unroll
                    for (int c = 0; c < K::NT; ++c) t[c] = terms[mine * 6 + c];
                } else {
                    K::terms(st, sj, r + l, a, t);   // beyond the buffer: evolved here
                }
#pragma unroll
                for (int c = 0; c < K::NT; ++c) tt[warp][c][l] = t[c];
            }
            e += __popc(word);
            __syncwarp();
            const int m = (nt - r) < 32 ? (nt - r) : 32;
            if (l < K::NT)
                for (int q = 0; q < m; ++q) acc = K::accum(l, acc, tt[warp][l][q]);
            __syncwarp();
        }
        __syncthreads();
    }
    double res[K::NT];
#pragma unroll
    for (int c = 0; c < K::NT; ++c) res[c] = __shfl_sync(0xffffffffu, acc, c);
    if (l == 0 && live) K::store_acc(res, st, a, i);
}

namespace {
struct SakuraSplit {
    size_t W, bits_b, count_b, off_b, cap, terms_b;
};
size_t align256(size_t x) { return (x + 255) / 256 * 256; }
SakuraSplit sakura_split_layout(size_t ni, size_t nj) {
    SakuraSplit L;
    L.W = (nj + 31) / 32;
    L.bits_b = align256(ni * L.W * sizeof(unsigned));
    L.count_b = align256(ni * sizeof(long long));
    L.off_b = align256((ni + 1) * sizeof(long long));
    // room for 1/32 of the pairs (65536 to 2^21 entries): Kepler pairs are a
    // few percent of a cluster's pairs; any excess is evolved inline
    size_t cap = ni * nj / 32;
    if (cap < 65536) cap = 65536;
    if (cap > ((size_t)1 << 21)) cap = (size_t)1 << 21;
    if (cap > ni * nj) cap = ni * nj;
    L.cap = cap;
    L.terms_b = align256(cap * 6 * sizeof(double));
    return L;
}
}  // namespace

bool sakura_split_applies(const PairArgs &a) {
    return (a.flag == 1 || a.flag == -1) && a.ni > 0 && a.nj > 0 &&
           (double)a.ni * (double)a.nj <= 1073741824.0;
}

size_t sakura_split_ws_bytes(size_t ni, size_t nj) {
    const SakuraSplit L = sakura_split_layout(ni, nj);
    return L.bits_b + L.count_b + L.off_b + L.terms_b;
}

cudaError_t launch_sakura_split(const PairArgs &a, void *ws, size_t ws_bytes, int sms, cudaStream_t s) {
    const SakuraSplit L = sakura_split_layout(a.ni, a.nj);
    if (L.bits_b + L.count_b + L.off_b + L.terms_b > ws_bytes) return cudaErrorInvalidValue;
    char *base = static_cast<char *>(ws);
    unsigned *bits = reinterpret_cast<unsigned *>(base);
    long long *count = reinterpret_cast<long long *>(base + L.bits_b);
    long long *off = reinterpret_cast<long long *>(base + L.bits_b + L.count_b);
    double *terms = reinterpret_cast<double *>(base + L.bits_b + L.count_b + L.off_b);
    const unsigned blocks = (unsigned)((a.ni + SAK_WARPS - 1) / SAK_WARPS);
    sakura_mark<<<blocks, F64W_THREADS, 0, s>>>(a, bits, L.W, count);
    sakura_scan<<<1, 1024, 0, s>>>(count, a.ni, off);
    sakura_solve<<<(unsigned)(sms > 0 ? sms * 8 : 1024), 128, 0, s>>>(a, bits, L.W, off, terms, (long long)L.cap);
    sakura_fold<<<blocks, F64W_THREADS, 0, s>>>(a, bits, L.W, off, terms, (long long)L.cap);
    return cudaGetLastError();
}

cudaError_t launch_fp64(int kernel, const PairArgs &a, int sms, cudaStream_t s) {
    switch (kernel) {
        case K_PHI: return run<Phi64>(a, sms, s);
        case K_ACC: return run<Acc64>(a, sms, s);
        case K_ACC_JERK: return run<AccJerk64>(a, sms, s);
        case K_SNAP_CRACKLE: return run<SnapCrackle64>(a, sms, s);
        case K_TSTEP: return run<Tstep64>(a, sms, s);
        case K_PNACC: return run<PNAcc64>(a, sms, s);
        case K_SAKURA: return run<Sakura64>(a, sms, s);
        case K_ACC_VJP: return run<AccVjp64>(a, sms, s);
        case K_NREG_X: return run<NregX64>(a, sms, s);
        case K_NREG_V: return run<NregV64>(a, sms, s);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace tg
