/*
 * tupan_oracle.c -- CPU restatement of Tupan's pairwise gravity kernels.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker for the GPU library:
 * it is compiled and called by tests/, by __graft_entry__.smoke() and by the
 * cpu_baseline / reference legs of bench.py, never by the product path.
 *
 * Each kernel restates the algorithm of the reference C backend
 * (tupan/lib/src/<name>_kernel.c + <name>_kernel_common.h + smoothing.h)
 * with the same per-pair operation order, so that with IEEE double
 * arithmetic and no FMA contraction (-ffp-contract=off) the FP64 results are
 * bit-identical to the reference on the same inputs.  The pin is checked by
 * tests/test_oracle_pin.py against the reference built from its own sources
 * (oracle/ref.mk) and against the golden fixtures in tests/golden/.
 *
 * Conventions (all follow tupan/lib/src/libtupan.h:2-246):
 *   - structure-of-arrays inputs, i-set then j-set, scalars, then outputs;
 *   - pair softening e2 = ie2 + je2, pair exclusion by r2 > 0;
 *   - every output is overwritten, nothing is accumulated across calls.
 * The extra trailing argument `nthreads` splits the i-range over POSIX
 * threads (the reference is single-threaded; slicing i does not change any
 * per-particle result because each i-sum runs over j in order).
 */
#define _POSIX_C_SOURCE 200809L
#define _GNU_SOURCE
#include <math.h>
#include <pthread.h>
#include <stddef.h>
#include <stdlib.h>
#include <string.h>

typedef double real;

/* ------------------------------------------------------------------------ */
/* Plummer-softened inverse distances, smoothing.h:10-183.                   */
/* inv_r2 = 1 / (r2 + e2), forced to 0 when r2 > 0 is false.                 */
/* ------------------------------------------------------------------------ */
static inline real soft_inv_r2(real r2, real e2)
{
    real q = 1 / (r2 + e2);
    return (r2 > 0) ? q : (real)0;
}

/* ------------------------------------------------------------------------ */
/* Threaded i-range driver.                                                  */
/* ------------------------------------------------------------------------ */
typedef void (*range_fn)(void *ctx, size_t i0, size_t i1);

struct slice_job { range_fn fn; void *ctx; size_t i0, i1; };

static void *slice_entry(void *p)
{
    struct slice_job *s = (struct slice_job *)p;
    s->fn(s->ctx, s->i0, s->i1);
    return NULL;
}

static void run_sliced(range_fn fn, void *ctx, size_t ni, int nthreads)
{
    if (nthreads <= 1 || ni < 2) { fn(ctx, 0, ni); return; }
    if ((size_t)nthreads > ni) nthreads = (int)ni;
    pthread_t *tid = (pthread_t *)malloc(sizeof(pthread_t) * (size_t)nthreads);
    struct slice_job *job = (struct slice_job *)malloc(sizeof(*job) * (size_t)nthreads);
    int started = 0;
    for (int t = 0; t < nthreads; ++t) {
        job[t].fn = fn; job[t].ctx = ctx;
        job[t].i0 = ni * (size_t)t / (size_t)nthreads;
        job[t].i1 = ni * (size_t)(t + 1) / (size_t)nthreads;
        if (t == 0) continue;
        if (pthread_create(&tid[t], NULL, slice_entry, &job[t]) == 0) {
            ++started;
        } else {
            fn(ctx, job[t].i0, job[t].i1);   /* run inline if no thread */
            job[t].fn = NULL;
        }
    }
    fn(ctx, job[0].i0, job[0].i1);
    for (int t = 1; t < nthreads; ++t)
        if (job[t].fn) pthread_join(tid[t], NULL);
    (void)started;
    free(tid); free(job);
}

/* A generic bag of pointers; each kernel reads the fields it needs. */
struct pset {
    const real *m, *rx, *ry, *rz, *e2, *vx, *vy, *vz;
    const real *ax, *ay, *az, *jx, *jy, *jz;
};

struct call {
    struct pset I, J;
    size_t nj;
    real *o[8];
    real eta, dt;
    long flag;
    unsigned long order;
    real inv[8];
};

/* ------------------------------------------------------------------------ */
/* Phi: phi_kernel_common.h:7-31, phi_kernel.c:5-34                          */
/* ------------------------------------------------------------------------ */
static void phi_range(void *p, size_t i0, size_t i1)
{
    struct call *c = (struct call *)p;
    for (size_t i = i0; i < i1; ++i) {
        real xi = c->I.rx[i], yi = c->I.ry[i], zi = c->I.rz[i], ei = c->I.e2[i];
        real acc = 0;
        for (size_t j = 0; j < c->nj; ++j) {
            real dx = xi - c->J.rx[j];
            real dy = yi - c->J.ry[j];
            real dz = zi - c->J.rz[j];
            real e2 = ei + c->J.e2[j];
            real r2 = dx * dx + dy * dy + dz * dz;
            real inv_r1 = sqrt(soft_inv_r2(r2, e2));
            acc -= c->J.m[j] * inv_r1;
        }
        c->o[0][i] = acc;
    }
}

/* ------------------------------------------------------------------------ */
/* Acc: acc_kernel_common.h:7-37, acc_kernel.c:5-40                          */
/* ------------------------------------------------------------------------ */
static void acc_range(void *p, size_t i0, size_t i1)
{
    struct call *c = (struct call *)p;
    for (size_t i = i0; i < i1; ++i) {
        real xi = c->I.rx[i], yi = c->I.ry[i], zi = c->I.rz[i], ei = c->I.e2[i];
        real ax = 0, ay = 0, az = 0;
        for (size_t j = 0; j < c->nj; ++j) {
            real dx = xi - c->J.rx[j];
            real dy = yi - c->J.ry[j];
            real dz = zi - c->J.rz[j];
            real e2 = ei + c->J.e2[j];
            real r2 = dx * dx + dy * dy + dz * dz;
            real q2 = soft_inv_r2(r2, e2);
            real q3 = q2 * sqrt(q2);
            q3 *= c->J.m[j];
            ax -= q3 * dx;
            ay -= q3 * dy;
            az -= q3 * dz;
        }
        c->o[0][i] = ax; c->o[1][i] = ay; c->o[2][i] = az;
    }
}

/* ------------------------------------------------------------------------ */
/* AccJerk: acc_jerk_kernel_common.h:7-55, acc_jerk_kernel.c:5-60            */
/* ------------------------------------------------------------------------ */
static void acc_jerk_range(void *p, size_t i0, size_t i1)
{
    struct call *c = (struct call *)p;
    for (size_t i = i0; i < i1; ++i) {
        real xi = c->I.rx[i], yi = c->I.ry[i], zi = c->I.rz[i], ei = c->I.e2[i];
        real ui = c->I.vx[i], vi = c->I.vy[i], wi = c->I.vz[i];
        real ax = 0, ay = 0, az = 0, jx = 0, jy = 0, jz = 0;
        for (size_t j = 0; j < c->nj; ++j) {
            real dx = xi - c->J.rx[j];
            real dy = yi - c->J.ry[j];
            real dz = zi - c->J.rz[j];
            real e2 = ei + c->J.e2[j];
            real du = ui - c->J.vx[j];
            real dv = vi - c->J.vy[j];
            real dw = wi - c->J.vz[j];
            real r2 = dx * dx + dy * dy + dz * dz;
            real rv = dx * du + dy * dv + dz * dw;
            real q2 = soft_inv_r2(r2, e2);
            real q3 = q2 * sqrt(q2);
            real alpha = 3 * rv * q2;
            du -= alpha * dx;
            dv -= alpha * dy;
            dw -= alpha * dz;
            q3 *= c->J.m[j];
            ax -= q3 * dx; ay -= q3 * dy; az -= q3 * dz;
            jx -= q3 * du; jy -= q3 * dv; jz -= q3 * dw;
        }
        c->o[0][i] = ax; c->o[1][i] = ay; c->o[2][i] = az;
        c->o[3][i] = jx; c->o[4][i] = jy; c->o[5][i] = jz;
    }
}

/* ------------------------------------------------------------------------ */
/* SnapCrackle: snap_crackle_kernel_common.h:7-94, snap_crackle_kernel.c     */
/* ------------------------------------------------------------------------ */
static void snap_crackle_range(void *p, size_t i0, size_t i1)
{
    struct call *c = (struct call *)p;
    const struct pset *I = &c->I, *J = &c->J;
    for (size_t i = i0; i < i1; ++i) {
        real sx = 0, sy = 0, sz = 0, kx = 0, ky = 0, kz = 0;
        for (size_t j = 0; j < c->nj; ++j) {
            real rx = I->rx[i] - J->rx[j], ry = I->ry[i] - J->ry[j], rz = I->rz[i] - J->rz[j];
            real e2 = I->e2[i] + J->e2[j];
            real vx = I->vx[i] - J->vx[j], vy = I->vy[i] - J->vy[j], vz = I->vz[i] - J->vz[j];
            real Ax = I->ax[i] - J->ax[j], Ay = I->ay[i] - J->ay[j], Az = I->az[i] - J->az[j];
            real Jx = I->jx[i] - J->jx[j], Jy = I->jy[i] - J->jy[j], Jz = I->jz[i] - J->jz[j];
            real r2 = rx * rx + ry * ry + rz * rz;
            real rv = rx * vx + ry * vy + rz * vz;
            real v2 = vx * vx + vy * vy + vz * vz;
            real rJ = rx * Jx + ry * Jy + rz * Jz;
            real rA = rx * Ax + ry * Ay + rz * Az;
            real vA = vx * Ax + vy * Ay + vz * Az;
            real q2 = soft_inv_r2(r2, e2);
            real q3 = q2 * sqrt(q2);
            real al = rv * q2;
            real al2 = al * al;
            real be = 3 * ((v2 + rA) * q2 + al2);
            real ga = (3 * vA + rJ) * q2 + al * (be - 4 * al2);
            al *= 3;
            ga *= 3;
            vx -= al * rx; vy -= al * ry; vz -= al * rz;
            real two_al = 2 * al;
            Ax -= two_al * vx + be * rx;
            Ay -= two_al * vy + be * ry;
            Az -= two_al * vz + be * rz;
            al *= 3;
            be *= 3;
            Jx -= al * Ax + be * vx + ga * rx;
            Jy -= al * Ay + be * vy + ga * ry;
            Jz -= al * Az + be * vz + ga * rz;
            q3 *= J->m[j];
            sx -= q3 * Ax; sy -= q3 * Ay; sz -= q3 * Az;
            kx -= q3 * Jx; ky -= q3 * Jy; kz -= q3 * Jz;
        }
        c->o[0][i] = sx; c->o[1][i] = sy; c->o[2][i] = sz;
        c->o[3][i] = kx; c->o[4][i] = ky; c->o[5][i] = kz;
    }
}

/* ------------------------------------------------------------------------ */
/* Tstep: tstep_kernel_common.h:7-59, tstep_kernel.c:5-49                    */
/* ------------------------------------------------------------------------ */
static void tstep_range(void *p, size_t i0, size_t i1)
{
    struct call *c = (struct call *)p;
    const struct pset *I = &c->I, *J = &c->J;
    const real eta = c->eta;
    for (size_t i = i0; i < i1; ++i) {
        real wsum = 0, wmax = 0;
        for (size_t j = 0; j < c->nj; ++j) {
            real rx = I->rx[i] - J->rx[j], ry = I->ry[i] - J->ry[j], rz = I->rz[i] - J->rz[j];
            real e2 = I->e2[i] + J->e2[j];
            real vx = I->vx[i] - J->vx[j], vy = I->vy[i] - J->vy[j], vz = I->vz[i] - J->vz[j];
            real m = I->m[i] + J->m[j];
            real r2 = rx * rx + ry * ry + rz * rz;
            real rv = rx * vx + ry * vy + rz * vz;
            real v2 = vx * vx + vy * vy + vz * vz;
            real q2 = soft_inv_r2(r2, e2);
            real q1 = sqrt(q2);
            /* a = 2 in the reference, so (1 + a/2) = 2 exactly */
            real b = 2 * q2;
            real phi = m * q1;
            real w2 = q2 * (v2 + 2 * phi);
            real gam = q2 * (w2 + b * phi);
            gam *= eta / sqrt(w2);
            w2 -= gam * rv;
            if (!(r2 > 0)) w2 = 0;
            wsum += w2;
            wmax = fmax(w2, wmax);
        }
        c->o[0][i] = eta / sqrt(1 + wsum);
        c->o[1][i] = eta / sqrt(1 + wmax);
    }
}

/* ------------------------------------------------------------------------ */
/* PNAcc: pnacc_kernel_common.h:8-69, pn_terms.h:126-567.                    */
/* The PN accelerations are evaluated from a monomial table (pn_table.h,     */
/* produced by oracle/gen_pn_table.py) instead of the reference's nested     */
/* Horner forms: same polynomial, independent rounding.                      */
/* ------------------------------------------------------------------------ */
#include "pn_table.h"

static real pn_eval(const struct pn_mono *t, int n, const real *var)
{
    /* sum of coeff * prod var[k]^e[k]; powers are small non-negative ints */
    real s = 0;
    for (int q = 0; q < n; ++q) {
        real term = t[q].c;
        for (int k = 0; k < PN_NVAR; ++k) {
            for (int e = 0; e < t[q].e[k]; ++e) term *= var[k];
        }
        s += term;
    }
    return s;
}

static void pnacc_range(void *p, size_t i0, size_t i1)
{
    struct call *c = (struct call *)p;
    const struct pset *I = &c->I, *J = &c->J;
    const unsigned long order = c->order;
    for (size_t i = i0; i < i1; ++i) {
        real ax = 0, ay = 0, az = 0;
        for (size_t j = 0; j < c->nj; ++j) {
            real rx = I->rx[i] - J->rx[j], ry = I->ry[i] - J->ry[j], rz = I->rz[i] - J->rz[j];
            real e2 = I->e2[i] + J->e2[j];
            real vx = I->vx[i] - J->vx[j], vy = I->vy[i] - J->vy[j], vz = I->vz[i] - J->vz[j];
            real r2 = rx * rx + ry * ry + rz * rz;
            real v2 = vx * vx + vy * vy + vz * vz;
            real q2 = soft_inv_r2(r2, e2);
            real q1 = sqrt(q2);
            real q3 = q2 * q1;
            real nx = rx * q1, ny = ry * q1, nz = rz * q1;
            real iv2 = I->vx[i] * I->vx[i] + I->vy[i] * I->vy[i] + I->vz[i] * I->vz[i];
            real jv2 = J->vx[j] * J->vx[j] + J->vy[j] * J->vy[j] + J->vz[j] * J->vz[j];
            real var[PN_NVAR];
            var[PN_IM] = I->m[i];
            var[PN_JM] = J->m[j];
            var[PN_IR] = q1;
            var[PN_IV2] = iv2;
            var[PN_JV2] = jv2;
            var[PN_IVJV] = I->vx[i] * J->vx[j] + I->vy[i] * J->vy[j] + I->vz[i] * J->vz[j];
            var[PN_NIV] = nx * I->vx[i] + ny * I->vy[i] + nz * I->vz[i];
            var[PN_NJV] = nx * J->vx[j] + ny * J->vy[j] + nz * J->vz[j];
            var[PN_NV] = nx * vx + ny * vy + nz * vz;
            var[PN_V2] = v2;
            real A = 0, B = 0;
            /* orders: 2 -> 1/c^2, 4 -> 1/c^4, 5 -> 1/c^5, 6 -> 1/c^6, 7 -> 1/c^7 */
            for (int k = 0; k < PN_NORDERS; ++k) {
                if (order < pn_orders[k].min_order) continue;
                real cpow = c->inv[pn_orders[k].cpow];
                A += cpow * pn_eval(pn_orders[k].a, pn_orders[k].na, var);
                B += cpow * pn_eval(pn_orders[k].b, pn_orders[k].nb, var);
            }
            A *= J->m[j] * q3;
            B *= J->m[j] * q2;
            ax += A * rx + B * vx;
            ay += A * ry + B * vy;
            az += A * rz + B * vz;
        }
        c->o[0][i] = ax; c->o[1][i] = ay; c->o[2][i] = az;
    }
}

/* ------------------------------------------------------------------------ */
/* Sakura: sakura_kernel_common.h:8-243 with the universal-variable Kepler   */
/* solver of universal_kepler_solver.h:17-614.                               */
/* ------------------------------------------------------------------------ */
#include "kepler_oracle.h"

static void sakura_range(void *p, size_t i0, size_t i1)
{
    struct call *c = (struct call *)p;
    const struct pset *I = &c->I, *J = &c->J;
    orc_set_caps(ORC_SPLIT_CAP, ORC_ENERGY_CAP, ORC_SOLVE_BUDGET);
    for (size_t i = i0; i < i1; ++i) {
        real d[6] = {0, 0, 0, 0, 0, 0};
        for (size_t j = 0; j < c->nj; ++j) {
            real r0[3] = {I->rx[i] - J->rx[j], I->ry[i] - J->ry[j], I->rz[i] - J->rz[j]};
            real e2 = I->e2[i] + J->e2[j];
            real v0[3] = {I->vx[i] - J->vx[j], I->vy[i] - J->vy[j], I->vz[i] - J->vz[j]};
            real m = I->m[i] + J->m[j];
            real r1[3], v1[3];
            orc_twobody_evolve(c->dt, c->flag, m, e2, r0, v0, r1, v1);
            real w = J->m[j] / m;
            for (int k = 0; k < 3; ++k) {
                d[k] += w * (r1[k] - r0[k]);
                d[3 + k] += w * (v1[k] - v0[k]);
            }
        }
        for (int k = 0; k < 6; ++k) c->o[k][i] = d[k];
    }
}

/* ------------------------------------------------------------------------ */
/* NREG_X: nreg_kernels_common.h:7-60, nreg_kernels.c:5-67.                  */
/* The pair separation is drifted by dt with the relative velocity before    */
/* use; outputs are sum m_j r_ij (mr), the softened acceleration and         */
/* u_i = m_i sum m_j / r_ij.                                                 */
/* ------------------------------------------------------------------------ */
static void nreg_x_range(void *p, size_t i0, size_t i1)
{
    struct call *c = (struct call *)p;
    const struct pset *I = &c->I, *J = &c->J;
    const real dt = c->dt;
    for (size_t i = i0; i < i1; ++i) {
        real mrx = 0, mry = 0, mrz = 0, ax = 0, ay = 0, az = 0, u = 0;
        for (size_t j = 0; j < c->nj; ++j) {
            real rx = I->rx[i] - J->rx[j];
            real ry = I->ry[i] - J->ry[j];
            real rz = I->rz[i] - J->rz[j];
            real e2 = I->e2[i] + J->e2[j];
            real vx = I->vx[i] - J->vx[j];
            real vy = I->vy[i] - J->vy[j];
            real vz = I->vz[i] - J->vz[j];
            rx += vx * dt;
            ry += vy * dt;
            rz += vz * dt;
            real r2 = rx * rx + ry * ry + rz * rz;
            real q2 = soft_inv_r2(r2, e2);
            real q1 = sqrt(q2);
            real q3 = q2 * q1;
            q3 *= J->m[j];
            mrx += J->m[j] * rx;
            mry += J->m[j] * ry;
            mrz += J->m[j] * rz;
            ax -= q3 * rx;
            ay -= q3 * ry;
            az -= q3 * rz;
            u += J->m[j] * q1;
        }
        c->o[0][i] = mrx; c->o[1][i] = mry; c->o[2][i] = mrz;
        c->o[3][i] = ax; c->o[4][i] = ay; c->o[5][i] = az;
        c->o[6][i] = I->m[i] * u;
    }
}

/* ------------------------------------------------------------------------ */
/* NREG_V: nreg_kernels_common.h:62-102, nreg_kernels.c:70-116.              */
/* The relative velocity is kicked by dt with the relative acceleration;     */
/* outputs are sum m_j v_ij (mv) and k_i = m_i sum m_j |v_ij|^2.             */
/* ------------------------------------------------------------------------ */
static void nreg_v_range(void *p, size_t i0, size_t i1)
{
    struct call *c = (struct call *)p;
    const struct pset *I = &c->I, *J = &c->J;
    const real dt = c->dt;
    for (size_t i = i0; i < i1; ++i) {
        real mvx = 0, mvy = 0, mvz = 0, k = 0;
        for (size_t j = 0; j < c->nj; ++j) {
            real vx = I->vx[i] - J->vx[j];
            real vy = I->vy[i] - J->vy[j];
            real vz = I->vz[i] - J->vz[j];
            real ax = I->ax[i] - J->ax[j];
            real ay = I->ay[i] - J->ay[j];
            real az = I->az[i] - J->az[j];
            vx += ax * dt;
            vy += ay * dt;
            vz += az * dt;
            real v2 = vx * vx + vy * vy + vz * vz;
            mvx += J->m[j] * vx;
            mvy += J->m[j] * vy;
            mvz += J->m[j] * vz;
            k += J->m[j] * v2;
        }
        c->o[0][i] = mvx; c->o[1][i] = mvy; c->o[2][i] = mvz;
        c->o[3][i] = I->m[i] * k;
    }
}

/* ------------------------------------------------------------------------ */
/* Kepler pair solver: kepler_solver_kernel_common.h:8-81 and                */
/* kepler_solver_kernel.c.  Pair p is elements 2p (i) and 2p+1 (j); the      */
/* centre of mass drifts freely and the relative orbit follows the bounded   */
/* universal-variable solver.  Outputs may alias the inputs.                 */
/* ------------------------------------------------------------------------ */
struct kcall {
    const real *m, *rx, *ry, *rz, *e2, *vx, *vy, *vz;
    real dt;
    real *o[6];
    int *capped;    /* per pair: 1 when a retry bound was reached (may be NULL) */
};

static void kepler_range(void *p, size_t k0, size_t k1)
{
    struct kcall *c = (struct kcall *)p;
    for (size_t k = k0; k < k1; ++k) {
        const size_t a = 2 * k, b = 2 * k + 1;
        real im = c->m[a], jm = c->m[b];
        real ir[3] = {c->rx[a], c->ry[a], c->rz[a]}, jr[3] = {c->rx[b], c->ry[b], c->rz[b]};
        real iv[3] = {c->vx[a], c->vy[a], c->vz[a]}, jv[3] = {c->vx[b], c->vy[b], c->vz[b]};
        real r0[3], v0[3], rcm[3], vcm[3], r1[3], v1[3];
        for (int q = 0; q < 3; ++q) { r0[q] = ir[q] - jr[q]; }
        real e2 = c->e2[a] + c->e2[b];
        for (int q = 0; q < 3; ++q) { v0[q] = iv[q] - jv[q]; }
        real m = im + jm;
        real imu = im / m, jmu = jm / m;
        for (int q = 0; q < 3; ++q) rcm[q] = imu * ir[q] + jmu * jr[q];
        for (int q = 0; q < 3; ++q) vcm[q] = imu * iv[q] + jmu * jv[q];
        for (int q = 0; q < 3; ++q) rcm[q] += vcm[q] * c->dt;
        orc_set_caps(ORC_PAIR_SPLIT_CAP, ORC_PAIR_ENERGY_CAP, ORC_PAIR_SOLVE_BUDGET);
        orc_solves = 0;
        orc_capped = 0;
        orc_kepler(c->dt, m, e2, r0, v0, r1, v1);
        if (c->capped) c->capped[k] = orc_capped;
        for (int q = 0; q < 3; ++q) {
            c->o[q][a] = rcm[q] + jmu * r1[q];
            c->o[3 + q][a] = vcm[q] + jmu * v1[q];
            c->o[q][b] = rcm[q] - imu * r1[q];
            c->o[3 + q][b] = vcm[q] - imu * v1[q];
        }
    }
}

/* ------------------------------------------------------------------------ */
/* Exported entry points: argument order of libtupan.h, plus nthreads.       */
/* ------------------------------------------------------------------------ */
#define SET5(S, m_, x_, y_, z_, e_) do { (S).m = m_; (S).rx = x_; (S).ry = y_; (S).rz = z_; (S).e2 = e_; } while (0)
#define SETV(S, u_, v_, w_) do { (S).vx = u_; (S).vy = v_; (S).vz = w_; } while (0)

void orc_phi(size_t ni, const real *im, const real *irx, const real *iry, const real *irz, const real *ie2,
             size_t nj, const real *jm, const real *jrx, const real *jry, const real *jrz, const real *je2,
             real *iphi, int nthreads)
{
    struct call c; memset(&c, 0, sizeof c);
    SET5(c.I, im, irx, iry, irz, ie2); SET5(c.J, jm, jrx, jry, jrz, je2);
    c.nj = nj; c.o[0] = iphi;
    run_sliced(phi_range, &c, ni, nthreads);
}

void orc_acc(size_t ni, const real *im, const real *irx, const real *iry, const real *irz, const real *ie2,
             size_t nj, const real *jm, const real *jrx, const real *jry, const real *jrz, const real *je2,
             real *iax, real *iay, real *iaz, int nthreads)
{
    struct call c; memset(&c, 0, sizeof c);
    SET5(c.I, im, irx, iry, irz, ie2); SET5(c.J, jm, jrx, jry, jrz, je2);
    c.nj = nj; c.o[0] = iax; c.o[1] = iay; c.o[2] = iaz;
    run_sliced(acc_range, &c, ni, nthreads);
}

void orc_acc_jerk(size_t ni, const real *im, const real *irx, const real *iry, const real *irz, const real *ie2,
                  const real *ivx, const real *ivy, const real *ivz,
                  size_t nj, const real *jm, const real *jrx, const real *jry, const real *jrz, const real *je2,
                  const real *jvx, const real *jvy, const real *jvz,
                  real *iax, real *iay, real *iaz, real *ijx, real *ijy, real *ijz, int nthreads)
{
    struct call c; memset(&c, 0, sizeof c);
    SET5(c.I, im, irx, iry, irz, ie2); SETV(c.I, ivx, ivy, ivz);
    SET5(c.J, jm, jrx, jry, jrz, je2); SETV(c.J, jvx, jvy, jvz);
    c.nj = nj;
    c.o[0] = iax; c.o[1] = iay; c.o[2] = iaz; c.o[3] = ijx; c.o[4] = ijy; c.o[5] = ijz;
    run_sliced(acc_jerk_range, &c, ni, nthreads);
}

void orc_snap_crackle(size_t ni, const real *im, const real *irx, const real *iry, const real *irz, const real *ie2,
                      const real *ivx, const real *ivy, const real *ivz,
                      const real *iax, const real *iay, const real *iaz,
                      const real *ijx, const real *ijy, const real *ijz,
                      size_t nj, const real *jm, const real *jrx, const real *jry, const real *jrz, const real *je2,
                      const real *jvx, const real *jvy, const real *jvz,
                      const real *jax, const real *jay, const real *jaz,
                      const real *jjx, const real *jjy, const real *jjz,
                      real *isx, real *isy, real *isz, real *icx, real *icy, real *icz, int nthreads)
{
    struct call c; memset(&c, 0, sizeof c);
    SET5(c.I, im, irx, iry, irz, ie2); SETV(c.I, ivx, ivy, ivz);
    c.I.ax = iax; c.I.ay = iay; c.I.az = iaz; c.I.jx = ijx; c.I.jy = ijy; c.I.jz = ijz;
    SET5(c.J, jm, jrx, jry, jrz, je2); SETV(c.J, jvx, jvy, jvz);
    c.J.ax = jax; c.J.ay = jay; c.J.az = jaz; c.J.jx = jjx; c.J.jy = jjy; c.J.jz = jjz;
    c.nj = nj;
    c.o[0] = isx; c.o[1] = isy; c.o[2] = isz; c.o[3] = icx; c.o[4] = icy; c.o[5] = icz;
    run_sliced(snap_crackle_range, &c, ni, nthreads);
}

void orc_tstep(size_t ni, const real *im, const real *irx, const real *iry, const real *irz, const real *ie2,
               const real *ivx, const real *ivy, const real *ivz,
               size_t nj, const real *jm, const real *jrx, const real *jry, const real *jrz, const real *je2,
               const real *jvx, const real *jvy, const real *jvz,
               real eta, real *idt_a, real *idt_b, int nthreads)
{
    struct call c; memset(&c, 0, sizeof c);
    SET5(c.I, im, irx, iry, irz, ie2); SETV(c.I, ivx, ivy, ivz);
    SET5(c.J, jm, jrx, jry, jrz, je2); SETV(c.J, jvx, jvy, jvz);
    c.nj = nj; c.eta = eta; c.o[0] = idt_a; c.o[1] = idt_b;
    run_sliced(tstep_range, &c, ni, nthreads);
}

void orc_pnacc(size_t ni, const real *im, const real *irx, const real *iry, const real *irz, const real *ie2,
               const real *ivx, const real *ivy, const real *ivz,
               size_t nj, const real *jm, const real *jrx, const real *jry, const real *jrz, const real *je2,
               const real *jvx, const real *jvy, const real *jvz,
               unsigned long order, real inv1, real inv2, real inv3, real inv4, real inv5, real inv6, real inv7,
               real *ipnax, real *ipnay, real *ipnaz, int nthreads)
{
    struct call c; memset(&c, 0, sizeof c);
    SET5(c.I, im, irx, iry, irz, ie2); SETV(c.I, ivx, ivy, ivz);
    SET5(c.J, jm, jrx, jry, jrz, je2); SETV(c.J, jvx, jvy, jvz);
    c.nj = nj; c.order = order;
    c.inv[1] = inv1; c.inv[2] = inv2; c.inv[3] = inv3; c.inv[4] = inv4;
    c.inv[5] = inv5; c.inv[6] = inv6; c.inv[7] = inv7;
    c.o[0] = ipnax; c.o[1] = ipnay; c.o[2] = ipnaz;
    run_sliced(pnacc_range, &c, ni, nthreads);
}

void orc_sakura(size_t ni, const real *im, const real *irx, const real *iry, const real *irz, const real *ie2,
                const real *ivx, const real *ivy, const real *ivz,
                size_t nj, const real *jm, const real *jrx, const real *jry, const real *jrz, const real *je2,
                const real *jvx, const real *jvy, const real *jvz,
                real dt, long flag,
                real *idrx, real *idry, real *idrz, real *idvx, real *idvy, real *idvz, int nthreads)
{
    struct call c; memset(&c, 0, sizeof c);
    SET5(c.I, im, irx, iry, irz, ie2); SETV(c.I, ivx, ivy, ivz);
    SET5(c.J, jm, jrx, jry, jrz, je2); SETV(c.J, jvx, jvy, jvz);
    c.nj = nj; c.dt = dt; c.flag = flag;
    c.o[0] = idrx; c.o[1] = idry; c.o[2] = idrz; c.o[3] = idvx; c.o[4] = idvy; c.o[5] = idvz;
    run_sliced(sakura_range, &c, ni, nthreads);
}

void orc_nreg_x(size_t ni, const real *im, const real *irx, const real *iry, const real *irz, const real *ie2,
                const real *ivx, const real *ivy, const real *ivz,
                size_t nj, const real *jm, const real *jrx, const real *jry, const real *jrz, const real *je2,
                const real *jvx, const real *jvy, const real *jvz,
                real dt, real *imrx, real *imry, real *imrz, real *iax, real *iay, real *iaz, real *iu,
                int nthreads)
{
    struct call c; memset(&c, 0, sizeof c);
    SET5(c.I, im, irx, iry, irz, ie2); SETV(c.I, ivx, ivy, ivz);
    SET5(c.J, jm, jrx, jry, jrz, je2); SETV(c.J, jvx, jvy, jvz);
    c.nj = nj; c.dt = dt;
    c.o[0] = imrx; c.o[1] = imry; c.o[2] = imrz; c.o[3] = iax; c.o[4] = iay; c.o[5] = iaz; c.o[6] = iu;
    run_sliced(nreg_x_range, &c, ni, nthreads);
}

void orc_nreg_v(size_t ni, const real *im, const real *ivx, const real *ivy, const real *ivz,
                const real *iax, const real *iay, const real *iaz,
                size_t nj, const real *jm, const real *jvx, const real *jvy, const real *jvz,
                const real *jax, const real *jay, const real *jaz,
                real dt, real *imvx, real *imvy, real *imvz, real *ik, int nthreads)
{
    struct call c; memset(&c, 0, sizeof c);
    c.I.m = im; SETV(c.I, ivx, ivy, ivz); c.I.ax = iax; c.I.ay = iay; c.I.az = iaz;
    c.J.m = jm; SETV(c.J, jvx, jvy, jvz); c.J.ax = jax; c.J.ay = jay; c.J.az = jaz;
    c.nj = nj; c.dt = dt;
    c.o[0] = imvx; c.o[1] = imvy; c.o[2] = imvz; c.o[3] = ik;
    run_sliced(nreg_v_range, &c, ni, nthreads);
}

/* npairs independent pairs (2 npairs particles); libtupan.h kepler_solver_kernel
 * is the npairs = 1 case. */
void orc_kepler_solver(size_t npairs, const real *m, const real *rx, const real *ry, const real *rz,
                       const real *e2, const real *vx, const real *vy, const real *vz, real dt,
                       real *r1x, real *r1y, real *r1z, real *v1x, real *v1y, real *v1z, int *capped,
                       int nthreads)
{
    struct kcall c;
    c.capped = capped;
    c.m = m; c.rx = rx; c.ry = ry; c.rz = rz; c.e2 = e2; c.vx = vx; c.vy = vy; c.vz = vz; c.dt = dt;
    c.o[0] = r1x; c.o[1] = r1y; c.o[2] = r1z; c.o[3] = v1x; c.o[4] = v1y; c.o[5] = v1z;
    run_sliced(kepler_range, &c, npairs, nthreads);
}
