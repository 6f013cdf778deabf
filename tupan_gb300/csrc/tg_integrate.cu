// tg_integrate.cu -- fused FP64 element-wise integrator updates.
//
// The integrators keep every particle attribute resident in HBM; between two
// pairwise-kernel calls they only need O(N) updates, fused here into one
// launch each instead of the dozen array operations of the numpy versions:
//
//   tg_drift / tg_kick       SIA drift r += v*tau and kick v += a*tau
//                            (tupan/integrator/sia.py:64-86)
//   tg_add_increments        r += dr, v += dv (Sakura, sakura.py:30-44)
//   tg_hermite_predict       Taylor predictor of order 2/4/6/8
//                            (tupan/integrator/hermite.py:24-36, 75-90,
//                            127-157, 200-235)
//   tg_hermite_correct       Hermite corrector of order 2/4/6/8
//                            (hermite.py:39-53, 93-119, 160-196, 238-283)
//   tg_div3                  x = mx / d for three arrays (NREG's r = mr / M,
//                            v = mv / M; nreg.py:27-29, 50-52)
//   tg_sum                   float64 sum in numpy's pairwise order, for the
//                            reductions that steer the reference integrators
//                            (total mass, energies; nreg.py:22-63)
//
// Every expression is evaluated with uncontracted IEEE operations in the
// order numpy evaluates the reference's Python expressions, so a GPU
// trajectory in FP64 is bit-identical to the reference integrator driven by
// the reference C kernels.
#include <cstring>

#include "../../include/tupan_gb300.h"
#include "tg_device.cuh"

namespace {

using tg::dadd;
using tg::ddiv;
using tg::dmul;
using tg::dsub;

struct Ptr3 { double *x[3]; };
struct CPtr3 { const double *x[3]; };

__global__ void k_drift(size_t n, Ptr3 r, CPtr3 v, double tau) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    for (int c = 0; c < 3; ++c) r.x[c][i] = dadd(r.x[c][i], dmul(v.x[c][i], tau));
}

__global__ void k_add(size_t n, Ptr3 r, Ptr3 v, CPtr3 dr, CPtr3 dv) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    for (int c = 0; c < 3; ++c) {
        r.x[c][i] = dadd(r.x[c][i], dr.x[c][i]);
        v.x[c][i] = dadd(v.x[c][i], dv.x[c][i]);
    }
}

// Predictor: with m = order/2 derivatives d[0..m-1] = a, j, s, c
//   r += ((((d[m-1] tau/(m+1) + d[m-2]) tau/m ...) + a) tau/2 + v) tau
//   v += (((d[m-1] tau/m + d[m-2]) ...) + a) tau
struct PredArgs {
    size_t n;
    double tau;
    int m;
    double *r[3], *v[3];
    const double *d[4][3];
};

__global__ void k_predict(PredArgs p) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n) return;
    const double tau = p.tau;
    for (int c = 0; c < 3; ++c) {
        const double v0 = p.v[c][i];
        double acc = p.d[p.m - 1][c][i];
        for (int q = p.m - 2; q >= 0; --q) acc = dadd(ddiv(dmul(acc, tau), (double)(q + 3)), p.d[q][c][i]);
        acc = dadd(ddiv(dmul(acc, tau), 2.0), v0);
        p.r[c][i] = dadd(p.r[c][i], dmul(acc, tau));
        double bcc = p.d[p.m - 1][c][i];
        for (int q = p.m - 2; q >= 0; --q) bcc = dadd(ddiv(dmul(bcc, tau), (double)(q + 2)), p.d[q][c][i]);
        p.v[c][i] = dadd(v0, dmul(bcc, tau));
    }
}

struct CorrArgs {
    size_t n;
    double tau;
    int order;
    const double *r0[3], *v0[3];
    const double *d0[4][3], *d1[4][3];   // a, j, s, c at the start and at the end
    double *r1[3], *v1[3];
};

__global__ void k_correct(CorrArgs p) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n) return;
    const double t = p.tau;
    for (int c = 0; c < 3; ++c) {
        const double r0 = p.r0[c][i], v0 = p.v0[c][i];
        const double a0 = p.d0[0][c][i], a1 = p.d1[0][c][i];
        double v1, r1;
        if (p.order == 2) {
            v1 = dadd(ddiv(dmul(dadd(a0, a1), t), 2.0), v0);
            r1 = dadd(ddiv(dmul(dadd(v0, v1), t), 2.0), r0);
        } else if (p.order == 4) {
            const double j0 = p.d0[1][c][i], j1 = p.d1[1][c][i];
            v1 = dadd(ddiv(dmul(dadd(ddiv(dmul(dsub(j0, j1), t), 6.0), dadd(a0, a1)), t), 2.0), v0);
            r1 = dadd(ddiv(dmul(dadd(ddiv(dmul(dsub(a0, a1), t), 6.0), dadd(v0, v1)), t), 2.0), r0);
        } else if (p.order == 6) {
            const double j0 = p.d0[1][c][i], j1 = p.d1[1][c][i];
            const double s0 = p.d0[2][c][i], s1 = p.d1[2][c][i];
            double w = dadd(ddiv(dmul(dadd(s0, s1), t), 12.0), dsub(j0, j1));
            w = dadd(ddiv(dmul(w, t), 5.0), dadd(a0, a1));
            v1 = dadd(ddiv(dmul(w, t), 2.0), v0);
            double u = dadd(ddiv(dmul(dadd(j0, j1), t), 12.0), dsub(a0, a1));
            u = dadd(ddiv(dmul(u, t), 5.0), dadd(v0, v1));
            r1 = dadd(ddiv(dmul(u, t), 2.0), r0);
        } else {
            const double j0 = p.d0[1][c][i], j1 = p.d1[1][c][i];
            const double s0 = p.d0[2][c][i], s1 = p.d1[2][c][i];
            const double c0 = p.d0[3][c][i], c1 = p.d1[3][c][i];
            double w = dadd(ddiv(dmul(dsub(c0, c1), t), 20.0), dadd(s0, s1));
            w = dadd(ddiv(dmul(w, t), 3.0), dmul(3.0, dsub(j0, j1)));
            w = dadd(ddiv(dmul(w, t), 14.0), dadd(a0, a1));
            v1 = dadd(ddiv(dmul(w, t), 2.0), v0);
            double u = dadd(ddiv(dmul(dsub(s0, s1), t), 20.0), dadd(j0, j1));
            u = dadd(ddiv(dmul(u, t), 3.0), dmul(3.0, dsub(a0, a1)));
            u = dadd(ddiv(dmul(u, t), 14.0), dadd(v0, v1));
            r1 = dadd(ddiv(dmul(u, t), 2.0), r0);
        }
        p.v1[c][i] = v1;
        p.r1[c][i] = r1;
    }
}

// numpy's float64 add-reduction of a contiguous array: blocks of at most 128
// elements are summed with eight interleaved accumulators combined as
// ((r0+r1)+(r2+r3))+((r4+r5)+(r6+r7)), then the tail in order; blocks of
// fewer than 8 elements are summed in order from 0; longer ranges split at
// n/2 rounded down to a multiple of 8 and add the halves; the reduction
// starts from the identity 0.  One thread walks the recursion with an
// explicit stack (depth <= 64): the reduction is O(n) adds with eight
// independent chains per block, negligible next to the O(n^2) kernels whose
// outputs it reduces.
__device__ double pw_block(const double *a, size_t n) {
    if (n < 8) {
        double r = 0.0;
        for (size_t i = 0; i < n; ++i) r = dadd(r, a[i]);
        return r;
    }
    double r[8];
    for (int j = 0; j < 8; ++j) r[j] = a[j];
    size_t i = 8;
    for (; i < n - (n % 8); i += 8)
        for (int j = 0; j < 8; ++j) r[j] = dadd(r[j], a[i + j]);
    double res = dadd(dadd(dadd(r[0], r[1]), dadd(r[2], r[3])), dadd(dadd(r[4], r[5]), dadd(r[6], r[7])));
    for (; i < n; ++i) res = dadd(res, a[i]);
    return res;
}

__global__ void k_sum_pairwise(size_t n, const double *a, double *out) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    struct Frame { size_t off, n; double left; int stage; };
    Frame st[64];
    int sp = 0;
    st[0] = Frame{0, n, 0.0, 0};
    double ret = 0.0;
    while (sp >= 0) {
        Frame &f = st[sp];
        if (f.n <= 128) { ret = pw_block(a + f.off, f.n); --sp; continue; }
        size_t n2 = f.n / 2;
        n2 -= n2 % 8;
        if (f.stage == 0) {
            f.stage = 1;
            st[++sp] = Frame{f.off, n2, 0.0, 0};
        } else if (f.stage == 1) {
            f.left = ret;
            f.stage = 2;
            st[++sp] = Frame{f.off + n2, f.n - n2, 0.0, 0};
        } else {
            ret = dadd(f.left, ret);
            --sp;
        }
    }
    *out = dadd(0.0, ret);
}

__global__ void k_div3(size_t n, Ptr3 x, CPtr3 mx, double d) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    for (int c = 0; c < 3; ++c) x.x[c][i] = ddiv(mx.x[c][i], d);
}

inline unsigned blocks_for(size_t n) { return (unsigned)((n + 255) / 256); }

int check_ptrs(const void *const *p, int k) {
    for (int q = 0; q < k; ++q)
        if (!p[q]) return TG_EINVAL;
    return TG_OK;
}

int launched() { return cudaGetLastError() == cudaSuccess ? TG_OK : TG_ECUDA; }

}  // namespace

extern "C" {

int tg_drift(size_t n, double *rx, double *ry, double *rz, const double *vx, const double *vy,
             const double *vz, double tau, void *stream) {
    if (n == 0) return TG_OK;
    const void *p[6] = {rx, ry, rz, vx, vy, vz};
    if (check_ptrs(p, 6)) return TG_EINVAL;
    k_drift<<<blocks_for(n), 256, 0, static_cast<cudaStream_t>(stream)>>>(n, Ptr3{{rx, ry, rz}}, CPtr3{{vx, vy, vz}}, tau);
    return launched();
}

int tg_kick(size_t n, double *vx, double *vy, double *vz, const double *ax, const double *ay,
            const double *az, double tau, void *stream) {
    return tg_drift(n, vx, vy, vz, ax, ay, az, tau, stream);
}

int tg_add_increments(size_t n, double *rx, double *ry, double *rz, double *vx, double *vy, double *vz,
                      const double *drx, const double *dry, const double *drz, const double *dvx,
                      const double *dvy, const double *dvz, void *stream) {
    if (n == 0) return TG_OK;
    const void *p[12] = {rx, ry, rz, vx, vy, vz, drx, dry, drz, dvx, dvy, dvz};
    if (check_ptrs(p, 12)) return TG_EINVAL;
    k_add<<<blocks_for(n), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        n, Ptr3{{rx, ry, rz}}, Ptr3{{vx, vy, vz}}, CPtr3{{drx, dry, drz}}, CPtr3{{dvx, dvy, dvz}});
    return launched();
}

int tg_hermite_predict(int order, size_t n, double tau, double *const *rv, const double *const *deriv,
                       void *stream) {
    if (order != 2 && order != 4 && order != 6 && order != 8) return TG_EINVAL;
    if (n == 0) return TG_OK;
    const int m = order / 2;
    if (!rv || !deriv || check_ptrs((const void *const *)rv, 6) || check_ptrs((const void *const *)deriv, 3 * m))
        return TG_EINVAL;
    PredArgs a;
    std::memset(&a, 0, sizeof a);
    a.n = n; a.tau = tau; a.m = m;
    for (int c = 0; c < 3; ++c) { a.r[c] = rv[c]; a.v[c] = rv[3 + c]; }
    for (int q = 0; q < m; ++q)
        for (int c = 0; c < 3; ++c) a.d[q][c] = deriv[3 * q + c];
    k_predict<<<blocks_for(n), 256, 0, static_cast<cudaStream_t>(stream)>>>(a);
    return launched();
}

int tg_hermite_correct(int order, size_t n, double tau, const double *const *rv0,
                       const double *const *deriv0, const double *const *deriv1, double *const *rv1,
                       void *stream) {
    if (order != 2 && order != 4 && order != 6 && order != 8) return TG_EINVAL;
    if (n == 0) return TG_OK;
    const int m = order / 2;
    if (!rv0 || !deriv0 || !deriv1 || !rv1 || check_ptrs((const void *const *)rv0, 6) ||
        check_ptrs((const void *const *)deriv0, 3 * m) || check_ptrs((const void *const *)deriv1, 3 * m) ||
        check_ptrs((const void *const *)rv1, 6))
        return TG_EINVAL;
    CorrArgs a;
    std::memset(&a, 0, sizeof a);
    a.n = n; a.tau = tau; a.order = order;
    for (int c = 0; c < 3; ++c) {
        a.r0[c] = rv0[c]; a.v0[c] = rv0[3 + c];
        a.r1[c] = rv1[c]; a.v1[c] = rv1[3 + c];
    }
    for (int q = 0; q < m; ++q)
        for (int c = 0; c < 3; ++c) { a.d0[q][c] = deriv0[3 * q + c]; a.d1[q][c] = deriv1[3 * q + c]; }
    k_correct<<<blocks_for(n), 256, 0, static_cast<cudaStream_t>(stream)>>>(a);
    return launched();
}

int tg_div3(size_t n, double *x, double *y, double *z, const double *mx, const double *my,
            const double *mz, double d, void *stream) {
    if (n == 0) return TG_OK;
    const void *p[6] = {x, y, z, mx, my, mz};
    if (check_ptrs(p, 6)) return TG_EINVAL;
    k_div3<<<blocks_for(n), 256, 0, static_cast<cudaStream_t>(stream)>>>(n, Ptr3{{x, y, z}}, CPtr3{{mx, my, mz}}, d);
    return launched();
}

int tg_sum(size_t n, const double *x, double *out, void *stream) {
    if (!out || (n > 0 && !x)) return TG_EINVAL;
    k_sum_pairwise<<<1, 32, 0, static_cast<cudaStream_t>(stream)>>>(n, x, out);
    return launched();
}

}  // extern "C"
