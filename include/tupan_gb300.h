/*
 * tupan_gb300.h -- C ABI of libtupan_gb300.so, the GB300 (sm_103a) backend
 * for Tupan's direct-summation pairwise kernels.
 *
 * Two families of entry points:
 *
 * 1. Drop-in host entry points with the exact signatures of the reference's
 *    C library (tupan/lib/src/libtupan.h:2-246, float64 build: UINT is
 *    unsigned long, INT is long, REAL is double).  They take HOST pointers,
 *    copy inputs to the GPU, run, copy outputs back and return when done, so
 *    the reference's cffi backend can load this library in place of its own
 *    build.  The arithmetic precision is chosen with
 *    tg_set_host_precision() (default TG_PREC_FP64).
 *
 * 2. Device entry points tg_<kernel>(...) with the same argument order but
 *    DEVICE pointers, a precision selector and a CUDA stream.  They are
 *    asynchronous (stream-ordered) and return TG_OK or a negative TG_E*
 *    code; device-side conditions (capped Kepler iterations, a bounded wait
 *    that timed out) accumulate in a per-device status word read by
 *    tg_sync_status().
 *
 * Common rules (libtupan.h conventions): structure-of-arrays float64 inputs,
 * i-set then j-set then scalars then outputs; pair softening e2 = ie2 + je2;
 * pairs with r2 == 0 (self pairs, coincident particles) contribute nothing;
 * every output is overwritten (never accumulated); outputs must not alias
 * inputs or each other; the i- and j-sets may be the same arrays.
 * ni == 0 is a no-op; nj == 0 yields the empty-sum results.
 */
#ifndef TUPAN_GB300_H
#define TUPAN_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* precision selectors */
#define TG_PREC_FP64 0 /* IEEE double, per-pair operations in the reference's order */
#define TG_PREC_DS32 1 /* split FP32: hi/lo positions, compensated FP32 sums */
#define TG_PREC_DS32X 2 /* double-single (float-float) arithmetic on the FP32 pipes, ~1e-12:
                           Acc, AccJerk and tg_acc_vjp only (other kernels: TG_EINVAL) */

/* return codes */
#define TG_OK 0
#define TG_EINVAL (-1)   /* bad argument: null pointer, size, precision, flag */
#define TG_ECUDA (-2)    /* CUDA runtime error (see tg_last_error) */
#define TG_ENOMEM (-3)   /* workspace allocation failed */
#define TG_ENODEV (-4)   /* no CUDA device */

/* status bits returned by tg_sync_status() */
#define TG_ST_MBAR_TIMEOUT 1u   /* a bounded shared-memory pipeline wait gave up */
#define TG_ST_KEPLER_CAP 2u     /* Sakura: Kepler retry bound reached, last iterate kept */

/* ---------------------------------------------------------------------- */
/* Library state                                                           */
/* ---------------------------------------------------------------------- */
const char *tg_version(void);
/* Text of the last error seen by this thread's calls ("" if none). */
const char *tg_last_error(void);
/* Synchronise `stream` and return (then clear) the status bits raised by
 * kernels on the current device since the last call, those of
 * tg_acc_jerk_noalloc included; negative on error. */
int tg_sync_status(void *stream);
/* Precision used by the drop-in host entry points (process-wide). */
int tg_set_host_precision(int prec);
int tg_get_host_precision(void);
/* Timing of the pairwise kernel (no counterpart in the reference;
 * process-wide, off by default).  While on, split-FP32 Acc and AccJerk calls
 * that take the ordered path (2^24 pairs and more) record CUDA events on
 * their stream around their pairwise kernel; tg_pair_kernel_time waits for
 * the recorded launches of `kernel` (TG_KERNEL_ACC or TG_KERNEL_ACC_JERK)
 * and returns their total milliseconds and count, then forgets them.
 * tg_time_pair_kernel returns the previous setting. */
#define TG_KERNEL_ACC 1
#define TG_KERNEL_ACC_JERK 2
int tg_time_pair_kernel(int on);
int tg_pair_kernel_time(int kernel, double *ms, long long *launches);
/* Accuracy control of split-FP32 Acc and AccJerk calls of 2^24 pairs and
 * more (no counterpart in the reference; process-wide).  Such a call
 * recomputes in double-single arithmetic every particle whose sum of term
 * magnitudes exceeds tau times its |a| (jerk: 2.5 tau times |j|), tau
 * scaled down with sqrt(nj / 65536) below 65536 j-particles.  The default,
 * 20, holds every particle of a Plummer-Salpeter sphere within 1e-6 of
 * FP64; 10 does so on multi-cluster and six-decade-mass-range sets as
 * well, at +20% time; a flat disk of equal masses needs 5 (4x the time).   Returns the previous tau, or -1 (unchanged)
 * unless 1 <= tau <= 1e6. */
double tg_set_recompute_threshold(double tau);
/* Sakura evaluation (no counterpart in the reference; process-wide): 1, the
 * default, solves the pairs that take the universal-variable Kepler solver
 * apart from the others (flags -1 and +1, ni * nj <= 2^30; uses the grow-only
 * workspace); 0 evaluates every pair in one pass and allocates nothing.  Both
 * return the same bits.  Returns the previous setting. */
int tg_set_sakura_split(int on);
/* Streaming multiprocessors of the current device (0 if none). */
int tg_device_sms(void);
/* Measurement helper with no counterpart in the reference: dense FMA issue
 * probe on the current device, returning TFLOP/s (2 flops per FMA) for FP32
 * (which = 0, packed FFMA2), FP64 (which = 1) or packed FFMA2 interleaved
 * with scalar FFMA (which = 2); negative on error.  It is
 * the measured denominator of the pairwise kernels' FP32 roofline. */
double tg_probe_fma_tflops(int which, int iters, void *stream);
/* Failure-detection check with no counterpart in the reference: one CTA
 * waits on a shared-memory barrier with the bounded poll the split-FP32
 * kernels use for their j-tile copies (`polls` polls; the kernels use
 * 2^18, about one second), and the barrier completes only if `arrive` is nonzero.  Returns the
 * status bits the wait raised (TG_ST_MBAR_TIMEOUT if it gave up, else 0) or
 * a negative TG_E* code, and stores the kernel time in *ms.  Synchronous,
 * default stream. */
int tg_check_bounded_wait(unsigned polls, int arrive, double *ms);

/* ---------------------------------------------------------------------- */
/* Device entry points (device pointers, asynchronous on `stream`)         */
/* ---------------------------------------------------------------------- */

/* replaces phi_kernel, tupan/lib/src/libtupan.h:2-15 */
int tg_phi(size_t ni, const double *im, const double *irx, const double *iry,
           const double *irz, const double *ie2,
           size_t nj, const double *jm, const double *jrx, const double *jry,
           const double *jrz, const double *je2,
           double *iphi, int prec, void *stream);

/* replaces acc_kernel, tupan/lib/src/libtupan.h:17-32 */
int tg_acc(size_t ni, const double *im, const double *irx, const double *iry,
           const double *irz, const double *ie2,
           size_t nj, const double *jm, const double *jrx, const double *jry,
           const double *jrz, const double *je2,
           double *iax, double *iay, double *iaz, int prec, void *stream);

/* replaces acc_jerk_kernel, tupan/lib/src/libtupan.h:34-58 */
int tg_acc_jerk(size_t ni, const double *im, const double *irx, const double *iry,
                const double *irz, const double *ie2,
                const double *ivx, const double *ivy, const double *ivz,
                size_t nj, const double *jm, const double *jrx, const double *jry,
                const double *jrz, const double *je2,
                const double *jvx, const double *jvy, const double *jvz,
                double *iax, double *iay, double *iaz,
                double *ijx, double *ijy, double *ijz, int prec, void *stream);

/* replaces snap_crackle_kernel, tupan/lib/src/libtupan.h:60-96 */
int tg_snap_crackle(size_t ni, const double *im, const double *irx, const double *iry,
                    const double *irz, const double *ie2,
                    const double *ivx, const double *ivy, const double *ivz,
                    const double *iax, const double *iay, const double *iaz,
                    const double *ijx, const double *ijy, const double *ijz,
                    size_t nj, const double *jm, const double *jrx, const double *jry,
                    const double *jrz, const double *je2,
                    const double *jvx, const double *jvy, const double *jvz,
                    const double *jax, const double *jay, const double *jaz,
                    const double *jjx, const double *jjy, const double *jjz,
                    double *isx, double *isy, double *isz,
                    double *icx, double *icy, double *icz, int prec, void *stream);

/* replaces tstep_kernel, tupan/lib/src/libtupan.h:98-119 */
int tg_tstep(size_t ni, const double *im, const double *irx, const double *iry,
             const double *irz, const double *ie2,
             const double *ivx, const double *ivy, const double *ivz,
             size_t nj, const double *jm, const double *jrx, const double *jry,
             const double *jrz, const double *je2,
             const double *jvx, const double *jvy, const double *jvz,
             double eta, double *idt_a, double *idt_b, int prec, void *stream);

/* replaces pnacc_kernel, tupan/lib/src/libtupan.h:121-150 */
int tg_pnacc(size_t ni, const double *im, const double *irx, const double *iry,
             const double *irz, const double *ie2,
             const double *ivx, const double *ivy, const double *ivz,
             size_t nj, const double *jm, const double *jrx, const double *jry,
             const double *jrz, const double *je2,
             const double *jvx, const double *jvy, const double *jvz,
             unsigned long order, double inv1, double inv2, double inv3, double inv4,
             double inv5, double inv6, double inv7,
             double *ipnax, double *ipnay, double *ipnaz, int prec, void *stream);

/* replaces sakura_kernel, tupan/lib/src/libtupan.h:203-229.  Always FP64
 * (the Kepler solve needs double); prec is accepted and ignored. */
int tg_sakura(size_t ni, const double *im, const double *irx, const double *iry,
              const double *irz, const double *ie2,
              const double *ivx, const double *ivy, const double *ivz,
              size_t nj, const double *jm, const double *jrx, const double *jry,
              const double *jrz, const double *je2,
              const double *jvx, const double *jvy, const double *jvz,
              double dt, long flag,
              double *idrx, double *idry, double *idrz,
              double *idvx, double *idvy, double *idvz, int prec, void *stream);

/* replaces nreg_Xkernel, tupan/lib/src/libtupan.h:152-178.  The pair
 * separation r_ij + v_ij dt feeds imr = sum m_j r_ij, the softened
 * acceleration and iu = m_i sum m_j / r_ij.  Always FP64 (the outputs are
 * positions, not small increments); prec is checked and otherwise ignored. */
int tg_nreg_x(size_t ni, const double *im, const double *irx, const double *iry,
              const double *irz, const double *ie2,
              const double *ivx, const double *ivy, const double *ivz,
              size_t nj, const double *jm, const double *jrx, const double *jry,
              const double *jrz, const double *je2,
              const double *jvx, const double *jvy, const double *jvz,
              double dt, double *imrx, double *imry, double *imrz,
              double *iax, double *iay, double *iaz, double *iu, int prec, void *stream);

/* replaces nreg_Vkernel, tupan/lib/src/libtupan.h:180-201.  The pair
 * velocity v_ij + a_ij dt feeds imv = sum m_j v_ij and
 * ik = m_i sum m_j |v_ij|^2.  Always FP64, like tg_nreg_x. */
int tg_nreg_v(size_t ni, const double *im, const double *ivx, const double *ivy,
              const double *ivz, const double *iax, const double *iay, const double *iaz,
              size_t nj, const double *jm, const double *jvx, const double *jvy,
              const double *jvz, const double *jax, const double *jay, const double *jaz,
              double dt, double *imvx, double *imvy, double *imvz, double *ik,
              int prec, void *stream);

/* replaces kepler_solver_kernel, tupan/lib/src/libtupan.h:231-246, for
 * npairs pairs at once (the reference call is npairs = 1): pair p is
 * particles 2p and 2p+1; after dt their centre of mass has drifted freely
 * and their relative orbit follows the universal-variable Kepler solver.
 * FP64.  The outputs may alias the inputs (in-place update, as the
 * reference's callers do).  The solver's retry loops are bounded (at most
 * 1024 sub-steps per retry loop and 65536 Kepler solves per pair); a pair
 * that reaches a bound keeps its last iterate and raises
 * TG_ST_KEPLER_CAP. */
int tg_kepler_solver(size_t npairs, const double *m, const double *rx, const double *ry,
                     const double *rz, const double *e2, const double *vx, const double *vy,
                     const double *vz, double dt, double *r1x, double *r1y, double *r1z,
                     double *v1x, double *v1y, double *v1z, void *stream);

/* ---------------------------------------------------------------------- */
/* Ensembles: many independent clusters in one launch.  No counterpart in  */
/* the reference (which calls its kernels once per particle set).          */
/* Cluster k is particles [start[k], start[k] + count[k]) of the arrays     */
/* passed to the segmented calls and interacts only with itself; results   */
/* per cluster equal the single-set calls (bit for bit in FP64).  The      */
/* split-FP32 form runs all clusters' (i-tile, j-tile) units as one         */
/* stream-K launch; its first call per kernel times a few tile/grid        */
/* variants on the stream and keeps the fastest (make it before any stream */
/* capture).  Later calls are capturable in a CUDA graph.                  */
/* ---------------------------------------------------------------------- */
typedef struct tg_segments tg_segments;
/* host arrays; segments must not overlap; NULL on error (tg_last_error) */
tg_segments *tg_segments_create(size_t nseg, const long long *start, const long long *count);
void tg_segments_destroy(tg_segments *seg);
int tg_phi_segmented(tg_segments *seg, const double *m, const double *rx, const double *ry,
                     const double *rz, const double *e2, double *phi, int prec, void *stream);
int tg_acc_segmented(tg_segments *seg, const double *m, const double *rx, const double *ry,
                     const double *rz, const double *e2, double *ax, double *ay, double *az,
                     int prec, void *stream);
int tg_acc_jerk_segmented(tg_segments *seg, const double *m, const double *rx, const double *ry,
                          const double *rz, const double *e2, const double *vx, const double *vy,
                          const double *vz, double *ax, double *ay, double *az,
                          double *jx, double *jy, double *jz, int prec, void *stream);
int tg_snap_crackle_segmented(tg_segments *seg, const double *m, const double *rx, const double *ry,
                              const double *rz, const double *e2, const double *vx, const double *vy,
                              const double *vz, const double *ax, const double *ay, const double *az,
                              const double *jx, const double *jy, const double *jz,
                              double *sx, double *sy, double *sz, double *cx, double *cy, double *cz,
                              int prec, void *stream);

/* No counterpart in the reference: vector-Jacobian product of acc_kernel
 * for one particle set (i-set = j-set).  Given the upstream gradient
 * g = dL/da, returns dL/dr (rb) and dL/dm (mb):
 *   rb_k = sum_j T_kj (m_k g_j - m_j g_k),  T = s^-3/2 I - 3 s^-5/2 r r^T,
 *   mb_k = sum_j g_j . (r_k - r_j) s^-3/2,  r = r_k - r_j, s = r^2 + e2_k + e2_j.
 * Same tiling and precisions as tg_acc. */
int tg_acc_vjp(size_t n, const double *m, const double *rx, const double *ry, const double *rz,
               const double *e2, const double *gx, const double *gy, const double *gz,
               double *rbx, double *rby, double *rbz, double *mb, int prec, void *stream);

/* ---------------------------------------------------------------------- */
/* Integrator updates (device pointers, FP64, asynchronous on `stream`).   */
/* Fused forms of the reference integrators' numpy updates, evaluated in   */
/* numpy's operation order so FP64 trajectories match bit for bit.         */
/* ---------------------------------------------------------------------- */

/* *out = sum of x[0..n) in numpy's float64 order (pairwise blocks of at
 * most 128 elements with eight interleaved accumulators, halves split at
 * multiples of 8), so reductions that steer the integrators (total mass,
 * energies, the NREG integrator's U, W and K) equal numpy.sum bit for bit.
 * n == 0 stores 0.  No counterpart in the reference's C library (numpy's
 * reduction in its Python layer). */
int tg_sum(size_t n, const double *x, double *out, void *stream);

/* x = mx / d, y = my / d, z = mz / d with IEEE division (the NREG
 * integrator's r = mr / M and v = mv / M, tupan/integrator/nreg.py:27-29,
 * 50-52); the outputs may alias the inputs. */
int tg_div3(size_t n, double *x, double *y, double *z, const double *mx, const double *my,
            const double *mz, double d, void *stream);

/* r += v * tau (drift_n, tupan/integrator/sia.py:64-73) */
int tg_drift(size_t n, double *rx, double *ry, double *rz, const double *vx, const double *vy,
             const double *vz, double tau, void *stream);
/* v += a * tau (kick_n, tupan/integrator/sia.py:77-86) */
int tg_kick(size_t n, double *vx, double *vy, double *vz, const double *ax, const double *ay,
            const double *az, double tau, void *stream);
/* r += dr, v += dv (sakura_step, tupan/integrator/sakura.py:30-44) */
int tg_add_increments(size_t n, double *rx, double *ry, double *rz, double *vx, double *vy, double *vz,
                      const double *drx, const double *dry, const double *drz, const double *dvx,
                      const double *dvy, const double *dvz, void *stream);
/* Hermite predictor of order 2/4/6/8 (H2/H4/H6/H8.epredict,
 * tupan/integrator/hermite.py:24-36, 75-90, 127-157, 200-235): updates
 * rv = {rx, ry, rz, vx, vy, vz} in place from deriv = {ax, ay, az, jx, ...,
 * cz} (3 * order/2 arrays: a, then j, s, c as the order needs). */
int tg_hermite_predict(int order, size_t n, double tau, double *const *rv, const double *const *deriv,
                       void *stream);
/* Hermite corrector of order 2/4/6/8 (H2..H8.ecorrect, hermite.py:39-53,
 * 93-119, 160-196, 238-283): rv1 = corrected {r, v} from the start state
 * rv0 = {r0, v0}, its derivatives deriv0 and the derivatives deriv1 at the
 * predicted state (same layouts as tg_hermite_predict). */
int tg_hermite_correct(int order, size_t n, double tau, const double *const *rv0,
                       const double *const *deriv0, const double *const *deriv1, double *const *rv1,
                       void *stream);

/* One step of the hierarchical SIA integrators (methods sia<NM>h.kdk and
 * sia<NM>h.dkd; SIA.recurse, tupan/integrator/sia.py:1092-1123, with split,
 * join, sf_kick and FewBody, sia.py:24-57, 175-230, fewbody.py:13-57),
 * driven from native code: per time-step level one Tstep call, one stable
 * slow/fast partition whose size is read back (the call waits for the
 * stream there), the scheme's kicks, drifts and cross kicks, and Kepler
 * pair solutions for two-particle subsets.  No counterpart in the
 * reference's C library (its recursion is Python).
 *   op_kind/op_coef: the scheme's symmetric operator sequence (nops <= 64;
 *     kind 0 opens and closes it): for kdk kind 0 is a kick and kind 1 a
 *     drift, for dkd the reverse; in the slow/fast bridge kind 0 advances
 *     the slow part and recurses on the fast part, kind 1 is the cross kick.
 *   prec_acc/prec_tstep: TG_PREC_* of the Acc and Tstep calls.
 *   real: rows_real rows of n float64 values, ld_real apart; ints: rows_int
 *     rows of n int64 values, ld_int apart; row_of[TG_SIA_ROW_*] gives each
 *     attribute's row (NSTEP in ints, the others in real).  Every row is
 *     permuted with the particles: on return the blocks hold the set after
 *     the step in the reference's order (slow before fast at every level).
 *   *t_curr: the integrator's current time, advanced as the reference's
 *     recursion advances it.
 * FP64 results are bit-identical to the same recursion over the Python
 * extension calls.  Level buffers are library-owned and grow on demand;
 * calls must not overlap in time. */
#define TG_SIA_ROW_MASS 0
#define TG_SIA_ROW_EPS2 1
#define TG_SIA_ROW_RX 2
#define TG_SIA_ROW_RY 3
#define TG_SIA_ROW_RZ 4
#define TG_SIA_ROW_VX 5
#define TG_SIA_ROW_VY 6
#define TG_SIA_ROW_VZ 7
#define TG_SIA_ROW_TIME 8
#define TG_SIA_ROW_TSTEP 9
#define TG_SIA_ROW_TSTEPIJ 10
#define TG_SIA_ROW_AX 11
#define TG_SIA_ROW_AY 12
#define TG_SIA_ROW_AZ 13
#define TG_SIA_ROW_NSTEP 14
#define TG_SIA_NROWS 15
int tg_sia_h_step(int nops, const int *op_kind, const double *op_coef, int kdk, double eta, double tau,
                  int prec_acc, int prec_tstep, size_t n, double *real, size_t ld_real, int rows_real,
                  long long *ints, size_t ld_int, int rows_int, const int *row_of, double *t_curr,
                  void *stream);

/* No counterpart in the reference.  Split-FP32 AccJerk (the unordered
 * stream-K kernels that tg_acc_jerk with TG_PREC_DS32 runs for calls below
 * 2^24 pairs) for callers that cannot let a library allocate GPU memory --
 * applications whose own pool owns the GPU's memory, or loops that must not
 * stall other streams on cudaMalloc/cudaFree.  It calls no allocator: its
 * scratch is a fixed 24 MiB __device__ array that every GPU loading the
 * library holds until exit.  Limits: ni <= 2^20, nj <= 2^17 (else
 * TG_EINVAL).  The first call on a device looks up the array's address with
 * that device current; make it before any stream capture.  Calls share the
 * array, so calls that overlap on the GPU race: order them on one stream.
 * A device-side wait that gave up is reported by tg_sync_status.  Device
 * pointers, asynchronous on `stream`. */
int tg_acc_jerk_noalloc(size_t ni, const double *im, const double *irx, const double *iry,
                        const double *irz, const double *ie2,
                        const double *ivx, const double *ivy, const double *ivz,
                        size_t nj, const double *jm, const double *jrx, const double *jry,
                        const double *jrz, const double *je2,
                        const double *jvx, const double *jvy, const double *jvz,
                        double *iax, double *iay, double *iaz,
                        double *ijx, double *ijy, double *ijz, void *stream);

/* ---------------------------------------------------------------------- */
/* Drop-in host entry points: exact libtupan.h signatures (float64 build)  */
/* ---------------------------------------------------------------------- */

/* tupan/lib/src/libtupan.h:2-15 */
void phi_kernel(const unsigned long ni, const double *_im, const double *_irx,
                const double *_iry, const double *_irz, const double *_ie2,
                const unsigned long nj, const double *_jm, const double *_jrx,
                const double *_jry, const double *_jrz, const double *_je2,
                double *_iphi);
/* tupan/lib/src/libtupan.h:17-32 */
void acc_kernel(const unsigned long ni, const double *_im, const double *_irx,
                const double *_iry, const double *_irz, const double *_ie2,
                const unsigned long nj, const double *_jm, const double *_jrx,
                const double *_jry, const double *_jrz, const double *_je2,
                double *_iax, double *_iay, double *_iaz);
/* tupan/lib/src/libtupan.h:34-58 */
void acc_jerk_kernel(const unsigned long ni, const double *_im, const double *_irx,
                     const double *_iry, const double *_irz, const double *_ie2,
                     const double *_ivx, const double *_ivy, const double *_ivz,
                     const unsigned long nj, const double *_jm, const double *_jrx,
                     const double *_jry, const double *_jrz, const double *_je2,
                     const double *_jvx, const double *_jvy, const double *_jvz,
                     double *_iax, double *_iay, double *_iaz,
                     double *_ijx, double *_ijy, double *_ijz);
/* tupan/lib/src/libtupan.h:60-96 */
void snap_crackle_kernel(const unsigned long ni, const double *_im, const double *_irx,
                         const double *_iry, const double *_irz, const double *_ie2,
                         const double *_ivx, const double *_ivy, const double *_ivz,
                         const double *_iax, const double *_iay, const double *_iaz,
                         const double *_ijx, const double *_ijy, const double *_ijz,
                         const unsigned long nj, const double *_jm, const double *_jrx,
                         const double *_jry, const double *_jrz, const double *_je2,
                         const double *_jvx, const double *_jvy, const double *_jvz,
                         const double *_jax, const double *_jay, const double *_jaz,
                         const double *_jjx, const double *_jjy, const double *_jjz,
                         double *_isx, double *_isy, double *_isz,
                         double *_icx, double *_icy, double *_icz);
/* tupan/lib/src/libtupan.h:98-119 */
void tstep_kernel(const unsigned long ni, const double *_im, const double *_irx,
                  const double *_iry, const double *_irz, const double *_ie2,
                  const double *_ivx, const double *_ivy, const double *_ivz,
                  const unsigned long nj, const double *_jm, const double *_jrx,
                  const double *_jry, const double *_jrz, const double *_je2,
                  const double *_jvx, const double *_jvy, const double *_jvz,
                  const double eta, double *_idt_a, double *_idt_b);
/* tupan/lib/src/libtupan.h:121-150 */
void pnacc_kernel(const unsigned long ni, const double *_im, const double *_irx,
                  const double *_iry, const double *_irz, const double *_ie2,
                  const double *_ivx, const double *_ivy, const double *_ivz,
                  const unsigned long nj, const double *_jm, const double *_jrx,
                  const double *_jry, const double *_jrz, const double *_je2,
                  const double *_jvx, const double *_jvy, const double *_jvz,
                  unsigned long order, const double inv1, const double inv2,
                  const double inv3, const double inv4, const double inv5,
                  const double inv6, const double inv7,
                  double *_ipnax, double *_ipnay, double *_ipnaz);
/* tupan/lib/src/libtupan.h:203-229 */
void sakura_kernel(const unsigned long ni, const double *_im, const double *_irx,
                   const double *_iry, const double *_irz, const double *_ie2,
                   const double *_ivx, const double *_ivy, const double *_ivz,
                   const unsigned long nj, const double *_jm, const double *_jrx,
                   const double *_jry, const double *_jrz, const double *_je2,
                   const double *_jvx, const double *_jvy, const double *_jvz,
                   const double dt, const long flag,
                   double *_idrx, double *_idry, double *_idrz,
                   double *_idvx, double *_idvy, double *_idvz);
/* tupan/lib/src/libtupan.h:152-178 */
void nreg_Xkernel(const unsigned long ni, const double *_im, const double *_irx,
                  const double *_iry, const double *_irz, const double *_ie2,
                  const double *_ivx, const double *_ivy, const double *_ivz,
                  const unsigned long nj, const double *_jm, const double *_jrx,
                  const double *_jry, const double *_jrz, const double *_je2,
                  const double *_jvx, const double *_jvy, const double *_jvz,
                  const double dt, double *_idrx, double *_idry, double *_idrz,
                  double *_iax, double *_iay, double *_iaz, double *_iu);
/* tupan/lib/src/libtupan.h:180-201 */
void nreg_Vkernel(const unsigned long ni, const double *_im, const double *_ivx,
                  const double *_ivy, const double *_ivz, const double *_iax,
                  const double *_iay, const double *_iaz,
                  const unsigned long nj, const double *_jm, const double *_jvx,
                  const double *_jvy, const double *_jvz, const double *_jax,
                  const double *_jay, const double *_jaz,
                  const double dt, double *_idvx, double *_idvy, double *_idvz, double *_ik);

/* tupan/lib/src/libtupan.h:231-246: two particles; the outputs may alias
 * the inputs */
void kepler_solver_kernel(const double *_im, const double *_irx, const double *_iry,
                          const double *_irz, const double *_ie2, const double *_ivx,
                          const double *_ivy, const double *_ivz, const double dt,
                          double *_ir1x, double *_ir1y, double *_ir1z,
                          double *_iv1x, double *_iv1y, double *_iv1z);

#ifdef __cplusplus
}
#endif
#endif /* TUPAN_GB300_H */
