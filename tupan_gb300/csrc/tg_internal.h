// tg_internal.h -- declarations shared by the library's translation units.
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

namespace tg {

// Particle attributes in the order of tupan/particles/body.py:26-39 plus the
// derivative fields the SnapCrackle kernel reads (extensions.py:290-300).
enum Field : int {
    F_M = 0, F_RX, F_RY, F_RZ, F_E2, F_VX, F_VY, F_VZ,
    F_AX, F_AY, F_AZ, F_JX, F_JY, F_JZ, F_COUNT
};

enum Kernel : int { K_PHI = 0, K_ACC, K_ACC_JERK, K_SNAP_CRACKLE, K_TSTEP, K_PNACC, K_SAKURA,
                    K_ACC_VJP, K_NREG_X, K_NREG_V, K_COUNT };
// K_ACC_VJP reads the upstream gradient of the acceleration from the
// F_AX..F_AZ slots of the particle set and writes r-bar (3) and m-bar (1).
// K_NREG_V reads m, v and a (F_M, F_VX..F_AZ); its F_RX..F_E2 slots are
// filled with the mass pointer so the contiguous field range stays valid.

// Number of leading per-particle field slots each kernel stages
// (libtupan.h:2-246; the slots follow the Field order).
constexpr int kernel_fields(int k) {
    return k == K_PHI || k == K_ACC ? 5
         : (k == K_SNAP_CRACKLE || k == K_ACC_VJP ? 14 : (k == K_NREG_V ? 11 : 8));
}
// Number of output arrays.
constexpr int kernel_outputs(int k) {
    return k == K_PHI ? 1
         : (k == K_ACC || k == K_PNACC ? 3
         : (k == K_TSTEP ? 2 : (k == K_ACC_VJP || k == K_NREG_V ? 4 : (k == K_NREG_X ? 7 : 6))));
}
constexpr int MAX_OUTPUTS = 7;

struct PSet {
    const double *f[F_COUNT];
};

struct PairArgs {
    PSet I, J;
    size_t ni, nj;
    double *out[MAX_OUTPUTS];
    double eta;               // Tstep
    double dt;                // Sakura, NREG_X, NREG_V
    long long flag;           // Sakura
    unsigned long order;      // PNAcc
    double inv[8];            // PNAcc: inv[k] = 1/c^k
    unsigned *status;         // device status word (tg::ST_* bits)
};

// Launchers (stream-ordered, asynchronous).  Return a cudaError_t.
cudaError_t launch_fp64(int kernel, const PairArgs &a, int sms, cudaStream_t s);
// Sakura with its Kepler pairs solved apart (bit-identical to launch_fp64's
// Sakura); applies to flags -1 and +1 and ni * nj <= 2^30.  Workspace:
// sakura_split_ws_bytes(ni, nj).
bool sakura_split_applies(const PairArgs &a);
size_t sakura_split_ws_bytes(size_t ni, size_t nj);
cudaError_t launch_sakura_split(const PairArgs &a, void *ws, size_t ws_bytes, int sms, cudaStream_t s);

// Kepler pair solver: pair p = particles 2p and 2p+1 of `in` (F_M..F_VZ);
// writes r, v after dt to out[0..5] (which may alias the inputs).
cudaError_t launch_kepler_pairs(size_t npairs, const PSet &in, double dt, double *const out[6],
                                unsigned *status, cudaStream_t s);

// Split-FP32 path: packs j-records into `ws` and runs the stream-K kernel.
struct Ds32Plan {
    size_t ws_bytes;
};
size_t ds32_workspace_bytes(int kernel, size_t ni, size_t nj, int sms);
cudaError_t launch_ds32(int kernel, const PairArgs &a, void *ws, size_t ws_bytes, int sms,
                        cudaStream_t s);
bool ds32_supported(int kernel);
// TG_PREC_DS32X (double-single for every particle): Acc, AccJerk, AccVjp
bool ds32x_supported(int kernel);
size_t ds32x_workspace_bytes(int kernel, size_t nj);
cudaError_t launch_ds32x(int kernel, const PairArgs &a, void *ws, size_t ws_bytes, int sms, cudaStream_t s);

// Segmented (ensemble) geometry for one kernel's i-tile size: C clusters,
// U units, NIT i-tiles, NJT j-tiles in total; `dev` holds the device tables
// unit_off[C+1], itile_off[C+1], rec_tile_off[C+1], seg_start[C], seg_n[C].
struct SegGeometry {
    long long C, U, NIT, NJT;
    const long long *dev;
};
int ds32_tile_i(int kernel, int ipt);
int ds32_tile_j();
size_t ds32_seg_workspace_bytes(int kernel, int ipt, const SegGeometry &g, int sms, int grid_mult);
cudaError_t launch_ds32_seg(int kernel, int ipt, const PairArgs &a, const SegGeometry &g, void *ws,
                            size_t ws_bytes, int sms, int grid_mult, cudaStream_t s);
// FP64 segmented launch: block_off[C+1] (device) maps CTAs of `threads`
// threads to clusters; seg_start/seg_n as above.
cudaError_t launch_fp64_seg(int kernel, const PairArgs &a, long long C, long long nblocks, int threads,
                            const long long *block_off, const long long *seg_start, const long long *seg_n,
                            cudaStream_t s);

// Spatial ordering of the particle sets for the ordered split-FP32 Acc and
// AccJerk (tg_order.cu).  pj: sorted j position -> j index (light particles
// in Hilbert order, then the heavy ones); pi: the same for the i-set (pj
// itself when `same`); *nlight: number of light j (device).
struct OrderOut {
    const int *pi, *pj;
    const unsigned *nlight;
};
size_t order_workspace_bytes(size_t ni, size_t nj, bool same);
cudaError_t build_order(const PSet &I, size_t ni, const PSet &J, size_t nj, bool same, void *ws,
                        size_t ws_bytes, OrderOut &out, cudaStream_t s);
// Inclusive prefix sum of n ints (cub::DeviceScan) in tmp_bytes of scratch.
size_t inclusive_sum_bytes(size_t n);
cudaError_t inclusive_sum(const int *in, int *out, size_t n, void *tmp, size_t tmp_bytes, cudaStream_t s);

// Record `msg` as this thread's tg_last_error() text.
void set_last_error(const char *msg);

// Split-FP32 launch on caller-provided scratch with the grid limited to
// `max_grid` CTAs (the caller sizes its scratch for that many).
size_t ds32_workspace_bytes_capped(int kernel, size_t ni, size_t nj, int sms, long long max_grid);
cudaError_t launch_ds32_capped(int kernel, const PairArgs &a, void *ws, size_t ws_bytes, int sms,
                               long long max_grid, cudaStream_t s);
// Timing of the ordered pairwise kernel (tg_time_pair_kernel).
// Ordered split-FP32 Acc/AccJerk: a particle whose sum of term magnitudes
// (proxy) exceeds tau |a| is recomputed in double-single; returns the
// previous tau, or -1 (unchanged) unless 1 <= tau <= 1e6.
double set_recompute_threshold(double tau);
int prof_enable(int on);
cudaError_t prof_read(int kernel, double *ms, long long *launches);

// Status bits tg_acc_jerk_noalloc left on the current device (read and
// cleared; no allocation).
cudaError_t noalloc_take_status(cudaStream_t s, unsigned *bits);

}  // namespace tg
