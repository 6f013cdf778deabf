// tg_sia.cu -- the hierarchical SIA step (modes "h", tupan/integrator/sia.py)
// driven from native host code.
//
// The reference's h. step is a recursion over time-step levels
// (sia.py:1092-1123): compute every particle's pairwise time step, split the
// set into the "slow" particles whose step is above the level's step and the
// "fast" rest (sia.py:24-43), advance the slow part with the scheme, the fast
// part recursively at the scheme's sub-steps, couple them with slow<->fast
// cross kicks (sia.py:200-230), and join them again, slow first
// (sia.py:46-57).  Subsets of at most two particles go to FewBody
// (fewbody.py:13-57): a free drift for one, the Kepler pair solver for two.
// On a small cluster one step is a thousand levels of a few particles each,
// so the cost is the per-operation overhead, not the arithmetic: here every
// level is a handful of kernel launches from C++ and one host read (the
// size of the slow part, which decides the recursion), with no Python in
// between.
//
// Layout: a particle set is a view of two blocks, float64 attributes
// (rows_real rows) and int64 attributes (rows_int rows), each row n
// contiguous values, rows ld apart.  A split gathers the set's columns into
// the level's own buffer, slow particles first then fast, each in their
// input order (a stable partition); the slow part is advanced in place
// there, the fast part recursed on in place there, and the buffer is copied
// back over the input view, which is the join: the result has the
// reference's particle order.  Buffers are per recursion depth (calls at one
// depth are sequential), grow on demand and stay with the library.
//
// Arithmetic: the same kernels, in the same order with the same scalar
// arguments (c * tau as the reference forms them), as the Python recursion
// over tupan_gb300.lib.extensions, so FP64 trajectories are bit-identical to
// that path and to the reference.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/tupan_gb300.h"
#include "tg_internal.h"

namespace {

constexpr int SPLIT_THREADS = 256;
constexpr int SPLIT_ITEMS = 4;
constexpr int SPLIT_CHUNK = SPLIT_THREADS * SPLIT_ITEMS;
constexpr int SIA_MAX_OPS = 64;
constexpr int SIA_MAX_DEPTH = 512;

// slow particles (|tstep| > thr) in chunk b -> cnt[b]
__global__ void k_split_count(size_t n, const double *tstep, double thr, int *cnt) {
    __shared__ int s_w[SPLIT_THREADS / 32];
    const size_t base = (size_t)blockIdx.x * SPLIT_CHUNK;
    int c = 0;
    for (int s = 0; s < SPLIT_ITEMS; ++s) {
        const size_t p = base + (size_t)s * SPLIT_THREADS + threadIdx.x;
        if (p < n && fabs(tstep[p]) > thr) ++c;
    }
    c = __reduce_add_sync(0xffffffffu, c);
    if ((threadIdx.x & 31) == 0) s_w[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        int t = 0;
        for (int w = 0; w < SPLIT_THREADS / 32; ++w) t += s_w[w];
        cnt[blockIdx.x] = t;
    }
}

struct SplitArgs {
    size_t n;
    const double *tstep;
    double thr;
    const int *cnt;
    int nchunks;
    const double *in_real;
    size_t ld_in_real;
    int rows_real;
    const long long *in_int;
    size_t ld_in_int;
    int rows_int;
    double *out_real;      // rows x n, row stride n
    long long *out_int;
    long long *nslow;      // device: the slow count
};

// Stable partition: column p goes to (slow particles before p) if slow, else
// to nslow + (fast particles before p).
__global__ void k_split_scatter(SplitArgs a) {
    __shared__ int s_w[SPLIT_THREADS / 32];
    __shared__ long long s_pre, s_tot;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    long long pre = 0, tot = 0;
    for (int b = tid; b < a.nchunks; b += SPLIT_THREADS) {
        const long long c = a.cnt[b];
        tot += c;
        if (b < (int)blockIdx.x) pre += c;
    }
    for (int o = 16; o > 0; o >>= 1) {
        pre += __shfl_xor_sync(0xffffffffu, pre, o);
        tot += __shfl_xor_sync(0xffffffffu, tot, o);
    }
    if (tid == 0) { s_pre = 0; s_tot = 0; }
    __syncthreads();
    if (lane == 0) {
        atomicAdd(reinterpret_cast<unsigned long long *>(&s_pre), (unsigned long long)pre);
        atomicAdd(reinterpret_cast<unsigned long long *>(&s_tot), (unsigned long long)tot);
    }
    __syncthreads();
    pre = s_pre;
    tot = s_tot;
    const size_t base = (size_t)blockIdx.x * SPLIT_CHUNK;
    long long run = 0;
    for (int s = 0; s < SPLIT_ITEMS; ++s) {
        const size_t p = base + (size_t)s * SPLIT_THREADS + tid;
        const bool slow = p < a.n && fabs(a.tstep[p]) > a.thr;
        const unsigned ball = __ballot_sync(0xffffffffu, slow);
        const int lane_pre = __popc(ball & ((1u << lane) - 1u));
        if (lane == 0) s_w[warp] = __popc(ball);
        __syncthreads();
        int warp_pre = 0, sub = 0;
        for (int w = 0; w < SPLIT_THREADS / 32; ++w) {
            if (w < warp) warp_pre += s_w[w];
            sub += s_w[w];
        }
        __syncthreads();   // s_w is rewritten by the next sub-chunk
        if (p < a.n) {
            const long long slow_before = pre + run + warp_pre + lane_pre;
            const size_t dst = slow ? (size_t)slow_before : (size_t)(tot + ((long long)p - slow_before));
            for (int r = 0; r < a.rows_real; ++r) a.out_real[r * a.n + dst] = a.in_real[r * a.ld_in_real + p];
            for (int r = 0; r < a.rows_int; ++r) a.out_int[r * a.n + dst] = a.in_int[r * a.ld_in_int + p];
        }
        run += sub;
    }
    if (blockIdx.x == 0 && tid == 0) *a.nslow = tot;
}

// dst rows <- src rows (the join: a level's buffer back over its input view)
__global__ void k_copy_rows(size_t n, int rows_real, const double *src_real, size_t ld_src_real, double *dst_real,
                            size_t ld_dst_real, int rows_int, const long long *src_int, size_t ld_src_int,
                            long long *dst_int, size_t ld_dst_int) {
    const size_t total = (size_t)(rows_real + rows_int) * n;
    for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < total; q += (size_t)gridDim.x * blockDim.x) {
        const size_t r = q / n, p = q % n;
        if (r < (size_t)rows_real) dst_real[r * ld_dst_real + p] = src_real[r * ld_src_real + p];
        else {
            const size_t ri = r - rows_real;
            dst_int[ri * ld_dst_int + p] = src_int[ri * ld_src_int + p];
        }
    }
}

// tstep = tau, time += tau, nstep += 1 for the slow part (sia.py:1117-1121)
__global__ void k_advance(size_t n, double *tstep, double *time, long long *nstep, double tau) {
    const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    tstep[p] = tau;
    time[p] = __dadd_rn(time[p], tau);
    nstep[p] += 1;
}

struct View {
    double *real;
    long long *ints;
    size_t ld_real, ld_int, n;
};

View cols(const View &v, size_t off, size_t n) {
    return View{v.real + off, v.ints + off, v.ld_real, v.ld_int, n};
}

// One buffer per recursion depth: [real rows x cap][int rows x cap][chunk counts][slow count].
struct Level {
    void *p = nullptr;
    size_t cap = 0, bytes = 0;
};

struct Pool {
    std::vector<Level> levels;
    long long *host = nullptr;   // pinned: the slow count read back
    int device = -1;
};
Pool g_pool;

size_t level_bytes(size_t n, int rows_real, int rows_int) {
    const size_t chunks = (n + SPLIT_CHUNK - 1) / SPLIT_CHUNK;
    return (size_t)rows_real * n * 8 + (size_t)rows_int * n * 8 + chunks * sizeof(int) + 256;
}

struct Engine {
    int nops;
    int kind[SIA_MAX_OPS];
    double coef[SIA_MAX_OPS];
    bool kdk;
    double eta;
    int prec_acc, prec_tstep;
    int rows_real, rows_int;
    int R[TG_SIA_NROWS];
    cudaStream_t s;
    void *sp;                  // the stream as the entry points take it
    double t_curr;
    int rc = TG_OK;

    double *row(const View &v, int which) const { return v.real + (size_t)R[which] * v.ld_real; }
    long long *nstep(const View &v) const { return v.ints + (size_t)R[TG_SIA_ROW_NSTEP] * v.ld_int; }

    // an entry point's error code (its message is already set)
    bool ok(int r) {
        if (r != TG_OK && rc == TG_OK) rc = r;
        return rc == TG_OK;
    }
    bool cuda_ok(cudaError_t e, const char *what) {
        if (e != cudaSuccess) {
            if (rc == TG_OK) {
                rc = e == cudaErrorMemoryAllocation ? TG_ENOMEM : TG_ECUDA;
                tg::set_last_error(what);
            }
            return false;
        }
        return rc == TG_OK;
    }

    // the particle's fields as tg_acc / tg_tstep take them
    void acc(const View &i, const View &j) {
        if (rc != TG_OK) return;
        ok(tg_acc(i.n, row(i, TG_SIA_ROW_MASS), row(i, TG_SIA_ROW_RX), row(i, TG_SIA_ROW_RY), row(i, TG_SIA_ROW_RZ),
                  row(i, TG_SIA_ROW_EPS2), j.n, row(j, TG_SIA_ROW_MASS), row(j, TG_SIA_ROW_RX), row(j, TG_SIA_ROW_RY),
                  row(j, TG_SIA_ROW_RZ), row(j, TG_SIA_ROW_EPS2), row(i, TG_SIA_ROW_AX), row(i, TG_SIA_ROW_AY),
                  row(i, TG_SIA_ROW_AZ), prec_acc, sp));
    }
    void set_tstep(const View &v) {
        if (rc != TG_OK) return;
        ok(tg_tstep(v.n, row(v, TG_SIA_ROW_MASS), row(v, TG_SIA_ROW_RX), row(v, TG_SIA_ROW_RY), row(v, TG_SIA_ROW_RZ),
                    row(v, TG_SIA_ROW_EPS2), row(v, TG_SIA_ROW_VX), row(v, TG_SIA_ROW_VY), row(v, TG_SIA_ROW_VZ), v.n,
                    row(v, TG_SIA_ROW_MASS), row(v, TG_SIA_ROW_RX), row(v, TG_SIA_ROW_RY), row(v, TG_SIA_ROW_RZ),
                    row(v, TG_SIA_ROW_EPS2), row(v, TG_SIA_ROW_VX), row(v, TG_SIA_ROW_VY), row(v, TG_SIA_ROW_VZ),
                    eta, row(v, TG_SIA_ROW_TSTEP), row(v, TG_SIA_ROW_TSTEPIJ), prec_tstep, sp));
    }
    void drift(const View &v, double tau) {   // sia.py:61-70
        if (rc != TG_OK || !v.n) return;
        ok(tg_drift(v.n, row(v, TG_SIA_ROW_RX), row(v, TG_SIA_ROW_RY), row(v, TG_SIA_ROW_RZ), row(v, TG_SIA_ROW_VX),
                    row(v, TG_SIA_ROW_VY), row(v, TG_SIA_ROW_VZ), tau, sp));
    }
    void kick_n(const View &v, double tau) {  // sia.py:73-82
        if (rc != TG_OK || !v.n) return;
        ok(tg_kick(v.n, row(v, TG_SIA_ROW_VX), row(v, TG_SIA_ROW_VY), row(v, TG_SIA_ROW_VZ), row(v, TG_SIA_ROW_AX),
                   row(v, TG_SIA_ROW_AY), row(v, TG_SIA_ROW_AZ), tau, sp));
    }
    void kick(const View &v, double tau) {    // sia.py:175-184
        acc(v, v);
        kick_n(v, tau);
    }
    void fewbody(const View &v, double tau) { // fewbody.py:13-57
        if (rc != TG_OK || v.n == 0) return;
        if (v.n == 1) { drift(v, tau); return; }
        double *rx = row(v, TG_SIA_ROW_RX), *ry = row(v, TG_SIA_ROW_RY), *rz = row(v, TG_SIA_ROW_RZ);
        double *vx = row(v, TG_SIA_ROW_VX), *vy = row(v, TG_SIA_ROW_VY), *vz = row(v, TG_SIA_ROW_VZ);
        ok(tg_kepler_solver(1, row(v, TG_SIA_ROW_MASS), rx, ry, rz, row(v, TG_SIA_ROW_EPS2), vx, vy, vz, tau, rx,
                            ry, rz, vx, vy, vz, sp));
    }
    void evolve(const View &v, double tau) {  // Scheme.kdk / Scheme.dkd
        if (v.n <= 2) { fewbody(v, tau); return; }
        for (int q = 0; q < nops && rc == TG_OK; ++q) {
            const double c = coef[q] * tau;
            if ((kind[q] == 0) == kdk) kick(v, c);
            else drift(v, c);
        }
    }
    void sf_kick(const View &slow, const View &fast, double tau) {   // sia.py:200-230
        if (!slow.n || !fast.n) return;
        acc(slow, fast);
        acc(fast, slow);
        kick_n(slow, tau);
        kick_n(fast, tau);
    }

    Level *level(int depth, size_t n) {
        if ((int)g_pool.levels.size() <= depth) g_pool.levels.resize(depth + 1);
        Level &L = g_pool.levels[depth];
        const size_t need = level_bytes(n, rows_real, rows_int);
        if (L.bytes < need) {
            if (L.p) {
                // the old buffer may still be read by queued kernels of an
                // earlier call at this depth
                if (!cuda_ok(cudaStreamSynchronize(s), "cudaStreamSynchronize")) return nullptr;
                cudaFree(L.p);
                L.p = nullptr;
                L.bytes = L.cap = 0;
            }
            const size_t grow = need + need / 2;
            if (!cuda_ok(cudaMalloc(&L.p, grow), "cudaMalloc (SIA level buffer)")) return nullptr;
            L.bytes = grow;
        }
        L.cap = n;
        return &L;
    }

    // split(ps) into the depth's buffer; returns the slow count, or -1
    long long split(const View &v, double thr, int depth, View &out) {
        Level *L = level(depth, v.n);
        if (!L) return -1;
        char *p = static_cast<char *>(L->p);
        double *real = reinterpret_cast<double *>(p);
        long long *ints = reinterpret_cast<long long *>(p + (size_t)rows_real * v.n * 8);
        int *cnt = reinterpret_cast<int *>(p + (size_t)(rows_real + rows_int) * v.n * 8);
        const int nchunks = (int)((v.n + SPLIT_CHUNK - 1) / SPLIT_CHUNK);
        long long *dn = reinterpret_cast<long long *>(
            p + (((size_t)(rows_real + rows_int) * v.n * 8 + (size_t)nchunks * sizeof(int) + 7) / 8) * 8);
        k_split_count<<<nchunks, SPLIT_THREADS, 0, s>>>(v.n, row(v, TG_SIA_ROW_TSTEP), thr, cnt);
        SplitArgs a{v.n, row(v, TG_SIA_ROW_TSTEP), thr, cnt, nchunks, v.real, v.ld_real, rows_real, v.ints,
                    v.ld_int, rows_int, real, ints, dn};
        k_split_scatter<<<nchunks, SPLIT_THREADS, 0, s>>>(a);
        if (!cuda_ok(cudaGetLastError(), "split launch")) return -1;
        if (!cuda_ok(cudaMemcpyAsync(g_pool.host, dn, sizeof(long long), cudaMemcpyDeviceToHost, s), "split count"))
            return -1;
        if (!cuda_ok(cudaStreamSynchronize(s), "cudaStreamSynchronize")) return -1;
        out = View{real, ints, v.n, v.n, v.n};
        return *g_pool.host;
    }

    void join(const View &from, const View &to) {
        if (rc != TG_OK || !to.n) return;
        const size_t total = (size_t)(rows_real + rows_int) * to.n;
        const unsigned blocks = (unsigned)std::min<size_t>((total + 255) / 256, 4096);
        k_copy_rows<<<blocks, 256, 0, s>>>(to.n, rows_real, from.real, from.ld_real, to.real, to.ld_real, rows_int,
                                           from.ints, from.ld_int, to.ints, to.ld_int);
        cuda_ok(cudaGetLastError(), "join launch");
    }

    void advance(const View &v, double tau) {
        if (rc != TG_OK || !v.n) return;
        k_advance<<<(unsigned)((v.n + 255) / 256), 256, 0, s>>>(v.n, row(v, TG_SIA_ROW_TSTEP), row(v, TG_SIA_ROW_TIME),
                                                              nstep(v), tau);
        cuda_ok(cudaGetLastError(), "advance launch");
    }

    void recurse(const View &ps, double tau, int depth) {   // sia.py:1092-1123
        if (rc != TG_OK || !ps.n) return;
        if (depth >= SIA_MAX_DEPTH) {
            rc = TG_EINVAL;
            tg::set_last_error("hierarchical SIA: more than 512 time-step levels");
            return;
        }
        set_tstep(ps);
        View slow = ps, fast = cols(ps, 0, 0), buf{};
        const bool whole = ps.n <= 2;    // a set of at most two particles stays whole
        if (!whole) {
            const long long k = split(ps, std::fabs(tau), depth, buf);
            if (k < 0) return;
            slow = cols(buf, 0, (size_t)k);
            fast = cols(buf, (size_t)k, ps.n - (size_t)k);
        }
        for (int q = 0; q < nops && rc == TG_OK; ++q) {   // Scheme.bridge
            const double c = coef[q] * tau;
            if (kind[q] == 0) {
                evolve(slow, c);
                recurse(fast, c, depth + 1);
            } else {
                sf_kick(slow, fast, c);
            }
        }
        if (fast.n == 0) t_curr += tau;
        advance(slow, tau);
        if (!whole) join(buf, ps);
    }
};

}  // namespace

extern "C" int tg_sia_h_step(int nops, const int *op_kind, const double *op_coef, int kdk, double eta, double tau,
                             int prec_acc, int prec_tstep, size_t n, double *real, size_t ld_real, int rows_real,
                             long long *ints, size_t ld_int, int rows_int, const int *row_of, double *t_curr,
                             void *stream) {
    tg::set_last_error("");
    if (nops < 1 || nops > SIA_MAX_OPS || !op_kind || !op_coef || !row_of || !t_curr) {
        tg::set_last_error("tg_sia_h_step: bad scheme or null pointer");
        return TG_EINVAL;
    }
    for (int q = 0; q < nops; ++q)
        if (op_kind[q] != 0 && op_kind[q] != 1) {
            tg::set_last_error("tg_sia_h_step: operator kinds are 0 or 1");
            return TG_EINVAL;
        }
    if (n == 0) return TG_OK;
    if (!real || !ints || rows_real < 1 || rows_int < 1 || ld_real < n || ld_int < n) {
        tg::set_last_error("tg_sia_h_step: bad particle blocks");
        return TG_EINVAL;
    }
    for (int q = 0; q < TG_SIA_NROWS; ++q) {
        const int lim = q == TG_SIA_ROW_NSTEP ? rows_int : rows_real;
        if (row_of[q] < 0 || row_of[q] >= lim) {
            tg::set_last_error("tg_sia_h_step: attribute row out of range");
            return TG_EINVAL;
        }
    }
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) return TG_ENODEV;
    if (g_pool.device != dev) {
        // level buffers of another device are not usable here: release them
        // (with unified addressing cudaFree finds their device)
        for (Level &L : g_pool.levels)
            if (L.p) cudaFree(L.p);
        g_pool.levels.clear();
        g_pool.device = dev;
    }
    if (!g_pool.host && cudaHostAlloc(reinterpret_cast<void **>(&g_pool.host), sizeof(long long),
                                      cudaHostAllocDefault) != cudaSuccess) {
        tg::set_last_error("cudaHostAlloc");
        return TG_ENOMEM;
    }
    Engine e;
    e.nops = nops;
    for (int q = 0; q < nops; ++q) {
        e.kind[q] = op_kind[q];
        e.coef[q] = op_coef[q];
    }
    e.kdk = kdk != 0;
    e.eta = eta;
    e.prec_acc = prec_acc;
    e.prec_tstep = prec_tstep;
    e.rows_real = rows_real;
    e.rows_int = rows_int;
    std::memcpy(e.R, row_of, sizeof e.R);
    e.s = static_cast<cudaStream_t>(stream);
    e.sp = stream;
    e.t_curr = *t_curr;
    e.recurse(View{real, ints, ld_real, ld_int, n}, tau, 0);
    if (e.rc == TG_OK) *t_curr = e.t_curr;
    return e.rc;
}
