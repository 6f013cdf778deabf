// tg_api.cu -- C ABI of libtupan_gb300.so (declared in include/tupan_gb300.h).
//
// Responsibilities: argument validation, per-device context (SM count,
// workspace, status word), dispatch to the FP64 or split-FP32 launchers, and
// the drop-in host entry points with the reference's libtupan.h signatures.
#include <cstdio>
#include <cstring>
#include <atomic>
#include <mutex>
#include <algorithm>
#include <string>
#include <utility>
#include <vector>

#include "../../include/tupan_gb300.h"
#include "tg_device.cuh"
#include "tg_internal.h"

namespace {

thread_local std::string g_err;

int fail(int code, const char *what, cudaError_t e = cudaSuccess) {
    char buf[512];
    if (e != cudaSuccess)
        snprintf(buf, sizeof buf, "%s: %s (%s)", what, cudaGetErrorString(e), cudaGetErrorName(e));
    else
        snprintf(buf, sizeof buf, "%s", what);
    g_err = buf;
    return code;
}

constexpr int MAX_DEV = 64;

struct DevCtx {
    std::mutex mu;
    bool ready = false;
    int sms = 0;
    void *ws = nullptr;
    size_t ws_bytes = 0;
    unsigned *status = nullptr;   // device word, sticky until tg_sync_status
};
DevCtx g_dev[MAX_DEV];
// Sakura evaluation: 1 = Kepler pairs solved apart, 0 = one pass (tg_set_sakura_split)
std::atomic<int> g_sakura_split{1};

int current_ctx(DevCtx **out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail(TG_ENODEV, "cudaGetDevice", e);
    if (dev < 0 || dev >= MAX_DEV) return fail(TG_ENODEV, "device index out of range");
    DevCtx &c = g_dev[dev];
    std::lock_guard<std::mutex> lk(c.mu);
    if (!c.ready) {
        e = cudaDeviceGetAttribute(&c.sms, cudaDevAttrMultiProcessorCount, dev);
        if (e != cudaSuccess) return fail(TG_ECUDA, "cudaDeviceGetAttribute", e);
        e = cudaMalloc(&c.status, sizeof(unsigned));
        if (e != cudaSuccess) return fail(TG_ENOMEM, "cudaMalloc(status)", e);
        e = cudaMemset(c.status, 0, sizeof(unsigned));
        if (e != cudaSuccess) return fail(TG_ECUDA, "cudaMemset(status)", e);
        c.ready = true;
    }
    *out = &c;
    return TG_OK;
}

// Grow-only workspace.  Calls that need scratch memory serialise on the
// context mutex on the host; GPU-side, two calls on different streams that
// overlap in time must not share a device (documented in the header).
int ensure_ws(DevCtx &c, size_t bytes, cudaStream_t s) {
    if (bytes <= c.ws_bytes) return TG_OK;
    if (c.ws) {
        cudaError_t e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return fail(TG_ECUDA, "cudaStreamSynchronize", e);
        cudaFree(c.ws);
        c.ws = nullptr;
        c.ws_bytes = 0;
    }
    size_t want = bytes + bytes / 4;
    cudaError_t e = cudaMalloc(&c.ws, want);
    if (e != cudaSuccess) return fail(TG_ENOMEM, "cudaMalloc(workspace)", e);
    c.ws_bytes = want;
    return TG_OK;
}

constexpr size_t MAX_N = (size_t)1 << 31;

int run(int kernel, tg::PairArgs &a, int prec, void *stream) {
    g_err.clear();
    if (prec != TG_PREC_FP64 && prec != TG_PREC_DS32 && prec != TG_PREC_DS32X)
        return fail(TG_EINVAL, "unknown precision");
    if (prec == TG_PREC_DS32X && !tg::ds32x_supported(kernel))
        return fail(TG_EINVAL, "TG_PREC_DS32X is available for Acc, AccJerk and tg_acc_vjp only");
    if (a.ni > MAX_N || a.nj > MAX_N) return fail(TG_EINVAL, "ni or nj above 2^31");
    const int nf = tg::kernel_fields(kernel), no = tg::kernel_outputs(kernel);
    if (a.ni > 0) {
        for (int f = 0; f < nf; ++f)
            if (!a.I.f[f]) return fail(TG_EINVAL, "null i-set pointer");
        for (int o = 0; o < no; ++o)
            if (!a.out[o]) return fail(TG_EINVAL, "null output pointer");
    }
    if (a.nj > 0)
        for (int f = 0; f < nf; ++f)
            if (!a.J.f[f]) return fail(TG_EINVAL, "null j-set pointer");
    if (a.ni == 0) return TG_OK;
    DevCtx *c = nullptr;
    int rc = current_ctx(&c);
    if (rc != TG_OK) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    a.status = c->status;
    cudaError_t e;
    if (kernel == tg::K_SAKURA && g_sakura_split.load() && tg::sakura_split_applies(a)) {
        // FP64 whatever `prec` asks; the Kepler pairs are solved apart
        std::lock_guard<std::mutex> lk(c->mu);
        rc = ensure_ws(*c, tg::sakura_split_ws_bytes(a.ni, a.nj), s);
        if (rc != TG_OK) return rc;
        e = tg::launch_sakura_split(a, c->ws, c->ws_bytes, c->sms, s);
    } else if (prec == TG_PREC_FP64 || !tg::ds32_supported(kernel) || a.nj == 0) {
        e = tg::launch_fp64(kernel, a, c->sms, s);
    } else if (prec == TG_PREC_DS32X) {
        std::lock_guard<std::mutex> lk(c->mu);
        rc = ensure_ws(*c, tg::ds32x_workspace_bytes(kernel, a.nj), s);
        if (rc != TG_OK) return rc;
        e = tg::launch_ds32x(kernel, a, c->ws, c->ws_bytes, c->sms, s);
    } else {
        std::lock_guard<std::mutex> lk(c->mu);
        const size_t need = tg::ds32_workspace_bytes(kernel, a.ni, a.nj, c->sms);
        rc = ensure_ws(*c, need, s);
        if (rc != TG_OK) return rc;
        e = tg::launch_ds32(kernel, a, c->ws, c->ws_bytes, c->sms, s);
    }
    if (e != cudaSuccess) return fail(TG_ECUDA, "kernel launch", e);
    return TG_OK;
}

void set5(tg::PSet &p, const double *m, const double *x, const double *y, const double *z,
          const double *e) {
    std::memset(&p, 0, sizeof p);
    p.f[tg::F_M] = m; p.f[tg::F_RX] = x; p.f[tg::F_RY] = y; p.f[tg::F_RZ] = z; p.f[tg::F_E2] = e;
}
void setv(tg::PSet &p, const double *u, const double *v, const double *w) {
    p.f[tg::F_VX] = u; p.f[tg::F_VY] = v; p.f[tg::F_VZ] = w;
}
tg::PairArgs blank() {
    tg::PairArgs a;
    std::memset(&a, 0, sizeof a);
    return a;
}

int g_host_prec = TG_PREC_FP64;

// ---------------------------------------------------------------------------
// Host staging for the drop-in entry points: one library stream and cached
// device buffers per device.
// ---------------------------------------------------------------------------
struct HostStage {
    std::mutex mu;
    cudaStream_t stream = nullptr;
    double *buf = nullptr;
    size_t cap = 0;   // doubles
};
HostStage g_stage[MAX_DEV];

struct HostCall {
    int nf;                 // input arrays per set, in the launch lambda's order
    int no;                 // output arrays
    size_t ni, nj;
    const double *in_i[14];
    const double *in_j[14];
    double *out[tg::MAX_OUTPUTS];
};

// Copies the host arrays in, runs `launch` on device copies, copies out.
template <class F>
void host_call(const HostCall &h, F launch) {
    g_err.clear();
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= MAX_DEV) {
        fail(TG_ENODEV, "no CUDA device for host entry point");
        fprintf(stderr, "tupan_gb300: %s\n", g_err.c_str());
        return;
    }
    HostStage &st = g_stage[dev];
    std::lock_guard<std::mutex> lk(st.mu);
    const int nf = h.nf, no = h.no;
    const size_t need = (size_t)nf * (h.ni + h.nj) + (size_t)no * h.ni + 8;
    cudaError_t e = cudaSuccess;
    if (!st.stream) e = cudaStreamCreateWithFlags(&st.stream, cudaStreamNonBlocking);
    if (e == cudaSuccess && need > st.cap) {
        if (st.buf) cudaFree(st.buf);
        st.buf = nullptr;
        st.cap = 0;
        e = cudaMalloc(&st.buf, need * sizeof(double));
        if (e == cudaSuccess) st.cap = need;
    }
    if (e != cudaSuccess) {
        fail(TG_ECUDA, "host entry point staging", e);
        fprintf(stderr, "tupan_gb300: %s\n", g_err.c_str());
        return;
    }
    double *p = st.buf;
    const double *di[14] = {}, *dj[14] = {};
    double *dout[tg::MAX_OUTPUTS] = {};
    for (int f = 0; f < nf && e == cudaSuccess; ++f) {
        if (h.ni) e = cudaMemcpyAsync(p, h.in_i[f], h.ni * sizeof(double), cudaMemcpyHostToDevice, st.stream);
        di[f] = p; p += h.ni;
    }
    for (int f = 0; f < nf && e == cudaSuccess; ++f) {
        if (h.nj == h.ni && h.in_j[f] == h.in_i[f]) {   // the same host array: one copy serves both
            dj[f] = di[f];
            continue;
        }
        if (h.nj) e = cudaMemcpyAsync(p, h.in_j[f], h.nj * sizeof(double), cudaMemcpyHostToDevice, st.stream);
        dj[f] = p; p += h.nj;
    }
    for (int o = 0; o < no; ++o) { dout[o] = p; p += h.ni; }
    int rc = (e == cudaSuccess) ? launch(di, dj, dout, st.stream) : TG_ECUDA;
    for (int o = 0; o < no && rc == TG_OK && e == cudaSuccess; ++o)
        if (h.ni) e = cudaMemcpyAsync(h.out[o], dout[o], h.ni * sizeof(double), cudaMemcpyDeviceToHost, st.stream);
    cudaError_t se = cudaStreamSynchronize(st.stream);
    if (e == cudaSuccess) e = se;
    if (rc != TG_OK || e != cudaSuccess) {
        if (e != cudaSuccess) fail(TG_ECUDA, "host entry point", e);
        fprintf(stderr, "tupan_gb300: %s\n", g_err.c_str());
    }
}

}  // namespace

namespace tg {
void set_last_error(const char *msg) { g_err = msg; }
}  // namespace tg

extern "C" {

const char *tg_version(void) { return "tupan_gb300 0.1.0 (sm_103a)"; }
const char *tg_last_error(void) { return g_err.c_str(); }

int tg_device_sms(void) {
    DevCtx *c = nullptr;
    if (current_ctx(&c) != TG_OK) return 0;
    return c->sms;
}

int tg_sync_status(void *stream) {
    DevCtx *c = nullptr;
    int rc = current_ctx(&c);
    if (rc != TG_OK) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    unsigned h = 0, na = 0;
    cudaError_t e = cudaMemcpyAsync(&h, c->status, sizeof h, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e == cudaSuccess) e = cudaMemsetAsync(c->status, 0, sizeof(unsigned), s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    // and the bits tg_acc_jerk_noalloc keeps in its own scratch
    if (e == cudaSuccess) e = tg::noalloc_take_status(s, &na);
    if (e != cudaSuccess) return fail(TG_ECUDA, "tg_sync_status", e);
    return (int)(h | na);
}

int tg_set_host_precision(int prec) {
    if (prec != TG_PREC_FP64 && prec != TG_PREC_DS32) return fail(TG_EINVAL, "unknown precision");
    g_host_prec = prec;
    return TG_OK;
}
int tg_get_host_precision(void) { return g_host_prec; }

int tg_set_sakura_split(int on) { return g_sakura_split.exchange(on ? 1 : 0); }

int tg_time_pair_kernel(int on) { return tg::prof_enable(on); }

double tg_set_recompute_threshold(double tau) { return tg::set_recompute_threshold(tau); }

int tg_pair_kernel_time(int kernel, double *ms, long long *launches) {
    if (!ms || !launches || (kernel != TG_KERNEL_ACC && kernel != TG_KERNEL_ACC_JERK))
        return fail(TG_EINVAL, "tg_pair_kernel_time: kernel must be TG_KERNEL_ACC or TG_KERNEL_ACC_JERK");
    cudaError_t e = tg::prof_read(kernel == TG_KERNEL_ACC ? tg::K_ACC : tg::K_ACC_JERK, ms, launches);
    if (e != cudaSuccess) return fail(TG_ECUDA, "tg_pair_kernel_time", e);
    return TG_OK;
}

int tg_phi(size_t ni, const double *im, const double *irx, const double *iry, const double *irz,
           const double *ie2, size_t nj, const double *jm, const double *jrx, const double *jry,
           const double *jrz, const double *je2, double *iphi, int prec, void *stream) {
    tg::PairArgs a = blank();
    set5(a.I, im, irx, iry, irz, ie2);
    set5(a.J, jm, jrx, jry, jrz, je2);
    a.ni = ni; a.nj = nj; a.out[0] = iphi;
    return run(tg::K_PHI, a, prec, stream);
}

int tg_acc(size_t ni, const double *im, const double *irx, const double *iry, const double *irz,
           const double *ie2, size_t nj, const double *jm, const double *jrx, const double *jry,
           const double *jrz, const double *je2, double *iax, double *iay, double *iaz, int prec,
           void *stream) {
    tg::PairArgs a = blank();
    set5(a.I, im, irx, iry, irz, ie2);
    set5(a.J, jm, jrx, jry, jrz, je2);
    a.ni = ni; a.nj = nj; a.out[0] = iax; a.out[1] = iay; a.out[2] = iaz;
    return run(tg::K_ACC, a, prec, stream);
}

int tg_acc_jerk(size_t ni, const double *im, const double *irx, const double *iry,
                const double *irz, const double *ie2, const double *ivx, const double *ivy,
                const double *ivz, size_t nj, const double *jm, const double *jrx,
                const double *jry, const double *jrz, const double *je2, const double *jvx,
                const double *jvy, const double *jvz, double *iax, double *iay, double *iaz,
                double *ijx, double *ijy, double *ijz, int prec, void *stream) {
    tg::PairArgs a = blank();
    set5(a.I, im, irx, iry, irz, ie2); setv(a.I, ivx, ivy, ivz);
    set5(a.J, jm, jrx, jry, jrz, je2); setv(a.J, jvx, jvy, jvz);
    a.ni = ni; a.nj = nj;
    a.out[0] = iax; a.out[1] = iay; a.out[2] = iaz; a.out[3] = ijx; a.out[4] = ijy; a.out[5] = ijz;
    return run(tg::K_ACC_JERK, a, prec, stream);
}

int tg_snap_crackle(size_t ni, const double *im, const double *irx, const double *iry,
                    const double *irz, const double *ie2, const double *ivx, const double *ivy,
                    const double *ivz, const double *iax, const double *iay, const double *iaz,
                    const double *ijx, const double *ijy, const double *ijz, size_t nj,
                    const double *jm, const double *jrx, const double *jry, const double *jrz,
                    const double *je2, const double *jvx, const double *jvy, const double *jvz,
                    const double *jax, const double *jay, const double *jaz, const double *jjx,
                    const double *jjy, const double *jjz, double *isx, double *isy, double *isz,
                    double *icx, double *icy, double *icz, int prec, void *stream) {
    tg::PairArgs a = blank();
    set5(a.I, im, irx, iry, irz, ie2); setv(a.I, ivx, ivy, ivz);
    a.I.f[tg::F_AX] = iax; a.I.f[tg::F_AY] = iay; a.I.f[tg::F_AZ] = iaz;
    a.I.f[tg::F_JX] = ijx; a.I.f[tg::F_JY] = ijy; a.I.f[tg::F_JZ] = ijz;
    set5(a.J, jm, jrx, jry, jrz, je2); setv(a.J, jvx, jvy, jvz);
    a.J.f[tg::F_AX] = jax; a.J.f[tg::F_AY] = jay; a.J.f[tg::F_AZ] = jaz;
    a.J.f[tg::F_JX] = jjx; a.J.f[tg::F_JY] = jjy; a.J.f[tg::F_JZ] = jjz;
    a.ni = ni; a.nj = nj;
    a.out[0] = isx; a.out[1] = isy; a.out[2] = isz; a.out[3] = icx; a.out[4] = icy; a.out[5] = icz;
    return run(tg::K_SNAP_CRACKLE, a, prec, stream);
}

int tg_tstep(size_t ni, const double *im, const double *irx, const double *iry, const double *irz,
             const double *ie2, const double *ivx, const double *ivy, const double *ivz, size_t nj,
             const double *jm, const double *jrx, const double *jry, const double *jrz,
             const double *je2, const double *jvx, const double *jvy, const double *jvz,
             double eta, double *idt_a, double *idt_b, int prec, void *stream) {
    tg::PairArgs a = blank();
    set5(a.I, im, irx, iry, irz, ie2); setv(a.I, ivx, ivy, ivz);
    set5(a.J, jm, jrx, jry, jrz, je2); setv(a.J, jvx, jvy, jvz);
    a.ni = ni; a.nj = nj; a.eta = eta; a.out[0] = idt_a; a.out[1] = idt_b;
    return run(tg::K_TSTEP, a, prec, stream);
}

int tg_pnacc(size_t ni, const double *im, const double *irx, const double *iry, const double *irz,
             const double *ie2, const double *ivx, const double *ivy, const double *ivz, size_t nj,
             const double *jm, const double *jrx, const double *jry, const double *jrz,
             const double *je2, const double *jvx, const double *jvy, const double *jvz,
             unsigned long order, double inv1, double inv2, double inv3, double inv4, double inv5,
             double inv6, double inv7, double *ipnax, double *ipnay, double *ipnaz, int prec,
             void *stream) {
    tg::PairArgs a = blank();
    set5(a.I, im, irx, iry, irz, ie2); setv(a.I, ivx, ivy, ivz);
    set5(a.J, jm, jrx, jry, jrz, je2); setv(a.J, jvx, jvy, jvz);
    a.ni = ni; a.nj = nj; a.order = order;
    a.inv[1] = inv1; a.inv[2] = inv2; a.inv[3] = inv3; a.inv[4] = inv4;
    a.inv[5] = inv5; a.inv[6] = inv6; a.inv[7] = inv7;
    a.out[0] = ipnax; a.out[1] = ipnay; a.out[2] = ipnaz;
    return run(tg::K_PNACC, a, prec, stream);
}

int tg_sakura(size_t ni, const double *im, const double *irx, const double *iry, const double *irz,
              const double *ie2, const double *ivx, const double *ivy, const double *ivz, size_t nj,
              const double *jm, const double *jrx, const double *jry, const double *jrz,
              const double *je2, const double *jvx, const double *jvy, const double *jvz, double dt,
              long flag, double *idrx, double *idry, double *idrz, double *idvx, double *idvy,
              double *idvz, int prec, void *stream) {
    tg::PairArgs a = blank();
    set5(a.I, im, irx, iry, irz, ie2); setv(a.I, ivx, ivy, ivz);
    set5(a.J, jm, jrx, jry, jrz, je2); setv(a.J, jvx, jvy, jvz);
    a.ni = ni; a.nj = nj; a.dt = dt; a.flag = flag;
    a.out[0] = idrx; a.out[1] = idry; a.out[2] = idrz; a.out[3] = idvx; a.out[4] = idvy; a.out[5] = idvz;
    (void)prec;
    return run(tg::K_SAKURA, a, TG_PREC_FP64, stream);
}

int tg_acc_vjp(size_t n, const double *m, const double *rx, const double *ry, const double *rz,
               const double *e2, const double *gx, const double *gy, const double *gz, double *rbx,
               double *rby, double *rbz, double *mb, int prec, void *stream) {
    tg::PairArgs a = blank();
    set5(a.I, m, rx, ry, rz, e2);
    // every field slot the kernel family validates must be non-null
    setv(a.I, rx, ry, rz);
    a.I.f[tg::F_AX] = gx; a.I.f[tg::F_AY] = gy; a.I.f[tg::F_AZ] = gz;
    a.I.f[tg::F_JX] = gx; a.I.f[tg::F_JY] = gy; a.I.f[tg::F_JZ] = gz;
    a.J = a.I;
    a.ni = n; a.nj = n;
    a.out[0] = rbx; a.out[1] = rby; a.out[2] = rbz; a.out[3] = mb;
    return run(tg::K_ACC_VJP, a, prec, stream);
}

int tg_nreg_x(size_t ni, const double *im, const double *irx, const double *iry, const double *irz,
              const double *ie2, const double *ivx, const double *ivy, const double *ivz, size_t nj,
              const double *jm, const double *jrx, const double *jry, const double *jrz,
              const double *je2, const double *jvx, const double *jvy, const double *jvz, double dt,
              double *imrx, double *imry, double *imrz, double *iax, double *iay, double *iaz,
              double *iu, int prec, void *stream) {
    tg::PairArgs a = blank();
    set5(a.I, im, irx, iry, irz, ie2); setv(a.I, ivx, ivy, ivz);
    set5(a.J, jm, jrx, jry, jrz, je2); setv(a.J, jvx, jvy, jvz);
    a.ni = ni; a.nj = nj; a.dt = dt;
    a.out[0] = imrx; a.out[1] = imry; a.out[2] = imrz;
    a.out[3] = iax; a.out[4] = iay; a.out[5] = iaz; a.out[6] = iu;
    if (prec != TG_PREC_FP64 && prec != TG_PREC_DS32) return fail(TG_EINVAL, "unknown precision");
    return run(tg::K_NREG_X, a, TG_PREC_FP64, stream);
}

int tg_nreg_v(size_t ni, const double *im, const double *ivx, const double *ivy, const double *ivz,
              const double *iax, const double *iay, const double *iaz, size_t nj, const double *jm,
              const double *jvx, const double *jvy, const double *jvz, const double *jax,
              const double *jay, const double *jaz, double dt, double *imvx, double *imvy,
              double *imvz, double *ik, int prec, void *stream) {
    tg::PairArgs a = blank();
    // slots F_RX..F_E2 carry the mass pointer (staged, never read)
    set5(a.I, im, im, im, im, im); setv(a.I, ivx, ivy, ivz);
    a.I.f[tg::F_AX] = iax; a.I.f[tg::F_AY] = iay; a.I.f[tg::F_AZ] = iaz;
    set5(a.J, jm, jm, jm, jm, jm); setv(a.J, jvx, jvy, jvz);
    a.J.f[tg::F_AX] = jax; a.J.f[tg::F_AY] = jay; a.J.f[tg::F_AZ] = jaz;
    a.ni = ni; a.nj = nj; a.dt = dt;
    a.out[0] = imvx; a.out[1] = imvy; a.out[2] = imvz; a.out[3] = ik;
    if (prec != TG_PREC_FP64 && prec != TG_PREC_DS32) return fail(TG_EINVAL, "unknown precision");
    return run(tg::K_NREG_V, a, TG_PREC_FP64, stream);
}

int tg_kepler_solver(size_t npairs, const double *m, const double *rx, const double *ry,
                     const double *rz, const double *e2, const double *vx, const double *vy,
                     const double *vz, double dt, double *r1x, double *r1y, double *r1z, double *v1x,
                     double *v1y, double *v1z, void *stream) {
    g_err.clear();
    if (npairs > MAX_N / 2) return fail(TG_EINVAL, "npairs above 2^30");
    if (npairs == 0) return TG_OK;
    const double *in[8] = {m, rx, ry, rz, e2, vx, vy, vz};
    double *out[6] = {r1x, r1y, r1z, v1x, v1y, v1z};
    for (const double *p : in)
        if (!p) return fail(TG_EINVAL, "null input pointer");
    for (double *p : out)
        if (!p) return fail(TG_EINVAL, "null output pointer");
    DevCtx *c = nullptr;
    int rc = current_ctx(&c);
    if (rc != TG_OK) return rc;
    tg::PSet ps;
    std::memset(&ps, 0, sizeof ps);
    for (int f = 0; f < 8; ++f) ps.f[f] = in[f];
    cudaError_t e = tg::launch_kepler_pairs(npairs, ps, dt, out, c->status, static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return fail(TG_ECUDA, "kernel launch", e);
    return TG_OK;
}

// ---------------------------------------------------------------------------
// Drop-in host entry points (libtupan.h signatures).
// ---------------------------------------------------------------------------
#define HC_BEGIN(K, NI, NJ)                        \
    HostCall h;                                    \
    std::memset(&h, 0, sizeof h);                  \
    h.nf = tg::kernel_fields(K); h.no = tg::kernel_outputs(K); h.ni = (NI); h.nj = (NJ);
#define I5(m, x, y, z, e) h.in_i[0] = m; h.in_i[1] = x; h.in_i[2] = y; h.in_i[3] = z; h.in_i[4] = e;
#define J5(m, x, y, z, e) h.in_j[0] = m; h.in_j[1] = x; h.in_j[2] = y; h.in_j[3] = z; h.in_j[4] = e;
#define IV(u, v, w) h.in_i[5] = u; h.in_i[6] = v; h.in_i[7] = w;
#define JV(u, v, w) h.in_j[5] = u; h.in_j[6] = v; h.in_j[7] = w;

void phi_kernel(const unsigned long ni, const double *_im, const double *_irx, const double *_iry,
                const double *_irz, const double *_ie2, const unsigned long nj, const double *_jm,
                const double *_jrx, const double *_jry, const double *_jrz, const double *_je2,
                double *_iphi) {
    HC_BEGIN(tg::K_PHI, ni, nj)
    I5(_im, _irx, _iry, _irz, _ie2) J5(_jm, _jrx, _jry, _jrz, _je2)
    h.out[0] = _iphi;
    host_call(h, [&](const double **i, const double **j, double **o, cudaStream_t s) {
        return tg_phi(ni, i[0], i[1], i[2], i[3], i[4], nj, j[0], j[1], j[2], j[3], j[4], o[0],
                      g_host_prec, s);
    });
}

void acc_kernel(const unsigned long ni, const double *_im, const double *_irx, const double *_iry,
                const double *_irz, const double *_ie2, const unsigned long nj, const double *_jm,
                const double *_jrx, const double *_jry, const double *_jrz, const double *_je2,
                double *_iax, double *_iay, double *_iaz) {
    HC_BEGIN(tg::K_ACC, ni, nj)
    I5(_im, _irx, _iry, _irz, _ie2) J5(_jm, _jrx, _jry, _jrz, _je2)
    h.out[0] = _iax; h.out[1] = _iay; h.out[2] = _iaz;
    host_call(h, [&](const double **i, const double **j, double **o, cudaStream_t s) {
        return tg_acc(ni, i[0], i[1], i[2], i[3], i[4], nj, j[0], j[1], j[2], j[3], j[4], o[0],
                      o[1], o[2], g_host_prec, s);
    });
}

void acc_jerk_kernel(const unsigned long ni, const double *_im, const double *_irx,
                     const double *_iry, const double *_irz, const double *_ie2,
                     const double *_ivx, const double *_ivy, const double *_ivz,
                     const unsigned long nj, const double *_jm, const double *_jrx,
                     const double *_jry, const double *_jrz, const double *_je2,
                     const double *_jvx, const double *_jvy, const double *_jvz, double *_iax,
                     double *_iay, double *_iaz, double *_ijx, double *_ijy, double *_ijz) {
    HC_BEGIN(tg::K_ACC_JERK, ni, nj)
    I5(_im, _irx, _iry, _irz, _ie2) IV(_ivx, _ivy, _ivz)
    J5(_jm, _jrx, _jry, _jrz, _je2) JV(_jvx, _jvy, _jvz)
    h.out[0] = _iax; h.out[1] = _iay; h.out[2] = _iaz; h.out[3] = _ijx; h.out[4] = _ijy; h.out[5] = _ijz;
    host_call(h, [&](const double **i, const double **j, double **o, cudaStream_t s) {
        return tg_acc_jerk(ni, i[0], i[1], i[2], i[3], i[4], i[5], i[6], i[7], nj, j[0], j[1], j[2],
                           j[3], j[4], j[5], j[6], j[7], o[0], o[1], o[2], o[3], o[4], o[5],
                           g_host_prec, s);
    });
}

void snap_crackle_kernel(const unsigned long ni, const double *_im, const double *_irx,
                         const double *_iry, const double *_irz, const double *_ie2,
                         const double *_ivx, const double *_ivy, const double *_ivz,
                         const double *_iax, const double *_iay, const double *_iaz,
                         const double *_ijx, const double *_ijy, const double *_ijz,
                         const unsigned long nj, const double *_jm, const double *_jrx,
                         const double *_jry, const double *_jrz, const double *_je2,
                         const double *_jvx, const double *_jvy, const double *_jvz,
                         const double *_jax, const double *_jay, const double *_jaz,
                         const double *_jjx, const double *_jjy, const double *_jjz, double *_isx,
                         double *_isy, double *_isz, double *_icx, double *_icy, double *_icz) {
    HC_BEGIN(tg::K_SNAP_CRACKLE, ni, nj)
    I5(_im, _irx, _iry, _irz, _ie2) IV(_ivx, _ivy, _ivz)
    J5(_jm, _jrx, _jry, _jrz, _je2) JV(_jvx, _jvy, _jvz)
    h.in_i[8] = _iax; h.in_i[9] = _iay; h.in_i[10] = _iaz;
    h.in_i[11] = _ijx; h.in_i[12] = _ijy; h.in_i[13] = _ijz;
    h.in_j[8] = _jax; h.in_j[9] = _jay; h.in_j[10] = _jaz;
    h.in_j[11] = _jjx; h.in_j[12] = _jjy; h.in_j[13] = _jjz;
    h.out[0] = _isx; h.out[1] = _isy; h.out[2] = _isz; h.out[3] = _icx; h.out[4] = _icy; h.out[5] = _icz;
    host_call(h, [&](const double **i, const double **j, double **o, cudaStream_t s) {
        return tg_snap_crackle(ni, i[0], i[1], i[2], i[3], i[4], i[5], i[6], i[7], i[8], i[9], i[10],
                               i[11], i[12], i[13], nj, j[0], j[1], j[2], j[3], j[4], j[5], j[6],
                               j[7], j[8], j[9], j[10], j[11], j[12], j[13], o[0], o[1], o[2], o[3],
                               o[4], o[5], g_host_prec, s);
    });
}

void tstep_kernel(const unsigned long ni, const double *_im, const double *_irx, const double *_iry,
                  const double *_irz, const double *_ie2, const double *_ivx, const double *_ivy,
                  const double *_ivz, const unsigned long nj, const double *_jm,
                  const double *_jrx, const double *_jry, const double *_jrz, const double *_je2,
                  const double *_jvx, const double *_jvy, const double *_jvz, const double eta,
                  double *_idt_a, double *_idt_b) {
    HC_BEGIN(tg::K_TSTEP, ni, nj)
    I5(_im, _irx, _iry, _irz, _ie2) IV(_ivx, _ivy, _ivz)
    J5(_jm, _jrx, _jry, _jrz, _je2) JV(_jvx, _jvy, _jvz)
    h.out[0] = _idt_a; h.out[1] = _idt_b;
    host_call(h, [&](const double **i, const double **j, double **o, cudaStream_t s) {
        return tg_tstep(ni, i[0], i[1], i[2], i[3], i[4], i[5], i[6], i[7], nj, j[0], j[1], j[2],
                        j[3], j[4], j[5], j[6], j[7], eta, o[0], o[1], g_host_prec, s);
    });
}

void pnacc_kernel(const unsigned long ni, const double *_im, const double *_irx, const double *_iry,
                  const double *_irz, const double *_ie2, const double *_ivx, const double *_ivy,
                  const double *_ivz, const unsigned long nj, const double *_jm,
                  const double *_jrx, const double *_jry, const double *_jrz, const double *_je2,
                  const double *_jvx, const double *_jvy, const double *_jvz, unsigned long order,
                  const double inv1, const double inv2, const double inv3, const double inv4,
                  const double inv5, const double inv6, const double inv7, double *_ipnax,
                  double *_ipnay, double *_ipnaz) {
    HC_BEGIN(tg::K_PNACC, ni, nj)
    I5(_im, _irx, _iry, _irz, _ie2) IV(_ivx, _ivy, _ivz)
    J5(_jm, _jrx, _jry, _jrz, _je2) JV(_jvx, _jvy, _jvz)
    h.out[0] = _ipnax; h.out[1] = _ipnay; h.out[2] = _ipnaz;
    host_call(h, [&](const double **i, const double **j, double **o, cudaStream_t s) {
        return tg_pnacc(ni, i[0], i[1], i[2], i[3], i[4], i[5], i[6], i[7], nj, j[0], j[1], j[2],
                        j[3], j[4], j[5], j[6], j[7], order, inv1, inv2, inv3, inv4, inv5, inv6,
                        inv7, o[0], o[1], o[2], g_host_prec, s);
    });
}

void sakura_kernel(const unsigned long ni, const double *_im, const double *_irx, const double *_iry,
                   const double *_irz, const double *_ie2, const double *_ivx, const double *_ivy,
                   const double *_ivz, const unsigned long nj, const double *_jm,
                   const double *_jrx, const double *_jry, const double *_jrz, const double *_je2,
                   const double *_jvx, const double *_jvy, const double *_jvz, const double dt,
                   const long flag, double *_idrx, double *_idry, double *_idrz, double *_idvx,
                   double *_idvy, double *_idvz) {
    HC_BEGIN(tg::K_SAKURA, ni, nj)
    I5(_im, _irx, _iry, _irz, _ie2) IV(_ivx, _ivy, _ivz)
    J5(_jm, _jrx, _jry, _jrz, _je2) JV(_jvx, _jvy, _jvz)
    h.out[0] = _idrx; h.out[1] = _idry; h.out[2] = _idrz; h.out[3] = _idvx; h.out[4] = _idvy; h.out[5] = _idvz;
    host_call(h, [&](const double **i, const double **j, double **o, cudaStream_t s) {
        return tg_sakura(ni, i[0], i[1], i[2], i[3], i[4], i[5], i[6], i[7], nj, j[0], j[1], j[2],
                         j[3], j[4], j[5], j[6], j[7], dt, flag, o[0], o[1], o[2], o[3], o[4], o[5],
                         TG_PREC_FP64, s);
    });
}

void nreg_Xkernel(const unsigned long ni, const double *_im, const double *_irx, const double *_iry,
                  const double *_irz, const double *_ie2, const double *_ivx, const double *_ivy,
                  const double *_ivz, const unsigned long nj, const double *_jm, const double *_jrx,
                  const double *_jry, const double *_jrz, const double *_je2, const double *_jvx,
                  const double *_jvy, const double *_jvz, const double dt, double *_idrx,
                  double *_idry, double *_idrz, double *_iax, double *_iay, double *_iaz,
                  double *_iu) {
    HC_BEGIN(tg::K_NREG_X, ni, nj)
    I5(_im, _irx, _iry, _irz, _ie2) IV(_ivx, _ivy, _ivz)
    J5(_jm, _jrx, _jry, _jrz, _je2) JV(_jvx, _jvy, _jvz)
    h.out[0] = _idrx; h.out[1] = _idry; h.out[2] = _idrz;
    h.out[3] = _iax; h.out[4] = _iay; h.out[5] = _iaz; h.out[6] = _iu;
    host_call(h, [&](const double **i, const double **j, double **o, cudaStream_t s) {
        return tg_nreg_x(ni, i[0], i[1], i[2], i[3], i[4], i[5], i[6], i[7], nj, j[0], j[1], j[2],
                         j[3], j[4], j[5], j[6], j[7], dt, o[0], o[1], o[2], o[3], o[4], o[5], o[6],
                         TG_PREC_FP64, s);
    });
}

void nreg_Vkernel(const unsigned long ni, const double *_im, const double *_ivx, const double *_ivy,
                  const double *_ivz, const double *_iax, const double *_iay, const double *_iaz,
                  const unsigned long nj, const double *_jm, const double *_jvx, const double *_jvy,
                  const double *_jvz, const double *_jax, const double *_jay, const double *_jaz,
                  const double dt, double *_idvx, double *_idvy, double *_idvz, double *_ik) {
    HC_BEGIN(tg::K_NREG_V, ni, nj)
    h.nf = 7;   // m, vx, vy, vz, ax, ay, az
    const double *ii[7] = {_im, _ivx, _ivy, _ivz, _iax, _iay, _iaz};
    const double *jj[7] = {_jm, _jvx, _jvy, _jvz, _jax, _jay, _jaz};
    for (int f = 0; f < 7; ++f) { h.in_i[f] = ii[f]; h.in_j[f] = jj[f]; }
    h.out[0] = _idvx; h.out[1] = _idvy; h.out[2] = _idvz; h.out[3] = _ik;
    host_call(h, [&](const double **i, const double **j, double **o, cudaStream_t s) {
        return tg_nreg_v(ni, i[0], i[1], i[2], i[3], i[4], i[5], i[6], nj, j[0], j[1], j[2], j[3],
                         j[4], j[5], j[6], dt, o[0], o[1], o[2], o[3], TG_PREC_FP64, s);
    });
}

void kepler_solver_kernel(const double *_im, const double *_irx, const double *_iry,
                          const double *_irz, const double *_ie2, const double *_ivx,
                          const double *_ivy, const double *_ivz, const double dt, double *_ir1x,
                          double *_ir1y, double *_ir1z, double *_iv1x, double *_iv1y,
                          double *_iv1z) {
    // one pair: two particles in, two out (the outputs may alias the inputs)
    HostCall h;
    std::memset(&h, 0, sizeof h);
    h.nf = 8; h.no = 6; h.ni = 2; h.nj = 0;
    const double *ii[8] = {_im, _irx, _iry, _irz, _ie2, _ivx, _ivy, _ivz};
    for (int f = 0; f < 8; ++f) h.in_i[f] = ii[f];
    h.out[0] = _ir1x; h.out[1] = _ir1y; h.out[2] = _ir1z; h.out[3] = _iv1x; h.out[4] = _iv1y; h.out[5] = _iv1z;
    host_call(h, [&](const double **i, const double **, double **o, cudaStream_t s) {
        return tg_kepler_solver(1, i[0], i[1], i[2], i[3], i[4], i[5], i[6], i[7], dt, o[0], o[1], o[2],
                                o[3], o[4], o[5], s);
    });
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Segmented (ensemble) entry points.
// ---------------------------------------------------------------------------
struct tg_segments {
    int dev = 0;
    long long C = 0, n_total = 0;
    std::vector<long long> start, count;
    long long *d_tab[2] = {nullptr, nullptr};   // ds32 tables for 1 and 2 i-particles per thread
    tg::SegGeometry geo[2];
    long long *d_fp64 = nullptr;                // block_off[C+1], seg_start[C], seg_n[C]
    long long fp64_blocks = 0;
    int fp64_threads = 128;
    struct Tune { int ipt = 0, mult = 0; };
    Tune tune[tg::K_COUNT];
};

namespace {

long long cdiv(long long a, long long b) { return (a + b - 1) / b; }

int upload(long long **dst, const std::vector<long long> &v) {
    if (cudaMalloc(dst, v.size() * sizeof(long long)) != cudaSuccess) return TG_ENOMEM;
    if (cudaMemcpy(*dst, v.data(), v.size() * sizeof(long long), cudaMemcpyHostToDevice) != cudaSuccess)
        return TG_ECUDA;
    return TG_OK;
}

// Candidates (i-particles per thread, grid multiple) timed on the first
// call outside stream capture; the fastest is kept for this ensemble.
const int TUNE_IPT[2] = {2, 1};
const int TUNE_MULT[2] = {1, 2};

int run_segmented(int kernel, tg_segments *sg, tg::PairArgs &a, int prec, void *stream) {
    g_err.clear();
    if (!sg) return fail(TG_EINVAL, "null segment table");
    if (prec != TG_PREC_FP64 && prec != TG_PREC_DS32) return fail(TG_EINVAL, "unknown precision");
    const int nf = tg::kernel_fields(kernel), no = tg::kernel_outputs(kernel);
    if (sg->n_total > 0) {
        for (int f = 0; f < nf; ++f)
            if (!a.I.f[f]) return fail(TG_EINVAL, "null particle pointer");
        for (int o = 0; o < no; ++o)
            if (!a.out[o]) return fail(TG_EINVAL, "null output pointer");
    }
    a.J = a.I;
    a.ni = a.nj = (size_t)sg->n_total;
    if (sg->n_total == 0) return TG_OK;
    DevCtx *c = nullptr;
    int rc = current_ctx(&c);
    if (rc != TG_OK) return rc;
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev != sg->dev) return fail(TG_EINVAL, "segment table was created on another device");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    a.status = c->status;
    cudaError_t e;
    if (prec == TG_PREC_FP64) {
        const long long *t = sg->d_fp64;
        e = tg::launch_fp64_seg(kernel, a, sg->C, sg->fp64_blocks, sg->fp64_threads, t, t + sg->C + 1,
                                t + 2 * sg->C + 1, s);
        if (e != cudaSuccess) return fail(TG_ECUDA, "segmented kernel launch", e);
        return TG_OK;
    }
    std::lock_guard<std::mutex> lk(c->mu);
    const int nipt = kernel == tg::K_SNAP_CRACKLE ? 1 : 2;
    size_t need = 0;
    for (int q = 0; q < nipt; ++q) {
        const int ipt = kernel == tg::K_SNAP_CRACKLE ? 1 : TUNE_IPT[q];
        for (int m = 0; m < 2; ++m) {
            const size_t b = tg::ds32_seg_workspace_bytes(kernel, ipt, sg->geo[ipt - 1], c->sms, TUNE_MULT[m]);
            need = b > need ? b : need;
        }
    }
    rc = ensure_ws(*c, need, s);
    if (rc != TG_OK) return rc;
    tg_segments::Tune &tu = sg->tune[kernel];
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaStreamIsCapturing(s, &cs);
    if (tu.ipt == 0 && cs == cudaStreamCaptureStatusNone) {
        cudaEvent_t e0, e1;
        cudaEventCreate(&e0);
        cudaEventCreate(&e1);
        float best = 1e30f;
        for (int q = 0; q < nipt; ++q) {
            const int ipt = kernel == tg::K_SNAP_CRACKLE ? 1 : TUNE_IPT[q];
            for (int m = 0; m < 2; ++m) {
                e = tg::launch_ds32_seg(kernel, ipt, a, sg->geo[ipt - 1], c->ws, c->ws_bytes, c->sms,
                                        TUNE_MULT[m], s);   // warm-up
                cudaEventRecord(e0, s);
                for (int rep = 0; rep < 2 && e == cudaSuccess; ++rep)
                    e = tg::launch_ds32_seg(kernel, ipt, a, sg->geo[ipt - 1], c->ws, c->ws_bytes, c->sms,
                                            TUNE_MULT[m], s);
                cudaEventRecord(e1, s);
                if (e != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess) {
                    cudaEventDestroy(e0);
                    cudaEventDestroy(e1);
                    return fail(TG_ECUDA, "segmented autotune launch", e);
                }
                float ms = 0.f;
                cudaEventElapsedTime(&ms, e0, e1);
                if (ms < best) { best = ms; tu.ipt = ipt; tu.mult = TUNE_MULT[m]; }
            }
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
    }
    const int ipt = tu.ipt ? tu.ipt : (kernel == tg::K_SNAP_CRACKLE ? 1 : 2);
    const int mult = tu.mult ? tu.mult : 1;
    e = tg::launch_ds32_seg(kernel, ipt, a, sg->geo[ipt - 1], c->ws, c->ws_bytes, c->sms, mult, s);
    if (e != cudaSuccess) return fail(TG_ECUDA, "segmented kernel launch", e);
    return TG_OK;
}

}  // namespace

extern "C" {

tg_segments *tg_segments_create(size_t nseg, const long long *start, const long long *count) {
    g_err.clear();
    if (nseg > 0 && (!start || !count)) { fail(TG_EINVAL, "null segment arrays"); return nullptr; }
    std::vector<std::pair<long long, long long>> iv;
    long long n_total = 0;
    for (size_t k = 0; k < nseg; ++k) {
        if (start[k] < 0 || count[k] < 0 || count[k] > (1LL << 31)) {
            fail(TG_EINVAL, "segment start/count out of range");
            return nullptr;
        }
        iv.push_back({start[k], start[k] + count[k]});
        n_total = std::max(n_total, start[k] + count[k]);
    }
    std::vector<std::pair<long long, long long>> sorted = iv;
    std::sort(sorted.begin(), sorted.end());
    long long max_end = 0;
    for (const auto &r : sorted) {
        if (r.second == r.first) continue;   // empty segments overlap nothing
        if (r.first < max_end) {
            fail(TG_EINVAL, "segments overlap");
            return nullptr;
        }
        max_end = std::max(max_end, r.second);
    }
    DevCtx *c = nullptr;
    if (current_ctx(&c) != TG_OK) return nullptr;
    tg_segments *sg = new tg_segments();
    cudaGetDevice(&sg->dev);
    sg->C = (long long)nseg;
    sg->n_total = n_total;
    sg->start.assign(start, start + nseg);
    sg->count.assign(count, count + nseg);
    const long long C = sg->C, TJ = tg::ds32_tile_j();
    int rc = TG_OK;
    for (int q = 0; q < 2 && rc == TG_OK; ++q) {
        const long long BI = tg::ds32_tile_i(tg::K_ACC_JERK, q + 1);
        std::vector<long long> tab;
        tab.reserve(5 * C + 3);
        long long u = 0, it = 0, rt = 0;
        std::vector<long long> uo(1, 0), io(1, 0), ro(1, 0);
        for (long long k = 0; k < C; ++k) {
            const long long n = sg->count[k];
            const long long nit = cdiv(n, BI), njt = cdiv(n, TJ);
            u += nit * njt; it += nit; rt += njt;
            uo.push_back(u); io.push_back(it); ro.push_back(rt);
        }
        tab.insert(tab.end(), uo.begin(), uo.end());
        tab.insert(tab.end(), io.begin(), io.end());
        tab.insert(tab.end(), ro.begin(), ro.end());
        tab.insert(tab.end(), sg->start.begin(), sg->start.end());
        tab.insert(tab.end(), sg->count.begin(), sg->count.end());
        rc = upload(&sg->d_tab[q], tab);
        sg->geo[q] = tg::SegGeometry{C, u, it, rt, sg->d_tab[q]};
    }
    // FP64: narrow CTAs while the ensemble would leave SMs idle
    int t = 128;
    auto blocks_for = [&](int th) {
        long long b = 0;
        for (long long k = 0; k < C; ++k) b += cdiv(sg->count[k], th);
        return b;
    };
    while (t > 32 && blocks_for(t) < c->sms) t /= 2;
    sg->fp64_threads = t;
    std::vector<long long> ft(1, 0);
    for (long long k = 0; k < C; ++k) ft.push_back(ft.back() + cdiv(sg->count[k], t));
    sg->fp64_blocks = ft.back();
    ft.insert(ft.end(), sg->start.begin(), sg->start.end());
    ft.insert(ft.end(), sg->count.begin(), sg->count.end());
    if (rc == TG_OK) rc = upload(&sg->d_fp64, ft);
    if (rc != TG_OK) {
        fail(rc, "segment table upload failed");
        tg_segments_destroy(sg);
        return nullptr;
    }
    return sg;
}

void tg_segments_destroy(tg_segments *sg) {
    if (!sg) return;
    for (int q = 0; q < 2; ++q)
        if (sg->d_tab[q]) cudaFree(sg->d_tab[q]);
    if (sg->d_fp64) cudaFree(sg->d_fp64);
    delete sg;
}

int tg_phi_segmented(tg_segments *sg, const double *m, const double *rx, const double *ry,
                     const double *rz, const double *e2, double *phi, int prec, void *stream) {
    tg::PairArgs a = blank();
    set5(a.I, m, rx, ry, rz, e2);
    a.out[0] = phi;
    return run_segmented(tg::K_PHI, sg, a, prec, stream);
}

int tg_acc_segmented(tg_segments *sg, const double *m, const double *rx, const double *ry,
                     const double *rz, const double *e2, double *ax, double *ay, double *az, int prec,
                     void *stream) {
    tg::PairArgs a = blank();
    set5(a.I, m, rx, ry, rz, e2);
    a.out[0] = ax; a.out[1] = ay; a.out[2] = az;
    return run_segmented(tg::K_ACC, sg, a, prec, stream);
}

int tg_acc_jerk_segmented(tg_segments *sg, const double *m, const double *rx, const double *ry,
                          const double *rz, const double *e2, const double *vx, const double *vy,
                          const double *vz, double *ax, double *ay, double *az, double *jx, double *jy,
                          double *jz, int prec, void *stream) {
    tg::PairArgs a = blank();
    set5(a.I, m, rx, ry, rz, e2); setv(a.I, vx, vy, vz);
    a.out[0] = ax; a.out[1] = ay; a.out[2] = az; a.out[3] = jx; a.out[4] = jy; a.out[5] = jz;
    return run_segmented(tg::K_ACC_JERK, sg, a, prec, stream);
}

int tg_snap_crackle_segmented(tg_segments *sg, const double *m, const double *rx, const double *ry,
                              const double *rz, const double *e2, const double *vx, const double *vy,
                              const double *vz, const double *ax, const double *ay, const double *az,
                              const double *jx, const double *jy, const double *jz, double *sx, double *sy,
                              double *sz, double *cx, double *cy, double *cz, int prec, void *stream) {
    tg::PairArgs a = blank();
    set5(a.I, m, rx, ry, rz, e2); setv(a.I, vx, vy, vz);
    a.I.f[tg::F_AX] = ax; a.I.f[tg::F_AY] = ay; a.I.f[tg::F_AZ] = az;
    a.I.f[tg::F_JX] = jx; a.I.f[tg::F_JY] = jy; a.I.f[tg::F_JZ] = jz;
    a.out[0] = sx; a.out[1] = sy; a.out[2] = sz; a.out[3] = cx; a.out[4] = cy; a.out[5] = cz;
    return run_segmented(tg::K_SNAP_CRACKLE, sg, a, prec, stream);
}

}  // extern "C"
