// tg_noalloc.cu -- split-FP32 AccJerk that allocates no GPU memory.
//
// Some callers cannot let a library call cudaMalloc: applications that hand
// all of the GPU's memory to their own pool or arena at start-up (a second
// allocator then fails or fragments it), and time-stepping loops that must
// not stall other streams, because cudaMalloc/cudaFree can synchronise the
// device.  tg_acc_jerk_noalloc serves them.  It runs the same split-FP32
// AccJerk kernels as tg_acc_jerk(..., TG_PREC_DS32, ...), but its scratch
// memory (packed j-records, stream-K partials, tickets) lives in the
// file-scope __device__ array below.  That array is part of the library's
// GPU image: every GPU that loads the library holds these 24 MiB until the
// process exits.
//
// Limits of the fixed scratch: ni <= 2^20 i-particles, nj <= 2^17
// j-particles, at most 320 CTAs (larger devices run 320).  Larger sizes are
// rejected with TG_EINVAL.
//
// Set-up: the first call on a device, with that device current, looks up
// the device address of the array (cudaGetSymbolAddress) and the SM count;
// make that first call before any stream capture.  Every call on a device
// shares the one array and leaves its contents behind (the tickets are
// cleared at the start of each call), so calls whose kernels overlap on the
// GPU -- e.g. issued on two streams without ordering -- race and corrupt
// each other's results.  Order them on one stream.
//
// Errors: arguments and launches are checked when the call is made (return
// code, tg_last_error).  A device-side bounded wait that gives up sets
// TG_ST_MBAR_TIMEOUT in a status word at the head of the array; the word is
// sticky and tg_sync_status(stream) reports it together with the other
// entry points' status bits, then clears it -- without allocating.
#include <cstring>
#include <mutex>

#include "../../include/tupan_gb300.h"
#include "tg_device.cuh"
#include "tg_internal.h"

namespace {

constexpr size_t NOALLOC_BYTES = (size_t)24 << 20;
constexpr size_t NOALLOC_HEADER = 256;             // status word
constexpr size_t NOALLOC_MAX_NI = (size_t)1 << 20;
constexpr size_t NOALLOC_MAX_NJ = (size_t)1 << 17;
constexpr long long NOALLOC_MAX_GRID = 320;
constexpr int NOALLOC_MAX_DEV = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_BYTES];

struct NoAllocDev {
    std::mutex mu;
    bool ready = false;
    unsigned char *base = nullptr;   // device address of g_noalloc_scratch
    int sms = 0;
};
NoAllocDev g_na[NOALLOC_MAX_DEV];

int na_fail(int code, const char *msg) {
    tg::set_last_error(msg);
    return code;
}

}  // namespace

namespace tg {
// Status bits that tg_acc_jerk_noalloc's kernels left in the scratch header
// of the current device (0 if the entry point never ran there); clears them.
// Ordered on `s`, then synchronised with it.
cudaError_t noalloc_take_status(cudaStream_t s, unsigned *bits) {
    *bits = 0;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || dev < 0 || dev >= NOALLOC_MAX_DEV) return e;
    NoAllocDev &d = g_na[dev];
    std::lock_guard<std::mutex> lk(d.mu);
    if (!d.ready) return cudaSuccess;
    unsigned h = 0;
    e = cudaMemcpyAsync(&h, d.base, sizeof h, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e == cudaSuccess) e = cudaMemsetAsync(d.base, 0, sizeof h, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e == cudaSuccess) *bits = h;
    return e;
}
}  // namespace tg

extern "C" int tg_acc_jerk_noalloc(size_t ni, const double *im, const double *irx, const double *iry,
                                   const double *irz, const double *ie2, const double *ivx,
                                   const double *ivy, const double *ivz, size_t nj, const double *jm,
                                   const double *jrx, const double *jry, const double *jrz,
                                   const double *je2, const double *jvx, const double *jvy,
                                   const double *jvz, double *iax, double *iay, double *iaz,
                                   double *ijx, double *ijy, double *ijz, void *stream) {
    tg::set_last_error("");
    if (ni > NOALLOC_MAX_NI || nj > NOALLOC_MAX_NJ)
        return na_fail(TG_EINVAL, "tg_acc_jerk_noalloc: ni must be <= 1048576 and nj <= 131072 "
                                  "(fixed 24 MiB scratch)");
    const double *ip[8] = {im, irx, iry, irz, ie2, ivx, ivy, ivz};
    const double *jp[8] = {jm, jrx, jry, jrz, je2, jvx, jvy, jvz};
    double *op[6] = {iax, iay, iaz, ijx, ijy, ijz};
    if (ni == 0) return TG_OK;
    for (int k = 0; k < 8; ++k)
        if (!ip[k] || (nj > 0 && !jp[k])) return na_fail(TG_EINVAL, "tg_acc_jerk_noalloc: null input pointer");
    for (int k = 0; k < 6; ++k)
        if (!op[k]) return na_fail(TG_EINVAL, "tg_acc_jerk_noalloc: null output pointer");
    if (nj == 0) {
        // empty j-set: the sums are zero; cudaMemsetAsync writes no scratch
        cudaStream_t s0 = static_cast<cudaStream_t>(stream);
        for (int k = 0; k < 6; ++k)
            if (cudaMemsetAsync(op[k], 0, ni * sizeof(double), s0) != cudaSuccess)
                return na_fail(TG_ECUDA, "tg_acc_jerk_noalloc: cudaMemsetAsync failed");
        return TG_OK;
    }

    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= NOALLOC_MAX_DEV)
        return na_fail(TG_ENODEV, "tg_acc_jerk_noalloc: no current CUDA device");
    NoAllocDev &d = g_na[dev];
    {
        std::lock_guard<std::mutex> lk(d.mu);
        if (!d.ready) {
            void *ptr = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
            if (e != cudaSuccess || ptr == nullptr)
                return na_fail(TG_ECUDA, "tg_acc_jerk_noalloc: cudaGetSymbolAddress failed");
            e = cudaDeviceGetAttribute(&d.sms, cudaDevAttrMultiProcessorCount, dev);
            if (e != cudaSuccess) return na_fail(TG_ECUDA, "tg_acc_jerk_noalloc: SM count query failed");
            d.base = static_cast<unsigned char *>(ptr);
            // the status word starts at zero and then stays sticky until
            // tg_sync_status reads it
            if (cudaMemsetAsync(d.base, 0, NOALLOC_HEADER, static_cast<cudaStream_t>(stream)) != cudaSuccess)
                return na_fail(TG_ECUDA, "tg_acc_jerk_noalloc: cudaMemsetAsync failed");
            d.ready = true;
        }
    }

    const size_t need = tg::ds32_workspace_bytes_capped(tg::K_ACC_JERK, ni, nj, d.sms, NOALLOC_MAX_GRID);
    if (need == 0 || need > NOALLOC_BYTES - NOALLOC_HEADER)
        return na_fail(TG_EINVAL, "tg_acc_jerk_noalloc: problem does not fit the fixed scratch");

    tg::PairArgs a;
    std::memset(&a, 0, sizeof a);
    for (int k = 0; k < 8; ++k) { a.I.f[k] = ip[k]; a.J.f[k] = jp[k]; }
    a.ni = ni;
    a.nj = nj;
    for (int k = 0; k < 6; ++k) a.out[k] = op[k];
    a.status = reinterpret_cast<unsigned *>(d.base);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    cudaError_t e = tg::launch_ds32_capped(tg::K_ACC_JERK, a, d.base + NOALLOC_HEADER,
                                           NOALLOC_BYTES - NOALLOC_HEADER, d.sms, NOALLOC_MAX_GRID, s);
    if (e != cudaSuccess) return na_fail(TG_ECUDA, "tg_acc_jerk_noalloc: kernel launch failed");
    return TG_OK;
}
