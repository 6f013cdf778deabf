// tg_order.cu -- per-call spatial ordering of the particle sets for the
// ordered split-FP32 Acc and AccJerk kernels (tg_ds32.cu).
//
// j-set: sorted by a 31-bit key, (heavy << 30) | Hilbert(x, y, z), so the
// light particles come first in Hilbert-curve order over 10 bits per axis
// and the heavy ones (mass above max(m) / 32 and above 16 min(m), so that
// a set of equal masses has none) follow, also in that order.
// (A Hilbert curve keeps neighbours in the key adjacent in space, without a
// Morton curve's jumps at octant boundaries: on a Plummer sphere of 65536
// particles 84% of (512-i tile, 64-j block) pairs come out far apart, 73%
// with Morton keys.)  The
// pairwise kernel then sees spatially compact 64-j blocks, which lets it use
// single-float separations for block pairs that are far apart, and it folds
// the terms of heavy particles (the large ones) into its compensated sums one
// record at a time.
// i-set: sorted by the Hilbert key alone (the same order as j when both are
// the same arrays), so i-tiles are compact too.
// Sorting is cub::DeviceRadixSort (stable, deterministic): equal keys keep
// their input order, so a call's result depends only on its inputs.
#include <algorithm>

#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

#include "tg_internal.h"

namespace tg {

namespace {

constexpr int ORD_THREADS = 256;
constexpr unsigned HEAVY_BIT = 1u << 30;
constexpr float HEAVY_FRACTION = 1.0f / 32.0f;   // of the largest mass
constexpr float HEAVY_OVER_MIN = 16.0f;           // times the smallest mass

__device__ __forceinline__ unsigned f2ord(float f) {
    const unsigned u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float ord2f(unsigned u) {
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

// scal[0..2] = min x, y, z; scal[3..5] = max; scal[6] = max mass; scal[8]
// = min mass (all as order-preserving unsigned); scal[7] = number of light j.
__global__ void ord_init(unsigned *scal) {
    const int t = threadIdx.x;
    if (t < 3 || t == 8) scal[t] = 0xffffffffu;
    else if (t < 8) scal[t] = 0u;
}

__global__ void ord_bounds(PSet S, size_t n, bool with_mass, unsigned *scal) {
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    float mmax = -INFINITY, mmin = INFINITY;
    for (size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += (size_t)gridDim.x * blockDim.x) {
        for (int k = 0; k < 3; ++k) {
            const float x = __double2float_rn(S.f[F_RX + k][p]);
            if (isfinite(x)) { lo[k] = fminf(lo[k], x); hi[k] = fmaxf(hi[k], x); }
        }
        if (with_mass) {
            const float m = __double2float_rn(S.f[F_M][p]);
            if (isfinite(m)) { mmax = fmaxf(mmax, m); mmin = fminf(mmin, m); }
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        for (int k = 0; k < 3; ++k) {
            lo[k] = fminf(lo[k], __shfl_xor_sync(0xffffffffu, lo[k], o));
            hi[k] = fmaxf(hi[k], __shfl_xor_sync(0xffffffffu, hi[k], o));
        }
        mmax = fmaxf(mmax, __shfl_xor_sync(0xffffffffu, mmax, o));
        mmin = fminf(mmin, __shfl_xor_sync(0xffffffffu, mmin, o));
    }
    if ((threadIdx.x & 31) == 0) {
        for (int k = 0; k < 3; ++k) {
            if (lo[k] <= hi[k]) {
                atomicMin(scal + k, f2ord(lo[k]));
                atomicMax(scal + 3 + k, f2ord(hi[k]));
            }
        }
        if (with_mass && mmax > -INFINITY) {
            atomicMax(scal + 6, f2ord(mmax));
            atomicMin(scal + 8, f2ord(mmin));
        }
    }
}

// Index of cell (x, y, z), 10 bits each, along a 3-d Hilbert curve: J.
// Skilling's transform of the coordinates into the curve's "transposed"
// index (Programming the Hilbert curve, AIP Conf. Proc. 707, 381 (2004)),
// then its bits interleaved, x most significant, into a 30-bit key.
__device__ __forceinline__ unsigned hilbert10(unsigned x0, unsigned x1, unsigned x2) {
    unsigned X[3] = {x0 & 0x3ffu, x1 & 0x3ffu, x2 & 0x3ffu};
    for (unsigned Q = 1u << 9; Q > 1u; Q >>= 1) {   // inverse undo
        const unsigned P = Q - 1u;
        for (int i = 0; i < 3; ++i) {
            if (X[i] & Q) {
                X[0] ^= P;                    // invert
            } else {
                const unsigned t = (X[0] ^ X[i]) & P;   // exchange
                X[0] ^= t;
                X[i] ^= t;
            }
        }
    }
    X[1] ^= X[0];                             // Gray encode
    X[2] ^= X[1];
    unsigned t = 0;
    for (unsigned Q = 1u << 9; Q > 1u; Q >>= 1)
        if (X[2] & Q) t ^= Q - 1u;
    for (int i = 0; i < 3; ++i) X[i] ^= t;
    unsigned key = 0;
    for (int b = 9; b >= 0; --b)
        for (int i = 0; i < 3; ++i) key = (key << 1) | ((X[i] >> b) & 1u);
    return key;
}

// keys[p] = (heavy bit if `heavy` and m > max(m) / 32) | Hilbert(position);
// vals[p] = p; counts the light particles into *nlight when `heavy`.
__global__ void ord_keys(PSet S, size_t n, bool heavy, const unsigned *scal, unsigned *keys, int *vals,
                         unsigned *nlight) {
    __shared__ unsigned s_light;
    if (threadIdx.x == 0) s_light = 0;
    __syncthreads();
    float lo[3], scale = 0.f;
    {
        float span = 0.f;
        for (int k = 0; k < 3; ++k) {
            const unsigned a = scal[k], b = scal[3 + k];
            lo[k] = (a == 0xffffffffu) ? 0.f : ord2f(a);
            const float h = (b == 0u) ? 0.f : ord2f(b);
            span = fmaxf(span, h - lo[k]);
        }
        if (span > 0.f && isfinite(span)) scale = 1023.999f / span;
    }
    const float mcut = (scal[6] == 0u) ? INFINITY
                                       : fmaxf(ord2f(scal[6]) * HEAVY_FRACTION, ord2f(scal[8]) * HEAVY_OVER_MIN);
    const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    unsigned light = 0;
    if (p < n) {
        unsigned c[3];
        for (int k = 0; k < 3; ++k) {
            const float x = __double2float_rn(S.f[F_RX + k][p]);
            float q = (x - lo[k]) * scale;
            q = (q > 0.f) ? fminf(q, 1023.f) : 0.f;   // NaN -> 0
            c[k] = (unsigned)q;
        }
        unsigned key = hilbert10(c[0], c[1], c[2]);
        if (heavy) {
            const float m = __double2float_rn(S.f[F_M][p]);
            if (m > mcut && mcut > 0.f) key |= HEAVY_BIT;
            else light = 1;
        }
        keys[p] = key;
        vals[p] = (int)p;
    }
    if (heavy) {
        light = __reduce_add_sync(0xffffffffu, light);
        if ((threadIdx.x & 31) == 0 && light) atomicAdd(&s_light, light);
        __syncthreads();
        if (threadIdx.x == 0 && s_light) atomicAdd(nlight, s_light);
    }
}

size_t align256(size_t x) { return (x + 255) / 256 * 256; }

size_t cub_bytes(size_t n) {
    size_t tmp = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, tmp, (const unsigned *)nullptr, (unsigned *)nullptr,
                                    (const int *)nullptr, (int *)nullptr, (int)n, 0, 31);
    return tmp;
}

}  // namespace

size_t order_workspace_bytes(size_t ni, size_t nj, bool same) {
    const size_t n = ni > nj ? ni : nj;
    size_t b = align256(16 * sizeof(unsigned));
    b += 4 * align256(nj * sizeof(unsigned));            // j keys in/out, values in/out
    if (!same) b += 4 * align256(ni * sizeof(unsigned)); // i keys in/out, values in/out
    b += align256(cub_bytes(n));
    return b;
}

size_t inclusive_sum_bytes(size_t n) {
    size_t tmp = 0;
    cub::DeviceScan::InclusiveSum(nullptr, tmp, (const int *)nullptr, (int *)nullptr, (int)n);
    return tmp;
}

cudaError_t inclusive_sum(const int *in, int *out, size_t n, void *tmp, size_t tmp_bytes, cudaStream_t s) {
    return cub::DeviceScan::InclusiveSum(tmp, tmp_bytes, in, out, (int)n, s);
}

cudaError_t build_order(const PSet &I, size_t ni, const PSet &J, size_t nj, bool same, void *ws,
                        size_t ws_bytes, OrderOut &out, cudaStream_t s) {
    if (order_workspace_bytes(ni, nj, same) > ws_bytes) return cudaErrorInvalidValue;
    char *p = static_cast<char *>(ws);
    unsigned *scal = reinterpret_cast<unsigned *>(p); p += align256(16 * sizeof(unsigned));
    unsigned *kj = reinterpret_cast<unsigned *>(p); p += align256(nj * sizeof(unsigned));
    unsigned *kj2 = reinterpret_cast<unsigned *>(p); p += align256(nj * sizeof(unsigned));
    int *vj = reinterpret_cast<int *>(p); p += align256(nj * sizeof(int));
    int *pj = reinterpret_cast<int *>(p); p += align256(nj * sizeof(int));
    unsigned *ki = nullptr, *ki2 = nullptr;
    int *vi = nullptr, *pi = pj;
    if (!same) {
        ki = reinterpret_cast<unsigned *>(p); p += align256(ni * sizeof(unsigned));
        ki2 = reinterpret_cast<unsigned *>(p); p += align256(ni * sizeof(unsigned));
        vi = reinterpret_cast<int *>(p); p += align256(ni * sizeof(int));
        pi = reinterpret_cast<int *>(p); p += align256(ni * sizeof(int));
    }
    void *tmp = p;
    size_t tmp_bytes = cub_bytes(ni > nj ? ni : nj);

    ord_init<<<1, 32, 0, s>>>(scal);
    ord_bounds<<<(unsigned)std::min<size_t>((nj + ORD_THREADS - 1) / ORD_THREADS, 1024), ORD_THREADS, 0, s>>>(
        J, nj, true, scal);
    if (!same)
        ord_bounds<<<(unsigned)std::min<size_t>((ni + ORD_THREADS - 1) / ORD_THREADS, 1024), ORD_THREADS, 0, s>>>(
            I, ni, false, scal);
    ord_keys<<<(unsigned)((nj + ORD_THREADS - 1) / ORD_THREADS), ORD_THREADS, 0, s>>>(J, nj, true, scal, kj, vj,
                                                                                     scal + 7);
    cudaError_t e = cub::DeviceRadixSort::SortPairs(tmp, tmp_bytes, kj, kj2, vj, pj, (int)nj, 0, 31, s);
    if (e != cudaSuccess) return e;
    if (!same) {
        ord_keys<<<(unsigned)((ni + ORD_THREADS - 1) / ORD_THREADS), ORD_THREADS, 0, s>>>(I, ni, false, scal, ki,
                                                                                         vi, nullptr);
        e = cub::DeviceRadixSort::SortPairs(tmp, tmp_bytes, ki, ki2, vi, pi, (int)ni, 0, 30, s);
        if (e != cudaSuccess) return e;
    }
    out.pi = pi;
    out.pj = pj;
    out.nlight = scal + 7;
    return cudaGetLastError();
}

}  // namespace tg
