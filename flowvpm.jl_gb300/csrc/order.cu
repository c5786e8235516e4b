// order.cu -- Morton (Z-order) ordering of the targets of a UJ / Estr call.
//
// The pair kernels give each warp 32 consecutive targets of this order, so a
// warp's targets sit in a small box: the far-field test of a source is then
// the same for the whole warp (no divergence), and the FP32 offsets of the
// mixed kernels, taken from a per-warp FP64 origin, stay small.  The order is
// internal: results are written back to each target's original index.
//
// Steps: per-block bounding boxes (bbox_partial), 63-bit Morton keys with 21
// bits per axis of the global box (morton_keys), CUB radix sort of (key,
// index), and a gather of the sorted positions into TgtPos records.
#include "internal.h"

#include <cub/device/device_radix_sort.cuh>

namespace vpm {

constexpr int BB_BLOCKS = 256;
constexpr int BB_THREADS = 256;

// Spread the low 21 bits of v so that bit i moves to bit 3i.
__device__ __forceinline__ uint64_t spread3(uint64_t v)
{
    v &= 0x1fffffULL;
    v = (v | (v << 32)) & 0x1f00000000ffffULL;
    v = (v | (v << 16)) & 0x1f0000ff0000ffULL;
    v = (v | (v << 8)) & 0x100f00f00f00f00fULL;
    v = (v | (v << 4)) & 0x10c30c30c30c30c3ULL;
    v = (v | (v << 2)) & 0x1249249249249249ULL;
    return v;
}

__global__ void __launch_bounds__(BB_THREADS)
bbox_partial(int64_t n, const double* __restrict__ x, double* __restrict__ part)
{
    __shared__ double red[6][BB_THREADS];
    double mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int64_t i = blockIdx.x * (int64_t)BB_THREADS + threadIdx.x; i < n; i += (int64_t)gridDim.x * BB_THREADS) {
#pragma unroll
        for (int k = 0; k < 3; k++) {
            const double v = x[3 * i + k];
            mn[k] = fmin(mn[k], v);
            mx[k] = fmax(mx[k], v);
        }
    }
#pragma unroll
    for (int k = 0; k < 3; k++) { red[k][threadIdx.x] = mn[k]; red[3 + k][threadIdx.x] = mx[k]; }
    __syncthreads();
    for (int off = BB_THREADS / 2; off > 0; off >>= 1) {
        if (threadIdx.x < off) {
#pragma unroll
            for (int k = 0; k < 3; k++) {
                red[k][threadIdx.x] = fmin(red[k][threadIdx.x], red[k][threadIdx.x + off]);
                red[3 + k][threadIdx.x] = fmax(red[3 + k][threadIdx.x], red[3 + k][threadIdx.x + off]);
            }
        }
        __syncthreads();
    }
    if (threadIdx.x < 6) part[blockIdx.x * 6 + threadIdx.x] = red[threadIdx.x][0];
}

__global__ void __launch_bounds__(BB_THREADS)
morton_keys(int64_t n, const double* __restrict__ x, const double* __restrict__ part,
            uint64_t* __restrict__ keys, int32_t* __restrict__ idx)
{
    __shared__ double box[6];
    if (threadIdx.x < 6) {
        double v = threadIdx.x < 3 ? INFINITY : -INFINITY;
        for (int b = 0; b < BB_BLOCKS; b++) {
            const double p = part[b * 6 + threadIdx.x];
            v = threadIdx.x < 3 ? fmin(v, p) : fmax(v, p);
        }
        box[threadIdx.x] = v;
    }
    __syncthreads();
    const int64_t i = blockIdx.x * (int64_t)BB_THREADS + threadIdx.x;
    if (i >= n) return;
    uint64_t key = 0;
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const double ext = box[3 + k] - box[k];
        double f = ext > 0.0 ? (x[3 * i + k] - box[k]) / ext : 0.0;
        f = fmin(fmax(f, 0.0), 1.0);
        const uint64_t q = (uint64_t)(f * 2097151.0);   // 2^21 - 1
        key |= spread3(q) << k;
    }
    keys[i] = key;
    idx[i] = (int32_t)i;
}

__global__ void gather_targets(int64_t n, const double* __restrict__ x, const int32_t* __restrict__ perm,
                               TgtPos* __restrict__ out)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int32_t j = perm ? perm[i] : (int32_t)i;
    TgtPos t;
    t.x = x[3 * (int64_t)j];
    t.y = x[3 * (int64_t)j + 1];
    t.z = x[3 * (int64_t)j + 2];
    t.idx = j;
    t.pad = 0;
    out[i] = t;
}

static inline size_t align256(size_t b) { return (b + 255) / 256 * 256; }

size_t order_bytes(int64_t nt)
{
    size_t tmp = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, tmp, (uint64_t*)nullptr, (uint64_t*)nullptr, (int32_t*)nullptr,
                                    (int32_t*)nullptr, (int)nt, 0, 63);
    return align256(BB_BLOCKS * 6 * sizeof(double)) + 2 * align256(nt * sizeof(uint64_t)) +
           2 * align256(nt * sizeof(int32_t)) + align256(tmp) + align256(nt * sizeof(TgtPos));
}

cudaError_t order_targets(int64_t nt, const double* xt, void* scratch, size_t scratch_bytes, cudaStream_t st,
                          int64_t* launches, const TgtPos** out)
{
    char* p = (char*)scratch;
    double* part = (double*)p;            p += align256(BB_BLOCKS * 6 * sizeof(double));
    uint64_t* k0 = (uint64_t*)p;          p += align256(nt * sizeof(uint64_t));
    uint64_t* k1 = (uint64_t*)p;          p += align256(nt * sizeof(uint64_t));
    int32_t* i0 = (int32_t*)p;            p += align256(nt * sizeof(int32_t));
    int32_t* i1 = (int32_t*)p;            p += align256(nt * sizeof(int32_t));
    size_t tmp = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, tmp, k0, k1, i0, i1, (int)nt, 0, 63);
    void* tmpp = p;                       p += align256(tmp);
    TgtPos* tp = (TgtPos*)p;              p += align256(nt * sizeof(TgtPos));
    if ((size_t)(p - (char*)scratch) > scratch_bytes) return cudaErrorInvalidValue;
    const unsigned nb = (unsigned)((nt + BB_THREADS - 1) / BB_THREADS);
    const int32_t* perm = nullptr;
    if (nt > 1) {
        bbox_partial<<<BB_BLOCKS, BB_THREADS, 0, st>>>(nt, xt, part);
        morton_keys<<<nb, BB_THREADS, 0, st>>>(nt, xt, part, k0, i0);
        *launches += 2;
        cudaError_t e = cub::DeviceRadixSort::SortPairs(tmpp, tmp, k0, k1, i0, i1, (int)nt, 0, 63, st);
        if (e != cudaSuccess) return e;
        *launches += 1;  // CUB's onesweep passes are counted as one library call
        perm = i1;
    }
    gather_targets<<<nb, BB_THREADS, 0, st>>>(nt, xt, perm, tp);
    *launches += 1;
    *out = tp;
    return cudaGetLastError();
}

}  // namespace vpm
