// noalloc.cu -- vpm_uj_dev_noalloc: the device-pointer UJ for callers that
// cannot allocate device memory.
//
// Some callers own all device memory through their own allocator (a
// framework's caching pool, an arena reserved at start-up) or must not
// allocate once they are running, so they cannot let the library call
// cudaMalloc.  This entry point needs no context and allocates nothing: the
// kernels' scratch (packed sources, the Morton ordering of the targets and
// the split-source partial sums) lives in one file-scope __device__ array of
// VPM_NOALLOC_SCRATCH_BYTES, which every GPU that loads this library's code
// for this entry point holds until the process exits.
//
// Host code cannot use the array's name as a device address (on the host it is
// only a stand-in), so the first call on each device, with that device
// current, looks the address up with cudaGetSymbolAddress and caches it.  Every
// call shares the one array and overwrites what it needs (nothing has to start at
// zero), so calls whose device work overlaps -- on different streams or from
// different threads -- race on it; serialise them.
#include "../../include/vpm_gb300.h"
#include "internal.h"

#include <chrono>
#include <cstdarg>
#include <cstdio>
#include <mutex>
#include <string>
#include <thread>

namespace {

__device__ __align__(256) unsigned char g_noalloc_scratch[VPM_NOALLOC_SCRATCH_BYTES];

constexpr int MAX_DEVICES = 64;
std::mutex g_setup_mu;
void* g_scratch_ptr[MAX_DEVICES] = {nullptr};

// Errors are reported through vpm_last_error(NULL), like vpm_ctx_create's.
int nerr(int code, const char* fmt, ...) __attribute__((format(printf, 2, 3)));
int nerr(int code, const char* fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    vpm::set_thread_error(buf);
    return code;
}

inline size_t align256(size_t b) { return (b + 255) / 256 * 256; }

// Device memory the kernels on device `dev` can use: managed memory, or device
// memory of `dev` itself (memory of another GPU is rejected, since the kernels
// run on the current device only).
bool is_device_ptr(const void* p, int dev)
{
    if (!p) return false;
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return at.type == cudaMemoryTypeManaged || (at.type == cudaMemoryTypeDevice && at.device == dev);
}

// Address of the scratch array on the current device (looked up once per device).
int scratch_address(int dev, void** out)
{
    if (dev < 0 || dev >= MAX_DEVICES) return nerr(VPM_ERR_ARG, "device %d out of range", dev);
    std::lock_guard<std::mutex> lk(g_setup_mu);
    if (!g_scratch_ptr[dev]) {
        void* ptr = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (e != cudaSuccess || !ptr) {
            cudaGetLastError();
            return nerr(VPM_ERR_CUDA, "cudaGetSymbolAddress of the scratch array failed: %s",
                        cudaGetErrorString(e));
        }
        g_scratch_ptr[dev] = ptr;
    }
    *out = g_scratch_ptr[dev];
    return VPM_OK;
}

}  // namespace

extern "C" {

int vpm_uj_dev_noalloc(int64_t nt, const double* xt, int64_t ns, const double* xs, const double* gs,
                       const double* sgs, double* U, double* J, int kernel, int precision, void* stream)
{
    vpm::TraceRange trace_("vpm_uj_dev_noalloc");
    if (nt < 0 || ns < 0 || nt > (int64_t)INT32_MAX || ns > (int64_t)INT32_MAX)
        return nerr(VPM_ERR_ARG, "vpm_uj_dev_noalloc: sizes out of range");
    if (kernel < VPM_KERNEL_SINGULAR || kernel > VPM_KERNEL_WINCKELMANS)
        return nerr(VPM_ERR_ARG, "vpm_uj_dev_noalloc: unknown kernel id %d", kernel);
    if (precision != VPM_FP64 && precision != VPM_FP32COMP)
        return nerr(VPM_ERR_ARG, "vpm_uj_dev_noalloc: unknown precision %d", precision);
    if (nt == 0 || ns == 0) return VPM_OK;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
        cudaGetLastError();
        return nerr(VPM_ERR_NODEVICE, "vpm_uj_dev_noalloc: no current CUDA device");
    }
    if (!is_device_ptr(xt, dev) || !is_device_ptr(xs, dev) || !is_device_ptr(gs, dev) || !is_device_ptr(sgs, dev) ||
        !is_device_ptr(U, dev) || !is_device_ptr(J, dev))
        return nerr(VPM_ERR_ARG, "vpm_uj_dev_noalloc: every array must be device memory of the current device %d",
                    dev);
    const int nsplit = vpm::uj_num_splits(nt, ns, sms);
    const size_t pack = align256(vpm::uj_src_pack_bytes(ns, precision));
    const size_t order = align256(vpm::order_bytes(nt));
    const size_t part = align256(vpm::uj_partial_bytes(nt, nsplit));
    if (pack + order + part > (size_t)VPM_NOALLOC_SCRATCH_BYTES)
        return nerr(VPM_ERR_CAPACITY,
                    "vpm_uj_dev_noalloc: %lld targets x %lld sources need %zu B of scratch; the static "
                    "scratch holds %llu B (use vpm_uj_dev for larger problems)",
                    (long long)nt, (long long)ns, pack + order + part,
                    (unsigned long long)VPM_NOALLOC_SCRATCH_BYTES);
    void* base = nullptr;
    int rc = scratch_address(dev, &base);
    if (rc != VPM_OK) return rc;
    char* p = (char*)base;
    vpm::Workspace w;
    w.src_pack = p;                   w.src_pack_bytes = pack;  p += pack;
    w.order = p;                      w.order_bytes = order;    p += order;
    w.partial = part ? (double*)p : nullptr; w.partial_bytes = part;
    vpm::UJArgs a;
    a.nt = nt; a.ns = ns; a.xt = xt; a.xs = xs; a.gs = gs; a.sgs = sgs;
    a.U = U; a.ldU = 3; a.J = J; a.ldJ = 9; a.kernel = kernel; a.precision = precision;
    a.self = (xt == xs) && (nt == ns);
    cudaStream_t st = (cudaStream_t)stream;
    int64_t launches = 0;
    cudaError_t e = vpm::launch_uj(a, w, sms, st, &launches);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return nerr(VPM_ERR_CUDA, "vpm_uj_dev_noalloc: launch failed: %s", cudaGetErrorString(e));
    }
    // bounded wait on the caller's stream (no event object is created)
    const auto t0 = std::chrono::steady_clock::now();
    int sleep_us = 2;
    for (;;) {
        e = cudaStreamQuery(st);
        if (e == cudaSuccess) return VPM_OK;
        if (e != cudaErrorNotReady) {
            cudaGetLastError();
            return nerr(VPM_ERR_CUDA, "vpm_uj_dev_noalloc: device work failed: %s", cudaGetErrorString(e));
        }
        if (std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count() > 3600.0)
            return nerr(VPM_ERR_TIMEOUT, "vpm_uj_dev_noalloc: device work did not finish within 3600 s");
        std::this_thread::sleep_for(std::chrono::microseconds(sleep_us));
        if (sleep_us < 1000) sleep_us *= 2;
    }
}

}  // extern "C"
