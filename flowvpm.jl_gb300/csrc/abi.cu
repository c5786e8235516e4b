// abi.cu -- the C ABI of libvpm_gb300.so (include/vpm_gb300.h): contexts,
// argument checking, host<->device staging of the reference's 46-row particle
// matrix, and dispatch to the UJ / Estr launchers.
#include "../../include/vpm_gb300.h"
#include "internal.h"
#include "vpm_math.cuh"
#include "tree.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <chrono>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

using namespace vpm;

namespace {

// 0-based rows of the particle column, src/FLOWVPM_particlefield.jl:239-252
enum : int { R_X = 0, R_G = 3, R_SIG = 6, R_U = 9, R_W = 12, R_J = 15, R_PSE = 24, R_SFS = 39, R_STATIC = 42 };

// Page-locked host staging memory that grows on demand.
struct PinBuf {
    void* p = nullptr;
    size_t cap = 0;
    cudaError_t grow(size_t bytes)
    {
        if (bytes <= cap) return cudaSuccess;
        if (p) cudaFreeHost(p);
        p = nullptr;
        cap = 0;
        const size_t want = bytes + bytes / 8;
        cudaError_t e = cudaHostAlloc(&p, want, cudaHostAllocDefault);
        if (e == cudaSuccess) cap = want;
        return e;
    }
    void release()
    {
        if (p) cudaFreeHost(p);
        p = nullptr;
        cap = 0;
    }
};

thread_local std::string g_create_error;

}  // namespace

void vpm::set_thread_error(const char* msg) { g_create_error = msg; }

struct vpm_ctx {
    int device = 0;
    int num_sms = 0;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
    double timeout_s = 3600.0;
    std::mutex mu;
    std::string err;
    bool broken = false;
    int64_t launches = 0;
    // device copies of host matrices and SoA views of them
    DevBuf mat, mat2, x, g, s, st, xt;
    // compact staging of the drop-in call: per particle X, Gamma, sigma, static in; U, J, SFS out
    PinBuf hin, hout;
    DevBuf din, dout;
    // packing and split-K scratch
    DevBuf src_pack, order, partial, flag;
    // near-field: packed particles, and the lists (built on the device or uploaded)
    DevBuf leaf;
    NearScratch near;
    // the lists (with warp groups) last built here from device positions, for VPM_REUSE_LISTS
    NearLists near_last;
    bool near_ok = false;
    int64_t near_n = 0;
    const double* near_x = nullptr;
    int near_leaf = 0;
    double near_theta = 0.0;
    int sync_rc = 0;     // VPM status of the last wait made for the list builder
};

namespace {

struct DeviceGuard {
    int prev = -1;
    explicit DeviceGuard(int dev)
    {
        cudaGetDevice(&prev);
        if (prev != dev) cudaSetDevice(dev);
    }
    ~DeviceGuard()
    {
        int cur = -1;
        cudaGetDevice(&cur);
        if (prev >= 0 && cur != prev) cudaSetDevice(prev);
    }
};

int fail(vpm_ctx* c, int code, const char* fmt, ...) __attribute__((format(printf, 3, 4)));
int fail(vpm_ctx* c, int code, const char* fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    if (c) c->err = buf;
    else g_create_error = buf;
    return code;
}

int cuda_fail(vpm_ctx* c, cudaError_t e, const char* what)
{
    // A sticky error (e.g. an illegal address) poisons the context for good.
    cudaError_t last = cudaGetLastError();
    (void)last;
    if (e == cudaErrorIllegalAddress || e == cudaErrorLaunchFailure || e == cudaErrorIllegalInstruction ||
        e == cudaErrorMisalignedAddress || e == cudaErrorHardwareStackError)
        c->broken = true;
    return fail(c, VPM_ERR_CUDA, "%s: %s (%s)", what, cudaGetErrorString(e), cudaGetErrorName(e));
}

#define CK(call, what)                                   \
    do {                                                 \
        cudaError_t e_ = (call);                         \
        if (e_ != cudaSuccess) return cuda_fail(c, e_, what); \
    } while (0)

// Wait for the context stream with a bound; the host never blocks forever.
int bounded_wait(vpm_ctx* c)
{
    CK(cudaEventRecord(c->done, c->stream), "cudaEventRecord");
    auto t0 = std::chrono::steady_clock::now();
    int sleep_us = 2;
    for (;;) {
        cudaError_t q = cudaEventQuery(c->done);
        if (q == cudaSuccess) return VPM_OK;
        if (q != cudaErrorNotReady) return cuda_fail(c, q, "device work");
        double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        if (el > c->timeout_s) {
            c->broken = true;
            return fail(c, VPM_ERR_TIMEOUT, "device work did not finish within %.1f s", c->timeout_s);
        }
        // short sleeps: a wait ends at most ~50 us after the work (a step makes dozens of waits)
        std::this_thread::sleep_for(std::chrono::microseconds(sleep_us));
        if (sleep_us < 50) sleep_us *= 2;
    }
}

// SyncFn for the near-field list builder: a bounded wait whose status is kept in the context
cudaError_t near_sync(void* p)
{
    vpm_ctx* c = (vpm_ctx*)p;
    c->sync_rc = bounded_wait(c);
    return c->sync_rc == VPM_OK ? cudaSuccess : cudaErrorLaunchTimeout;
}

// a failure of the list builder: the wait's own status, a capacity error, or a CUDA error
int near_fail(vpm_ctx* c, cudaError_t e, const char* what)
{
    if (c->sync_rc != VPM_OK) return c->sync_rc;
    if (e == cudaErrorMemoryAllocation) {
        cudaGetLastError();
        return fail(c, VPM_ERR_CAPACITY, "%s: out of device memory", what);
    }
    return cuda_fail(c, e, what);
}

bool is_device_ptr(const void* p)
{
    if (!p) return false;
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

// ------------------------------------------------------------ matrix kernels
// Gather X, Gamma, sigma, static of the 46-row columns into SoA arrays and apply
// _reset_particles / _reset_particles_sfs (src/FLOWVPM_particlefield.jl:464-507).
__global__ void unpack_matrix(int64_t np, double* __restrict__ mat, int flags, double* __restrict__ x,
                              double* __restrict__ g, double* __restrict__ s, uint8_t* __restrict__ st)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= np) return;
    double* p = mat + (int64_t)VPM_NFIELDS * i;
    for (int k = 0; k < 3; k++) { x[3 * i + k] = p[R_X + k]; g[3 * i + k] = p[R_G + k]; }
    s[i] = p[R_SIG];
    const bool is_static = p[R_STATIC] != 0.0;
    st[i] = is_static ? 1 : 0;
    if (!is_static) {
        if (flags & VPM_RESET)
            for (int k = R_U; k < R_PSE + 3; k++) p[k] = 0.0;
        if (flags & VPM_RESET_SFS)
            for (int k = R_SFS; k < R_SFS + 3; k++) p[k] = 0.0;
    }
}

// the compact input rows (X, Gamma, sigma, static: 8 doubles a particle) to SoA
__global__ void unpack_compact(int64_t np, const double* __restrict__ in, double* __restrict__ x,
                               double* __restrict__ g, double* __restrict__ s, uint8_t* __restrict__ st)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= np) return;
    const double* p = in + 8 * i;
    for (int k = 0; k < 3; k++) { x[3 * i + k] = p[k]; g[3 * i + k] = p[3 + k]; }
    s[i] = p[6];
    st[i] = p[7] != 0.0 ? 1 : 0;
}

__global__ void positions_of_matrix(int64_t np, const double* __restrict__ mat, double* __restrict__ x)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= np) return;
    for (int k = 0; k < 3; k++) x[3 * i + k] = mat[(int64_t)VPM_NFIELDS * i + R_X + k];
}

// out[i] = a * in[i] (core sizes of the test filter)
__global__ void scale_copy(int64_t n, const double* __restrict__ in, double a, double* __restrict__ out)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) out[i] = a * in[i];
}

// out[i] = a[i] - b[i]
__global__ void sub_arrays(int64_t n, const double* __restrict__ a, const double* __restrict__ b, double* __restrict__ out)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) out[i] = a[i] - b[i];
}

// rows [r0, r1) of every column set to zero
__global__ void zero_rows(int64_t np, double* __restrict__ mat, int r0, int r1)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= np) return;
    for (int r = r0; r < r1; r++) mat[i * VPM_NFIELDS + r] = 0.0;
}

// Sets *flag if any of rows [r0, r1) of the first np columns is not finite.
__global__ void check_rows_finite(int64_t np, const double* __restrict__ mat, int r0, int r1, int* flag)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= np) return;
    const double* p = mat + (int64_t)VPM_NFIELDS * i;
    for (int k = r0; k < r1; k++)
        if (!isfinite(p[k])) { atomicOr(flag, 1); return; }
}

// FP32 pipe probe: 8 independent FFMA chains per thread, 16x unrolled.
__global__ void ffma_probe_kernel(float* out, int iters, float a, float b)
{
    float x[8];
#pragma unroll
    for (int k = 0; k < 8; k++) x[k] = threadIdx.x * 1e-3f + k;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int u = 0; u < 16; u++) {
#pragma unroll
            for (int k = 0; k < 8; k++) x[k] = fmaf(x[k], a, b);
        }
    }
    float s = 0.f;
#pragma unroll
    for (int k = 0; k < 8; k++) s += x[k];
    if (s == 1234.5678f) out[0] = s;  // keeps the chains live; never true in practice
}

// FP64 pipe probe: 8 independent DFMA chains per thread, 8x unrolled.
__global__ void dfma_probe_kernel(double* out, int iters, double a, double b)
{
    double x[8];
#pragma unroll
    for (int k = 0; k < 8; k++) x[k] = threadIdx.x * 1e-3 + k;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int u = 0; u < 8; u++) {
#pragma unroll
            for (int k = 0; k < 8; k++) x[k] = fma(x[k], a, b);
        }
    }
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < 8; k++) s += x[k];
    if (s == 1234.5678) out[0] = s;  // keeps the chains live; never true in practice
}

constexpr int EB = 256;  // threads per block of the O(N) helper kernels
inline unsigned nblk(int64_t n) { return (unsigned)((n + EB - 1) / EB); }

int check_kernel(vpm_ctx* c, int kernel, int precision)
{
    if (kernel < VPM_KERNEL_SINGULAR || kernel > VPM_KERNEL_WINCKELMANS)
        return fail(c, VPM_ERR_ARG, "unknown kernel id %d (expected 0..3: singular, gaussian, gaussianerf, winckelmans)", kernel);
    if (precision != VPM_FP64 && precision != VPM_FP32COMP)
        return fail(c, VPM_ERR_ARG, "unknown precision %d (expected 0 = FP64, 1 = FP32-comp)", precision);
    return VPM_OK;
}

// Grow the packing / scratch buffers for a UJ and (optionally) an Estr pass.
int ensure_work(vpm_ctx* c, int64_t nt, int64_t ns, int precision, bool estr, Workspace* w)
{
    size_t sp = uj_src_pack_bytes(ns, precision);
    if (estr) { size_t e = estr_src_pack_bytes(ns, precision); if (e > sp) sp = e; }
    const size_t ob = order_bytes(nt);
    const int nsplit = uj_num_splits(nt, ns, c->num_sms);
    const size_t pb = uj_partial_bytes(nt, nsplit);
    if (c->src_pack.grow(sp) != cudaSuccess || c->order.grow(ob) != cudaSuccess ||
        (pb && c->partial.grow(pb) != cudaSuccess)) {
        cudaGetLastError();
        return fail(c, VPM_ERR_CAPACITY, "could not allocate %zu B of packing/scratch memory", sp + ob + pb);
    }
    w->src_pack = c->src_pack.p; w->src_pack_bytes = c->src_pack.cap;
    w->order = c->order.p; w->order_bytes = c->order.cap;
    w->partial = (double*)c->partial.p; w->partial_bytes = c->partial.cap;
    return VPM_OK;
}

int grow(vpm_ctx* c, DevBuf& b, size_t bytes, const char* what)
{
    if (b.grow(bytes) != cudaSuccess) {
        cudaGetLastError();
        return fail(c, VPM_ERR_CAPACITY, "could not allocate %zu B for %s", bytes, what);
    }
    return VPM_OK;
}

#define RC(call)                   \
    do {                           \
        int rc_ = (call);          \
        if (rc_ != VPM_OK) return rc_; \
    } while (0)

int enter(vpm_ctx* c)
{
    if (c->broken) return fail(c, VPM_ERR_STATE, "context is unusable after an earlier device error: %s", c->err.c_str());
    c->err.clear();
    return VPM_OK;
}

}  // namespace

// =================================================================== ABI
// Host rows <-> compact staging, split over host threads.
template <class F>
static void host_parallel(int64_t n, F f)
{
    const unsigned hw = std::thread::hardware_concurrency();
    int nth = (int)std::min<int64_t>(hw ? hw : 1, 16);
    if (n < (1 << 15)) nth = 1;
    if (nth <= 1) { f(0, n); return; }
    std::vector<std::thread> th;
    const int64_t chunk = (n + nth - 1) / nth;
    for (int t = 0; t < nth; t++) {
        const int64_t a = t * chunk, b = std::min(n, a + chunk);
        if (a < b) th.emplace_back(f, a, b);
    }
    for (auto& x : th) x.join();
}

extern "C" {

int vpm_abi_version(void) { return VPM_ABI_VERSION; }

const char* vpm_build_info(void)
{
    return "libvpm_gb300 abi " "1" " sm_103a; UJ fp64 + fp32comp, Estr fp64 + fp32comp";
}

int vpm_ctx_create(vpm_ctx** out, int device)
{
    vpm::TraceRange trace_("vpm_ctx_create");
    if (!out) return fail(nullptr, VPM_ERR_ARG, "vpm_ctx_create: out is NULL");
    *out = nullptr;
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0) {
        cudaGetLastError();
        return fail(nullptr, VPM_ERR_NODEVICE, "no CUDA device available (%s)", cudaGetErrorString(e));
    }
    if (device < 0 || device >= n) return fail(nullptr, VPM_ERR_ARG, "device %d out of range (0..%d)", device, n - 1);
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, device) != cudaSuccess)
        return fail(nullptr, VPM_ERR_NODEVICE, "cudaGetDeviceProperties failed");
    if (!(prop.major == 10 && prop.minor == 3))
        return fail(nullptr, VPM_ERR_NODEVICE, "device %d is sm_%d%d; this library is built for sm_103a only",
                    device, prop.major, prop.minor);
    DeviceGuard dg(device);
    vpm_ctx* c = new vpm_ctx();
    c->device = device;
    c->num_sms = prop.multiProcessorCount;
    // a blocking stream: ordered with the legacy default stream's work both ways, so that
    // callers who queue their own work there (frameworks' default streams) need no events
    if (cudaStreamCreateWithFlags(&c->own_stream, cudaStreamDefault) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->done, cudaEventDisableTiming) != cudaSuccess) {
        cudaGetLastError();
        delete c;
        return fail(nullptr, VPM_ERR_CUDA, "could not create a stream/event on device %d", device);
    }
    c->stream = c->own_stream;
    *out = c;
    return VPM_OK;
}

int vpm_ctx_destroy(vpm_ctx* c)
{
    vpm::TraceRange trace_("vpm_ctx_destroy");
    if (!c) return VPM_OK;
    {
        std::lock_guard<std::mutex> lk(c->mu);
        DeviceGuard dg(c->device);
        if (!c->broken) cudaStreamSynchronize(c->stream);
        for (DevBuf* b : {&c->mat, &c->mat2, &c->x, &c->g, &c->s, &c->st, &c->xt, &c->src_pack, &c->order,
                          &c->partial, &c->flag, &c->leaf})
            b->release();
        c->near.release_all();
        for (DevBuf* b : {&c->din, &c->dout}) b->release();
        c->hin.release();
        c->hout.release();
        if (c->done) cudaEventDestroy(c->done);
        if (c->own_stream) cudaStreamDestroy(c->own_stream);
        cudaGetLastError();
    }
    delete c;
    return VPM_OK;
}

const char* vpm_last_error(const vpm_ctx* c) { return c ? c->err.c_str() : g_create_error.c_str(); }

int vpm_ctx_set_stream(vpm_ctx* c, void* stream)
{
    if (!c) return fail(nullptr, VPM_ERR_ARG, "vpm_ctx_set_stream: ctx is NULL");
    std::lock_guard<std::mutex> lk(c->mu);
    c->stream = stream ? (cudaStream_t)stream : c->own_stream;
    return VPM_OK;
}

int vpm_ctx_set_timeout(vpm_ctx* c, double seconds)
{
    if (!c) return fail(nullptr, VPM_ERR_ARG, "vpm_ctx_set_timeout: ctx is NULL");
    if (!(seconds > 0)) return fail(c, VPM_ERR_ARG, "timeout must be > 0 s");
    std::lock_guard<std::mutex> lk(c->mu);
    c->timeout_s = seconds;
    return VPM_OK;
}

int vpm_ctx_set_near_capacity(vpm_ctx* c, int64_t frontier_pairs, int64_t near_pairs)
{
    if (!c) return fail(nullptr, VPM_ERR_ARG, "vpm_ctx_set_near_capacity: ctx is NULL");
    if (frontier_pairs < 1 || near_pairs < 1 || frontier_pairs > ((int64_t)1 << 34) || near_pairs > ((int64_t)1 << 34))
        return fail(c, VPM_ERR_ARG, "vpm_ctx_set_near_capacity: capacities must be in 1..2^34 pairs");
    std::lock_guard<std::mutex> lk(c->mu);
    c->near.capF = (size_t)frontier_pairs;
    c->near.capN = (size_t)near_pairs;
    return VPM_OK;
}

int64_t vpm_launch_count(const vpm_ctx* c) { return c ? c->launches : 0; }

int vpm_probe_ffma(vpm_ctx* c, double* tflops)
{
    vpm::TraceRange trace_("vpm_probe_ffma");
    if (!c || !tflops) return fail(c, VPM_ERR_ARG, "vpm_probe_ffma: NULL argument");
    std::lock_guard<std::mutex> lk(c->mu);
    RC(enter(c));
    DeviceGuard dg(c->device);
    RC(grow(c, c->flag, sizeof(int), "flag"));
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0), "cudaEventCreate");
    CK(cudaEventCreate(&e1), "cudaEventCreate");
    const int blocks = c->num_sms * 8, threads = 256, iters = 4096;
    double best = 0.0;
    for (int rep = 0; rep < 4; rep++) {
        CK(cudaEventRecord(e0, c->stream), "cudaEventRecord");
        ffma_probe_kernel<<<blocks, threads, 0, c->stream>>>((float*)c->flag.p, iters, 0.9999999f, 1e-7f);
        CK(cudaEventRecord(e1, c->stream), "cudaEventRecord");
        c->launches++;
        RC(bounded_wait(c));
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, e0, e1), "cudaEventElapsedTime");
        const double flops = 2.0 * 16 * 8 * (double)iters * blocks * threads;
        if (rep > 0 && ms > 0) best = std::max(best, flops / (ms * 1e-3) / 1e12);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *tflops = best;
    return VPM_OK;
}

int vpm_probe_dfma(vpm_ctx* c, double* tflops)
{
    vpm::TraceRange trace_("vpm_probe_dfma");
    if (!c || !tflops) return fail(c, VPM_ERR_ARG, "vpm_probe_dfma: NULL argument");
    std::lock_guard<std::mutex> lk(c->mu);
    RC(enter(c));
    DeviceGuard dg(c->device);
    RC(grow(c, c->flag, sizeof(double), "flag"));
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0), "cudaEventCreate");
    CK(cudaEventCreate(&e1), "cudaEventCreate");
    const int blocks = c->num_sms * 8, threads = 256, iters = 256;
    double best = 0.0;
    for (int rep = 0; rep < 4; rep++) {
        CK(cudaEventRecord(e0, c->stream), "cudaEventRecord");
        dfma_probe_kernel<<<blocks, threads, 0, c->stream>>>((double*)c->flag.p, iters, 0.9999999, 1e-7);
        CK(cudaEventRecord(e1, c->stream), "cudaEventRecord");
        c->launches++;
        RC(bounded_wait(c));
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, e0, e1), "cudaEventElapsedTime");
        const double flops = 2.0 * 8 * 8 * (double)iters * blocks * threads;
        if (rep > 0 && ms > 0) best = std::max(best, flops / (ms * 1e-3) / 1e12);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *tflops = best;
    return VPM_OK;
}

// ------------------------------------------------------------- UJ_direct drop-in
// The drop-in call through the whole particle matrix: the matrix goes to the
// device, the kernels update its rows in place, the touched rows come back.
// Used when the old J of every particle feeds Estr (SFS without RESET).
static int uj_full_matrix(vpm_ctx* c, double* particles, int64_t np, int kernel, int precision, int flags)
{
    cudaStream_t st = c->stream;
    const size_t mat_bytes = (size_t)VPM_NFIELDS * np * sizeof(double);
    RC(grow(c, c->mat, mat_bytes, "particle matrix"));
    RC(grow(c, c->x, 3 * np * sizeof(double), "positions"));
    RC(grow(c, c->g, 3 * np * sizeof(double), "strengths"));
    RC(grow(c, c->s, np * sizeof(double), "core sizes"));
    RC(grow(c, c->st, np, "static flags"));
    RC(grow(c, c->flag, sizeof(int), "flag"));
    Workspace w;
    const bool sfs = (flags & VPM_SFS) != 0;
    RC(ensure_work(c, np, np, precision, sfs, &w));
    double* mat = (double*)c->mat.p;
    double* x = (double*)c->x.p;
    double* g = (double*)c->g.p;
    double* s = (double*)c->s.p;
    uint8_t* stf = (uint8_t*)c->st.p;

    CK(cudaMemcpyAsync(mat, particles, mat_bytes, cudaMemcpyHostToDevice, st), "H2D particle matrix");
    unpack_matrix<<<nblk(np), EB, 0, st>>>(np, mat, flags, x, g, s, stf);
    c->launches++;
    CK(cudaGetLastError(), "unpack_matrix");

    UJArgs a;
    a.nt = np; a.ns = np; a.xt = x; a.xs = x; a.gs = g; a.sgs = s;
    a.U = mat + R_U; a.ldU = VPM_NFIELDS; a.J = mat + R_J; a.ldJ = VPM_NFIELDS;
    a.kernel = kernel; a.precision = precision; a.self = true;
    CK(launch_uj(a, w, c->num_sms, st, &c->launches), "UJ kernels");
    if (sfs) {
        EstrArgs e;
        e.nt = np; e.ns = np;
        e.xt = x; e.Jt = mat + R_J; e.ldJt = VPM_NFIELDS; e.static_t = stf;
        e.xs = x; e.gs = g; e.sgs = s; e.Js = mat + R_J; e.ldJs = VPM_NFIELDS; e.static_s = stf;
        e.SFS = mat + R_SFS; e.ldS = VPM_NFIELDS;
        e.kernel = kernel; e.precision = precision;
        e.transposed = (flags & VPM_TRANSPOSED) != 0; e.self = true;
        CK(launch_estr(e, w, c->num_sms, st, &c->launches), "Estr kernels");
    }
    int* dflag = (int*)c->flag.p;
    if (flags & VPM_CHECK_FINITE) {
        CK(cudaMemsetAsync(dflag, 0, sizeof(int), st), "memset flag");
        check_rows_finite<<<nblk(np), EB, 0, st>>>(np, mat, R_U, R_PSE + 3, dflag);
        c->launches++;
        if (sfs) { check_rows_finite<<<nblk(np), EB, 0, st>>>(np, mat, R_SFS, R_SFS + 3, dflag); c->launches++; }
        CK(cudaGetLastError(), "check_rows_finite");
    }
    RC(bounded_wait(c));
    // rows 10:27 (U, vorticity, J, PSE) and, when touched, rows 40:42 (SFS)
    const size_t pitch = VPM_NFIELDS * sizeof(double);
    CK(cudaMemcpy2DAsync(particles + R_U, pitch, mat + R_U, pitch, 18 * sizeof(double), (size_t)np,
                         cudaMemcpyDeviceToHost, st), "D2H rows 10:27");
    if (flags & (VPM_SFS | VPM_RESET_SFS))
        CK(cudaMemcpy2DAsync(particles + R_SFS, pitch, mat + R_SFS, pitch, 3 * sizeof(double), (size_t)np,
                             cudaMemcpyDeviceToHost, st), "D2H rows 40:42");
    int hflag = 0;
    if (flags & VPM_CHECK_FINITE)
        CK(cudaMemcpyAsync(&hflag, dflag, sizeof(int), cudaMemcpyDeviceToHost, st), "D2H flag");
    CK(cudaStreamSynchronize(st), "D2H");
    if (hflag) return fail(c, VPM_ERR_NONFINITE, "vpm_uj: NaN or Inf in the computed U/J/SFS");
    return VPM_OK;
}

// The drop-in call with compact staging: only X, Gamma, sigma and the static
// flag go to the device (64 B a particle instead of the 368 B column), the
// kernels compute the U, J (and SFS) sums from zero, and the host applies them
// to the matrix with UJ_direct's rules: with RESET the non-static particles'
// rows 10:27 restart from zero, static ones accumulate; likewise RESET_SFS for
// rows 40:42.  Valid whenever Estr does not need the old J (RESET or no SFS):
// Estr reads J only of non-static particles, whose J is then the new sum.
static int uj_staged(vpm_ctx* c, double* particles, int64_t np, int kernel, int precision, int flags)
{
    cudaStream_t st = c->stream;
    const bool sfs = (flags & VPM_SFS) != 0;
    const int nout = sfs ? 15 : 12;
    RC(grow(c, c->x, 3 * np * sizeof(double), "positions"));
    RC(grow(c, c->g, 3 * np * sizeof(double), "strengths"));
    RC(grow(c, c->s, np * sizeof(double), "core sizes"));
    RC(grow(c, c->st, np, "static flags"));
    RC(grow(c, c->din, (size_t)8 * np * sizeof(double), "staged inputs"));
    RC(grow(c, c->dout, (size_t)15 * np * sizeof(double), "staged outputs"));
    if (c->hin.grow((size_t)8 * np * sizeof(double)) != cudaSuccess ||
        c->hout.grow((size_t)15 * np * sizeof(double)) != cudaSuccess) {
        cudaGetLastError();
        return fail(c, VPM_ERR_CAPACITY, "could not allocate %lld B of pinned host staging", (long long)(23 * 8 * np));
    }
    Workspace w;
    RC(ensure_work(c, np, np, precision, sfs, &w));
    double* hin = (double*)c->hin.p;
    double* hout = (double*)c->hout.p;
    host_parallel(np, [&](int64_t a, int64_t b) {
        for (int64_t i = a; i < b; i++) {
            const double* p = particles + (int64_t)VPM_NFIELDS * i;
            double* q = hin + 8 * i;
            for (int k = 0; k < 7; k++) q[k] = p[k];
            q[7] = p[R_STATIC];
        }
    });
    double* din = (double*)c->din.p;
    double* dU = (double*)c->dout.p;
    double* dJ = dU + 3 * np;
    double* dS = dJ + 9 * np;
    double* x = (double*)c->x.p;
    double* g = (double*)c->g.p;
    double* s = (double*)c->s.p;
    uint8_t* stf = (uint8_t*)c->st.p;
    CK(cudaMemcpyAsync(din, hin, (size_t)8 * np * sizeof(double), cudaMemcpyHostToDevice, st), "H2D staged inputs");
    unpack_compact<<<nblk(np), EB, 0, st>>>(np, din, x, g, s, stf);
    c->launches++;
    CK(cudaMemsetAsync(dU, 0, (size_t)nout * np * sizeof(double), st), "memset staged outputs");
    UJArgs a;
    a.nt = np; a.ns = np; a.xt = x; a.xs = x; a.gs = g; a.sgs = s;
    a.U = dU; a.ldU = 3; a.J = dJ; a.ldJ = 9;
    a.kernel = kernel; a.precision = precision; a.self = true;
    CK(launch_uj(a, w, c->num_sms, st, &c->launches), "UJ kernels");
    if (sfs) {
        EstrArgs e;
        e.nt = np; e.ns = np;
        e.xt = x; e.Jt = dJ; e.ldJt = 9; e.static_t = stf;
        e.xs = x; e.gs = g; e.sgs = s; e.Js = dJ; e.ldJs = 9; e.static_s = stf;
        e.SFS = dS; e.ldS = 3;
        e.kernel = kernel; e.precision = precision;
        e.transposed = (flags & VPM_TRANSPOSED) != 0; e.self = true;
        CK(launch_estr(e, w, c->num_sms, st, &c->launches), "Estr kernels");
    }
    CK(cudaMemcpyAsync(hout, dU, (size_t)nout * np * sizeof(double), cudaMemcpyDeviceToHost, st), "D2H staged outputs");
    RC(bounded_wait(c));
    const bool reset = (flags & VPM_RESET) != 0, reset_sfs = (flags & VPM_RESET_SFS) != 0;
    const double* hU = hout;
    const double* hJ = hU + 3 * np;
    const double* hS = hJ + 9 * np;
    std::atomic<int> bad{0};
    host_parallel(np, [&](int64_t a0, int64_t b0) {
        int nonfinite = 0;
        for (int64_t i = a0; i < b0; i++) {
            double* p = particles + (int64_t)VPM_NFIELDS * i;
            const bool is_static = p[R_STATIC] != 0.0;
            if (reset && !is_static)
                for (int k = R_U; k < R_PSE + 3; k++) p[k] = 0.0;
            for (int k = 0; k < 3; k++) p[R_U + k] += hU[3 * i + k];
            for (int k = 0; k < 9; k++) p[R_J + k] += hJ[9 * i + k];
            if (reset_sfs && !is_static)
                for (int k = 0; k < 3; k++) p[R_SFS + k] = 0.0;
            if (sfs)
                for (int k = 0; k < 3; k++) p[R_SFS + k] += hS[3 * i + k];
            if (flags & VPM_CHECK_FINITE) {
                for (int k = R_U; k < R_PSE + 3; k++) nonfinite |= !std::isfinite(p[k]);
                if (sfs)
                    for (int k = 0; k < 3; k++) nonfinite |= !std::isfinite(p[R_SFS + k]);
            }
        }
        if (nonfinite) bad = 1;
    });
    if (bad) return fail(c, VPM_ERR_NONFINITE, "vpm_uj: NaN or Inf in the computed U/J/SFS");
    return VPM_OK;
}

int vpm_uj(vpm_ctx* c, double* particles, int64_t ld, int64_t np, int kernel, int precision, int flags)
{
    vpm::TraceRange trace_("vpm_uj");
    if (!c) return fail(nullptr, VPM_ERR_ARG, "vpm_uj: ctx is NULL");
    std::lock_guard<std::mutex> lk(c->mu);
    RC(enter(c));
    if (!particles && np > 0) return fail(c, VPM_ERR_ARG, "vpm_uj: particles is NULL");
    if (ld != VPM_NFIELDS) return fail(c, VPM_ERR_ARG, "vpm_uj: ld must be %d (got %lld)", VPM_NFIELDS, (long long)ld);
    if (np < 0 || np > (int64_t)INT32_MAX) return fail(c, VPM_ERR_ARG, "vpm_uj: np=%lld out of range", (long long)np);
    if (flags & ~(VPM_RESET | VPM_RESET_SFS | VPM_SFS | VPM_TRANSPOSED | VPM_CHECK_FINITE))
        return fail(c, VPM_ERR_ARG, "vpm_uj: unknown flag bits 0x%x", flags);
    RC(check_kernel(c, kernel, precision));
    if (np == 0) return VPM_OK;
    DeviceGuard dg(c->device);
    if ((flags & VPM_SFS) && !(flags & VPM_RESET)) return uj_full_matrix(c, particles, np, kernel, precision, flags);
    return uj_staged(c, particles, np, kernel, precision, flags);
}

int vpm_uj_cross(vpm_ctx* c, const double* src, int64_t ld_src, int64_t ns, double* tgt, int64_t ld_tgt,
                 int64_t nt, int kernel, int precision)
{
    vpm::TraceRange trace_("vpm_uj_cross");
    if (!c) return fail(nullptr, VPM_ERR_ARG, "vpm_uj_cross: ctx is NULL");
    std::lock_guard<std::mutex> lk(c->mu);
    RC(enter(c));
    if ((!src && ns > 0) || (!tgt && nt > 0)) return fail(c, VPM_ERR_ARG, "vpm_uj_cross: NULL matrix");
    if (ld_src != VPM_NFIELDS || ld_tgt != VPM_NFIELDS)
        return fail(c, VPM_ERR_ARG, "vpm_uj_cross: ld must be %d", VPM_NFIELDS);
    if (ns < 0 || nt < 0 || ns > (int64_t)INT32_MAX || nt > (int64_t)INT32_MAX)
        return fail(c, VPM_ERR_ARG, "vpm_uj_cross: sizes out of range");
    RC(check_kernel(c, kernel, precision));
    if (ns == 0 || nt == 0) return VPM_OK;
    DeviceGuard dg(c->device);
    cudaStream_t st = c->stream;
    RC(grow(c, c->mat, (size_t)VPM_NFIELDS * ns * sizeof(double), "source matrix"));
    RC(grow(c, c->mat2, (size_t)VPM_NFIELDS * nt * sizeof(double), "target matrix"));
    RC(grow(c, c->x, 3 * ns * sizeof(double), "positions"));
    RC(grow(c, c->g, 3 * ns * sizeof(double), "strengths"));
    RC(grow(c, c->s, ns * sizeof(double), "core sizes"));
    RC(grow(c, c->st, ns, "static flags"));
    RC(grow(c, c->xt, 3 * nt * sizeof(double), "target positions"));
    Workspace w;
    RC(ensure_work(c, nt, ns, precision, false, &w));
    double* ms = (double*)c->mat.p;
    double* mt = (double*)c->mat2.p;
    CK(cudaMemcpyAsync(ms, src, (size_t)VPM_NFIELDS * ns * sizeof(double), cudaMemcpyHostToDevice, st), "H2D src");
    CK(cudaMemcpyAsync(mt, tgt, (size_t)VPM_NFIELDS * nt * sizeof(double), cudaMemcpyHostToDevice, st), "H2D tgt");
    unpack_matrix<<<nblk(ns), EB, 0, st>>>(ns, ms, 0, (double*)c->x.p, (double*)c->g.p, (double*)c->s.p,
                                           (uint8_t*)c->st.p);
    positions_of_matrix<<<nblk(nt), EB, 0, st>>>(nt, mt, (double*)c->xt.p);
    c->launches += 2;
    CK(cudaGetLastError(), "unpack");
    UJArgs a;
    a.nt = nt; a.ns = ns; a.xt = (double*)c->xt.p; a.xs = (double*)c->x.p; a.gs = (double*)c->g.p;
    a.sgs = (double*)c->s.p; a.U = mt + R_U; a.ldU = VPM_NFIELDS; a.J = mt + R_J; a.ldJ = VPM_NFIELDS;
    a.kernel = kernel; a.precision = precision; a.self = false;
    CK(launch_uj(a, w, c->num_sms, st, &c->launches), "UJ kernels");
    RC(bounded_wait(c));
    const size_t pitch = VPM_NFIELDS * sizeof(double);
    CK(cudaMemcpy2DAsync(tgt + R_U, pitch, mt + R_U, pitch, 15 * sizeof(double), (size_t)nt,
                         cudaMemcpyDeviceToHost, st), "D2H rows 10:24");
    CK(cudaStreamSynchronize(st), "D2H");
    return VPM_OK;
}

// --------------------------------------------------------- device-pointer API
int vpm_uj_dev(vpm_ctx* c, int64_t nt, const double* xt, int64_t ns, const double* xs, const double* gs,
               const double* sgs, double* U, double* J, int kernel, int precision)
{
    vpm::TraceRange trace_("vpm_uj_dev");
    if (!c) return fail(nullptr, VPM_ERR_ARG, "vpm_uj_dev: ctx is NULL");
    std::lock_guard<std::mutex> lk(c->mu);
    RC(enter(c));
    if (nt < 0 || ns < 0 || nt > (int64_t)INT32_MAX || ns > (int64_t)INT32_MAX)
        return fail(c, VPM_ERR_ARG, "vpm_uj_dev: sizes out of range");
    RC(check_kernel(c, kernel, precision));
    if (nt == 0 || ns == 0) return VPM_OK;
    DeviceGuard dg(c->device);
    if (!is_device_ptr(xt) || !is_device_ptr(xs) || !is_device_ptr(gs) || !is_device_ptr(sgs) ||
        !is_device_ptr(U) || !is_device_ptr(J))
        return fail(c, VPM_ERR_ARG, "vpm_uj_dev: every array must be a device pointer");
    Workspace w;
    const bool self = (xt == xs) && (nt == ns);
    RC(ensure_work(c, nt, ns, precision, false, &w));
    UJArgs a;
    a.nt = nt; a.ns = ns; a.xt = xt; a.xs = xs; a.gs = gs; a.sgs = sgs;
    a.U = U; a.ldU = 3; a.J = J; a.ldJ = 9; a.kernel = kernel; a.precision = precision; a.self = self;
    CK(launch_uj(a, w, c->num_sms, c->stream, &c->launches), "UJ kernels");
    return bounded_wait(c);
}

int vpm_estr_dev(vpm_ctx* c, int64_t nt, const double* xt, const double* Jt, const uint8_t* static_t, int64_t ns,
                 const double* xs, const double* gs, const double* sgs, const double* Js, const uint8_t* static_s,
                 double* SFS, int kernel, int precision, int flags)
{
    vpm::TraceRange trace_("vpm_estr_dev");
    if (!c) return fail(nullptr, VPM_ERR_ARG, "vpm_estr_dev: ctx is NULL");
    std::lock_guard<std::mutex> lk(c->mu);
    RC(enter(c));
    if (nt < 0 || ns < 0 || nt > (int64_t)INT32_MAX || ns > (int64_t)INT32_MAX)
        return fail(c, VPM_ERR_ARG, "vpm_estr_dev: sizes out of range");
    if (flags & ~VPM_TRANSPOSED) return fail(c, VPM_ERR_ARG, "vpm_estr_dev: only VPM_TRANSPOSED is accepted in flags");
    RC(check_kernel(c, kernel, precision));
    if (nt == 0 || ns == 0) return VPM_OK;
    DeviceGuard dg(c->device);
    if (!is_device_ptr(xt) || !is_device_ptr(Jt) || !is_device_ptr(xs) || !is_device_ptr(gs) ||
        !is_device_ptr(sgs) || !is_device_ptr(Js) || !is_device_ptr(SFS) ||
        (static_t && !is_device_ptr(static_t)) || (static_s && !is_device_ptr(static_s)))
        return fail(c, VPM_ERR_ARG, "vpm_estr_dev: every array must be a device pointer");
    Workspace w;
    RC(ensure_work(c, nt, ns, precision, true, &w));
    EstrArgs e;
    e.nt = nt; e.ns = ns; e.xt = xt; e.Jt = Jt; e.ldJt = 9; e.static_t = static_t;
    e.xs = xs; e.gs = gs; e.sgs = sgs; e.Js = Js; e.ldJs = 9; e.static_s = static_s;
    e.SFS = SFS; e.ldS = 3; e.kernel = kernel; e.precision = precision;
    e.transposed = (flags & VPM_TRANSPOSED) != 0;
    e.self = (xt == xs) && (nt == ns);
    CK(launch_estr(e, w, c->num_sms, c->stream, &c->launches), "Estr kernels");
    return bounded_wait(c);
}

// --------------------------------------------------------------- zeta (RBF basis)
int vpm_zeta_dev(vpm_ctx* c, int64_t nt, const double* xt, int64_t ns, const double* xs, const double* gs,
                 const double* sgs, double* W, int kernel, int precision)
{
    vpm::TraceRange trace_("vpm_zeta_dev");
    if (!c) return fail(nullptr, VPM_ERR_ARG, "vpm_zeta_dev: ctx is NULL");
    std::lock_guard<std::mutex> lk(c->mu);
    RC(enter(c));
    if (nt < 0 || ns < 0 || nt > (int64_t)INT32_MAX || ns > (int64_t)INT32_MAX)
        return fail(c, VPM_ERR_ARG, "vpm_zeta_dev: sizes out of range");
    RC(check_kernel(c, kernel, precision));
    if (nt == 0 || ns == 0) return VPM_OK;
    DeviceGuard dg(c->device);
    if (!is_device_ptr(xt) || !is_device_ptr(xs) || !is_device_ptr(gs) || !is_device_ptr(sgs) || !is_device_ptr(W))
        return fail(c, VPM_ERR_ARG, "vpm_zeta_dev: every array must be a device pointer");
    Workspace w;
    RC(ensure_work(c, nt, ns, precision, true, &w));
    EstrArgs e;
    e.nt = nt; e.ns = ns; e.xt = xt; e.Jt = nullptr; e.ldJt = 9; e.static_t = nullptr;
    e.xs = xs; e.gs = gs; e.sgs = sgs; e.Js = nullptr; e.ldJs = 9; e.static_s = nullptr;
    e.SFS = W; e.ldS = 3; e.kernel = kernel; e.precision = precision;
    e.transposed = true; e.self = (xt == xs) && (nt == ns); e.zeta = true;
    CK(launch_estr(e, w, c->num_sms, c->stream, &c->launches), "zeta kernels");
    return bounded_wait(c);
}

int vpm_zeta(vpm_ctx* c, double* particles, int64_t ld, int64_t np, int kernel, int precision)
{
    vpm::TraceRange trace_("vpm_zeta");
    if (!c) return fail(nullptr, VPM_ERR_ARG, "vpm_zeta: ctx is NULL");
    std::lock_guard<std::mutex> lk(c->mu);
    RC(enter(c));
    if (!particles && np > 0) return fail(c, VPM_ERR_ARG, "vpm_zeta: particles is NULL");
    if (ld != VPM_NFIELDS) return fail(c, VPM_ERR_ARG, "vpm_zeta: ld must be %d (got %lld)", VPM_NFIELDS, (long long)ld);
    if (np < 0 || np > (int64_t)INT32_MAX) return fail(c, VPM_ERR_ARG, "vpm_zeta: np=%lld out of range", (long long)np);
    RC(check_kernel(c, kernel, precision));
    if (np == 0) return VPM_OK;
    DeviceGuard dg(c->device);
    cudaStream_t st = c->stream;
    const size_t mat_bytes = (size_t)VPM_NFIELDS * np * sizeof(double);
    RC(grow(c, c->mat, mat_bytes, "particle matrix"));
    RC(grow(c, c->x, 3 * np * sizeof(double), "positions"));
    RC(grow(c, c->g, 3 * np * sizeof(double), "strengths"));
    RC(grow(c, c->s, np * sizeof(double), "core sizes"));
    RC(grow(c, c->st, np, "static flags"));
    Workspace w;
    RC(ensure_work(c, np, np, precision, true, &w));
    double* mat = (double*)c->mat.p;
    double* x = (double*)c->x.p;
    double* g = (double*)c->g.p;
    double* s = (double*)c->s.p;
    CK(cudaMemcpyAsync(mat, particles, mat_bytes, cudaMemcpyHostToDevice, st), "H2D particle matrix");
    unpack_matrix<<<nblk(np), EB, 0, st>>>(np, mat, 0, x, g, s, (uint8_t*)c->st.p);
    zero_rows<<<nblk(np), EB, 0, st>>>(np, mat, R_J, R_J + 3);   // J[1:3] of every particle, statics included
    c->launches += 2;
    CK(cudaGetLastError(), "unpack_matrix");
    EstrArgs e;
    e.nt = np; e.ns = np; e.xt = x; e.Jt = nullptr; e.ldJt = VPM_NFIELDS; e.static_t = nullptr;
    e.xs = x; e.gs = g; e.sgs = s; e.Js = nullptr; e.ldJs = VPM_NFIELDS; e.static_s = nullptr;
    e.SFS = mat + R_J; e.ldS = VPM_NFIELDS; e.kernel = kernel; e.precision = precision;
    e.transposed = true; e.self = true; e.zeta = true;
    CK(launch_estr(e, w, c->num_sms, st, &c->launches), "zeta kernels");
    RC(bounded_wait(c));
    const size_t pitch = VPM_NFIELDS * sizeof(double);
    CK(cudaMemcpy2DAsync(particles + R_J, pitch, mat + R_J, pitch, 3 * sizeof(double), (size_t)np,
                         cudaMemcpyDeviceToHost, st), "D2H rows 16:18");
    return bounded_wait(c);
}

// ------------------------------------------------- dynamic SFS test-filter differences
int vpm_dynamic_diff_dev(vpm_ctx* c, int64_t n, const double* x, const double* gam, const double* sig,
                         const double* J, double alpha, double* dJ, double* dSFS, int kernel, int precision,
                         int flags)
{
    vpm::TraceRange trace_("vpm_dynamic_diff_dev");
    const char* fn = "vpm_dynamic_diff_dev";
    if (!c) return fail(nullptr, VPM_ERR_ARG, "%s: ctx is NULL", fn);
    std::lock_guard<std::mutex> lk(c->mu);
    RC(enter(c));
    if (n < 0 || n > (int64_t)INT32_MAX) return fail(c, VPM_ERR_ARG, "%s: n out of range", fn);
    if (!(alpha > 0.0 && alpha < 1.0)) return fail(c, VPM_ERR_ARG, "%s: alpha must be in (0, 1)", fn);
    if (flags & ~VPM_TRANSPOSED) return fail(c, VPM_ERR_ARG, "%s: only VPM_TRANSPOSED is accepted in flags", fn);
    RC(check_kernel(c, kernel, precision));
    if (n == 0) return VPM_OK;
    DeviceGuard dg(c->device);
    if (!is_device_ptr(x) || !is_device_ptr(gam) || !is_device_ptr(sig) || !is_device_ptr(J) || !is_device_ptr(dJ) ||
        !is_device_ptr(dSFS))
        return fail(c, VPM_ERR_ARG, "%s: every array must be a device pointer", fn);
    cudaStream_t st = c->stream;
    Workspace w;
    RC(ensure_work(c, n, n, precision, true, &w));
    RC(grow(c, c->s, n * sizeof(double), "test-filter core sizes"));
    double* sig_a = (double*)c->s.p;
    scale_copy<<<nblk(n), EB, 0, st>>>(n, sig, alpha, sig_a);
    c->launches++;
    const bool tr = (flags & VPM_TRANSPOSED) != 0;
    EstrArgs e;
    e.nt = n; e.ns = n; e.xt = x; e.ldJt = 9; e.static_t = nullptr;
    e.xs = x; e.gs = gam; e.ldJs = 9; e.static_s = nullptr;
    e.ldS = 3; e.kernel = kernel; e.precision = precision; e.transposed = tr; e.self = true;
    if (precision == VPM_FP32COMP) {
        CK(cudaMemsetAsync(dJ, 0, 9 * n * sizeof(double), st), "memset dJ");
        CK(cudaMemsetAsync(dSFS, 0, 3 * n * sizeof(double), st), "memset dSFS");
        CK(launch_uj_filter_diff(n, x, gam, sig, alpha, dJ, kernel, w, st, &c->launches), "filter-difference UJ");
        // the weight difference at J, then an ordinary Estr of dJ at alpha sigma
        e.Jt = J; e.Js = J; e.sgs = sig; e.SFS = dSFS; e.dz_alpha = alpha;
        CK(launch_estr(e, w, c->num_sms, st, &c->launches), "weight-difference Estr");
        e.Jt = dJ; e.Js = dJ; e.sgs = sig_a; e.dz_alpha = 0.0;
        CK(launch_estr(e, w, c->num_sms, st, &c->launches), "test-filter Estr");
    } else {
        // FP64: the reference's two evaluations, then their differences
        RC(grow(c, c->mat2, (size_t)18 * n * sizeof(double), "test-filter scratch"));
        double* Ua = (double*)c->mat2.p;
        double* Ja = Ua + 3 * n;
        double* Sa = Ja + 9 * n;
        double* S0 = Sa + 3 * n;
        CK(cudaMemsetAsync(Ua, 0, (size_t)18 * n * sizeof(double), st), "memset scratch");
        UJArgs a;
        a.nt = n; a.ns = n; a.xt = x; a.xs = x; a.gs = gam; a.sgs = sig_a;
        a.U = Ua; a.ldU = 3; a.J = Ja; a.ldJ = 9; a.kernel = kernel; a.precision = precision; a.self = true;
        CK(launch_uj(a, w, c->num_sms, st, &c->launches), "test-filter UJ");
        e.Jt = Ja; e.Js = Ja; e.sgs = sig_a; e.SFS = Sa;
        CK(launch_estr(e, w, c->num_sms, st, &c->launches), "test-filter Estr");
        e.Jt = J; e.Js = J; e.sgs = sig; e.SFS = S0;
        CK(launch_estr(e, w, c->num_sms, st, &c->launches), "Estr");
        sub_arrays<<<nblk(9 * n), EB, 0, st>>>(9 * n, Ja, J, dJ);
        sub_arrays<<<nblk(3 * n), EB, 0, st>>>(3 * n, Sa, S0, dSFS);
        c->launches += 2;
        CK(cudaGetLastError(), "differences");
    }
    return bounded_wait(c);
}

static int near_check(vpm_ctx* c, const char* fn, int64_t n, const double* x, const double* gam,
                      const double* sig, const uint8_t* static_flags, double* U, double* J, double* SFS,
                      int kernel, int precision, int flags)
{
    if (n < 0 || n > (int64_t)1 << 30) return fail(c, VPM_ERR_ARG, "%s: n out of range", fn);
    if (flags & ~(VPM_SFS | VPM_TRANSPOSED))
        return fail(c, VPM_ERR_ARG, "%s: only VPM_SFS and VPM_TRANSPOSED are accepted", fn);
    RC(check_kernel(c, kernel, precision));
    if (n == 0) return VPM_OK;
    const bool sfs = (flags & VPM_SFS) != 0;
    if (!is_device_ptr(x) || !is_device_ptr(gam) || !is_device_ptr(sig) || !is_device_ptr(U) ||
        !is_device_ptr(J) || (sfs && !is_device_ptr(SFS)) || (static_flags && !is_device_ptr(static_flags)))
        return fail(c, VPM_ERR_ARG, "%s: every array must be a device pointer", fn);
    return VPM_OK;
}

// The near lists and warp groups of the positions x: the context's last ones when the
// caller asks (VPM_REUSE_LISTS) and they were built from the same array, size, leaf size
// and theta, else built now (and kept for the next call).
static int near_lists(vpm_ctx* c, int64_t n, const double* x, int leaf_size, double theta, bool reuse,
                      NearLists* L)
{
    if (reuse && c->near_ok && c->near_n == n && c->near_x == x && c->near_leaf == leaf_size &&
        c->near_theta == theta) {
        *L = c->near_last;
        return VPM_OK;
    }
    c->near_ok = false;
    cudaError_t e = near_build(c->near, n, x, leaf_size, theta, c->stream, near_sync, c, L, &c->launches);
    if (e != cudaSuccess) return near_fail(c, e, "octree and leaf-pair lists");
    e = near_groups(c->near, L, c->stream, near_sync, c, &c->launches);
    if (e != cudaSuccess) return near_fail(c, e, "near-field warp groups");
    c->near_last = *L;
    c->near_ok = true;
    c->near_n = n; c->near_x = x; c->near_leaf = leaf_size; c->near_theta = theta;
    return VPM_OK;
}

static int near_run(vpm_ctx* c, NearLists& L, int64_t n, const double* x, const double* gam, const double* sig,
                    const uint8_t* static_flags, double* U, double* J, double* SFS, int kernel, int precision,
                    int flags, int64_t* stats)
{
    RC(grow(c, c->leaf, leaf_work_bytes(n), "near-field packs"));
    LeafArgs a;
    a.n = n; a.x = x; a.gam = gam; a.sig = sig; a.U = U; a.J = J; a.SFS = SFS; a.static_flags = static_flags;
    a.kernel = kernel; a.precision = precision; a.sfs = (flags & VPM_SFS) != 0;
    a.transposed = (flags & VPM_TRANSPOSED) != 0;
    CK(launch_leaflist(a, L, c->leaf.p, c->stream, &c->launches), "near-field P2P kernels");
    RC(bounded_wait(c));
    if (stats) {
        stats[0] = L.nleaves;
        stats[1] = L.nlpairs;
        stats[2] = L.pairs;
    }
    return VPM_OK;
}

int vpm_p2p_leaflist_dev(vpm_ctx* c, int64_t n, const double* x, const double* gam, const double* sig,
                         const uint8_t* static_flags, double* U, double* J, double* SFS, int leaf_size,
                         double theta, int kernel, int precision, int flags, int64_t* stats)
{
    vpm::TraceRange trace_("vpm_p2p_leaflist_dev");
    const char* fn = "vpm_p2p_leaflist_dev";
    if (!c) return fail(nullptr, VPM_ERR_ARG, "%s: ctx is NULL", fn);
    std::lock_guard<std::mutex> lk(c->mu);
    RC(enter(c));
    if (stats) stats[0] = stats[1] = stats[2] = 0;
    if (leaf_size < 1 || leaf_size > LEAF_SIZE_MAX)
        return fail(c, VPM_ERR_ARG, "%s: leaf_size must be in 1..%d", fn, LEAF_SIZE_MAX);
    if (!(theta >= 0.0 && theta <= 1.0e6)) return fail(c, VPM_ERR_ARG, "%s: bad theta", fn);
    DeviceGuard dg(c->device);
    RC(near_check(c, fn, n, x, gam, sig, static_flags, U, J, SFS, kernel, precision, flags & ~VPM_REUSE_LISTS));
    if (n == 0) return VPM_OK;
    NearLists L;
    RC(near_lists(c, n, x, leaf_size, theta, (flags & VPM_REUSE_LISTS) != 0, &L));
    return near_run(c, L, n, x, gam, sig, static_flags, U, J, SFS, kernel, precision, flags & ~VPM_REUSE_LISTS,
                    stats);
}

int vpm_rk3_stage_dev(vpm_ctx* c, int64_t n, double a, double b, double dt, const double* Uinf, double f, double g,
                      double zeta0, double nu, int flags, double* x, double* gam, double* sig, const double* U,
                      const double* J, const double* SFS, const double* C, double* M)
{
    vpm::TraceRange trace_("vpm_rk3_stage_dev");
    const char* fn = "vpm_rk3_stage_dev";
    if (!c) return fail(nullptr, VPM_ERR_ARG, "%s: ctx is NULL", fn);
    std::lock_guard<std::mutex> lk(c->mu);
    RC(enter(c));
    if (n < 0 || n > (int64_t)INT32_MAX) return fail(c, VPM_ERR_ARG, "%s: n out of range", fn);
    if (flags & ~VPM_TRANSPOSED) return fail(c, VPM_ERR_ARG, "%s: only VPM_TRANSPOSED is accepted in flags", fn);
    if (!Uinf) return fail(c, VPM_ERR_ARG, "%s: Uinf is NULL", fn);
    if (!(std::isfinite(a) && std::isfinite(b) && std::isfinite(dt) && std::isfinite(f) && std::isfinite(g) &&
          std::isfinite(zeta0) && zeta0 != 0.0 && std::isfinite(nu) && 1.0 + 3.0 * f != 0.0))
        return fail(c, VPM_ERR_ARG, "%s: bad scalar argument", fn);
    if (n == 0) return VPM_OK;
    DeviceGuard dg(c->device);
    if (!is_device_ptr(x) || !is_device_ptr(gam) || !is_device_ptr(sig) || !is_device_ptr(U) || !is_device_ptr(J) ||
        !is_device_ptr(M) || (SFS && (!is_device_ptr(SFS) || !C || !is_device_ptr(C))))
        return fail(c, VPM_ERR_ARG, "%s: every array must be a device pointer (C with SFS)", fn);
    StageArgs s;
    s.n = n; s.a = a; s.b = b; s.dt = dt; s.f = f; s.g = g; s.zeta0 = zeta0; s.nu = nu;
    for (int k = 0; k < 3; k++) s.uinf[k] = Uinf[k];
    s.transposed = (flags & VPM_TRANSPOSED) != 0;
    s.x = x; s.gam = gam; s.sig = sig; s.U = U; s.J = J; s.SFS = SFS; s.C = SFS ? C : nullptr; s.M = M;
    CK(launch_rk3_stage(s, c->stream, &c->launches), "RK3 stage");
    return bounded_wait(c);
}

int vpm_relax_dev(vpm_ctx* c, int64_t n, double rlxf, const double* J, double* gam)
{
    vpm::TraceRange trace_("vpm_relax_dev");
    const char* fn = "vpm_relax_dev";
    if (!c) return fail(nullptr, VPM_ERR_ARG, "%s: ctx is NULL", fn);
    std::lock_guard<std::mutex> lk(c->mu);
    RC(enter(c));
    if (n < 0 || n > (int64_t)INT32_MAX) return fail(c, VPM_ERR_ARG, "%s: n out of range", fn);
    if (!std::isfinite(rlxf)) return fail(c, VPM_ERR_ARG, "%s: bad rlxf", fn);
    if (n == 0) return VPM_OK;
    DeviceGuard dg(c->device);
    if (!is_device_ptr(J) || !is_device_ptr(gam)) return fail(c, VPM_ERR_ARG, "%s: device pointers required", fn);
    CK(launch_relax(n, rlxf, J, gam, c->stream, &c->launches), "relaxation");
    return bounded_wait(c);
}

int vpm_dynamic_after_dev(vpm_ctx* c, int64_t n, double alpha, double rlxf, double minC, double maxC, double zeta0,
                          int flags, const double* gam, const double* sig, const double* J, const double* SFS,
                          double* C, double* M)
{
    vpm::TraceRange trace_("vpm_dynamic_after_dev");
    const char* fn = "vpm_dynamic_after_dev";
    if (!c) return fail(nullptr, VPM_ERR_ARG, "%s: ctx is NULL", fn);
    std::lock_guard<std::mutex> lk(c->mu);
    RC(enter(c));
    if (n < 0 || n > (int64_t)INT32_MAX) return fail(c, VPM_ERR_ARG, "%s: n out of range", fn);
    if (flags & ~(VPM_TRANSPOSED | VPM_DYN_FORCE_POSITIVE | VPM_DYN_CLIP_BACKSCATTER | VPM_DYN_SUBTRACT))
        return fail(c, VPM_ERR_ARG, "%s: unknown flags", fn);
    if (!(std::isfinite(alpha) && std::isfinite(rlxf) && !std::isnan(minC) && !std::isnan(maxC) &&
          std::isfinite(zeta0) && zeta0 != 0.0))
        return fail(c, VPM_ERR_ARG, "%s: bad scalar argument", fn);
    // the reference's error cases (src/FLOWVPM_subfilterscale.jl:549-556)
    if (minC < 0.0) return fail(c, VPM_ERR_ARG, "Invalid C bounds: Got a negative bound for minC (%g)", minC);
    if (maxC < 0.0) return fail(c, VPM_ERR_ARG, "Invalid C bounds: Got a negative bound for maxC (%g)", maxC);
    if (minC > maxC) return fail(c, VPM_ERR_ARG, "Invalid C bounds: minC > maxC (%g > %g)", minC, maxC);
    if (n == 0) return VPM_OK;
    DeviceGuard dg(c->device);
    if (!is_device_ptr(gam) || !is_device_ptr(sig) || !is_device_ptr(SFS) || !is_device_ptr(C) ||
        !is_device_ptr(M) || ((flags & VPM_DYN_SUBTRACT) && !is_device_ptr(J)))
        return fail(c, VPM_ERR_ARG, "%s: device pointers required", fn);
    RC(grow(c, c->flag, sizeof(int), "flag"));
    int* dflag = (int*)c->flag.p;
    CK(cudaMemsetAsync(dflag, 0, sizeof(int), c->stream), "memset flag");
    DynAfterArgs d;
    d.n = n; d.alpha = alpha; d.rlxf = rlxf; d.minC = minC; d.maxC = maxC; d.zeta0 = zeta0; d.flags = flags;
    d.gam = gam; d.sig = sig; d.J = J; d.SFS = SFS; d.C = C; d.M = M;
    CK(launch_dynamic_after(d, dflag, c->stream, &c->launches), "dynamic procedure");
    RC(bounded_wait(c));   // the kernel has finished: the flag's copy cannot block on it
    int hflag = 0;
    CK(cudaMemcpy(&hflag, dflag, sizeof(int), cudaMemcpyDeviceToHost), "D2H flag");
    if (hflag) return fail(c, VPM_ERR_NONFINITE, "%s: NaN in dynamicprocedure_pseudo3level_afterUJ", fn);
    return VPM_OK;
}

int vpm_zeta_leaflist_dev(vpm_ctx* c, int64_t n, const double* x, const double* gam, const double* sig, double* W,
                          int leaf_size, double theta, int kernel, int precision, int flags, int64_t* stats)
{
    vpm::TraceRange trace_("vpm_zeta_leaflist_dev");
    const char* fn = "vpm_zeta_leaflist_dev";
    if (!c) return fail(nullptr, VPM_ERR_ARG, "%s: ctx is NULL", fn);
    std::lock_guard<std::mutex> lk(c->mu);
    RC(enter(c));
    if (stats) stats[0] = stats[1] = stats[2] = 0;
    if (leaf_size < 1 || leaf_size > LEAF_SIZE_MAX)
        return fail(c, VPM_ERR_ARG, "%s: leaf_size must be in 1..%d", fn, LEAF_SIZE_MAX);
    if (!(theta >= 0.0 && theta <= 1.0e6)) return fail(c, VPM_ERR_ARG, "%s: bad theta", fn);
    if (flags & ~VPM_REUSE_LISTS) return fail(c, VPM_ERR_ARG, "%s: only VPM_REUSE_LISTS is accepted in flags", fn);
    if (n < 0 || n > (int64_t)1 << 30) return fail(c, VPM_ERR_ARG, "%s: n out of range", fn);
    RC(check_kernel(c, kernel, precision));
    if (n == 0) return VPM_OK;
    DeviceGuard dg(c->device);
    if (!is_device_ptr(x) || !is_device_ptr(gam) || !is_device_ptr(sig) || !is_device_ptr(W))
        return fail(c, VPM_ERR_ARG, "%s: every array must be a device pointer", fn);
    NearLists L;
    RC(near_lists(c, n, x, leaf_size, theta, (flags & VPM_REUSE_LISTS) != 0, &L));
    RC(grow(c, c->leaf, leaf_work_bytes(n), "near-field packs"));
    LeafArgs a;
    a.n = n; a.x = x; a.gam = gam; a.sig = sig; a.U = nullptr; a.J = nullptr; a.SFS = nullptr;
    a.static_flags = nullptr; a.kernel = kernel; a.precision = precision; a.sfs = false; a.transposed = true;
    CK(launch_leaf_zeta(a, L, W, c->leaf.p, c->stream, &c->launches), "near-field zeta");
    RC(bounded_wait(c));
    if (stats) {
        stats[0] = L.nleaves;
        stats[1] = L.nlpairs;
        stats[2] = L.pairs;
    }
    return VPM_OK;
}

int vpm_dynamic_diff_leaflist_dev(vpm_ctx* c, int64_t n, const double* x, const double* gam, const double* sig,
                                  const uint8_t* static_flags, const double* J, double alpha, double* dJ,
                                  double* dSFS, int leaf_size, double theta, int kernel, int precision, int flags,
                                  int64_t* stats)
{
    vpm::TraceRange trace_("vpm_dynamic_diff_leaflist_dev");
    const char* fn = "vpm_dynamic_diff_leaflist_dev";
    if (!c) return fail(nullptr, VPM_ERR_ARG, "%s: ctx is NULL", fn);
    std::lock_guard<std::mutex> lk(c->mu);
    RC(enter(c));
    if (stats) stats[0] = stats[1] = stats[2] = 0;
    if (leaf_size < 1 || leaf_size > LEAF_SIZE_MAX)
        return fail(c, VPM_ERR_ARG, "%s: leaf_size must be in 1..%d", fn, LEAF_SIZE_MAX);
    if (!(theta >= 0.0 && theta <= 1.0e6)) return fail(c, VPM_ERR_ARG, "%s: bad theta", fn);
    if (!(alpha > 0.0 && alpha < 1.0)) return fail(c, VPM_ERR_ARG, "%s: alpha must be in (0, 1)", fn);
    if (flags & ~(VPM_TRANSPOSED | VPM_REUSE_LISTS))
        return fail(c, VPM_ERR_ARG, "%s: only VPM_TRANSPOSED and VPM_REUSE_LISTS are accepted in flags", fn);
    if (n < 0 || n > (int64_t)1 << 30) return fail(c, VPM_ERR_ARG, "%s: n out of range", fn);
    RC(check_kernel(c, kernel, precision));
    if (n == 0) return VPM_OK;
    DeviceGuard dg(c->device);
    if (!is_device_ptr(x) || !is_device_ptr(gam) || !is_device_ptr(sig) || !is_device_ptr(J) || !is_device_ptr(dJ) ||
        !is_device_ptr(dSFS) || (static_flags && !is_device_ptr(static_flags)))
        return fail(c, VPM_ERR_ARG, "%s: every array must be a device pointer", fn);
    cudaStream_t st = c->stream;
    NearLists L;
    RC(near_lists(c, n, x, leaf_size, theta, (flags & VPM_REUSE_LISTS) != 0, &L));
    RC(grow(c, c->leaf, leaf_work_bytes(n), "near-field packs"));
    RC(grow(c, c->s, n * sizeof(double), "test-filter core sizes"));
    double* sig_a = (double*)c->s.p;
    scale_copy<<<nblk(n), EB, 0, st>>>(n, sig, alpha, sig_a);
    c->launches++;
    CK(cudaMemsetAsync(dJ, 0, 9 * n * sizeof(double), st), "memset dJ");
    CK(cudaMemsetAsync(dSFS, 0, 3 * n * sizeof(double), st), "memset dSFS");
    LeafArgs a;
    a.n = n; a.x = x; a.gam = gam; a.sig = sig; a.U = nullptr; a.J = const_cast<double*>(J); a.SFS = dSFS;
    a.static_flags = static_flags; a.kernel = kernel; a.precision = precision; a.sfs = true;
    a.transposed = (flags & VPM_TRANSPOSED) != 0;
    if (precision == VPM_FP32COMP) {
        CK(launch_leaf_dynamic(a, L, alpha, sig_a, dJ, dSFS, c->leaf.p, st, &c->launches),
           "near-field test-filter differences");
    } else {
        // FP64: the near-field leg at alpha sigma, the Estr pass at sigma with J, then the differences
        RC(grow(c, c->mat2, (size_t)18 * n * sizeof(double), "test-filter scratch"));
        double* Ua = (double*)c->mat2.p;
        double* Ja = Ua + 3 * n;
        double* Sa = Ja + 9 * n;
        double* S0 = Sa + 3 * n;
        CK(cudaMemsetAsync(Ua, 0, (size_t)18 * n * sizeof(double), st), "memset scratch");
        LeafArgs b = a;
        b.sig = sig_a; b.U = Ua; b.J = Ja; b.SFS = Sa;
        CK(launch_leaflist(b, L, c->leaf.p, st, &c->launches), "test-filter near field");
        LeafArgs z = a;
        z.uj = false; z.SFS = S0;
        CK(launch_leaflist(z, L, c->leaf.p, st, &c->launches), "near-field Estr");
        sub_arrays<<<nblk(9 * n), EB, 0, st>>>(9 * n, Ja, J, dJ);
        sub_arrays<<<nblk(3 * n), EB, 0, st>>>(3 * n, Sa, S0, dSFS);
        c->launches += 2;
        CK(cudaGetLastError(), "differences");
    }
    RC(bounded_wait(c));
    if (stats) {
        stats[0] = L.nleaves;
        stats[1] = L.nlpairs;
        stats[2] = L.pairs;
    }
    return VPM_OK;
}

int vpm_p2p_lists_dev(vpm_ctx* c, int64_t n, const double* x, const double* gam, const double* sig,
                      const uint8_t* static_flags, double* U, double* J, double* SFS, const int32_t* perm,
                      int64_t nl, const int64_t* leaf_begin, const int64_t* leaf_end, const int64_t* row,
                      const int32_t* col, int kernel, int precision, int flags, int64_t* stats)
{
    vpm::TraceRange trace_("vpm_p2p_lists_dev");
    const char* fn = "vpm_p2p_lists_dev";
    if (!c) return fail(nullptr, VPM_ERR_ARG, "%s: ctx is NULL", fn);
    std::lock_guard<std::mutex> lk(c->mu);
    RC(enter(c));
    if (stats) stats[0] = stats[1] = stats[2] = 0;
    DeviceGuard dg(c->device);
    RC(near_check(c, fn, n, x, gam, sig, static_flags, U, J, SFS, kernel, precision, flags));
    if (n == 0) return VPM_OK;
    // the lists must describe a partition of the n tree positions into leaves
    if (!perm || !leaf_begin || !leaf_end || !row || nl < 1 || nl > n)
        return fail(c, VPM_ERR_ARG, "%s: missing or empty lists", fn);
    {
        std::vector<uint8_t> seen(n, 0);
        for (int64_t p = 0; p < n; p++) {
            if (perm[p] < 0 || perm[p] >= n || seen[perm[p]])
                return fail(c, VPM_ERR_ARG, "%s: perm is not a permutation of 0..n-1", fn);
            seen[perm[p]] = 1;
        }
    }
    for (int64_t l = 0; l < nl; l++)
        if (leaf_begin[l] != (l == 0 ? 0 : leaf_end[l - 1]) || leaf_end[l] <= leaf_begin[l])
            return fail(c, VPM_ERR_ARG, "%s: leaf %lld is not the next non-empty range", fn, (long long)l);
    if (leaf_end[nl - 1] != n) return fail(c, VPM_ERR_ARG, "%s: the leaves do not cover 0..n-1", fn);
    if (row[0] != 0) return fail(c, VPM_ERR_ARG, "%s: row[0] must be 0", fn);
    for (int64_t l = 0; l < nl; l++)
        if (row[l + 1] < row[l]) return fail(c, VPM_ERR_ARG, "%s: row is not monotone", fn);
    if (row[nl] > (int64_t)INT32_MAX) return fail(c, VPM_ERR_CAPACITY, "%s: 2^31 or more leaf pairs", fn);
    if (row[nl] > 0 && !col) return fail(c, VPM_ERR_ARG, "%s: col is NULL", fn);
    std::vector<int32_t> cs(col, col + row[nl]);
    for (int64_t l = 0; l < nl; l++) {
        std::sort(cs.begin() + row[l], cs.begin() + row[l + 1]);
        for (int64_t j = row[l]; j < row[l + 1]; j++) {
            if (cs[j] < 0 || cs[j] >= nl) return fail(c, VPM_ERR_ARG, "%s: source leaf out of range", fn);
            if (j > row[l] && cs[j] == cs[j - 1])
                return fail(c, VPM_ERR_ARG, "%s: leaf %lld lists source leaf %d twice", fn, (long long)l, cs[j]);
        }
    }
    NearLists L;
    c->near_ok = false;
    cudaError_t e = near_upload(c->near, n, perm, nl, leaf_begin, leaf_end, row, cs.data(), c->stream, near_sync, c,
                                &L, &c->launches);
    if (e != cudaSuccess) return near_fail(c, e, "leaf-pair lists");
    e = near_groups(c->near, &L, c->stream, near_sync, c, &c->launches);
    if (e != cudaSuccess) return near_fail(c, e, "near-field warp groups");
    return near_run(c, L, n, x, gam, sig, static_flags, U, J, SFS, kernel, precision, flags, stats);
}

int vpm_leaflist_dev(vpm_ctx* c, int64_t n, const double* x, int leaf_size, double theta, int32_t* perm,
                     int64_t* leaf_begin, int64_t* leaf_end, int64_t* row, int32_t* col, int64_t* sizes)
{
    vpm::TraceRange trace_("vpm_leaflist_dev");
    const char* fn = "vpm_leaflist_dev";
    if (!c) return fail(nullptr, VPM_ERR_ARG, "%s: ctx is NULL", fn);
    std::lock_guard<std::mutex> lk(c->mu);
    RC(enter(c));
    if (!sizes || n <= 0 || n > (int64_t)1 << 30 || leaf_size < 1 || leaf_size > LEAF_SIZE_MAX ||
        !(theta >= 0.0 && theta <= 1.0e6))
        return fail(c, VPM_ERR_ARG, "%s: bad arguments", fn);
    DeviceGuard dg(c->device);
    if (!is_device_ptr(x)) return fail(c, VPM_ERR_ARG, "%s: x must be a device pointer", fn);
    NearLists L;
    c->near_ok = false;
    cudaError_t e = near_build(c->near, n, x, leaf_size, theta, c->stream, near_sync, c, &L, &c->launches);
    if (e != cudaSuccess) return near_fail(c, e, "octree and leaf-pair lists");
    sizes[0] = L.nleaves;
    sizes[1] = L.nlpairs;
    sizes[2] = L.pairs;
    if (!perm) return VPM_OK;
    if (!leaf_begin || !leaf_end || !row || !col) return fail(c, VPM_ERR_ARG, "%s: NULL output", fn);
    const int64_t nl = L.nleaves, m = L.nlpairs;
    std::vector<int32_t> b(nl), en(nl), r(nl + 1);
    CK(cudaMemcpyAsync(perm, L.perm, n * sizeof(int32_t), cudaMemcpyDeviceToHost, c->stream), "D2H lists");
    CK(cudaMemcpyAsync(b.data(), L.leaf_begin, nl * sizeof(int32_t), cudaMemcpyDeviceToHost, c->stream), "D2H lists");
    CK(cudaMemcpyAsync(en.data(), L.leaf_end, nl * sizeof(int32_t), cudaMemcpyDeviceToHost, c->stream), "D2H lists");
    CK(cudaMemcpyAsync(r.data(), L.row, (nl + 1) * sizeof(int32_t), cudaMemcpyDeviceToHost, c->stream), "D2H lists");
    if (m > 0) CK(cudaMemcpyAsync(col, L.col, m * sizeof(int32_t), cudaMemcpyDeviceToHost, c->stream), "D2H lists");
    RC(bounded_wait(c));
    for (int64_t l = 0; l < nl; l++) { leaf_begin[l] = b[l]; leaf_end[l] = en[l]; }
    for (int64_t l = 0; l <= nl; l++) row[l] = r[l];
    return VPM_OK;
}

int vpm_leaflist_host(int64_t n, const double* x, int leaf_size, double theta, int32_t* perm,
                      int64_t* leaf_begin, int64_t* leaf_end, int64_t* row, int32_t* col, int64_t* sizes)
{
    vpm::TraceRange trace_("vpm_leaflist_host");
    if (!x || !sizes || n <= 0 || leaf_size < 1 || leaf_size > LEAF_SIZE_MAX || !(theta >= 0.0))
        return fail(nullptr, VPM_ERR_ARG, "vpm_leaflist_host: bad arguments");
    LeafLists L;
    if (build_leaf_lists(n, x, leaf_size, theta, &L) != 0)
        return fail(nullptr, VPM_ERR_ARG, "vpm_leaflist_host: octree construction failed");
    const int64_t nl = (int64_t)L.leaf_begin.size();
    sizes[0] = nl;
    sizes[1] = (int64_t)L.col.size();
    if (!perm) return VPM_OK;
    if (!leaf_begin || !leaf_end || !row || !col) return fail(nullptr, VPM_ERR_ARG, "vpm_leaflist_host: NULL output");
    std::memcpy(perm, L.perm.data(), n * sizeof(int32_t));
    std::memcpy(leaf_begin, L.leaf_begin.data(), nl * sizeof(int64_t));
    std::memcpy(leaf_end, L.leaf_end.data(), nl * sizeof(int64_t));
    std::memcpy(row, L.row.data(), (nl + 1) * sizeof(int64_t));
    std::memcpy(col, L.col.data(), L.col.size() * sizeof(int32_t));
    return VPM_OK;
}

int vpm_uj_adjoint_dev(vpm_ctx* c, int64_t n, const double* x, const double* gam, const double* sig,
                       const double* Ubar, const double* Jbar, double* xbar, double* gbar, double* sbar,
                       int kernel, int precision)
{
    vpm::TraceRange trace_("vpm_uj_adjoint_dev");
    if (!c) return fail(nullptr, VPM_ERR_ARG, "vpm_uj_adjoint_dev: ctx is NULL");
    std::lock_guard<std::mutex> lk(c->mu);
    RC(enter(c));
    if (n < 0 || n > (int64_t)INT32_MAX) return fail(c, VPM_ERR_ARG, "vpm_uj_adjoint_dev: n out of range");
    RC(check_kernel(c, kernel, precision));
    if (precision == VPM_FP32COMP && kernel == VPM_KERNEL_GAUSSIAN)
        return fail(c, VPM_ERR_ARG, "vpm_uj_adjoint_dev: the FP32-comp adjoint covers the singular, Gaussian-erf "
                                    "and Winckelmans kernels (the Gaussian kernel needs VPM_FP64)");
    if (n == 0) return VPM_OK;
    DeviceGuard dg(c->device);
    if (!is_device_ptr(x) || !is_device_ptr(gam) || !is_device_ptr(sig) || !is_device_ptr(Ubar) ||
        !is_device_ptr(Jbar) || !is_device_ptr(xbar) || !is_device_ptr(gbar) || !is_device_ptr(sbar))
        return fail(c, VPM_ERR_ARG, "vpm_uj_adjoint_dev: every array must be a device pointer");
    Workspace w;
    RC(ensure_work(c, n, n, VPM_FP64, false, &w));
    AdjArgs a;
    a.n = n; a.x = x; a.gam = gam; a.sig = sig; a.Ubar = Ubar; a.Jbar = Jbar;
    a.xbar = xbar; a.gbar = gbar; a.sbar = sbar; a.kernel = kernel; a.precision = precision;
    CK(launch_uj_adjoint(a, w, c->num_sms, c->stream, &c->launches), "UJ adjoint kernels");
    return bounded_wait(c);
}

int vpm_estr_adjoint_dev(vpm_ctx* c, int64_t n, const double* x, const double* gam, const double* sig,
                         const double* J, const uint8_t* static_flags, const double* SFSbar, double* xbar,
                         double* gbar, double* sbar, double* Jbar, int kernel, int precision, int flags)
{
    vpm::TraceRange trace_("vpm_estr_adjoint_dev");
    const char* fn = "vpm_estr_adjoint_dev";
    if (!c) return fail(nullptr, VPM_ERR_ARG, "%s: ctx is NULL", fn);
    std::lock_guard<std::mutex> lk(c->mu);
    RC(enter(c));
    if (n < 0 || n > (int64_t)INT32_MAX) return fail(c, VPM_ERR_ARG, "%s: n out of range", fn);
    if (flags & ~VPM_TRANSPOSED) return fail(c, VPM_ERR_ARG, "%s: only VPM_TRANSPOSED is accepted in flags", fn);
    RC(check_kernel(c, kernel, precision));
    if (n == 0) return VPM_OK;
    DeviceGuard dg(c->device);
    if (!is_device_ptr(x) || !is_device_ptr(gam) || !is_device_ptr(sig) || !is_device_ptr(J) ||
        !is_device_ptr(SFSbar) || !is_device_ptr(xbar) || !is_device_ptr(gbar) || !is_device_ptr(sbar) ||
        !is_device_ptr(Jbar) || (static_flags && !is_device_ptr(static_flags)))
        return fail(c, VPM_ERR_ARG, "%s: every array must be a device pointer", fn);
    const EstrAdjSizes z = estr_adjoint_sizes(n, c->num_sms);
    RC(grow(c, c->order, order_bytes(n), "Morton ordering"));
    RC(grow(c, c->src_pack, 2 * z.pack, "adjoint packs"));
    RC(grow(c, c->partial, z.partial, "adjoint partial sums"));
    EstrAdjWork w;
    w.order = c->order.p; w.order_bytes = c->order.cap;
    w.pack1 = c->src_pack.p; w.pack2 = (char*)c->src_pack.p + z.pack;
    w.partial = (double*)c->partial.p;
    EstrAdjArgs a;
    a.n = n; a.x = x; a.gam = gam; a.sig = sig; a.J = J; a.static_flags = static_flags; a.Sbar = SFSbar;
    a.xbar = xbar; a.gbar = gbar; a.sbar = sbar; a.Jbar = Jbar; a.kernel = kernel; a.precision = precision;
    a.transposed = (flags & VPM_TRANSPOSED) != 0;
    CK(launch_estr_adjoint(a, w, c->num_sms, c->stream, &c->launches), "Estr adjoint kernels");
    return bounded_wait(c);
}

}  // extern "C"
