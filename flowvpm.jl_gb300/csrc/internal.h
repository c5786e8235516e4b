// internal.h -- declarations shared by the translation units of libvpm_gb300.so.
// Not part of the public ABI (include/vpm_gb300.h).
#pragma once
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>
#include <stdint.h>

namespace vpm {

// One NVTX range per library call, named after the entry point, so that a
// profiler's timeline shows each UJ / Estr / adjoint call around its kernels.
// Without a tool attached a push/pop is a null-pointer check.
struct TraceRange {
    explicit TraceRange(const char* name) { nvtxRangePushA(name); }
    ~TraceRange() { nvtxRangePop(); }
    TraceRange(const TraceRange&) = delete;
    TraceRange& operator=(const TraceRange&) = delete;
};

// A target in Morton order: FP64 position and its index in the caller's arrays.
struct __align__(16) TgtPos { double x, y, z; int32_t idx, pad; };

// Packed source of the mixed (FP32-comp) UJ kernel, 48 B:
//   a   = (x_hi, y_hi, z_hi, sigma^2)     position as a double-float x_hi + x_lo
//   b   = (x_lo, y_lo, z_lo, 1/sigma)
//   gam = -Gamma/(4 pi)            for kernels with a singular tail (all but Winckelmans)
//         -Gamma/(4 pi sigma^3)    for Winckelmans
// For the singular kernel sigma is taken as 1 (g == 1 does not depend on it).
struct __align__(16) SrcMixed { float4 a, b, gam; };

// Packed source of the FP64 UJ kernel, 64 B.
struct __align__(16) SrcF64 { double2 xy, z_isig, gxy, gz_sig; };

// Packed source of the all-pairs and near-field mixed Estr kernels, 64 B:
// position as a double-float (a.xyz + b.xyz), a.w = 1/sigma^2,
// g = ZNORM Gamma / sigma^3 and v = ZNORM (J^T Gamma) / sigma^3 (or J Gamma), in
// FP32; g = v = 0 for static sources.
struct __align__(16) SrcEstrDF { float4 a, b, g, v; };

// Packed source of the FP64 Estr kernel, 80 B:
//   (x, y), (z, 1/sigma), (Gamma_x, Gamma_y), (Gamma_z, v_x), (v_y, v_z)
// with Gamma and v = J^T Gamma zero for static sources.
struct __align__(16) SrcEstrF64 { double2 xy, z_isig, gxy, gz_vx, vyz; };

constexpr int UJ_THREADS = 128;   // targets per block, one per thread
constexpr int UJ_WARPS = UJ_THREADS / 32;
constexpr int UJ_TILE = 128;      // sources staged in shared memory per tile
constexpr int UJ_BLOCK = 64;      // sources summed in FP32 per inner block
constexpr int UJ_FLUSH_TILES = 2; // tiles summed in FP32 before the FP64 add

// Problem description handed from the ABI layer to the kernel launchers.
struct UJArgs {
    int64_t nt, ns;
    const double* xt;     // targets [nt,3]
    const double* xs;     // sources [ns,3]
    const double* gs;     // [ns,3]
    const double* sgs;    // [ns]
    double* U; int64_t ldU;   // U of target t at U[t*ldU + k]
    double* J; int64_t ldJ;   // J of target t at J[t*ldJ + k]
    int kernel, precision;
    bool self;            // targets are the sources (same arrays)
};

struct EstrArgs {
    int64_t nt, ns;
    const double* xt; const double* Jt; int64_t ldJt; const uint8_t* static_t;
    const double* xs; const double* gs; const double* sgs;
    const double* Js; int64_t ldJs; const uint8_t* static_s;
    double* SFS; int64_t ldS;
    int kernel, precision;
    bool transposed, self;
    bool zeta = false;    // zeta_direct instead: SFS receives W = sum zeta Gamma (J unused, statics included)
    double dz_alpha = 0.0;   // > 0: the weight difference zeta~(r, alpha sigma) - zeta~(r, sigma) (mixed only)
};

// Reverse mode of the self-induced UJ of one particle set.
struct AdjArgs {
    int64_t n;
    const double* x; const double* gam; const double* sig;   // [n,3], [n,3], [n]
    const double* Ubar; const double* Jbar;                  // [n,3], [n,9]
    double* xbar; double* gbar; double* sbar;                // += outputs
    int kernel, precision;
};

// Reverse mode of the self-induced Estr of one particle set (estr_adjoint.cu).
struct EstrAdjArgs {
    int64_t n;
    const double* x; const double* gam; const double* sig; const double* J;   // [n,3], [n,3], [n], [n,9]
    const uint8_t* static_flags;                                              // [n] or null
    const double* Sbar;                                                       // [n,3] = dL/dSFS
    double* xbar; double* gbar; double* sbar; double* Jbar;                   // += outputs
    int kernel, precision;
    bool transposed;
};
struct EstrAdjWork {
    void* order; size_t order_bytes;          // Morton ordering of the particles
    void* pack1; void* pack2;                 // EstrAdjSizes::pack bytes each
    double* partial;                          // EstrAdjSizes::partial bytes
};
struct EstrAdjSizes { size_t pack, partial; };
EstrAdjSizes estr_adjoint_sizes(int64_t n, int num_sms);
cudaError_t launch_estr_adjoint(const EstrAdjArgs& a, const EstrAdjWork& w, int num_sms, cudaStream_t st,
                                int64_t* launches);

// Near-field P2P over octree leaf pairs (leaflist.cu).
struct LeafArgs {
    int64_t n;
    const double* x; const double* gam; const double* sig;   // [n,3], [n,3], [n]
    double* U; double* J; double* SFS;                        // += outputs, original order
    const uint8_t* static_flags;                              // [n] or null
    int kernel, precision;
    bool sfs, transposed;
    bool uj = true;                                           // false: the Estr pass alone (J is input)
};

// Scratch and packing buffers supplied by the caller (the context).
struct Workspace {
    void* src_pack; size_t src_pack_bytes;
    void* order; size_t order_bytes;          // Morton ordering of the targets
    double* partial; size_t partial_bytes;    // split-source partial sums
};

size_t uj_src_pack_bytes(int64_t ns, int precision);
size_t estr_src_pack_bytes(int64_t ns, int precision);
size_t order_bytes(int64_t nt);
int uj_num_splits(int64_t nt, int64_t ns, int num_sms);
size_t uj_partial_bytes(int64_t nt, int nsplit);

// Morton-order the nt targets xt; *out receives nt TgtPos records in scratch.
cudaError_t order_targets(int64_t nt, const double* xt, void* scratch, size_t scratch_bytes, cudaStream_t st,
                          int64_t* launches, const TgtPos** out);

// Sets the calling thread's context-free error text (vpm_last_error(NULL)).
void set_thread_error(const char* msg);

// Launchers; return cudaError_t of the launches and count kernel launches.
cudaError_t launch_uj(const UJArgs& a, const Workspace& w, int num_sms, cudaStream_t st,
                      int64_t* launches);
cudaError_t launch_estr(const EstrArgs& a, const Workspace& w, int num_sms, cudaStream_t st,
                        int64_t* launches);
cudaError_t launch_uj_adjoint(const AdjArgs& a, const Workspace& w, int num_sms, cudaStream_t st,
                              int64_t* launches);
// dJ[n,9] += J(alpha sigma) - J(sigma) of one particle set, all pairs, FP32-comp (dynamic.cu)
size_t dyn_src_pack_bytes(int64_t ns);
cudaError_t launch_uj_filter_diff(int64_t n, const double* x, const double* gam, const double* sig, double alpha,
                                  double* dJ, int kernel, const Workspace& w, cudaStream_t st, int64_t* launches);

// ------------------------------------------------------------------ near field
// A device allocation that grows on demand and never shrinks.
struct DevBuf {
    void* p = nullptr;
    size_t cap = 0;
    cudaError_t grow(size_t bytes)
    {
        if (bytes <= cap) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
        const size_t want = bytes + bytes / 8;   // some headroom
        cudaError_t e = cudaMalloc(&p, want);
        if (e == cudaSuccess) cap = want;
        return e;
    }
    void release()
    {
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
    }
    template <class T> T* as() const { return (T*)p; }
};

// Leaf-pair lists on the device.  Particles are numbered by their Morton
// position p (perm[p] = caller index); leaves are Morton-ordered ranges
// [leaf_begin[l], leaf_end[l]); row/col is the CSR list of the source leaves
// of every target leaf.  For the kernels, targets are cut into warp groups of
// 32 consecutive Morton positions; group g's sources are the intervals
// ivs[grp_row[g] .. grp_row[g+1]) = (p0, p1, mask, 0): particle range [p0, p1)
// needed by the target leaves whose bit (leaf - leaf_of[32 g]) is set in mask.
struct NearLists {
    int64_t n = 0, nleaves = 0, nlpairs = 0, ngroups = 0, nivs = 0;
    int64_t pairs = 0;                 // particle pairs over all leaf pairs
    int64_t nodes = 0;                 // octree nodes (0 for lists given by the caller)
    const int32_t* perm = nullptr;     // [n]
    const int32_t* leaf_of = nullptr;  // [n]
    const int32_t* leaf_begin = nullptr;
    const int32_t* leaf_end = nullptr; // [nleaves]
    const int32_t* row = nullptr;      // [nleaves + 1]
    const int32_t* col = nullptr;      // [nlpairs]
    const int32_t* grp_row = nullptr;  // [ngroups + 1]
    const int4* ivs = nullptr;         // [nivs]
};

// Device scratch of the list builder (owned by the context).
struct NearScratch {
    DevBuf keys, keys2, idx, perm, xs, part, nodes, node_lvl, node_box, node_cr, node_leaf, ctr;
    DevBuf flag, leaf_of, lb, le, row, col, fr0, fr1, near0, near1, grp_cnt, grp_row, ivs, cub;
    int64_t* hctr = nullptr;          // pinned host copy of the builder's counters
    size_t capF = 0, capN = 0;        // traversal capacities (pairs)
    void release_all();
};

// A bounded wait for the stream, supplied by the ABI layer (cudaSuccess or an error).
typedef cudaError_t (*SyncFn)(void* ctx);

// Octree (leaf size, Morton keys of 21 bits per axis) and near leaf pairs
// (theta |c_A - c_B| < R_A + R_B) of the n device positions x[n,3].
cudaError_t near_build(NearScratch& s, int64_t n, const double* x, int leaf_size, double theta, cudaStream_t st,
                       SyncFn sync, void* sync_ctx, NearLists* out, int64_t* launches);
// Lists supplied by the caller on the host (checked there): copied to the device.
cudaError_t near_upload(NearScratch& s, int64_t n, const int32_t* perm, int64_t nleaves, const int64_t* leaf_begin,
                        const int64_t* leaf_end, const int64_t* row, const int32_t* col, cudaStream_t st,
                        SyncFn sync, void* sync_ctx, NearLists* out, int64_t* launches);
// The warp-group source intervals of lists built or uploaded above.
cudaError_t near_groups(NearScratch& s, NearLists* L, cudaStream_t st, SyncFn sync, void* sync_ctx,
                        int64_t* launches);

constexpr int LEAF_SIZE_MAX = 4096;
size_t leaf_work_bytes(int64_t n);
cudaError_t launch_leaflist(const LeafArgs& a, const NearLists& L, void* work, cudaStream_t st, int64_t* launches);
// The per-particle work of an RK3 step (step.cu).
struct StageArgs {
    int64_t n;
    double a, b, dt, uinf[3], f, g, zeta0, nu;   // nu < 0: no core spreading
    bool transposed;
    double* x; double* gam; double* sig;
    const double* U; const double* J; const double* SFS; const double* C;
    double* M;
};
struct DynAfterArgs {
    int64_t n;
    double alpha, rlxf, minC, maxC, zeta0;
    int flags;
    const double* gam; const double* sig; const double* J; const double* SFS;
    double* C; double* M;
};
cudaError_t launch_rk3_stage(const StageArgs& a, cudaStream_t st, int64_t* launches);
cudaError_t launch_relax(int64_t n, double rlxf, const double* J, double* gam, cudaStream_t st, int64_t* launches);
cudaError_t launch_dynamic_after(const DynAfterArgs& a, int* nan_flag, cudaStream_t st, int64_t* launches);

// zeta_fmm's near-field sum: W[n,3] += sum over the near lists of zeta(r/sigma_s)/sigma_s^3 Gamma_s.
cudaError_t launch_leaf_zeta(const LeafArgs& a, const NearLists& L, double* W, void* work, cudaStream_t st,
                             int64_t* launches);
// The dynamic procedure's test-filter differences over the near lists (FP32-comp):
// dJ, dSFS (+=, original order) from a.x, a.gam, a.sig, a.J and sig_a = alpha sig.
cudaError_t launch_leaf_dynamic(const LeafArgs& a, const NearLists& L, double alpha, const double* sig_a, double* dJ,
                                double* dSFS, void* work, cudaStream_t st, int64_t* launches);

}  // namespace vpm
