// internal.h -- declarations shared by the translation units of libvpm_gb300.so.
// Not part of the public ABI (include/vpm_gb300.h).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace vpm {

// Packed source payload of the mixed (FP32-comp) UJ kernel, 48 B per source:
//   a = (x_hi, y_hi, z_hi, 1/sigma^2)
//   b = (x_lo, y_lo, z_lo, 0)           x = x_hi + x_lo (double-float position)
//   c = (-Gamma/(4 pi sigma^3), 0)
// For the singular kernel sigma is taken as 1 (g == 1 does not depend on it).
struct __align__(16) SrcMixed { float4 a, b, c; };

// Packed source payload of the FP64 UJ kernel, 64 B per source.
struct __align__(16) SrcF64 { double2 xy, z_isig, gxy, gz_sig; };

// Packed source payload of the mixed Estr kernel, 64 B per source:
//   a = (x_hi, y_hi, z_hi, 1/sigma^2), b = (x_lo, y_lo, z_lo, 0)
//   c = (Gt_x, Gt_y, Gt_z, vt_x), d = (vt_y, vt_z, 0, 0)
// with Gt = ZNORM * Gamma / sigma^3 and vt = ZNORM * v / sigma^3, v = J^T Gamma
// (transposed scheme) or J Gamma; zero for static sources.
struct __align__(16) SrcEstrMixed { float4 a, b, c, d; };

// Packed source payload of the FP64 Estr kernel, 80 B per source:
//   (x, y), (z, 1/sigma), (Gamma_x, Gamma_y), (Gamma_z, v_x), (v_y, v_z)
// with Gamma and v = J^T Gamma zero for static sources.
struct __align__(16) SrcEstrF64 { double2 xy, z_isig, gxy, gz_vx, vyz; };

constexpr int UJ_THREADS = 128;   // targets per block, one per thread
constexpr int UJ_TILE = 128;      // sources staged in shared memory per tile
constexpr int UJ_BLOCK = 64;      // sources summed in FP32 before the FP64 add

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
};

// Scratch and packing buffers supplied by the caller (the context).
struct Workspace {
    void* src_pack; size_t src_pack_bytes;
    void* tgt_pack; size_t tgt_pack_bytes;
    double* partial; size_t partial_bytes;   // split-K partial sums
};

// Bytes of workspace needed for a problem (computed on the host).
size_t uj_src_pack_bytes(int64_t ns, int precision);
size_t uj_tgt_pack_bytes(int64_t nt, int precision);
size_t estr_src_pack_bytes(int64_t ns, int precision);
// Number of source splits used for nt targets / ns sources and partial bytes.
int uj_num_splits(int64_t nt, int64_t ns, int num_sms);
size_t uj_partial_bytes(int64_t nt, int nsplit);

// Launchers; return cudaError_t of the launches and count kernel launches.
cudaError_t launch_uj(const UJArgs& a, const Workspace& w, int num_sms, cudaStream_t st,
                      int64_t* launches);
cudaError_t launch_estr(const EstrArgs& a, const Workspace& w, int num_sms, cudaStream_t st,
                        int64_t* launches);

}  // namespace vpm
