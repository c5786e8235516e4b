// nearfield.cu -- the near-field leaf-pair lists of the FMM path, built on the
// device.
//
// UJ_fmm (src/FLOWVPM_UJ.jl:62-129) evaluates by direct P2P every pair of
// octree leaves that fails the multipole acceptance criterion, which FLOWVPM
// documents as "if theta*r < R1+R2 the interaction between two cells is
// resolved through P2P, where r is the distance between cell centers, and R1
// and R2 are each cell radius" (src/FLOWVPM_particlefield.jl:28-36).  The
// octree itself belongs to FastMultipole.jl, which is not available; the tree
// defined here is this library's own and is specified once, in tree.cpp (the
// host builder, kept as the readable statement of it).  This file builds the
// identical lists on the GPU:
//
//   1. bounding box, Morton keys (21 bits per axis, one extent for all axes),
//      stable radix sort of (key, index);
//   2. nodes = key-prefix ranges, split breadth-first while they hold more than
//      leaf_size particles; a range whose particles share the next octant is
//      not a new node (the split descends a level in place);
//   3. geometry: bounding box of each node's particles (leaves directly,
//      inner nodes as the union of their children), centre = box centre,
//      R = half the box diagonal;
//   4. dual-tree traversal from (root, root), one frontier of node pairs per
//      step: far when A != B and theta*r >= R_A + R_B, a near leaf pair when
//      both are leaves, otherwise the larger non-leaf node (the target on a
//      tie) is split;
//   5. the near pairs sorted into CSR rows per target leaf, and the warp-group
//      source intervals used by the kernels of leaflist.cu.
//
// The result equals tree.cpp's bit for bit: the same keys, the same node
// ranges, and geometry computed with the same IEEE operations in the same
// order (round-to-nearest intrinsics, so nothing is contracted into an FMA;
// the host side is compiled with -ffp-contract=off).  The set of near pairs
// does not depend on the order in which the frontier is processed.
#include "internal.h"

#include <cub/cub.cuh>

#include <algorithm>
#include <cstring>
#include <vector>

namespace vpm {

namespace {

constexpr int KEY_LEVELS = 21;                 // 3 x 21 = 63 key bits
constexpr int MAX_DEPTH = KEY_LEVELS + 1;      // breadth-first node depths
constexpr int TRAV_STEPS = 2 * MAX_DEPTH + 2;  // each step descends one side
constexpr int GS_THREADS = 256;
constexpr int GS_BLOCKS = 8 * 152;

// counters in NearScratch::ctr (unsigned 64-bit)
enum : int {
    C_NODES = 0, C_NEAR = 1, C_OVF = 2, C_PAIRS = 3, C_NL = 4,
    C_OVFN = 5,                                 // the near list overflowed (the traversal itself stays valid)
    C_LVL = 8,                                  // [C_LVL + 2d, C_LVL + 2d + 1) = node ids of depth d
    C_F = C_LVL + 2 * (MAX_DEPTH + 2),          // C_F + s = frontier size of traversal step s
    C_COUNT = C_F + TRAV_STEPS + 2
};

typedef unsigned long long ull;

// what the traversal reads of a node, in one 64-B record: centre, radius,
// first child, number of children (0: a leaf) and the leaf's index
struct __align__(64) TravNode { double x, y, z, w; int first, nkid, leaf; float w32; int pad[4]; };

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

__device__ __forceinline__ int64_t gtid() { return blockIdx.x * (int64_t)blockDim.x + threadIdx.x; }
__device__ __forceinline__ int64_t gstride() { return (int64_t)gridDim.x * blockDim.x; }

// Every thread of the block calls this (no early exit: it holds barriers);
// returns the thread's slot in a shared append counter, with one atomic per
// block.  sw: GS_THREADS/32 words of shared memory, sb: one.
__device__ __forceinline__ ull block_append(ull* ctr, unsigned k, unsigned* sw, ull* sb)
{
    const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    unsigned incl = k;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= (unsigned)o) incl += v;
    }
    if (lane == 31) sw[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        const unsigned t = lane < nw ? sw[lane] : 0u;
        unsigned w = t;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned v = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= (unsigned)o) w += v;
        }
        if (lane < nw) sw[lane] = w - t;                  // exclusive offset of each warp
        if (lane == nw - 1) *sb = w ? atomicAdd(ctr, (ull)w) : 0ull;
    }
    __syncthreads();
    const ull slot = *sb + sw[warp] + incl - k;
    __syncthreads();                                      // sw, sb are reused by the next call
    return slot;
}

// ------------------------------------------------------------------ keys
__global__ void nt_bbox_partial(int64_t n, const double* __restrict__ x, double* __restrict__ part)
{
    double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int64_t i = gtid(); i < n; i += gstride())
        for (int k = 0; k < 3; k++) {
            const double v = x[3 * i + k];
            lo[k] = fmin(lo[k], v);
            hi[k] = fmax(hi[k], v);
        }
    __shared__ double s[6][GS_THREADS];
    for (int k = 0; k < 3; k++) { s[k][threadIdx.x] = lo[k]; s[3 + k][threadIdx.x] = hi[k]; }
    __syncthreads();
    for (int m = GS_THREADS / 2; m > 0; m >>= 1) {
        if ((int)threadIdx.x < m)
            for (int k = 0; k < 3; k++) {
                s[k][threadIdx.x] = fmin(s[k][threadIdx.x], s[k][threadIdx.x + m]);
                s[3 + k][threadIdx.x] = fmax(s[3 + k][threadIdx.x], s[3 + k][threadIdx.x + m]);
            }
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int k = 0; k < 6; k++) part[6 * blockIdx.x + k] = s[k][0];
}

// box = (lo_x, lo_y, lo_z, ext): the cube of side ext = the largest extent (one block of GS_THREADS)
__global__ void nt_bbox_final(int nb, const double* __restrict__ part, double* __restrict__ box)
{
    double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int b = threadIdx.x; b < nb; b += blockDim.x)
        for (int k = 0; k < 3; k++) {
            lo[k] = fmin(lo[k], part[6 * b + k]);
            hi[k] = fmax(hi[k], part[6 * b + 3 + k]);
        }
    __shared__ double s[6][GS_THREADS];
    for (int k = 0; k < 3; k++) { s[k][threadIdx.x] = lo[k]; s[3 + k][threadIdx.x] = hi[k]; }
    __syncthreads();
    for (int m = GS_THREADS / 2; m > 0; m >>= 1) {
        if ((int)threadIdx.x < m)
            for (int k = 0; k < 3; k++) {
                s[k][threadIdx.x] = fmin(s[k][threadIdx.x], s[k][threadIdx.x + m]);
                s[3 + k][threadIdx.x] = fmax(s[3 + k][threadIdx.x], s[3 + k][threadIdx.x + m]);
            }
        __syncthreads();
    }
    if (threadIdx.x != 0) return;
    double ext = 0.0;
    for (int k = 0; k < 3; k++) ext = fmax(ext, __dsub_rn(s[3 + k][0], s[k][0]));
    if (!(ext > 0.0)) ext = 1.0;
    box[0] = s[0][0]; box[1] = s[1][0]; box[2] = s[2][0]; box[3] = ext;
}

__global__ void nt_keys(int64_t n, const double* __restrict__ x, const double* __restrict__ box,
                        uint64_t* __restrict__ key, int32_t* __restrict__ idx)
{
    const double ext = box[3];
    for (int64_t i = gtid(); i < n; i += gstride()) {
        uint64_t kk = 0;
        for (int k = 0; k < 3; k++) {
            double f = __ddiv_rn(__dsub_rn(x[3 * i + k], box[k]), ext);
            f = fmin(fmax(f, 0.0), 1.0);
            kk |= spread3((uint64_t)__dmul_rn(f, 2097151.0)) << (2 - k);
        }
        key[i] = kk;
        idx[i] = (int32_t)i;
    }
}

__global__ void nt_gather_x(int64_t n, const double* __restrict__ x, const int32_t* __restrict__ perm,
                            double* __restrict__ xs)
{
    for (int64_t i = gtid(); i < n; i += gstride()) {
        const int64_t j = perm[i];
        xs[3 * i] = x[3 * j]; xs[3 * i + 1] = x[3 * j + 1]; xs[3 * i + 2] = x[3 * j + 2];
    }
}

// ----------------------------------------------------------------- nodes
// node = (begin, end, first child, number of children); a leaf has no children
__global__ void nt_init(int64_t n, int4* __restrict__ nodes, int32_t* __restrict__ lvl, ull* __restrict__ ctr)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    nodes[0] = make_int4(0, (int)n, -1, 0);
    lvl[0] = 0;
    ctr[C_NODES] = 1;
    ctr[C_LVL] = 0;
    ctr[C_LVL + 1] = 1;
    ctr[C_F] = 1;
}

// first position in [lo, hi) whose octant digit at `shift` is >= oct (digits are sorted there)
__device__ __forceinline__ int digit_lower_bound(const uint64_t* __restrict__ key, int lo, int hi, int shift, unsigned oct)
{
    while (lo < hi) {
        const int mid = lo + ((hi - lo) >> 1);
        if ((unsigned)((key[mid] >> shift) & 7u) < oct) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

__global__ void nt_split(int d, const uint64_t* __restrict__ key, int leaf_size, int4* __restrict__ nodes,
                         int32_t* __restrict__ lvl, ull* __restrict__ ctr)
{
    const int64_t s = (int64_t)ctr[C_LVL + 2 * d], e = (int64_t)ctr[C_LVL + 2 * d + 1];
    for (int64_t id = s + gtid(); id < e; id += gstride()) {
        const int4 nd = nodes[id];
        int L = lvl[id];
        if (nd.y - nd.x <= leaf_size || L >= KEY_LEVELS) continue;
        int st[9];
        int nk = 0;
        for (;;) {
            const int shift = 3 * (KEY_LEVELS - 1 - L);
            st[0] = nd.x;
            st[8] = nd.y;
            for (unsigned oct = 1; oct < 8; oct++) st[oct] = digit_lower_bound(key, st[oct - 1], nd.y, shift, oct);
            nk = 0;
            for (int o = 0; o < 8; o++) nk += st[o + 1] > st[o];
            if (nk >= 2) break;
            if (++L >= KEY_LEVELS) { nk = 0; break; }   // one octant down to the last key bit: a leaf
        }
        if (nk == 0) continue;
        const int64_t slot = (int64_t)atomicAdd(&ctr[C_NODES], (ull)nk);
        int j = 0;
        for (int o = 0; o < 8; o++)
            if (st[o + 1] > st[o]) {
                nodes[slot + j] = make_int4(st[o], st[o + 1], -1, 0);
                lvl[slot + j] = L + 1;
                j++;
            }
        nodes[id] = make_int4(nd.x, nd.y, (int)slot, nk);
    }
}

__global__ void nt_mark(int d, ull* __restrict__ ctr)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    ctr[C_LVL + 2 * (d + 1)] = ctr[C_LVL + 2 * d + 1];
    ctr[C_LVL + 2 * (d + 1) + 1] = ctr[C_NODES];
}

__global__ void nt_leaf_flag(const int4* __restrict__ nodes, const ull* __restrict__ ctr, int32_t* __restrict__ flag)
{
    const int64_t nn = (int64_t)ctr[C_NODES];
    for (int64_t id = gtid(); id < nn; id += gstride())
        if (nodes[id].w == 0) flag[nodes[id].x] = 1;
}

// incl = inclusive sum of the leaf-start flags: the leaf of Morton position p is incl[p] - 1
__global__ void nt_leaf_ids(int64_t n, const int4* __restrict__ nodes, const int32_t* __restrict__ incl,
                            int32_t* __restrict__ lb, int32_t* __restrict__ le, int32_t* __restrict__ node_leaf,
                            ull* __restrict__ ctr)
{
    const int64_t nn = (int64_t)ctr[C_NODES];
    if (gtid() == 0) ctr[C_NL] = (ull)incl[n - 1];
    for (int64_t id = gtid(); id < nn; id += gstride()) {
        const int4 nd = nodes[id];
        if (nd.w != 0) { node_leaf[id] = -1; continue; }
        const int l = incl[nd.x] - 1;
        lb[l] = nd.x;
        le[l] = nd.y;
        node_leaf[id] = l;
    }
}

__global__ void nt_leaf_of(int64_t n, int32_t* __restrict__ incl_to_leaf)
{
    for (int64_t p = gtid(); p < n; p += gstride()) incl_to_leaf[p] -= 1;
}

// node boxes: [6 id .. 6 id + 6) = lo_x, lo_y, lo_z, hi_x, hi_y, hi_z
__global__ void nt_box_leaf(const int4* __restrict__ nodes, const ull* __restrict__ ctr, const double* __restrict__ xs,
                            double* __restrict__ box)
{
    const int64_t nn = (int64_t)ctr[C_NODES];
    for (int64_t id = gtid(); id < nn; id += gstride()) {
        const int4 nd = nodes[id];
        if (nd.w != 0) continue;
        double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
        for (int64_t i = nd.x; i < nd.y; i++)
            for (int k = 0; k < 3; k++) {
                lo[k] = fmin(lo[k], xs[3 * i + k]);
                hi[k] = fmax(hi[k], xs[3 * i + k]);
            }
        for (int k = 0; k < 3; k++) { box[6 * id + k] = lo[k]; box[6 * id + 3 + k] = hi[k]; }
    }
}

__global__ void nt_box_inner(int d, const int4* __restrict__ nodes, const ull* __restrict__ ctr, double* __restrict__ box)
{
    const int64_t s = (int64_t)ctr[C_LVL + 2 * d], e = (int64_t)ctr[C_LVL + 2 * d + 1];
    for (int64_t id = s + gtid(); id < e; id += gstride()) {
        const int4 nd = nodes[id];
        if (nd.w == 0) continue;
        double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
        for (int c = nd.z; c < nd.z + nd.w; c++)
            for (int k = 0; k < 3; k++) {
                lo[k] = fmin(lo[k], box[6 * (int64_t)c + k]);
                hi[k] = fmax(hi[k], box[6 * (int64_t)c + 3 + k]);
            }
        for (int k = 0; k < 3; k++) { box[6 * id + k] = lo[k]; box[6 * id + 3 + k] = hi[k]; }
    }
}

// centre and radius, in tree.cpp's operation order: c = 0.5 (lo + hi), R = 0.5 sqrt(sum (hi - lo)^2)
__global__ void nt_cr(const ull* __restrict__ ctr, const double* __restrict__ box, const int4* __restrict__ nodes,
                      const int32_t* __restrict__ node_leaf, TravNode* __restrict__ cr)
{
    const int64_t nn = (int64_t)ctr[C_NODES];
    for (int64_t id = gtid(); id < nn; id += gstride()) {
        const double* b = box + 6 * id;
        double c[3], d2 = 0.0;
        for (int k = 0; k < 3; k++) {
            c[k] = __dmul_rn(0.5, __dadd_rn(b[k], b[3 + k]));
            const double w = __dsub_rn(b[3 + k], b[k]);
            d2 = __dadd_rn(d2, __dmul_rn(w, w));
        }
        const int4 nd = nodes[id];
        TravNode t;
        t.x = c[0]; t.y = c[1]; t.z = c[2]; t.w = __dmul_rn(0.5, __dsqrt_rn(d2));
        t.first = nd.z; t.nkid = nd.w; t.leaf = node_leaf[id];
        t.w32 = (float)t.w;
        for (int k = 0; k < 4; k++) t.pad[k] = 0;
        cr[id] = t;
    }
}

// -------------------------------------------------------------- traversal
// The acceptance test theta r >= R_A + R_B is decided in FP32 on the squares,
// from the FP64 centre differences (each rounded once to FP32): the FP32 sides
// carry < 2^-20 relative error, so a difference above 2^-17 of their sum gives
// tree.cpp's FP64 decision; closer calls, and A = B, take the FP64 test itself
// (GB300's FP64 pipe runs at 1/64 of the FP32 rate: the FP64 test was most of
// this kernel's time).
__global__ void nt_trav(int step, double theta, const TravNode* __restrict__ cr, const int2* __restrict__ fin,
                        int2* __restrict__ fout, uint64_t* __restrict__ near, ull* __restrict__ ctr, ull capF, ull capN)
{
    __shared__ unsigned sw[GS_THREADS / 32];
    __shared__ ull sb;
    __shared__ int stop;
    // After an overflow in an earlier step, the slots of this step's frontier past the last
    // write were counted but never written: read nothing, the host grows the buffers and
    // repeats the traversal.  One read per block keeps the exit block-uniform (block_append
    // holds barriers); the flag is read once, before this launch writes anything.
    if (threadIdx.x == 0) stop = ctr[C_OVF] != 0ull;
    __syncthreads();
    if (stop) return;
    const float th2 = (float)(theta * theta);
    const ull raw = ctr[C_F + step];
    const int64_t cnt = (int64_t)(raw < capF ? raw : capF);
    // block-strided so that every thread of a block runs the same iterations (block_append)
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < cnt; base += gstride()) {
        const int64_t i = base + threadIdx.x;
        unsigned knear = 0, ksplit = 0;
        int A = 0, B = 0, first = 0, la_leaf = 0, lb_leaf = 0;
        bool split_a = false;
        if (i < cnt) {
            const int2 ab = fin[i];
            A = ab.x;
            B = ab.y;
            const TravNode a = cr[A], c = cr[B];
            const double dx = __dsub_rn(a.x, c.x), dy = __dsub_rn(a.y, c.y), dz = __dsub_rn(a.z, c.z);
            const float fx = (float)dx, fy = (float)dy, fz = (float)dz;
            const float lhs = th2 * fmaf(fx, fx, fmaf(fy, fy, fz * fz));
            const float rs = a.w32 + c.w32;
            const float rhs = rs * rs;
            bool far;
            if (A != B && fabsf(lhs - rhs) > 7.62939453125e-06f * (lhs + rhs)) {
                far = lhs > rhs;
            } else {   // tree.cpp's FP64 test, in its operation order
                const double r = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)),
                                                      __dmul_rn(dz, dz)));
                far = (A != B) && (__dmul_rn(theta, r) >= __dadd_rn(a.w, c.w));
            }
            if (!far) {
                const bool la = a.nkid == 0, lb = c.nkid == 0;
                if (la && lb) {
                    knear = 1;
                    la_leaf = a.leaf;
                    lb_leaf = c.leaf;
                } else {
                    split_a = !la && (lb || a.w >= c.w);
                    first = split_a ? a.first : c.first;
                    ksplit = (unsigned)(split_a ? a.nkid : c.nkid);
                }
            }
        }
        const ull sn = block_append(&ctr[C_NEAR], knear, sw, &sb);
        if (knear) {
            if (sn < capN) near[sn] = ((uint64_t)(uint32_t)la_leaf << 32) | (uint32_t)lb_leaf;
            else ctr[C_OVFN] = 1;
        }
        const ull sf = block_append(&ctr[C_F + step + 1], ksplit, sw, &sb);
        if (ksplit) {
            if (sf + ksplit <= capF) {
                for (unsigned k = 0; k < ksplit; k++) {
                    const int ch = first + (int)k;
                    fout[sf + k] = split_a ? make_int2(ch, B) : make_int2(A, ch);
                }
            } else {
                ctr[C_OVF] = 1;
            }
        }
    }
}

// the root pair starts the traversal; every frontier count and the near count are reset
__global__ void nt_trav_init(int2* __restrict__ fr0, ull* __restrict__ ctr)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    fr0[0] = make_int2(0, 0);
    ctr[C_NEAR] = 0;
    ctr[C_OVF] = 0;
    ctr[C_OVFN] = 0;
    for (int k = 0; k < TRAV_STEPS + 2; k++) ctr[C_F + k] = 0;
    ctr[C_F] = 1;
}

// ------------------------------------------------------------------- CSR
__global__ void nt_csr_col(int64_t m, const uint64_t* __restrict__ keys, int32_t* __restrict__ col)
{
    for (int64_t i = gtid(); i < m; i += gstride()) col[i] = (int32_t)(uint32_t)(keys[i] & 0xffffffffULL);
}

__global__ void nt_csr_row(int64_t m, int64_t nl, const uint64_t* __restrict__ keys, int32_t* __restrict__ row)
{
    for (int64_t l = gtid(); l <= nl; l += gstride()) {
        const uint64_t want = (uint64_t)l << 32;
        int64_t lo = 0, hi = m;
        while (lo < hi) {
            const int64_t mid = lo + ((hi - lo) >> 1);
            if (keys[mid] < want) lo = mid + 1;
            else hi = mid;
        }
        row[l] = (int32_t)lo;
    }
}

// particle pairs over all leaf pairs
__global__ void nt_pairs(int64_t nl, const int32_t* __restrict__ lb, const int32_t* __restrict__ le,
                         const int32_t* __restrict__ row, const int32_t* __restrict__ col, ull* __restrict__ ctr)
{
    ull acc = 0;
    for (int64_t l = gtid(); l < nl; l += gstride()) {
        ull s = 0;
        for (int j = row[l]; j < row[l + 1]; j++) s += (ull)(le[col[j]] - lb[col[j]]);
        acc += s * (ull)(le[l] - lb[l]);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0 && acc) atomicAdd(&ctr[C_PAIRS], acc);
}

__global__ void nt_leaf_of_lists(int64_t nl, const int32_t* __restrict__ lb, const int32_t* __restrict__ le,
                                 int32_t* __restrict__ leaf_of)
{
    for (int64_t l = gtid(); l < nl; l += gstride())
        for (int p = lb[l]; p < le[l]; p++) leaf_of[p] = (int32_t)l;
}

// ------------------------------------------------------------ warp groups
// One warp per group of 32 Morton positions: lane i walks the source list of
// the group's i-th leaf; each step takes the smallest source leaf among the
// lanes' heads (a k-way merge), with the mask of the lanes that hold it.
// Consecutive source leaves with the same mask are joined into one interval.
template <bool WRITE>
__global__ void nt_groups(int64_t n, int64_t ngroups, const int32_t* __restrict__ leaf_of,
                          const int32_t* __restrict__ row, const int32_t* __restrict__ col,
                          const int32_t* __restrict__ lb, const int32_t* __restrict__ le,
                          int32_t* __restrict__ grp_cnt, const int32_t* __restrict__ grp_row, int4* __restrict__ ivs)
{
    const unsigned lane = threadIdx.x & 31;
    const int64_t g = gtid() >> 5;
    if (g >= ngroups) return;
    const int64_t p0 = 32 * g;
    const int64_t p1 = (p0 + 32 < n ? p0 + 32 : n) - 1;
    const int l0 = leaf_of[p0], l1 = leaf_of[p1];
    const int k = l1 - l0 + 1;                     // <= 32: every leaf holds a particle of the group
    int cur = 0, end = 0;
    if ((int)lane < k) { cur = row[l0 + lane]; end = row[l0 + lane + 1]; }
    int count = 0, first = -1, last = -1;
    unsigned omask = 0;
    int64_t out = WRITE ? grp_row[g] : 0;
    for (;;) {
        const unsigned head = cur < end ? (unsigned)col[cur] : 0xffffffffu;
        const unsigned m = __reduce_min_sync(0xffffffffu, head);
        if (m == 0xffffffffu) break;
        const bool hit = head == m;
        const unsigned mask = __ballot_sync(0xffffffffu, hit);
        if (hit) cur++;
        if (first >= 0 && (int)m == last + 1 && mask == omask) {
            last = (int)m;
        } else {
            if (first >= 0) {
                if (WRITE && lane == 0) ivs[out + count] = make_int4(lb[first], le[last], (int)omask, 0);
                count++;
            }
            first = last = (int)m;
            omask = mask;
        }
    }
    if (first >= 0) {
        if (WRITE && lane == 0) ivs[out + count] = make_int4(lb[first], le[last], (int)omask, 0);
        count++;
    }
    if (!WRITE && lane == 0) grp_cnt[g] = count;
}

cudaError_t grow_cub(NearScratch& s, size_t bytes) { return s.cub.grow(bytes < 256 ? 256 : bytes); }

inline unsigned gs_blocks(int64_t work)
{
    const int64_t b = (work + GS_THREADS - 1) / GS_THREADS;
    return (unsigned)(b < 1 ? 1 : (b > GS_BLOCKS ? GS_BLOCKS : b));
}

#define NT_TRY(call)                         \
    do {                                     \
        cudaError_t e_ = (call);             \
        if (e_ != cudaSuccess) return e_;    \
    } while (0)

cudaError_t read_counters(NearScratch& s, cudaStream_t st, SyncFn sync, void* sync_ctx)
{
    NT_TRY(cudaMemcpyAsync(s.hctr, s.ctr.p, C_COUNT * sizeof(ull), cudaMemcpyDeviceToHost, st));
    return sync(sync_ctx);
}

// CSR rows, pair count and leaf_of from the leaf lists already on the device
cudaError_t finish_lists(NearScratch& s, NearLists* L, cudaStream_t st, SyncFn sync, void* sync_ctx, int64_t* launches)
{
    const int64_t nl = L->nleaves;
    NT_TRY(cudaMemsetAsync((char*)s.ctr.p + C_PAIRS * sizeof(ull), 0, sizeof(ull), st));
    nt_pairs<<<gs_blocks(nl), GS_THREADS, 0, st>>>(nl, L->leaf_begin, L->leaf_end, L->row, L->col, s.ctr.as<ull>());
    *launches += 1;
    NT_TRY(cudaGetLastError());
    NT_TRY(read_counters(s, st, sync, sync_ctx));
    L->pairs = s.hctr[C_PAIRS];
    return cudaSuccess;
}

}  // namespace

void NearScratch::release_all()
{
    for (DevBuf* b : {&keys, &keys2, &idx, &perm, &xs, &part, &nodes, &node_lvl, &node_box, &node_cr, &node_leaf,
                      &ctr, &flag, &leaf_of, &lb, &le, &row, &col, &fr0, &fr1, &near0, &near1, &grp_cnt, &grp_row,
                      &ivs, &cub})
        b->release();
    if (hctr) cudaFreeHost(hctr);
    hctr = nullptr;
    capF = capN = 0;
}

static cudaError_t common_alloc(NearScratch& s, int64_t n)
{
    NT_TRY(s.ctr.grow(C_COUNT * sizeof(ull)));
    if (!s.hctr) NT_TRY(cudaHostAlloc((void**)&s.hctr, C_COUNT * sizeof(ull), cudaHostAllocDefault));
    NT_TRY(s.perm.grow(n * sizeof(int32_t)));
    NT_TRY(s.leaf_of.grow(n * sizeof(int32_t)));
    return cudaSuccess;
}

cudaError_t near_build(NearScratch& s, int64_t n, const double* x, int leaf_size, double theta, cudaStream_t st,
                       SyncFn sync, void* sync_ctx, NearLists* L, int64_t* launches)
{
    *L = NearLists();
    L->n = n;
    NT_TRY(common_alloc(s, n));
    const int64_t ncap = 2 * n + 2;   // every split makes >= 2 children: < 2n nodes
    NT_TRY(s.keys.grow(n * sizeof(uint64_t)));
    NT_TRY(s.keys2.grow(n * sizeof(uint64_t)));
    NT_TRY(s.idx.grow(n * sizeof(int32_t)));
    NT_TRY(s.xs.grow(3 * n * sizeof(double)));
    NT_TRY(s.part.grow(6 * GS_BLOCKS * sizeof(double) + 64));
    NT_TRY(s.nodes.grow(ncap * sizeof(int4)));
    NT_TRY(s.node_lvl.grow(ncap * sizeof(int32_t)));
    NT_TRY(s.node_box.grow(6 * ncap * sizeof(double)));
    NT_TRY(s.node_cr.grow(ncap * sizeof(TravNode)));
    NT_TRY(s.node_leaf.grow(ncap * sizeof(int32_t)));
    NT_TRY(s.flag.grow(n * sizeof(int32_t)));
    NT_TRY(s.lb.grow(n * sizeof(int32_t)));
    NT_TRY(s.le.grow(n * sizeof(int32_t)));
    ull* ctr = s.ctr.as<ull>();
    double* box = s.part.as<double>() + 6 * GS_BLOCKS;
    NT_TRY(cudaMemsetAsync(ctr, 0, C_COUNT * sizeof(ull), st));

    // 1. keys and the Morton order
    const unsigned gb = gs_blocks(n);
    nt_bbox_partial<<<gb, GS_THREADS, 0, st>>>(n, x, s.part.as<double>());
    nt_bbox_final<<<1, GS_THREADS, 0, st>>>((int)gb, s.part.as<double>(), box);
    nt_keys<<<gb, GS_THREADS, 0, st>>>(n, x, box, s.keys.as<uint64_t>(), s.idx.as<int32_t>());
    size_t tb = 0;
    NT_TRY(cub::DeviceRadixSort::SortPairs(nullptr, tb, s.keys.as<uint64_t>(), s.keys2.as<uint64_t>(),
                                           s.idx.as<int32_t>(), s.perm.as<int32_t>(), (int)n, 0, 63, st));
    NT_TRY(grow_cub(s, tb));
    NT_TRY(cub::DeviceRadixSort::SortPairs(s.cub.p, tb, s.keys.as<uint64_t>(), s.keys2.as<uint64_t>(),
                                           s.idx.as<int32_t>(), s.perm.as<int32_t>(), (int)n, 0, 63, st));
    const uint64_t* skey = s.keys2.as<uint64_t>();
    nt_gather_x<<<gb, GS_THREADS, 0, st>>>(n, x, s.perm.as<int32_t>(), s.xs.as<double>());
    *launches += 6;

    // 2. nodes, breadth first
    int4* nodes = s.nodes.as<int4>();
    nt_init<<<1, 32, 0, st>>>(n, nodes, s.node_lvl.as<int32_t>(), ctr);
    for (int d = 0; d < MAX_DEPTH; d++) {
        nt_split<<<gs_blocks(n / 2 + 1), GS_THREADS, 0, st>>>(d, skey, leaf_size, nodes, s.node_lvl.as<int32_t>(), ctr);
        nt_mark<<<1, 32, 0, st>>>(d, ctr);
    }
    // leaves in Morton order
    NT_TRY(cudaMemsetAsync(s.flag.p, 0, n * sizeof(int32_t), st));
    nt_leaf_flag<<<gs_blocks(n), GS_THREADS, 0, st>>>(nodes, ctr, s.flag.as<int32_t>());
    NT_TRY(cub::DeviceScan::InclusiveSum(nullptr, tb, s.flag.as<int32_t>(), s.leaf_of.as<int32_t>(), (int)n, st));
    NT_TRY(grow_cub(s, tb));
    NT_TRY(cub::DeviceScan::InclusiveSum(s.cub.p, tb, s.flag.as<int32_t>(), s.leaf_of.as<int32_t>(), (int)n, st));
    nt_leaf_ids<<<gs_blocks(2 * n), GS_THREADS, 0, st>>>(n, nodes, s.leaf_of.as<int32_t>(), s.lb.as<int32_t>(),
                                                          s.le.as<int32_t>(), s.node_leaf.as<int32_t>(), ctr);
    nt_leaf_of<<<gb, GS_THREADS, 0, st>>>(n, s.leaf_of.as<int32_t>());
    // 3. geometry
    double* nbox = s.node_box.as<double>();
    nt_box_leaf<<<gs_blocks(2 * n), GS_THREADS, 0, st>>>(nodes, ctr, s.xs.as<double>(), nbox);
    for (int d = MAX_DEPTH; d >= 0; d--) nt_box_inner<<<gs_blocks(n / 2 + 1), GS_THREADS, 0, st>>>(d, nodes, ctr, nbox);
    nt_cr<<<gs_blocks(2 * n), GS_THREADS, 0, st>>>(ctr, nbox, nodes, s.node_leaf.as<int32_t>(),
                                                   s.node_cr.as<TravNode>());
    *launches += 2 * MAX_DEPTH + 1 + 4 + (MAX_DEPTH + 1) + 2;
    NT_TRY(cudaGetLastError());

    // 4. traversal; on overflow of a frontier or of the near list, grow and repeat
    // a uniform cloud at leaf size 64 and theta 0.4 needs ~32 n frontier pairs and ~16 n near pairs
    if (s.capF == 0) s.capF = (size_t)(n < 4096 ? 4096 : n) * 40;
    if (s.capN == 0) s.capN = (size_t)(n < 4096 ? 4096 : n) * 24;
    for (int attempt = 0;; attempt++) {
        NT_TRY(s.fr0.grow(s.capF * sizeof(int2)));
        NT_TRY(s.fr1.grow(s.capF * sizeof(int2)));
        NT_TRY(s.near0.grow(s.capN * sizeof(uint64_t)));
        NT_TRY(s.near1.grow(s.capN * sizeof(uint64_t)));
        nt_trav_init<<<1, 32, 0, st>>>(s.fr0.as<int2>(), ctr);
        for (int k = 0; k < TRAV_STEPS; k++) {
            const int2* fin = (k & 1) ? s.fr1.as<int2>() : s.fr0.as<int2>();
            int2* fout = (k & 1) ? s.fr0.as<int2>() : s.fr1.as<int2>();
            nt_trav<<<GS_BLOCKS, GS_THREADS, 0, st>>>(k, theta, s.node_cr.as<TravNode>(), fin, fout,
                                                       s.near0.as<uint64_t>(), ctr, (ull)s.capF, (ull)s.capN);
        }
        *launches += TRAV_STEPS + 1;
        NT_TRY(cudaGetLastError());
        NT_TRY(read_counters(s, st, sync, sync_ctx));
        const ull* h = (const ull*)s.hctr;
        if (!h[C_OVF] && !h[C_OVFN] && h[C_F + TRAV_STEPS] == 0) break;
        // The counters hold the full sizes of every frontier up to the one that overflowed
        // (appends are counted even when they do not fit) and the near pairs found so far:
        // grow past them, so that each retry gets at least one step further.
        if (attempt >= TRAV_STEPS + 2) return cudaErrorMemoryAllocation;
        ull maxF = 0;
        for (int k = 0; k <= TRAV_STEPS; k++) maxF = h[C_F + k] > maxF ? h[C_F + k] : maxF;
        const size_t needF = (size_t)maxF + (size_t)maxF / 4, needN = (size_t)h[C_NEAR] + (size_t)h[C_NEAR] / 4;
        s.capF = std::max(2 * s.capF, needF);
        s.capN = std::max(h[C_NEAR] >= s.capN ? 2 * s.capN : s.capN, needN);
    }
    const ull* h = (const ull*)s.hctr;
    L->nodes = (int64_t)h[C_NODES];
    L->nleaves = (int64_t)h[C_NL];
    L->nlpairs = (int64_t)h[C_NEAR];
    if (L->nlpairs > (int64_t)INT32_MAX) return cudaErrorMemoryAllocation;
    const int64_t nl = L->nleaves, m = L->nlpairs;

    // 5. CSR: sort the (target leaf, source leaf) keys
    int hb = 1;
    while (((int64_t)1 << hb) <= nl) hb++;
    NT_TRY(cub::DeviceRadixSort::SortKeys(nullptr, tb, s.near0.as<uint64_t>(), s.near1.as<uint64_t>(), (int)m, 0,
                                          32 + hb, st));
    NT_TRY(grow_cub(s, tb));
    NT_TRY(cub::DeviceRadixSort::SortKeys(s.cub.p, tb, s.near0.as<uint64_t>(), s.near1.as<uint64_t>(), (int)m, 0,
                                          32 + hb, st));
    NT_TRY(s.row.grow((nl + 1) * sizeof(int32_t)));
    NT_TRY(s.col.grow((m > 0 ? m : 1) * sizeof(int32_t)));
    nt_csr_col<<<gs_blocks(m), GS_THREADS, 0, st>>>(m, s.near1.as<uint64_t>(), s.col.as<int32_t>());
    nt_csr_row<<<gs_blocks(nl + 1), GS_THREADS, 0, st>>>(m, nl, s.near1.as<uint64_t>(), s.row.as<int32_t>());
    *launches += 4;
    NT_TRY(cudaGetLastError());
    L->perm = s.perm.as<int32_t>();
    L->leaf_of = s.leaf_of.as<int32_t>();
    L->leaf_begin = s.lb.as<int32_t>();
    L->leaf_end = s.le.as<int32_t>();
    L->row = s.row.as<int32_t>();
    L->col = s.col.as<int32_t>();
    return finish_lists(s, L, st, sync, sync_ctx, launches);
}

cudaError_t near_upload(NearScratch& s, int64_t n, const int32_t* perm, int64_t nl, const int64_t* leaf_begin,
                        const int64_t* leaf_end, const int64_t* row, const int32_t* col, cudaStream_t st,
                        SyncFn sync, void* sync_ctx, NearLists* L, int64_t* launches)
{
    *L = NearLists();
    L->n = n;
    L->nleaves = nl;
    L->nlpairs = row[nl];
    NT_TRY(common_alloc(s, n));
    NT_TRY(s.lb.grow(nl * sizeof(int32_t)));
    NT_TRY(s.le.grow(nl * sizeof(int32_t)));
    NT_TRY(s.row.grow((nl + 1) * sizeof(int32_t)));
    NT_TRY(s.col.grow((L->nlpairs > 0 ? L->nlpairs : 1) * sizeof(int32_t)));
    std::vector<int32_t> b32(nl), e32(nl), r32(nl + 1);
    for (int64_t l = 0; l < nl; l++) { b32[l] = (int32_t)leaf_begin[l]; e32[l] = (int32_t)leaf_end[l]; }
    for (int64_t l = 0; l <= nl; l++) r32[l] = (int32_t)row[l];
    NT_TRY(cudaMemcpyAsync(s.perm.p, perm, n * sizeof(int32_t), cudaMemcpyHostToDevice, st));
    NT_TRY(cudaMemcpyAsync(s.lb.p, b32.data(), nl * sizeof(int32_t), cudaMemcpyHostToDevice, st));
    NT_TRY(cudaMemcpyAsync(s.le.p, e32.data(), nl * sizeof(int32_t), cudaMemcpyHostToDevice, st));
    NT_TRY(cudaMemcpyAsync(s.row.p, r32.data(), (nl + 1) * sizeof(int32_t), cudaMemcpyHostToDevice, st));
    if (L->nlpairs > 0)
        NT_TRY(cudaMemcpyAsync(s.col.p, col, L->nlpairs * sizeof(int32_t), cudaMemcpyHostToDevice, st));
    nt_leaf_of_lists<<<gs_blocks(nl), GS_THREADS, 0, st>>>(nl, s.lb.as<int32_t>(), s.le.as<int32_t>(),
                                                            s.leaf_of.as<int32_t>());
    *launches += 1;
    NT_TRY(cudaGetLastError());
    // the host vectors must outlive the copies: finish_lists waits for the stream
    L->perm = s.perm.as<int32_t>();
    L->leaf_of = s.leaf_of.as<int32_t>();
    L->leaf_begin = s.lb.as<int32_t>();
    L->leaf_end = s.le.as<int32_t>();
    L->row = s.row.as<int32_t>();
    L->col = s.col.as<int32_t>();
    return finish_lists(s, L, st, sync, sync_ctx, launches);
}

cudaError_t near_groups(NearScratch& s, NearLists* L, cudaStream_t st, SyncFn sync, void* sync_ctx, int64_t* launches)
{
    const int64_t n = L->n, ng = (n + 31) / 32;
    L->ngroups = ng;
    NT_TRY(s.grp_cnt.grow((ng + 1) * sizeof(int32_t)));
    NT_TRY(s.grp_row.grow((ng + 1) * sizeof(int32_t)));
    NT_TRY(cudaMemsetAsync(s.grp_cnt.p, 0, (ng + 1) * sizeof(int32_t), st));
    const unsigned blocks = (unsigned)((ng * 32 + GS_THREADS - 1) / GS_THREADS);
    nt_groups<false><<<blocks, GS_THREADS, 0, st>>>(n, ng, L->leaf_of, L->row, L->col, L->leaf_begin, L->leaf_end,
                                                    s.grp_cnt.as<int32_t>(), nullptr, nullptr);
    size_t tb = 0;
    NT_TRY(cub::DeviceScan::ExclusiveSum(nullptr, tb, s.grp_cnt.as<int32_t>(), s.grp_row.as<int32_t>(), (int)(ng + 1), st));
    NT_TRY(grow_cub(s, tb));
    NT_TRY(cub::DeviceScan::ExclusiveSum(s.cub.p, tb, s.grp_cnt.as<int32_t>(), s.grp_row.as<int32_t>(), (int)(ng + 1), st));
    NT_TRY(cudaGetLastError());
    int32_t total = 0;
    NT_TRY(cudaMemcpyAsync(s.hctr, s.grp_row.as<int32_t>() + ng, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    NT_TRY(sync(sync_ctx));
    std::memcpy(&total, s.hctr, sizeof(int32_t));
    L->nivs = total;
    NT_TRY(s.ivs.grow((total > 0 ? total : 1) * sizeof(int4)));
    nt_groups<true><<<blocks, GS_THREADS, 0, st>>>(n, ng, L->leaf_of, L->row, L->col, L->leaf_begin, L->leaf_end,
                                                   nullptr, s.grp_row.as<int32_t>(), s.ivs.as<int4>());
    *launches += 3;
    NT_TRY(cudaGetLastError());
    L->grp_row = s.grp_row.as<int32_t>();
    L->ivs = s.ivs.as<int4>();
    return cudaSuccess;
}

}  // namespace vpm
