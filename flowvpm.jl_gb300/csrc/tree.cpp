// tree.cpp -- host octree and near-field leaf-pair lists for the FMM path.
//
// UJ_fmm (src/FLOWVPM_UJ.jl:62-129) hands FastMultipole.jl an octree of the
// particles (leaf size ncrit) and evaluates by direct P2P every pair of leaves
// that fails the multipole acceptance criterion; FLOWVPM documents that
// criterion as "if theta*r < R1+R2 the interaction between two cells is
// resolved through P2P, where r is the distance between cell centers, and R1
// and R2 are each cell radius" (src/FLOWVPM_particlefield.jl:28-36).  This file
// builds the same kind of structure on the host:
//   * particles in Morton order (21 bits per axis of the bounding box);
//   * an octree whose nodes are key-prefix ranges, split while a node holds
//     more than leaf_size particles (or until the keys run out of bits);
//   * node geometry: center = center of the node's particle bounding box,
//     R = half its diagonal;
//   * a dual-tree traversal from (root, root): a pair is far when
//     theta * |c_A - c_B| >= R_A + R_B, is a P2P leaf pair when both are leaves,
//     and otherwise the larger node is split.
// The result is a CSR list: for every target leaf, the source leaves it
// interacts with directly (itself included).  The far field (the multipole
// part of UJ_fmm) is not computed by this library.
#include "tree.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <vector>

namespace vpm {

namespace {

inline uint64_t spread3_host(uint64_t v)
{
    v &= 0x1fffffULL;
    v = (v | (v << 32)) & 0x1f00000000ffffULL;
    v = (v | (v << 16)) & 0x1f0000ff0000ffULL;
    v = (v | (v << 8)) & 0x100f00f00f00f00fULL;
    v = (v | (v << 4)) & 0x10c30c30c30c30c3ULL;
    v = (v | (v << 2)) & 0x1249249249249249ULL;
    return v;
}

struct Node {
    int64_t begin, end;    // particle range in Morton order
    int first_child;       // index of the first child, -1 for a leaf
    int nchild;
    double c[3], R;
};

struct Builder {
    const std::vector<uint64_t>& keys;
    const double* xs;      // positions in Morton order [n][3]
    int leaf_size;
    std::vector<Node> nodes;

    void geometry(Node& nd) const
    {
        double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
        for (int64_t i = nd.begin; i < nd.end; i++)
            for (int k = 0; k < 3; k++) {
                lo[k] = std::min(lo[k], xs[3 * i + k]);
                hi[k] = std::max(hi[k], xs[3 * i + k]);
            }
        double d2 = 0;
        for (int k = 0; k < 3; k++) {
            nd.c[k] = 0.5 * (lo[k] + hi[k]);
            d2 += (hi[k] - lo[k]) * (hi[k] - lo[k]);
        }
        nd.R = 0.5 * std::sqrt(d2);
    }

    // Split node `id` on key bits [3*level .. 3*level+2] counted from the top.
    void split(int id, int level)
    {
        Node nd = nodes[id];
        if (nd.end - nd.begin <= leaf_size || level >= 21) return;
        const int shift = 3 * (20 - level);
        int64_t b = nd.begin;
        std::vector<Node> kids;
        for (int oct = 0; oct < 8 && b < nd.end; oct++) {
            // particles of this octant form a contiguous run of the sorted keys
            int64_t e = b;
            while (e < nd.end && (int)((keys[e] >> shift) & 7u) == oct) e++;
            if (e > b) {
                Node ch;
                ch.begin = b; ch.end = e; ch.first_child = -1; ch.nchild = 0;
                geometry(ch);
                kids.push_back(ch);
            }
            b = e;
        }
        if (kids.size() == 1) {   // all in one octant: descend without a new level of nodes
            split_inplace(id, level + 1);
            return;
        }
        const int first = (int)nodes.size();
        nodes[id].first_child = first;
        nodes[id].nchild = (int)kids.size();
        for (auto& k : kids) nodes.push_back(k);
        for (int i = 0; i < (int)kids.size(); i++) split(first + i, level + 1);
    }
    void split_inplace(int id, int level) { split(id, level); }
};

}  // namespace

int build_leaf_lists(int64_t n, const double* x, int leaf_size, double theta, LeafLists* out)
{
    if (n <= 0 || leaf_size < 1 || !(theta >= 0)) return -1;
    // bounding box and Morton keys
    double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int64_t i = 0; i < n; i++)
        for (int k = 0; k < 3; k++) {
            lo[k] = std::min(lo[k], x[3 * i + k]);
            hi[k] = std::max(hi[k], x[3 * i + k]);
        }
    double ext = 0;
    for (int k = 0; k < 3; k++) ext = std::max(ext, hi[k] - lo[k]);
    if (!(ext > 0)) ext = 1.0;
    std::vector<uint64_t> key(n);
    for (int64_t i = 0; i < n; i++) {
        uint64_t kk = 0;
        for (int k = 0; k < 3; k++) {
            double f = (x[3 * i + k] - lo[k]) / ext;   // cubic cells: one extent for all axes
            f = std::min(std::max(f, 0.0), 1.0);
            kk |= spread3_host((uint64_t)(f * 2097151.0)) << (2 - k);
        }
        key[i] = kk;
    }
    out->perm.resize(n);
    std::iota(out->perm.begin(), out->perm.end(), 0);
    std::stable_sort(out->perm.begin(), out->perm.end(), [&](int32_t a, int32_t b) { return key[a] < key[b]; });
    std::vector<uint64_t> skey(n);
    std::vector<double> xs(3 * n);
    for (int64_t i = 0; i < n; i++) {
        skey[i] = key[out->perm[i]];
        for (int k = 0; k < 3; k++) xs[3 * i + k] = x[3 * (int64_t)out->perm[i] + k];
    }
    Builder b{skey, xs.data(), leaf_size, {}};
    Node root;
    root.begin = 0; root.end = n; root.first_child = -1; root.nchild = 0;
    b.geometry(root);
    b.nodes.push_back(root);
    b.split(0, 0);
    const std::vector<Node>& nd = b.nodes;
    // leaves in Morton order
    std::vector<int> leaf_of_node(nd.size(), -1);
    out->leaf_begin.clear();
    out->leaf_end.clear();
    for (int i = 0; i < (int)nd.size(); i++) (void)i;
    std::vector<int> stack{0};
    std::vector<int> leaves;
    // depth-first, children in octant order = Morton order of the leaves
    while (!stack.empty()) {
        const int id = stack.back();
        stack.pop_back();
        if (nd[id].first_child < 0) {
            leaves.push_back(id);
        } else {
            for (int c = nd[id].nchild - 1; c >= 0; c--) stack.push_back(nd[id].first_child + c);
        }
    }
    for (int l = 0; l < (int)leaves.size(); l++) {
        leaf_of_node[leaves[l]] = l;
        out->leaf_begin.push_back(nd[leaves[l]].begin);
        out->leaf_end.push_back(nd[leaves[l]].end);
    }
    // dual-tree traversal
    const int nl = (int)leaves.size();
    std::vector<std::vector<int>> near(nl);
    std::vector<std::pair<int, int>> work{{0, 0}};
    int64_t far_pairs = 0;
    while (!work.empty()) {
        const auto [A, B] = work.back();
        work.pop_back();
        const Node& a = nd[A];
        const Node& c = nd[B];
        const double dx = a.c[0] - c.c[0], dy = a.c[1] - c.c[1], dz = a.c[2] - c.c[2];
        const double r = std::sqrt(dx * dx + dy * dy + dz * dz);
        if (A != B && theta * r >= a.R + c.R) { far_pairs++; continue; }
        const bool la = a.first_child < 0, lb = c.first_child < 0;
        if (la && lb) { near[leaf_of_node[A]].push_back(leaf_of_node[B]); continue; }
        // split the larger non-leaf node (the target when equal)
        const bool split_a = !la && (lb || a.R >= c.R);
        if (split_a) {
            for (int k = 0; k < a.nchild; k++) work.push_back({a.first_child + k, B});
        } else {
            for (int k = 0; k < c.nchild; k++) work.push_back({A, c.first_child + k});
        }
    }
    out->row.assign(nl + 1, 0);
    for (int l = 0; l < nl; l++) {
        std::sort(near[l].begin(), near[l].end());
        out->row[l + 1] = out->row[l] + (int64_t)near[l].size();
    }
    out->col.resize(out->row[nl]);
    out->pairs = 0;
    for (int l = 0; l < nl; l++) {
        std::copy(near[l].begin(), near[l].end(), out->col.begin() + out->row[l]);
        const int64_t nt = out->leaf_end[l] - out->leaf_begin[l];
        for (int s : near[l]) out->pairs += nt * (out->leaf_end[s] - out->leaf_begin[s]);
    }
    out->far_node_pairs = far_pairs;
    out->nodes = (int64_t)nd.size();
    return 0;
}

}  // namespace vpm
