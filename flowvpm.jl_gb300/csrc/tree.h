// tree.h -- host octree and near-field leaf-pair lists (tree.cpp).
#pragma once
#include <cstdint>
#include <vector>

namespace vpm {

struct LeafLists {
    std::vector<int32_t> perm;                   // perm[i] = original index of the i-th particle (Morton order)
    std::vector<int64_t> leaf_begin, leaf_end;   // particle ranges of the leaves, in Morton order
    std::vector<int64_t> row;                    // CSR over target leaves: row[l]..row[l+1]
    std::vector<int32_t> col;                    //   source leaves of target leaf l
    int64_t pairs = 0;                           // particle pairs over all leaf pairs
    int64_t far_node_pairs = 0;                  // node pairs accepted as far field
    int64_t nodes = 0;
};

// Octree of the n positions x[n][3] with leaves of at most leaf_size particles,
// and the leaf pairs with theta * |c_A - c_B| < R_A + R_B.  Returns 0 or -1.
int build_leaf_lists(int64_t n, const double* x, int leaf_size, double theta, LeafLists* out);

}  // namespace vpm
