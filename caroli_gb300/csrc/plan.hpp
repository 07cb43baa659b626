// Host-side symbolic phase of the nested-dissection transmission: the elimination tree of each
// independent block, the variables of every front, and how each front is assembled. Produces
// flat, device-ready descriptors (FrontDesc, child index maps, H-entry lists).
//
// Follows crates/caroli-green/src/nested.rs of caroli:
//   geometric bisection      split       nested.rs:1049-1093 (LEAF_ORBITALS = 16, nested.rs:34)
//   boundaries               symbolic    nested.rs:1095-1122
//   front variables          front_vars  nested.rs:144-158
//   H entries of a front     separator_entries nested.rs:160-179
//   root on the lead slices  Tree::root  nested.rs:246-281 and root_with_leads :806-845
//   pivot delay              Tree::front nested.rs:356-373 (a refused front goes up whole)
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace caroli {

// One H entry of a front: F[a, b] -= conj ? conj(vals[q]) : vals[q].
struct Entry {
  int32_t a, b;
  int32_t conj, pad;
  int64_t q;
};

// Device-ready description of one front (and of the root, which is the last front).
struct FrontDesc {
  int32_t n;          // variables of the front
  int32_t ne;         // eliminated here (0: nothing eliminated, the whole front goes to the parent)
  int32_t nchild;     // 0..2
  int32_t level;      // execution level (children run at lower levels)
  int32_t child[2];   // front indices of the children
  int32_t child_dim[2];  // size of the block a child hands over (its boundary, or all of it)
  int64_t child_off[2];  // element offset of that block inside the child's front
  int64_t map_off[2];    // offset of the child's index map in `maps` (n entries: child index or -1)
  int64_t own_off;       // offset of the own-separator flags in `own` (n entries)
  int64_t ent_off;       // entries [ent_off, ent_off + ent_cnt) in `entries`
  int64_t ent_cnt;
  int64_t arena_off;     // element offset of the front inside a solve's arena (n x n, column-major)
  int64_t var_off;       // block-local indices of the front's variables in `vidx` (n entries)
  int64_t toff;          // row offset of the front's ne x c block in a solve's forward buffer
  int64_t hoff;          // row offset of its (n - ne) x c handed block in a solve's update buffer
};

struct SystemDesc {
  int64_t n;
  const int64_t* row_ptr;
  const uint32_t* cols;
  int64_t nsites;
  int dim;
  const int64_t* cells;
  const int64_t* site_offsets;
  const int64_t* site_orbitals;
  int64_t range[3];
  int64_t n_interior;
  const int64_t* interior;
  int nblocks;
  const int32_t* labels;
  const int64_t* left_ptr;
  const int64_t* left;
  const int64_t* right_ptr;
  const int64_t* right;
};

struct TreeNode {
  std::vector<int64_t> eliminate, boundary;
  std::vector<int32_t> children;
};

// The symbolic data of one block, and one front plan (static, or with delayed fronts).
struct BlockTree {
  std::vector<TreeNode> nodes;  // post-order
  std::vector<int32_t> top;     // children of the root
  std::vector<int64_t> left, right;
  // Block-local numbering (for refinement solves): the block's orbitals in increasing order, the
  // local index of every orbital of the system (-1 outside the block), and H restricted to the
  // block as CSR with local columns and the index of each entry in the system's value array.
  std::vector<int64_t> orbitals;
  std::vector<int32_t> local;
  std::vector<int32_t> csr_ptr, csr_col;
  std::vector<int64_t> csr_q;
  std::vector<int32_t> left_local, right_local;
};

// Where a refinement sweep finds row i of a front (one 16-byte load per row): `own` = block-local
// row of the right-hand side when the variable is the front's own separator variable, else -1;
// `h0`, `h1` = rows of the children's handed vectors in the update buffer (child hoff + index in
// the child's handed block), else -1; `var` = block-local row of the variable.
struct SweepRow {
  int32_t own, h0, h1, var;
};

struct FrontPlan {
  std::vector<FrontDesc> fronts;  // tree fronts in post-order, then the root
  std::vector<int32_t> maps;
  std::vector<uint8_t> own;
  std::vector<Entry> entries;
  std::vector<std::vector<int64_t>> vars;  // variables of each front (elim then rest)
  std::vector<int32_t> vidx;               // block-local index of each front variable
  std::vector<SweepRow> srows;             // parallel to vidx
  int64_t sum_ne = 0, sum_nb = 0;          // rows of the forward and update buffers
  int32_t levels = 0;                      // the root runs at level `levels - 1`
  int64_t arena_elems = 0;
  int32_t root = 0;
  int32_t nl = 0, nr = 0, rpos = 0, nd = 0;  // root: [nd delayed][nl left][right at nd + rpos]
  int64_t max_ne = 0, max_n = 0;
};

// Builds the site tree once and the orbital tree of every block.
std::vector<BlockTree> build_trees(const SystemDesc& d);

// The plan of a block; `delayed[k]` marks tree fronts that eliminate nothing (empty: none).
FrontPlan make_plan(const SystemDesc& d, const BlockTree& t, const std::vector<uint8_t>& delayed);

}  // namespace caroli
