// Host symbolic phase (see plan.hpp for the reference map).
#include "plan.hpp"

#include <algorithm>
#include <climits>
#include <stdexcept>
#include <unordered_map>

namespace caroli {
namespace {

constexpr int64_t LEAF_ORBITALS = 16;

struct SiteNode {
  std::vector<int64_t> sites;
  std::vector<int32_t> children;
};

// Recursive bisection of the longest extent (ties: lowest axis); the separator is as thick as
// the hopping range along that axis; domains of at most LEAF_ORBITALS orbitals are leaves.
int32_t bisect(const SystemDesc& d, std::vector<int64_t> sites, std::vector<SiteNode>& out) {
  if (sites.empty()) return -1;
  int64_t orbitals = 0;
  for (int64_t i : sites) orbitals += d.site_orbitals[i];
  int axis = 0;
  int64_t lo = 0, hi = -1, ext = -1;
  for (int a = 0; a < d.dim; ++a) {
    int64_t l = INT64_MAX, h = INT64_MIN;
    for (int64_t i : sites) {
      int64_t c = d.cells[i * 3 + a];
      l = std::min(l, c);
      h = std::max(h, c);
    }
    if (h - l > ext) { ext = h - l; axis = a; lo = l; hi = h; }
  }
  if (orbitals <= LEAF_ORBITALS || hi - lo < d.range[axis]) {
    out.push_back({std::move(sites), {}});
    return (int32_t)out.size() - 1;
  }
  const int64_t thick = d.range[axis];
  const int64_t mid = lo + (hi - lo + 1 - thick) / 2;
  std::vector<int64_t> a, sep, b;
  for (int64_t i : sites) {
    int64_t c = d.cells[i * 3 + axis];
    (c < mid ? a : (c < mid + thick ? sep : b)).push_back(i);
  }
  std::vector<int32_t> kids;
  int32_t ka = bisect(d, std::move(a), out);
  if (ka >= 0) kids.push_back(ka);
  int32_t kb = bisect(d, std::move(b), out);
  if (kb >= 0) kids.push_back(kb);
  out.push_back({std::move(sep), std::move(kids)});
  return (int32_t)out.size() - 1;
}

// Boundary of each node: columns of its eliminated rows and its children's boundaries, minus
// what is eliminated at or below it.
void boundaries(const SystemDesc& d, std::vector<TreeNode>& nodes) {
  constexpr int64_t NEVER = INT64_MAX;
  std::vector<int64_t> rank(d.n, NEVER), last(nodes.size());
  int64_t next = 0;
  for (size_t k = 0; k < nodes.size(); ++k) {
    for (int64_t o : nodes[k].eliminate) rank[o] = next++;
    last[k] = next;
  }
  for (size_t k = 0; k < nodes.size(); ++k) {
    std::vector<int64_t> bnd;
    for (int64_t o : nodes[k].eliminate)
      for (int64_t q = d.row_ptr[o]; q < d.row_ptr[o + 1]; ++q) bnd.push_back(d.cols[q]);
    for (int32_t c : nodes[k].children)
      bnd.insert(bnd.end(), nodes[c].boundary.begin(), nodes[c].boundary.end());
    std::vector<int64_t> keep;
    keep.reserve(bnd.size());
    for (int64_t o : bnd)
      if (rank[o] == NEVER || rank[o] >= last[k]) keep.push_back(o);
    std::sort(keep.begin(), keep.end());
    keep.erase(std::unique(keep.begin(), keep.end()), keep.end());
    nodes[k].boundary = std::move(keep);
  }
}

bool has(const std::vector<int64_t>& sorted, int64_t x) { return std::binary_search(sorted.begin(), sorted.end(), x); }

// Position lookup for the variables of one front.
struct Index {
  std::unordered_map<int64_t, int32_t> m;
  explicit Index(const std::vector<int64_t>& vars) {
    m.reserve(vars.size() * 2);
    for (size_t k = 0; k < vars.size(); ++k) m.emplace(vars[k], (int32_t)k);
  }
  int32_t get(int64_t x) const {
    auto it = m.find(x);
    return it == m.end() ? -1 : it->second;
  }
};

}  // namespace

std::vector<BlockTree> build_trees(const SystemDesc& d) {
  std::vector<SiteNode> site_nodes;
  std::vector<int64_t> interior(d.interior, d.interior + d.n_interior);
  int32_t top = bisect(d, interior, site_nodes);
  std::vector<BlockTree> out;
  for (int b = 0; b < d.nblocks; ++b) {
    BlockTree t;
    t.nodes.resize(site_nodes.size());
    for (size_t k = 0; k < site_nodes.size(); ++k) {
      auto& node = t.nodes[k];
      for (int64_t i : site_nodes[k].sites)
        for (int64_t o = d.site_offsets[i]; o < d.site_offsets[i] + d.site_orbitals[i]; ++o)
          if (d.labels[o] == b) node.eliminate.push_back(o);
      std::sort(node.eliminate.begin(), node.eliminate.end());
      node.children = site_nodes[k].children;
    }
    if (top >= 0) t.top.push_back(top);
    boundaries(d, t.nodes);
    t.left.assign(d.left + d.left_ptr[b], d.left + d.left_ptr[b + 1]);
    t.right.assign(d.right + d.right_ptr[b], d.right + d.right_ptr[b + 1]);
    t.local.assign(d.n, -1);
    for (int64_t o = 0; o < d.n; ++o)
      if (d.labels[o] == b) {
        t.local[o] = (int32_t)t.orbitals.size();
        t.orbitals.push_back(o);
      }
    t.csr_ptr.push_back(0);
    for (int64_t o : t.orbitals) {
      for (int64_t q = d.row_ptr[o]; q < d.row_ptr[o + 1]; ++q) {
        int32_t c = t.local[d.cols[q]];
        if (c < 0) continue;  // an explicit zero coupling another block
        t.csr_col.push_back(c);
        t.csr_q.push_back(q);
      }
      t.csr_ptr.push_back((int32_t)t.csr_col.size());
    }
    for (int64_t o : t.left) t.left_local.push_back(t.local[o]);
    for (int64_t o : t.right) t.right_local.push_back(t.local[o]);
    out.push_back(std::move(t));
  }
  return out;
}

FrontPlan make_plan(const SystemDesc& d, const BlockTree& t, const std::vector<uint8_t>& delayed) {
  FrontPlan p;
  const size_t nn = t.nodes.size();
  p.fronts.resize(nn + 1);
  p.vars.resize(nn + 1);
  std::vector<int32_t> height(nn, 0);
  // What each front hands to its parent: its boundary, or all its variables when delayed.
  std::vector<std::vector<int64_t>> handed(nn);
  int64_t arena = 0;

  auto add_child = [&](FrontDesc& f, int slot, int32_t c, const Index& pos) {
    const FrontDesc& cf = p.fronts[c];
    const auto& hv = handed[c];
    f.child[slot] = c;
    f.child_dim[slot] = (int32_t)hv.size();
    // A child that eliminated ne_c variables hands its trailing (n_c - ne_c) block.
    f.child_off[slot] = (int64_t)cf.ne * cf.n + cf.ne;
    f.map_off[slot] = (int64_t)p.maps.size();
    std::vector<int32_t> map(f.n, -1);
    for (size_t a = 0; a < hv.size(); ++a) {
      int32_t pa = pos.get(hv[a]);
      if (pa < 0) throw std::runtime_error("child variable missing from its parent front");
      map[pa] = (int32_t)a;
    }
    p.maps.insert(p.maps.end(), map.begin(), map.end());
  };

  for (size_t k = 0; k < nn; ++k) {
    const TreeNode& node = t.nodes[k];
    // front_vars: own separator and what children could not eliminate (sorted), then boundary.
    std::vector<int64_t> elim = node.eliminate;
    for (int32_t c : node.children)
      for (int64_t o : handed[c])
        if (!has(node.boundary, o)) elim.push_back(o);
    std::sort(elim.begin(), elim.end());
    elim.erase(std::unique(elim.begin(), elim.end()), elim.end());
    std::vector<int64_t> vars = elim;
    vars.insert(vars.end(), node.boundary.begin(), node.boundary.end());
    Index pos(vars);
    FrontDesc& f = p.fronts[k];
    f.n = (int32_t)vars.size();
    bool delay = !delayed.empty() && delayed[k];
    f.ne = delay ? 0 : (int32_t)elim.size();
    f.nchild = (int32_t)node.children.size();
    if (f.nchild > 2) throw std::runtime_error("a front with more than two children");
    for (int s = 0; s < f.nchild; ++s) {
      int32_t c = node.children[s];
      height[k] = std::max(height[k], height[c] + 1);
      add_child(f, s, c, pos);
    }
    f.level = height[k];
    // Own separator flags (z on the diagonal).
    f.own_off = (int64_t)p.own.size();
    std::vector<uint8_t> own(f.n, 0);
    for (int64_t i : node.eliminate) own[pos.get(i)] = 1;
    p.own.insert(p.own.end(), own.begin(), own.end());
    // H entries of the separator with every later variable (the rest of the separator after it,
    // and the boundary); delayed variables of children already carry theirs.
    f.ent_off = (int64_t)p.entries.size();
    for (int64_t i : node.eliminate) {
      int32_t pi = pos.get(i);
      for (int64_t q = d.row_ptr[i]; q < d.row_ptr[i + 1]; ++q) {
        int64_t j = d.cols[q];
        if (j == i) {
          p.entries.push_back({pi, pi, 0, 0, q});
          continue;
        }
        int32_t pj = pos.get(j);
        if (pj < 0) continue;
        bool later = has(node.eliminate, j) ? j > i : has(node.boundary, j);
        if (later) {
          p.entries.push_back({pi, pj, 0, 0, q});
          p.entries.push_back({pj, pi, 1, 0, q});
        }
      }
    }
    f.ent_cnt = (int64_t)p.entries.size() - f.ent_off;
    f.arena_off = arena;
    arena += (int64_t)f.n * f.n;
    f.var_off = (int64_t)p.vidx.size();
    for (int64_t v : vars) p.vidx.push_back(t.local[v]);
    f.toff = p.sum_ne;
    f.hoff = p.sum_nb;
    p.sum_ne += f.ne;
    p.sum_nb += f.n - f.ne;
    p.max_ne = std::max<int64_t>(p.max_ne, f.ne);
    p.max_n = std::max<int64_t>(p.max_n, f.n);
    handed[k] = delay ? vars : node.boundary;
    p.vars[k] = std::move(vars);
  }

  // Root: variables delayed up to it, then the kept orbitals (left slice, then the right one
  // unless both slices are the same).
  const bool same = t.left == t.right;
  std::vector<int64_t> kept = t.left;
  if (!same) kept.insert(kept.end(), t.right.begin(), t.right.end());
  std::vector<int64_t> kept_sorted = kept;
  std::sort(kept_sorted.begin(), kept_sorted.end());
  std::vector<int64_t> del;
  for (int32_t c : t.top)
    for (int64_t o : handed[c])
      if (!has(kept_sorted, o)) del.push_back(o);
  std::sort(del.begin(), del.end());
  del.erase(std::unique(del.begin(), del.end()), del.end());
  std::vector<int64_t> vars = del;
  vars.insert(vars.end(), kept.begin(), kept.end());
  Index pos(vars);
  FrontDesc& r = p.fronts[nn];
  r.n = (int32_t)vars.size();
  r.ne = 0;
  r.nchild = (int32_t)t.top.size();
  int32_t lvl = 0;
  for (int s = 0; s < r.nchild; ++s) {
    add_child(r, s, t.top[s], pos);
    lvl = std::max(lvl, height[t.top[s]] + 1);
  }
  r.level = lvl;
  r.own_off = (int64_t)p.own.size();
  std::vector<uint8_t> own(r.n, 0);
  for (int64_t i : kept) own[pos.get(i)] = 1;
  p.own.insert(p.own.end(), own.begin(), own.end());
  // Entries of z - H between kept orbitals: every entry of their rows whose column is kept.
  r.ent_off = (int64_t)p.entries.size();
  for (int64_t i : kept) {
    int32_t pi = pos.get(i);
    for (int64_t q = d.row_ptr[i]; q < d.row_ptr[i + 1]; ++q) {
      if (!has(kept_sorted, d.cols[q])) continue;
      p.entries.push_back({pi, pos.get((int64_t)d.cols[q]), 0, 0, q});
    }
  }
  r.ent_cnt = (int64_t)p.entries.size() - r.ent_off;
  r.arena_off = arena;
  arena += (int64_t)r.n * r.n;
  r.var_off = (int64_t)p.vidx.size();
  for (int64_t v : vars) p.vidx.push_back(t.local[v]);
  r.toff = p.sum_ne;
  r.hoff = p.sum_nb;
  p.arena_elems = arena;
  p.max_n = std::max<int64_t>(p.max_n, r.n);
  p.vars[nn] = std::move(vars);
  // Sweep gather rows of every front (the children's hoff are final now).
  p.srows.resize(p.vidx.size());
  for (size_t k = 0; k <= nn; ++k) {
    const FrontDesc& f = p.fronts[k];
    for (int32_t i = 0; i < f.n; ++i) {
      SweepRow& g = p.srows[f.var_off + i];
      g.var = p.vidx[f.var_off + i];
      g.own = p.own[f.own_off + i] ? g.var : -1;
      g.h0 = g.h1 = -1;
      for (int c = 0; c < f.nchild; ++c) {
        const int32_t a = p.maps[f.map_off[c] + i];
        if (a < 0) continue;
        const int32_t h = (int32_t)(p.fronts[f.child[c]].hoff + a);
        if (c == 0) g.h0 = h; else g.h1 = h;
      }
    }
  }
  p.root = (int32_t)nn;
  p.levels = lvl + 1;
  p.nd = (int32_t)del.size();
  p.nl = (int32_t)t.left.size();
  p.nr = (int32_t)t.right.size();
  p.rpos = same ? 0 : p.nl;
  return p;
}

}  // namespace caroli
