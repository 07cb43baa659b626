// ORACLE — test infrastructure only. Not part of the product path.
//
// CPU restatement of caroli's nested-dissection two-terminal transmission
// (crates/caroli-green/src/nested.rs), used by the tests, by the GPU smoke check and by the
// CPU-baseline leg of bench.py to check and time the GPU path. Nothing in caroli_gb300/
// links or calls this file.
//
// What it restates, function by function (reference file:line):
//   split                -> nested.rs:1049-1093   geometric bisection, separators as thick as the hopping range
//   symbolic             -> nested.rs:1095-1122   boundaries from the sparsity of H and the children
//   front_vars           -> nested.rs:144-158
//   separator_entries    -> nested.rs:160-179
//   runs / add_runs      -> nested.rs:1135-1162   extend-add of a child's Schur complement
//   Tree::front          -> nested.rs:302-374     planned and delayed assembly, pivot delay
//   small_schur          -> nested.rs:1164-1223   in-place elimination, n < SMALL_FRONT (64)
//   schur (Field::schur) -> caroli-dense/src/field.rs:79-105 (c64), :129-137 + :140-170 (c32)
//   Tree::root           -> nested.rs:246-281
//   root_with_leads      -> nested.rs:806-845
//   lead_green           -> nested.rs:783-802
//   broadening           -> caroli-green/src/lib.rs:67-71
//   caroli_trace         -> caroli-green/src/lib.rs:106-113
// Constants: LEAF_ORBITALS = 16 (nested.rs:34), SMALL_FRONT = 64 (:37),
// PIVOT_TOL = 1e-11 for c64 (field.rs:61) and 1e-5 for c32 (field.rs:111).
//
// The dense LU of large fronts and of the root is faer's partial-pivoting LU in the reference
// (faer 0.24.4, not vendored); this file uses its own partial-pivoting LU with the same pivot
// test, so results agree to rounding, not bitwise.
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

using c64 = std::complex<double>;
using c32 = std::complex<float>;
constexpr size_t LEAF_ORBITALS = 16;
constexpr size_t SMALL_FRONT = 64;
constexpr size_t NEVER = SIZE_MAX;

template <typename T> struct Field;
template <> struct Field<c64> {
  static constexpr double PIVOT_TOL = 1e-11;
  static c64 from(c64 z) { return z; }
  static double modulus(c64 z) { return std::abs(z); }
};
template <> struct Field<c32> {
  static constexpr double PIVOT_TOL = 1e-5;
  static c32 from(c64 z) { return c32((float)z.real(), (float)z.imag()); }
  static double modulus(c32 z) { return std::hypot((double)z.real(), (double)z.imag()); }
};

// Column-major dense matrix.
template <typename T> struct Mat {
  size_t r = 0, c = 0;
  std::vector<T> a;
  Mat() = default;
  Mat(size_t r_, size_t c_) : r(r_), c(c_), a(r_ * c_, T(0)) {}
  T& operator()(size_t i, size_t j) { return a[i + j * r]; }
  const T& operator()(size_t i, size_t j) const { return a[i + j * r]; }
};

struct Csr {
  size_t n;
  const int64_t* row_ptr;
  const uint32_t* cols;
};

struct Node {
  std::vector<size_t> eliminate, boundary;
  std::vector<size_t> children;
};

struct PlanEntry { size_t a, b; int64_t k; bool conj; };
struct Run { size_t src, dst, len; };

struct Plan {
  std::vector<size_t> vars;
  size_t ne = 0;
  std::vector<size_t> diagonal;
  std::vector<PlanEntry> entries;  // value = conj ? conj(vals[k]) : vals[k]
  std::vector<std::vector<Run>> children;
};

// Sorted index for binary search: position of each variable (nested.rs:511-524).
struct Positions {
  std::vector<std::pair<size_t, size_t>> v;
  explicit Positions(const std::vector<size_t>& vars) {
    v.reserve(vars.size());
    for (size_t k = 0; k < vars.size(); ++k) v.push_back({vars[k], k});
    std::sort(v.begin(), v.end());
  }
  long get(size_t x) const {
    auto it = std::lower_bound(v.begin(), v.end(), std::make_pair(x, (size_t)0));
    if (it != v.end() && it->first == x) return (long)it->second;
    return -1;
  }
};

static bool contains_sorted(const std::vector<size_t>& v, size_t x) {
  return std::binary_search(v.begin(), v.end(), x);
}

struct Geometry {
  size_t nsites;
  int dim;
  const int64_t* cells;    // nsites x 3
  const int64_t* offsets;  // first orbital of each site
  const int64_t* norbs;    // orbitals of each site
  int64_t range[3];
};

static long split(const Geometry& g, std::vector<size_t> sites,
                  std::vector<std::pair<std::vector<size_t>, std::vector<size_t>>>& nodes) {
  if (sites.empty()) return -1;
  size_t orbitals = 0;
  for (size_t i : sites) orbitals += (size_t)g.norbs[i];
  // Longest extent; ties go to the lowest axis (max_by_key with Reverse(d)).
  int best_d = 0;
  int64_t best_lo = 0, best_hi = -1, best_ext = -1;
  for (int d = 0; d < g.dim; ++d) {
    int64_t lo = INT64_MAX, hi = INT64_MIN;
    for (size_t i : sites) {
      int64_t c = g.cells[i * 3 + d];
      lo = std::min(lo, c);
      hi = std::max(hi, c);
    }
    if (hi - lo > best_ext) { best_ext = hi - lo; best_d = d; best_lo = lo; best_hi = hi; }
  }
  int d = best_d;
  int64_t lo = best_lo, hi = best_hi;
  if (orbitals <= LEAF_ORBITALS || hi - lo < g.range[d]) {
    nodes.push_back({std::move(sites), {}});
    return (long)nodes.size() - 1;
  }
  int64_t mid = lo + (hi - lo + 1 - g.range[d]) / 2;
  std::vector<size_t> a, sep, b;
  for (size_t i : sites) {
    int64_t c = g.cells[i * 3 + d];
    if (c < mid) a.push_back(i);
    else if (c < mid + g.range[d]) sep.push_back(i);
    else b.push_back(i);
  }
  std::vector<size_t> children;
  long ka = split(g, std::move(a), nodes);
  if (ka >= 0) children.push_back((size_t)ka);
  long kb = split(g, std::move(b), nodes);
  if (kb >= 0) children.push_back((size_t)kb);
  nodes.push_back({std::move(sep), std::move(children)});
  return (long)nodes.size() - 1;
}

static void symbolic(const Csr& h, std::vector<Node>& nodes) {
  std::vector<size_t> rank(h.n, NEVER), last_rank(nodes.size());
  size_t next = 0;
  for (size_t k = 0; k < nodes.size(); ++k) {
    for (size_t o : nodes[k].eliminate) rank[o] = next++;
    last_rank[k] = next;
  }
  for (size_t k = 0; k < nodes.size(); ++k) {
    std::vector<size_t> bnd;
    for (size_t o : nodes[k].eliminate)
      for (int64_t q = h.row_ptr[o]; q < h.row_ptr[o + 1]; ++q) bnd.push_back(h.cols[q]);
    for (size_t c : nodes[k].children)
      bnd.insert(bnd.end(), nodes[c].boundary.begin(), nodes[c].boundary.end());
    std::vector<size_t> kept;
    for (size_t o : bnd)
      if (rank[o] == NEVER || rank[o] >= last_rank[k]) kept.push_back(o);
    std::sort(kept.begin(), kept.end());
    kept.erase(std::unique(kept.begin(), kept.end()), kept.end());
    nodes[k].boundary = std::move(kept);
  }
}

static std::pair<std::vector<size_t>, size_t> front_vars(const Node& node,
                                                         const std::vector<const std::vector<size_t>*>& children) {
  std::vector<size_t> elim = node.eliminate;
  for (auto* vars : children)
    for (size_t o : *vars)
      if (!contains_sorted(node.boundary, o)) elim.push_back(o);
  std::sort(elim.begin(), elim.end());
  elim.erase(std::unique(elim.begin(), elim.end()), elim.end());
  size_t ne = elim.size();
  elim.insert(elim.end(), node.boundary.begin(), node.boundary.end());
  return {elim, ne};
}

template <typename F>
static void separator_entries(const Csr& h, const Node& node, const Positions& pos, F add) {
  for (size_t i : node.eliminate) {
    size_t pi = (size_t)pos.get(i);
    for (int64_t q = h.row_ptr[i]; q < h.row_ptr[i + 1]; ++q) {
      size_t j = h.cols[q];
      if (j == i) {
        add(pi, pi, q, false);
      } else {
        long pj = pos.get(j);
        if (pj < 0) continue;
        bool later = contains_sorted(node.eliminate, j) ? j > i : contains_sorted(node.boundary, j);
        if (later) {
          add(pi, (size_t)pj, q, false);
          add((size_t)pj, pi, q, true);
        }
      }
    }
  }
}

static std::vector<Run> runs(const std::vector<size_t>& vars, const Positions& pos) {
  std::vector<Run> out;
  for (size_t a = 0; a < vars.size(); ++a) {
    long pa = pos.get(vars[a]);
    if (pa < 0) throw std::runtime_error("child variable missing from the parent front");
    if (!out.empty() && out.back().src + out.back().len == a && out.back().dst + out.back().len == (size_t)pa)
      out.back().len += 1;
    else
      out.push_back({a, (size_t)pa, 1});
  }
  return out;
}

template <typename T>
static void add_runs(Mat<T>& f, const std::vector<Run>& rs, const Mat<T>& s) {
  for (const Run& cb : rs)
    for (size_t b = 0; b < cb.len; ++b)
      for (const Run& ra : rs)
        for (size_t a = 0; a < ra.len; ++a) f(ra.dst + a, cb.dst + b) += s(ra.src + a, cb.src + b);
}

// small_schur (nested.rs:1167-1223): Gaussian elimination in a copy, partial pivoting within the
// separator rows, refused when a pivot is not above PIVOT_TOL times the largest entry of F11.
template <typename T>
static bool small_schur(const Mat<T>& f, size_t ne, Mat<T>& s_out) {
  size_t n = f.r, nb = n - ne;
  double scale = 0.0;
  for (size_t j = 0; j < ne; ++j)
    for (size_t i = 0; i < ne; ++i) scale = std::max(scale, Field<T>::modulus(f(i, j)));
  Mat<T> w = f;
  for (size_t k = 0; k < ne; ++k) {
    size_t p = k;
    double big = -1.0;
    for (size_t i = k; i < ne; ++i) {
      double m = Field<T>::modulus(w(i, k));
      if (m > big) { big = m; p = i; }
    }
    if (!(big > Field<T>::PIVOT_TOL * scale)) return false;
    if (p != k)
      for (size_t j = 0; j < n; ++j) std::swap(w(p, j), w(k, j));
    T inv = T(1) / w(k, k);
    for (size_t i = k + 1; i < n; ++i) w(i, k) *= inv;
    for (size_t j = k + 1; j < n; ++j) {
      T ukj = w(k, j);
      if (ukj != T(0))
        for (size_t i = k + 1; i < n; ++i) w(i, j) -= w(i, k) * ukj;
    }
  }
  s_out = Mat<T>(nb, nb);
  for (size_t j = 0; j < nb; ++j)
    for (size_t i = 0; i < nb; ++i) s_out(i, j) = w(ne + i, ne + j);
  return true;
}

// Partial-pivoting LU of a square matrix; `piv[k]` is the row swapped with k at step k.
template <typename T> struct Lu {
  Mat<T> lu;
  std::vector<size_t> piv;
  explicit Lu(const Mat<T>& a) : lu(a), piv(a.r) {
    size_t n = a.r;
    for (size_t k = 0; k < n; ++k) {
      size_t p = k;
      double big = -1.0;
      for (size_t i = k; i < n; ++i) {
        double m = Field<T>::modulus(lu(i, k));
        if (m > big) { big = m; p = i; }
      }
      piv[k] = p;
      if (p != k)
        for (size_t j = 0; j < n; ++j) std::swap(lu(p, j), lu(k, j));
      T d = lu(k, k);
      if (d == T(0)) continue;  // singular: the solve returns non-finite values
      T inv = T(1) / d;
      for (size_t i = k + 1; i < n; ++i) lu(i, k) *= inv;
      for (size_t j = k + 1; j < n; ++j) {
        T ukj = lu(k, j);
        if (ukj != T(0))
          for (size_t i = k + 1; i < n; ++i) lu(i, j) -= lu(i, k) * ukj;
      }
    }
  }
  double min_pivot() const {
    double m = INFINITY;
    for (size_t i = 0; i < lu.r; ++i) m = std::min(m, Field<T>::modulus(lu(i, i)));
    return m;
  }
  void solve(Mat<T>& b) const {
    size_t n = lu.r;
    for (size_t c = 0; c < b.c; ++c) {
      for (size_t k = 0; k < n; ++k)
        if (piv[k] != k) std::swap(b(k, c), b(piv[k], c));
      for (size_t k = 0; k < n; ++k) {
        T v = b(k, c);
        if (v != T(0))
          for (size_t i = k + 1; i < n; ++i) b(i, c) -= lu(i, k) * v;
      }
      for (size_t k = n; k-- > 0;) {
        b(k, c) /= lu(k, k);
        T v = b(k, c);
        if (v != T(0))
          for (size_t i = 0; i < k; ++i) b(i, c) -= lu(i, k) * v;
      }
    }
  }
};

// Field::schur (field.rs:79-105): S = F22 - F21 F11^-1 F12, refused when the smallest pivot of
// the LU of F11 is not above PIVOT_TOL times the largest entry of F11.
template <typename T>
static bool big_schur(const Mat<T>& f, size_t ne, Mat<T>& s_out) {
  size_t n = f.r, nb = n - ne;
  Mat<T> f11(ne, ne);
  double scale = 0.0;
  for (size_t j = 0; j < ne; ++j)
    for (size_t i = 0; i < ne; ++i) {
      f11(i, j) = f(i, j);
      scale = std::max(scale, Field<T>::modulus(f(i, j)));
    }
  Lu<T> lu(f11);
  if (!(lu.min_pivot() > Field<T>::PIVOT_TOL * scale)) return false;
  s_out = Mat<T>(nb, nb);
  if (nb == 0) return true;
  Mat<T> x(ne, nb);
  for (size_t j = 0; j < nb; ++j)
    for (size_t i = 0; i < ne; ++i) x(i, j) = f(i, ne + j);
  lu.solve(x);
  for (size_t j = 0; j < nb; ++j)
    for (size_t i = 0; i < nb; ++i) s_out(i, j) = f(ne + i, ne + j);
  for (size_t j = 0; j < nb; ++j)
    for (size_t k = 0; k < ne; ++k) {
      T xkj = x(k, j);
      for (size_t i = 0; i < nb; ++i) s_out(i, j) -= f(ne + i, k) * xkj;
    }
  return true;
}

template <typename T> struct Front {
  std::vector<size_t> vars;
  Mat<T> s;
};

struct Tree {
  std::vector<Node> nodes;
  std::vector<size_t> top;
  std::vector<Plan> plans;
};

struct BlockInfo {
  Tree tree;
  std::vector<size_t> left, right;
};

struct System {
  Csr h;
  std::vector<int64_t> row_ptr;
  std::vector<uint32_t> cols;
  std::vector<BlockInfo> blocks;
};

static Plan make_plan(const Csr& h, const std::vector<Node>& nodes, size_t k) {
  const Node& node = nodes[k];
  std::vector<const std::vector<size_t>*> kids;
  for (size_t c : node.children) kids.push_back(&nodes[c].boundary);
  Plan p;
  auto fv = front_vars(node, kids);
  p.vars = fv.first;
  p.ne = fv.second;
  Positions pos(p.vars);
  separator_entries(h, node, pos, [&](size_t a, size_t b, int64_t q, bool cj) { p.entries.push_back({a, b, q, cj}); });
  for (size_t i : node.eliminate) p.diagonal.push_back((size_t)pos.get(i));
  for (auto* vars : kids) p.children.push_back(runs(*vars, pos));
  return p;
}

template <typename T> struct Solver {
  const System& sys;
  const Tree& tree;
  const c64* vals;
  c64 z;
  bool failed = false;

  c64 value(int64_t q, bool cj) const { return cj ? std::conj(vals[q]) : vals[q]; }

  std::vector<Front<T>> fronts(const std::vector<size_t>& ks) {
    std::vector<Front<T>> out;
    for (size_t k : ks) out.push_back(front(k));
    return out;
  }

  Front<T> front(size_t k) {
    const Node& node = tree.nodes[k];
    std::vector<Front<T>> kids = fronts(node.children);
    const Plan& plan = tree.plans[k];
    bool planned = true;
    for (size_t c = 0; c < kids.size(); ++c)
      if (kids[c].vars != tree.nodes[node.children[c]].boundary) planned = false;
    T zt = Field<T>::from(z);
    std::vector<size_t> vars;
    size_t ne;
    Mat<T> f;
    if (planned) {
      vars = plan.vars;
      ne = plan.ne;
      size_t n = vars.size();
      f = Mat<T>(n, n);
      for (const PlanEntry& e : plan.entries) f(e.a, e.b) -= Field<T>::from(value(e.k, e.conj));
      for (size_t a : plan.diagonal) f(a, a) += zt;
      for (size_t c = 0; c < kids.size(); ++c) add_runs(f, plan.children[c], kids[c].s);
    } else {
      std::vector<const std::vector<size_t>*> handed;
      for (auto& kid : kids) handed.push_back(&kid.vars);
      auto fv = front_vars(node, handed);
      vars = fv.first;
      ne = fv.second;
      Positions pos(vars);
      f = Mat<T>(vars.size(), vars.size());
      separator_entries(sys.h, node, pos, [&](size_t a, size_t b, int64_t q, bool cj) {
        f(a, b) -= Field<T>::from(value(q, cj));
      });
      for (size_t i : node.eliminate) {
        size_t pi = (size_t)pos.get(i);
        f(pi, pi) += zt;
      }
      for (auto& kid : kids) add_runs(f, runs(kid.vars, pos), kid.s);
    }
    if (ne == 0) return {vars, std::move(f)};
    Mat<T> s;
    bool ok = f.r < SMALL_FRONT ? small_schur(f, ne, s) : big_schur(f, ne, s);
    if (ok) return {node.boundary, std::move(s)};
    return {vars, std::move(f)};  // singular separator block: the whole front goes up
  }
};

template <typename T> static Mat<c64> to_c64(const Mat<T>& m) {
  Mat<c64> out(m.r, m.c);
  for (size_t i = 0; i < m.a.size(); ++i) out.a[i] = c64(m.a[i].real(), m.a[i].imag());
  return out;
}

// Status codes shared with the product's C ABI.
enum { ST_OK = 0, ST_SINGULAR = 2, ST_NONFINITE = 3 };

template <typename T>
static int solve_block(const System& sys, const BlockInfo& blk, const c64* vals, double energy,
                       const c64* sigma_l, const c64* sigma_r, double* t_out, c64* g_out,
                       long* delayed_out) {
  const Tree& tree = blk.tree;
  c64 z(energy, 0.0);
  Solver<T> solver{sys, tree, vals, z};
  std::vector<Front<T>> kids = solver.fronts(tree.top);
  // Tree::root (nested.rs:246-281).
  const auto& left = blk.left;
  const auto& right = blk.right;
  bool same = left == right;
  std::vector<size_t> kept = left;
  if (!same) kept.insert(kept.end(), right.begin(), right.end());
  Positions in_kept(kept);
  std::vector<size_t> delayed;
  for (auto& kid : kids)
    for (size_t o : kid.vars)
      if (in_kept.get(o) < 0) delayed.push_back(o);
  std::sort(delayed.begin(), delayed.end());
  delayed.erase(std::unique(delayed.begin(), delayed.end()), delayed.end());
  std::vector<size_t> vars = delayed;
  vars.insert(vars.end(), kept.begin(), kept.end());
  Positions pos(vars);
  size_t m = vars.size();
  Mat<c64> f(m, m);
  for (size_t i : kept) {
    size_t pi = (size_t)pos.get(i);
    f(pi, pi) += z;
    for (int64_t q = sys.h.row_ptr[i]; q < sys.h.row_ptr[i + 1]; ++q) {
      size_t j = sys.h.cols[q];
      if (in_kept.get(j) >= 0) f(pi, (size_t)pos.get(j)) -= vals[q];
    }
  }
  for (auto& kid : kids) add_runs(f, runs(kid.vars, pos), to_c64(kid.s));
  // root_with_leads (nested.rs:806-845).
  size_t nd = delayed.size(), nl = left.size(), nr = right.size();
  size_t rpos = same ? 0 : nl;
  for (size_t c = 0; c < nl; ++c)
    for (size_t a = 0; a < nl; ++a) f(nd + a, nd + c) -= sigma_l[a + c * nl];
  for (size_t c = 0; c < nr; ++c)
    for (size_t a = 0; a < nr; ++a) f(nd + rpos + a, nd + rpos + c) -= sigma_r[a + c * nr];
  Mat<c64> s;
  if (nd > 0) {
    bool ok = m < SMALL_FRONT ? small_schur(f, nd, s) : big_schur(f, nd, s);
    if (!ok) return ST_SINGULAR;
  } else {
    s = std::move(f);
  }
  if (delayed_out) *delayed_out = (long)nd;
  // lead_green (nested.rs:783-802).
  size_t k = s.r;
  Mat<c64> rhs(k, nr);
  for (size_t j = 0; j < nr; ++j) rhs(rpos + j, j) = 1.0;
  Lu<c64> lu(s);
  lu.solve(rhs);
  for (c64 v : rhs.a)
    if (!std::isfinite(v.real()) || !std::isfinite(v.imag())) return ST_SINGULAR;
  Mat<c64> g(nl, nr);
  for (size_t j = 0; j < nr; ++j)
    for (size_t i = 0; i < nl; ++i) g(i, j) = rhs(i, j);
  if (g_out)
    for (size_t i = 0; i < g.a.size(); ++i) g_out[i] = g.a[i];
  // broadening + caroli_trace (lib.rs:67-71, :106-113): T = sum_ij (Γ_L G)_ij conj((G Γ_R)_ij).
  Mat<c64> gl(nl, nl), gr(nr, nr);
  const c64 I(0.0, 1.0);
  for (size_t j = 0; j < nl; ++j)
    for (size_t i = 0; i < nl; ++i) gl(i, j) = I * (sigma_l[i + j * nl] - std::conj(sigma_l[j + i * nl]));
  for (size_t j = 0; j < nr; ++j)
    for (size_t i = 0; i < nr; ++i) gr(i, j) = I * (sigma_r[i + j * nr] - std::conj(sigma_r[j + i * nr]));
  Mat<c64> a(nl, nr), b(nl, nr);
  for (size_t j = 0; j < nr; ++j)
    for (size_t kk = 0; kk < nl; ++kk) {
      c64 gkj = g(kk, j);
      for (size_t i = 0; i < nl; ++i) a(i, j) += gl(i, kk) * gkj;
    }
  for (size_t j = 0; j < nr; ++j)
    for (size_t kk = 0; kk < nr; ++kk) {
      c64 rkj = gr(kk, j);
      for (size_t i = 0; i < nl; ++i) b(i, j) += g(i, kk) * rkj;
    }
  double t = 0.0;
  for (size_t j = 0; j < nr; ++j) {
    double col = 0.0;
    for (size_t i = 0; i < nl; ++i) col += (a(i, j) * std::conj(b(i, j))).real();
    t += col;
  }
  *t_out = t;
  return std::isfinite(t) ? ST_OK : ST_NONFINITE;
}

}  // namespace

extern "C" {

// Builds the trees of every block of a two-terminal system.
//   n, row_ptr[n+1], cols[nnz]     CSR pattern of H (values are given per solve)
//   nsites, dim, cells[nsites*3], site_offsets[nsites], site_orbitals[nsites], range[3]
//   n_interior, interior[]         sites of the tree (all but the two lead slices)
//   nblocks, labels[n]             block index of each orbital (-1: none)
//   left_ptr[nblocks+1], left[]    device orbitals of the first slice per block (lead-cell order)
//   right_ptr[nblocks+1], right[]  same for the last slice
int oracle_build(int64_t n, const int64_t* row_ptr, const uint32_t* cols, int64_t nsites, int dim,
                 const int64_t* cells, const int64_t* site_offsets, const int64_t* site_orbitals,
                 const int64_t* range, int64_t n_interior, const int64_t* interior, int nblocks,
                 const int32_t* labels, const int64_t* left_ptr, const int64_t* left,
                 const int64_t* right_ptr, const int64_t* right, void** out) {
  try {
    auto sys = std::make_unique<System>();
    sys->row_ptr.assign(row_ptr, row_ptr + n + 1);
    sys->cols.assign(cols, cols + row_ptr[n]);
    sys->h = Csr{(size_t)n, sys->row_ptr.data(), sys->cols.data()};
    Geometry g{(size_t)nsites, dim, cells, site_offsets, site_orbitals, {range[0], range[1], range[2]}};
    std::vector<std::pair<std::vector<size_t>, std::vector<size_t>>> site_nodes;
    std::vector<size_t> sites(interior, interior + n_interior);
    long top = split(g, sites, site_nodes);
    for (int b = 0; b < nblocks; ++b) {
      BlockInfo blk;
      Tree& t = blk.tree;
      for (auto& sn : site_nodes) {
        Node node;
        for (size_t i : sn.first)
          for (int64_t o = site_offsets[i]; o < site_offsets[i] + site_orbitals[i]; ++o)
            if (labels[o] == b) node.eliminate.push_back((size_t)o);
        std::sort(node.eliminate.begin(), node.eliminate.end());
        node.children = sn.second;
        t.nodes.push_back(std::move(node));
      }
      if (top >= 0) t.top.push_back((size_t)top);
      symbolic(sys->h, t.nodes);
      for (size_t k = 0; k < t.nodes.size(); ++k) t.plans.push_back(make_plan(sys->h, t.nodes, k));
      blk.left.assign(left + left_ptr[b], left + left_ptr[b + 1]);
      blk.right.assign(right + right_ptr[b], right + right_ptr[b + 1]);
      sys->blocks.push_back(std::move(blk));
    }
    *out = sys.release();
    return 0;
  } catch (...) {
    return 1;
  }
}

void oracle_free(void* h) { delete static_cast<System*>(h); }

// T of one block at one energy. vals: complex128 values of H (interleaved, on the build's
// pattern); sigma_l / sigma_r: column-major complex128 (nl x nl, nr x nr). precision 0: c64
// fronts, 1: c32 fronts below the root (the root stays c64, nested.rs:244-261).
// g_out (optional): G_LR, column-major nl x nr complex128.
int oracle_solve(void* handle, int block, double energy, const double* vals, const double* sigma_l,
                 const double* sigma_r, int precision, double* t_out, double* g_out, int64_t* delayed) {
  const System& sys = *static_cast<System*>(handle);
  const BlockInfo& blk = sys.blocks[block];
  long nd = 0;
  int st;
  try {
    if (precision == 0)
      st = solve_block<c64>(sys, blk, (const c64*)vals, energy, (const c64*)sigma_l, (const c64*)sigma_r, t_out,
                            (c64*)g_out, &nd);
    else
      st = solve_block<c32>(sys, blk, (const c64*)vals, energy, (const c64*)sigma_l, (const c64*)sigma_r, t_out,
                            (c64*)g_out, &nd);
  } catch (...) {
    return 9;
  }
  if (delayed) *delayed = nd;
  return st;
}

// Many independent solves on `threads` OpenMP threads (one solve per thread at a time, the
// reference's data parallelism over energies and configurations, run.rs:41-45).
int oracle_solve_batch(void* handle, int64_t count, const int32_t* blocks, const double* energies,
                       const double* const* vals, const double* const* sigma_l, const double* const* sigma_r,
                       int precision, int threads, double* t_out, int32_t* status) {
#ifdef _OPENMP
  if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel for schedule(dynamic, 1)
#endif
  for (int64_t i = 0; i < count; ++i)
    status[i] = oracle_solve(handle, blocks[i], energies[i], vals[i], sigma_l[i], sigma_r[i], precision, &t_out[i],
                             nullptr, nullptr);
  return 0;
}

// Sizes of the planned fronts of a block in post-order: n = separator + boundary, ne = separator.
int oracle_tree_fronts(void* handle, int block, int64_t capacity, int32_t* n, int32_t* ne) {
  const System& sys = *static_cast<System*>(handle);
  const Tree& t = sys.blocks[block].tree;
  for (size_t k = 0; k < t.nodes.size() && (int64_t)k < capacity; ++k) {
    n[k] = (int32_t)(t.plans[k].vars.size());
    ne[k] = (int32_t)t.plans[k].ne;
  }
  return (int)t.nodes.size();
}

int oracle_tree_info(void* handle, int block, int64_t* nodes, int64_t* max_ne, int64_t* max_nb) {
  const System& sys = *static_cast<System*>(handle);
  const Tree& t = sys.blocks[block].tree;
  *nodes = (int64_t)t.nodes.size();
  *max_ne = 0;
  *max_nb = 0;
  for (auto& nd : t.nodes) {
    *max_ne = std::max<int64_t>(*max_ne, (int64_t)nd.eliminate.size());
    *max_nb = std::max<int64_t>(*max_nb, (int64_t)nd.boundary.size());
  }
  return 0;
}

}  // extern "C"
