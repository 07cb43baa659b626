// Device kernels of the nested-dissection transmission (sm_103a).
//
// Every front lives in a per-solve arena as an n x n column-major complex matrix, interleaved
// (re, im). After elimination of its ne leading variables a front holds
//     [ F11^-1          | X = F11^-1 F12 ]
//     [ W = -F21 F11^-1 | S = F22 - F21 X ]
// The parent gathers S (the trailing nb x nb block) through an index map; a refinement solve
// reads F11^-1, X and W (forward: t = F11^-1 r_e, r_b += W r_e; backward: x_e = t - X x_b).
//
// The elimination is the reference's partial-pivoting Schur step (nested.rs:1167-1223,
// caroli-dense/src/field.rs:79-105) written as an in-place Gauss-Jordan sweep: the pivots (and so
// the stability test |pivot| > PIVOT_TOL * max|F11|) are those of the LU with partial pivoting
// within the separator rows.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "plan.hpp"

namespace caroli {

enum Status : int32_t {
  ST_OK = 0,
  ST_PIVOT_DELAYED = 1,  // a front refused its pivots: the solve is redone with delayed fronts
  ST_SINGULAR = 2,       // the root (or a delayed block at the root) is singular
  ST_NONFINITE = 3,      // T is not finite
  ST_REFINE_STALLED = 4, // mixed precision: refinement did not reach its tolerance
  ST_TIMEOUT = 5,
};

// One solve (one block of one instance) as the kernels see it.
struct JobDesc {
  const FrontDesc* fronts;
  const int32_t* maps;
  const uint8_t* own;
  const Entry* entries;
  void* arena;             // tree fronts, in the precision of the fronts
  void* root_arena;        // the root front (m x m), in the precision of the root
  const double2* vals;     // H values of the configuration (on the system's pattern)
  const double2* sigma_l;  // nl x nl, column-major
  const double2* sigma_r;  // nr x nr
  const double2* gamma_l;  // i (Σ_L - Σ_L^†)
  const double2* gamma_r;
  uint8_t* fail;           // one flag per front: refused pivots
  double energy;
  int32_t root, nl, nr, rpos, nd;
  int32_t nfronts;
};

struct Task {
  int32_t job, front;
  const FrontDesc* fd;  // the front's descriptor (device), read without going through the job
};

template <typename T> struct Cx;
template <> struct Cx<double> { using V = double2; };
template <> struct Cx<float> { using V = float2; };

template <typename V> __device__ __forceinline__ V cx(double re, double im) { V v; v.x = re; v.y = im; return v; }
template <typename V> __device__ __forceinline__ V cadd(V a, V b) { a.x += b.x; a.y += b.y; return a; }
template <typename V> __device__ __forceinline__ V csub(V a, V b) { a.x -= b.x; a.y -= b.y; return a; }
template <typename V> __device__ __forceinline__ V cmul(V a, V b) {
  V r; r.x = a.x * b.x - a.y * b.y; r.y = a.x * b.y + a.y * b.x; return r;
}
// acc - a b
template <typename V> __device__ __forceinline__ V cfms(V acc, V a, V b) {
  acc.x = fma(-a.x, b.x, fma(a.y, b.y, acc.x));
  acc.y = fma(-a.x, b.y, fma(-a.y, b.x, acc.y));
  return acc;
}
// acc + a b
template <typename V> __device__ __forceinline__ V cfma(V acc, V a, V b) {
  acc.x = fma(a.x, b.x, fma(-a.y, b.y, acc.x));
  acc.y = fma(a.x, b.y, fma(a.y, b.x, acc.y));
  return acc;
}
// The same multiply-adds with each pair of component FMAs issued as one packed f32x2 FMA for
// complex f32 (fma.rn.f32x2): the same two rounding steps per component, so identical results.
// Used where measured faster (the panel sweep of large fronts); FP64 falls back to cfms/cfma.
__device__ __forceinline__ float2 fma_f32x2(float2 a, float2 b, float2 c) {
  unsigned long long ra, rb, rc, rd;
  asm("mov.b64 %0, {%1, %2};" : "=l"(ra) : "f"(a.x), "f"(a.y));
  asm("mov.b64 %0, {%1, %2};" : "=l"(rb) : "f"(b.x), "f"(b.y));
  asm("mov.b64 %0, {%1, %2};" : "=l"(rc) : "f"(c.x), "f"(c.y));
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(rd) : "l"(ra), "l"(rb), "l"(rc));
  float2 d;
  asm("mov.b64 {%0, %1}, %2;" : "=f"(d.x), "=f"(d.y) : "l"(rd));
  return d;
}
template <typename V> __device__ __forceinline__ V cfms_pk(V acc, V a, V b) { return cfms(acc, a, b); }
template <> __device__ __forceinline__ float2 cfms_pk<float2>(float2 acc, float2 a, float2 b) {
  acc = fma_f32x2(make_float2(a.y, -a.y), make_float2(b.y, b.x), acc);
  return fma_f32x2(make_float2(-a.x, -a.x), b, acc);
}

// |a|^2 in the precision of a (comparisons of pivot candidates; FP64 is 1/64 rate on GB300).
template <typename V> __device__ __forceinline__ auto cnorm(V a) -> decltype(a.x) { return a.x * a.x + a.y * a.y; }

// 1 / a with a scaling step (Smith's method) against overflow of |a|^2.
template <typename V> __device__ __forceinline__ V cinv(V a) {
  V r;
  if (fabs(a.x) >= fabs(a.y)) {
    auto q = a.y / a.x;
    auto d = a.x + a.y * q;
    r.x = 1 / d; r.y = -q / d;
  } else {
    auto q = a.x / a.y;
    auto d = a.x * q + a.y;
    r.x = q / d; r.y = -1 / d;
  }
  return r;
}
template <typename V> __device__ __forceinline__ double cabs2(V a) {
  return (double)a.x * (double)a.x + (double)a.y * (double)a.y;
}
template <typename V> __device__ __forceinline__ V from64(double2 z) { return cx<V>(z.x, z.y); }

// ---- block reductions -------------------------------------------------------------------------
__device__ __forceinline__ double block_max(double v, double* red) {
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = (blockDim.x + 31) >> 5;
  __syncthreads();
  if (l == 0) red[w] = v;
  __syncthreads();
  if (w == 0) {
    v = l < nw ? red[l] : 0.0;
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    if (l == 0) red[0] = v;
  }
  __syncthreads();
  double r = red[0];
  __syncthreads();
  return r;
}

// Largest value, ties to the smaller index (the reference keeps the first maximum). NaN values
// never win, so a column of NaN reports -1 and fails the pivot test.
__device__ __forceinline__ void argmax_pair(double& v, int& i, double v2, int i2) {
  if (v2 > v || (v2 == v && i2 < i)) { v = v2; i = i2; }
}
__device__ __forceinline__ int block_argmax(double v, int i, double* redv, int* redi, double* out_v) {
  for (int o = 16; o > 0; o >>= 1) {
    double v2 = __shfl_xor_sync(0xffffffffu, v, o);
    int i2 = __shfl_xor_sync(0xffffffffu, i, o);
    argmax_pair(v, i, v2, i2);
  }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = (blockDim.x + 31) >> 5;
  __syncthreads();
  if (l == 0) { redv[w] = v; redi[w] = i; }
  __syncthreads();
  if (w == 0) {
    v = l < nw ? redv[l] : -1.0;
    i = l < nw ? redi[l] : 0x7fffffff;
    for (int o = 16; o > 0; o >>= 1) {
      double v2 = __shfl_xor_sync(0xffffffffu, v, o);
      int i2 = __shfl_xor_sync(0xffffffffu, i, o);
      argmax_pair(v, i, v2, i2);
    }
    if (l == 0) { redv[0] = v; redi[0] = i; }
  }
  __syncthreads();
  int r = redi[0];
  *out_v = redv[0];
  __syncthreads();
  return r;
}

// ---- assembly -----------------------------------------------------------------------------------
// Assembly: element (i, j) of a front before its H entries is the children's handed blocks through
// their index maps, plus z on the diagonal of the own separator, minus Σ on the root.
// The children's handed blocks of a front, hoisted out of the per-element assembly loops:
// element (i, j) = Σ_c S_c[map_c(i), map_c(j)] (both mapped), S_c a column-major block with
// leading dimension ld[c].
template <typename TC>
struct ChildBlocks {
  const typename Cx<TC>::V* base[2];
  const int32_t* map[2];
  int32_t ld[2];
  int nchild;
  __device__ __forceinline__ ChildBlocks(const JobDesc& J, const FrontDesc& f) {
    nchild = f.nchild;
    const typename Cx<TC>::V* arena = static_cast<const typename Cx<TC>::V*>(J.arena);
    for (int c = 0; c < 2; ++c) {
      if (c < nchild) {
        const FrontDesc& cf = J.fronts[f.child[c]];
        base[c] = arena + cf.arena_off + f.child_off[c];
        ld[c] = cf.n;
        map[c] = J.maps + f.map_off[c];
      } else {
        base[c] = nullptr;
        ld[c] = 0;
        map[c] = nullptr;
      }
    }
  }
  // Row maps of row i (or column maps of column j): -1 where the child has no such variable.
  __device__ __forceinline__ void index(int i, int (&a)[2]) const {
    a[0] = nchild > 0 ? map[0][i] : -1;
    a[1] = nchild > 1 ? map[1][i] : -1;
  }
  template <typename T>
  __device__ __forceinline__ typename Cx<T>::V at(const int (&a)[2], const int (&b)[2]) const {
    typename Cx<T>::V v = cx<typename Cx<T>::V>(0.0, 0.0);
#pragma unroll
    for (int c = 0; c < 2; ++c)
      if (a[c] >= 0 && b[c] >= 0) {
        const auto w = base[c][a[c] + (int64_t)b[c] * ld[c]];
        v.x += (T)w.x;
        v.y += (T)w.y;
      }
    return v;
  }
};

template <typename T>
__device__ __forceinline__ void apply_entries(const JobDesc& J, const FrontDesc& f, typename Cx<T>::V* F, int ld,
                                              int col0, int col1) {
  using V = typename Cx<T>::V;
  for (int64_t e = threadIdx.x; e < f.ent_cnt; e += blockDim.x) {
    Entry en = J.entries[f.ent_off + e];
    if (en.b < col0 || en.b >= col1) continue;
    double2 h = J.vals[en.q];
    if (en.conj) h.y = -h.y;
    V& d = F[en.a + (int64_t)en.b * ld];
    d = csub(d, from64<V>(h));
  }
}

// ---- Gauss-Jordan sweep -------------------------------------------------------------------------
// Largest value of a warp, ties to the smaller index (the reference keeps the first maximum); NaN
// never wins, so a column of NaN reports -1 and fails the pivot test.
// v is a lane's largest |c|^2 (never NaN) or -1 for no candidate. In f32 two warp reductions do
// it: the maximum of v's bits (non-negative floats order as unsigned integers; +1 so that 0 means
// no candidate), then the minimum index among the lanes holding it.
template <typename T> __device__ __forceinline__ void warp_argmax(T& v, int& i) {
  if constexpr (sizeof(T) == 4) {
    const unsigned key = v >= 0 ? __float_as_uint((float)v) + 1u : 0u;
    const unsigned top = __reduce_max_sync(0xffffffffu, key);
    i = __reduce_min_sync(0xffffffffu, key == top ? i : 0x7fffffff);
    v = top ? (T)__uint_as_float(top - 1u) : (T)-1;
  } else {
    for (int o = 16; o > 0; o >>= 1) {
      const T v2 = __shfl_xor_sync(0xffffffffu, v, o);
      const int i2 = __shfl_xor_sync(0xffffffffu, i, o);
      if (v2 > v || (v2 == v && i2 < i)) { v = v2; i = i2; }
    }
  }
}

// In-place Gauss-Jordan sweep of the leading `npiv` columns of a rows x cols matrix F (column-major,
// leading dimension ld), the pivot of step k chosen among rows [k, cand) of column k. On exit
// (before the column interchanges) the swept rows hold, for the pivot block P (rows in pivot
// order) and the other rows a: [P^-1 | P^-1 B] and [-a P^-1 | b - a P^-1 B].
//
// One __syncthreads per pivot: warp w owns the columns j = w (mod warps), lane l the rows l,
// l + 32, ...; column k itself is read from the double buffer `cb` (2 x rows), which the owner of
// column k + 1 fills while it updates it, so no warp reads a column another warp writes in the
// same step. The row interchange of step k is folded into the update (row k receives the pivot
// row, row p the old row k). `cb[0:rows]` must hold column 0 and be visible to the block.
// piv[k] receives the pivot row of step k; with `prows`, prows[k * cols + j] receives the scaled
// pivot row of step k (1 / pivot at j = k), from which other rows replay the same elimination.
//
// Returns false when a pivot is not above tol * sqrt(scale2) (uniform in the block: every warp
// searches the same column). With `perturb` such a pivot is replaced by tol * sqrt(scale2) in its
// own direction (static pivoting, counted in *perturbed) and the sweep goes on: the factors then
// only precondition an iterative refinement that removes the perturbation.
template <typename T>
__device__ bool gj_sweep(typename Cx<T>::V* F, int ld, int rows, int cols, int npiv, int cand, double scale2,
                         double tol, typename Cx<T>::V* cb, int* piv, bool perturb, int* perturbed,
                         typename Cx<T>::V* prows = nullptr) {
  using V = typename Cx<T>::V;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const double thresh = tol * tol * scale2;
  for (int k = 0; k < npiv; ++k) {
    const V* ck = cb + (k & 1) * rows;
    V* cn = cb + ((k + 1) & 1) * rows;
    T best = -1;
    int p = 0x7fffffff;
    for (int i = k + lane; i < cand; i += 32) {
      const T m = cnorm(ck[i]);
      if (m > best) { best = m; p = i; }
    }
    warp_argmax(best, p);
    const double big = (double)best;
    V d;
    if (!(big > thresh) || p >= cand) {
      // NaN or an empty column: nothing sensible to perturb.
      if (!perturb || !(big >= 0.0) || !(scale2 > 0.0) || p >= cand) return false;
      d = ck[p];
      const double mag = sqrt(big), target = tol * sqrt(scale2);
      if (mag > 0.0) { d.x = (T)(d.x / mag * target); d.y = (T)(d.y / mag * target); }
      else { d.x = (T)target; d.y = (T)0; }
      if (threadIdx.x == 0 && perturbed) atomicAdd(perturbed, 1);
    } else {
      d = ck[p];
    }
    if (threadIdx.x == 0) piv[k] = p;
    const V inv = cinv(d);
    const V ckk = ck[k];  // old row k of column k (moves to row p)
    for (int j = w; j < cols; j += nw) {
      V* Fj = F + (int64_t)j * ld;
      const bool fill = (j == k + 1) && (j < npiv);
      if (j == k) {
        if (prows && lane == 0) prows[k * cols + j] = inv;
        for (int i = lane; i < rows; i += 32) {
          const V c = (i == p) ? ckk : ck[i];
          const V nv = (i == k) ? inv : cmul(cx<V>(-c.x, -c.y), inv);
          Fj[i] = nv;
        }
        continue;
      }
      const V pr = cmul(Fj[p], inv);
      const V rk = Fj[k];
      if (prows && lane == 0) prows[k * cols + j] = pr;
      __syncwarp();  // rows k and p are read by every lane before their owners write them
      for (int i = lane; i < rows; i += 32) {
        V nv;
        if (i == k) {
          nv = pr;
        } else {
          const V c = (i == p) ? ckk : ck[i];
          nv = cfms_pk((i == p) ? rk : Fj[i], c, pr);
        }
        Fj[i] = nv;
        if (fill) cn[i] = nv;
      }
    }
    __syncthreads();
  }
  return true;
}

// Column order after undoing the row interchanges of a sweep as column interchanges of the
// inverse, last first: the result's column j is column cperm[j] of the swept matrix.
__device__ __forceinline__ void column_order(const int* piv, int npiv, int* cperm) {
  for (int k = npiv - 1; k >= 0; --k) {
    const int p = piv[k];
    if (p != k) { const int a = cperm[k]; cperm[k] = cperm[p]; cperm[p] = a; }
  }
}

// Gauss-Jordan sweep of the leading rows x cols block of F (the pivot candidates of a small front)
// by the first ceil(cols / 32) warps, a lane per column, synchronised by named barrier 1: same
// pivots and operations as gj_sweep(F, ld, rows, cols, rows, rows, ...). The pivot of step k is the
// largest |F[i, k]| over i in [k, rows), row k receives the pivot row and row p the old row k, and
// the scaled pivot row of every step goes to prows (rows x cols). Column k is read from the double
// buffer cb (2 x rows; cb[0:rows] must hold column 0), which the owner of column k + 1 fills while
// it updates it. The calling warps must be exactly the first ceil(cols / 32).
//
// Every lane runs the same loop each step, so the warp holding the pivot column does not execute
// two divergent loops: a column j != k becomes F[i, j] - c_i pr_j (pr_j = F[p, j] / pivot), the
// pivot column -c_i / pivot, which is the same update from a zero column (`zeros`, rows zeros in
// shared memory) with pr = 1 / pivot. Rows k and p, which the interchange treats apart, are
// rewritten after the loop.
template <typename T>
__device__ bool gj_sweep_cols(typename Cx<T>::V* F, int ld, int rows, int cols, double scale2, double tol,
                              typename Cx<T>::V* cb, int* piv, bool perturb, int* perturbed,
                              typename Cx<T>::V* prows, const typename Cx<T>::V* zeros) {
  using V = typename Cx<T>::V;
  const int lane = threadIdx.x & 31;
  const int j = threadIdx.x;  // this lane's column
  const int nthreads = ((cols + 31) / 32) * 32;
  const double thresh = tol * tol * scale2;
  V* Fj = F + (int64_t)j * ld;
  for (int k = 0; k < rows; ++k) {
    const V* ck = cb + (k & 1) * rows;
    V* cn = cb + ((k + 1) & 1) * rows;
    T best = -1;
    int p = 0x7fffffff;
    if (sizeof(T) == 4 && rows - k <= 32) {
      // One candidate per lane: the largest |c|^2 by a warp max of its bits (non-negative floats
      // order as unsigned integers; +1 so that 0 means no candidate or NaN), the smallest row
      // among equal maxima by a ballot. Same result as the shuffle reduction below.
      const int i = k + lane;
      const float m = i < rows ? (float)cnorm(ck[i]) : -1.f;
      const unsigned key = (i < rows && m == m) ? __float_as_uint(m) + 1u : 0u;
      const unsigned top = __reduce_max_sync(0xffffffffu, key);
      if (top != 0u) {
        p = k + __ffs(__ballot_sync(0xffffffffu, key == top)) - 1;
        best = (T)__uint_as_float(top - 1u);
      }
    } else {
      for (int i = k + lane; i < rows; i += 32) {
        const T m = cnorm(ck[i]);
        if (m > best) { best = m; p = i; }
      }
      warp_argmax(best, p);
    }
    const double big = (double)best;
    V d;
    if (!(big > thresh) || p >= rows) {
      if (!perturb || !(big >= 0.0) || !(scale2 > 0.0) || p >= rows) return false;
      d = ck[p];
      const double mag = sqrt(big), target = tol * sqrt(scale2);
      if (mag > 0.0) { d.x = (T)(d.x / mag * target); d.y = (T)(d.y / mag * target); }
      else { d.x = (T)target; d.y = (T)0; }
      if (threadIdx.x == 0 && perturbed) atomicAdd(perturbed, 1);
    } else {
      d = ck[p];
    }
    if (threadIdx.x == 0) piv[k] = p;
    const V inv = cinv(d);
    const V ckk = ck[k];
    if (j < cols) {
      const bool pc = j == k;
      const V* src = pc ? zeros : Fj;
      const V rk = pc ? cx<V>(0.0, 0.0) : Fj[k];
      const V pr = pc ? inv : cmul(Fj[p], inv);
      prows[k * cols + j] = pr;
      const bool fill = j == k + 1;
#pragma unroll 4
      for (int i = 0; i < rows; ++i) {
        const V nv = cfms(src[i], ck[i], pr);
        Fj[i] = nv;
        if (fill) cn[i] = nv;
      }
      if (p != k) {
        const V nv = cfms(rk, ckk, pr);
        Fj[p] = nv;
        if (fill) cn[p] = nv;
      }
      Fj[k] = pr;
      if (fill) cn[k] = pr;
    }
    asm volatile("bar.sync 1, %0;" ::"r"(nthreads) : "memory");
  }
  return true;
}

// Boundary rows of a small front: the recorded steps replayed, a warp per NR rows (two in f32, one
// in FP64 for registers), lane l holding columns l + 32 q (q < RQ, RQ = ceil(n / 32)). Step k
// leaves a row r as r - a prows[k] with a = r[k], and -a prows[k][k] in column k (r[k] is cleared
// before the subtraction), the operations of the sweep itself. The step's entry a comes from lane
// k % 32 of register k / 32, a compile-time register in each 32-step segment. Loads of prows past
// column n run into the buffers after it in shared memory (at most 31 entries past the last row)
// and are never stored.
template <typename T, int RQ>
__device__ __forceinline__ void replay_boundary(typename Cx<T>::V* F, int ld, int n, int ne,
                                                const typename Cx<T>::V* prows) {
  using V = typename Cx<T>::V;
  constexpr int NR = sizeof(T) == 4 ? 2 : 1;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int i0 = ne + NR * w; i0 < n; i0 += NR * nw) {
    V r[NR][RQ];
#pragma unroll
    for (int u = 0; u < NR; ++u)
#pragma unroll
      for (int q = 0; q < RQ; ++q) {
        const int col = lane + 32 * q;
        r[u][q] = (i0 + u < n && col < n) ? F[i0 + u + col * ld] : cx<V>(0.0, 0.0);
      }
#pragma unroll
    for (int qk = 0; qk < RQ; ++qk) {
      const int k1 = min(ne, 32 * qk + 32);
      for (int k = 32 * qk; k < k1; ++k) {
        const int kl = k & 31;
        V a[NR];
#pragma unroll
        for (int u = 0; u < NR; ++u) {
          a[u] = cx<V>(__shfl_sync(0xffffffffu, r[u][qk].x, kl), __shfl_sync(0xffffffffu, r[u][qk].y, kl));
          if (lane == kl) r[u][qk] = cx<V>(0.0, 0.0);
        }
        const V* pk = prows + (int64_t)k * n + lane;
#pragma unroll
        for (int q = 0; q < RQ; ++q) {
          const V b = pk[32 * q];
#pragma unroll
          for (int u = 0; u < NR; ++u) r[u][q] = cfms(r[u][q], a[u], b);
        }
      }
    }
#pragma unroll
    for (int u = 0; u < NR; ++u)
#pragma unroll
      for (int q = 0; q < RQ; ++q) {
        const int col = lane + 32 * q;
        if (i0 + u < n && col < n) F[i0 + u + col * ld] = r[u][q];
      }
  }
}

// ---- small fronts: assembly and elimination in shared memory, one CTA per front ---------------
// The Gauss-Jordan sweep runs in two phases. The ne separator rows (the pivot candidates) are
// swept with the block's barriers, recording the scaled pivot row of every step (prows). The
// nb boundary rows never pivot and never interchange, so each of them then replays the ne steps
// on its own from prows, a warp per row, without barriers: the same operations in the same order
// as a sweep of the whole front.
// Shared memory: the front (n x (n | 1)), prows (ne x n), the column buffer (2n), n zeros, 32
// doubles, piv and cperm (n), the children's index maps (2n).
__host__ __device__ inline size_t small_smem_bytes(int n, int ne, size_t vbytes) {
  const int ld = n | 1;
  return ((size_t)ld * n + (size_t)ne * n + 3 * (size_t)n) * vbytes + 32 * 8 + 4 * (size_t)n * 4 + 16;
}

template <typename T, bool KEEP, bool PREFETCH>
__device__ __forceinline__ void small_front_body(const JobDesc* __restrict__ jobs, const Task* __restrict__ tasks,
                                                 double tol, int perturb, int* __restrict__ perturbed) {
  using V = typename Cx<T>::V;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const Task t = tasks[blockIdx.x];
  const JobDesc& J = jobs[t.job];
  const FrontDesc f = *t.fd;  // copied at once: its fields load together, not on first use
  const int n = f.n, ne = f.ne;
  const int ld = n | 1;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  V* F = reinterpret_cast<V*>(smem_raw);
  V* prows = F + (int64_t)ld * n;
  V* cb = prows + (int64_t)ne * n;
  V* zeros = cb + 2 * n;
  double* red = reinterpret_cast<double*>(zeros + n);
  int* piv = reinterpret_cast<int*>(red + 32);
  int* cperm = piv + n;
  int* cmap = cperm + n;  // 2 x n: child c's position of variable i, -1 where it has none
  // With PREFETCH, the first blockDim.x H entries and their values are requested before the
  // assembly, so that their loads overlap its loads (where registers allow).
  const bool has0 = PREFETCH && threadIdx.x < f.ent_cnt;
  Entry en0{};
  double2 h0 = make_double2(0.0, 0.0);
  if (has0) {
    en0 = J.entries[f.ent_off + threadIdx.x];
    h0 = J.vals[en0.q];
  }
  {
    // The children's index maps are read once into shared memory; a lane keeps those of its rows
    // (lane + 32 q) in registers, so the value loads of all its rows of a column issue together
    // instead of each waiting for its own index load.
    const ChildBlocks<T> kids(J, f);
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      int a[2];
      kids.index(i, a);
      cmap[i] = a[0];
      cmap[n + i] = a[1];
    }
    int ar[3][2];
    bool own[3];
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      const int i = lane + 32 * q;
      own[q] = i < n && J.own[f.own_off + i];
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      const int i = lane + 32 * q;
      ar[q][0] = i < n ? cmap[i] : -1;
      ar[q][1] = i < n ? cmap[n + i] : -1;
    }
    for (int j = w; j < n; j += nw) {
      const int bj[2] = {cmap[j], cmap[n + j]};
      V v[3];
#pragma unroll
      for (int q = 0; q < 3; ++q) v[q] = kids.template at<T>(ar[q], bj);
#pragma unroll
      for (int q = 0; q < 3; ++q) {
        const int i = lane + 32 * q;
        if (i >= n) continue;
        if (i == j && own[q]) v[q].x += (T)J.energy;
        F[i + j * ld] = v[q];
      }
    }
  }
  __syncthreads();
  if (has0) {
    if (en0.conj) h0.y = -h0.y;
    V& d = F[en0.a + (int64_t)en0.b * ld];
    d = csub(d, from64<V>(h0));
  }
  for (int64_t e = threadIdx.x + (PREFETCH ? blockDim.x : 0); e < f.ent_cnt; e += blockDim.x) {
    const Entry en = J.entries[f.ent_off + e];
    double2 h = J.vals[en.q];
    if (en.conj) h.y = -h.y;
    V& d = F[en.a + (int64_t)en.b * ld];
    d = csub(d, from64<V>(h));
  }
  __syncthreads();
  V* out = static_cast<V*>(J.arena) + f.arena_off;
  if (ne == 0) {
    for (int j = w; j < n; j += nw)
      for (int i = lane; i < n; i += 32) out[i + (int64_t)j * n] = F[i + j * ld];
    return;
  }
  T local = 0;
  for (int j = w; j < ne; j += nw)
    for (int i = lane; i < ne; i += 32) local = fmax(local, cnorm(F[i + j * ld]));
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    if (i < ne) cb[i] = F[i];
    zeros[i] = cx<V>(0.0, 0.0);
  }
  const double scale2 = block_max((double)local, red);  // also publishes cb
  // Pivot rows: a lane per column in the first ceil(n / 32) warps (named barrier per pivot); the
  // other warps wait at the block barrier.
  __shared__ int ok_flag;
  if (w < (n + 31) / 32) {
    const bool okc = gj_sweep_cols<T>(F, ld, ne, n, scale2, tol, cb, piv, perturb != 0,
                                      perturbed ? perturbed + t.job : nullptr, prows, zeros);
    if (threadIdx.x == 0) ok_flag = okc ? 1 : 0;
  }
  __syncthreads();
  const bool ok = ok_flag != 0;
  if (!ok) {
    if (threadIdx.x == 0) J.fail[t.front] = 1;
    return;
  }
  // Boundary rows: the recorded steps replayed.
  if (n <= 32) replay_boundary<T, 1>(F, ld, n, ne, prows);
  else if (n <= 64) replay_boundary<T, 2>(F, ld, n, ne, prows);
  else replay_boundary<T, 3>(F, ld, n, ne, prows);
  // Column order, a column per thread of the last warps (the replay gives them the fewest rows):
  // the interchanges undone on the columns, last first, leave in column j the swept column
  // sigma_{ne-1}(... sigma_0(j)), sigma_k the transposition (k piv[k]) (as column_order).
  for (int j = (int)blockDim.x - 1 - (int)threadIdx.x; j < n; j += blockDim.x) {
    int pos = j;
    for (int k = 0; k < ne; ++k) {
      const int p = piv[k];
      pos = pos == k ? p : (pos == p ? k : pos);
    }
    cperm[j] = pos;
  }
  __syncthreads();
  for (int j = w; j < n; j += nw) {
    const V* Fj = F + cperm[j] * ld;
    for (int i = lane; i < n; i += 32) {
      if (!KEEP && (i < ne || j < ne)) continue;
      out[i + (int64_t)j * n] = Fj[i];
    }
  }
}

// One CTA of 256 threads per front (f32: registers for five CTAs per SM, as many as their shared
// memory allows for fronts of up to 64 variables); small_front_wide_kernel: 512 threads, for the
// largest bucket (fronts of 64 to 96 variables, two CTAs per SM by their shared memory), where
// twice the warps replay the boundary rows.
template <typename T, bool KEEP>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? 5 : 2)
    small_front_kernel(const JobDesc* __restrict__ jobs, const Task* __restrict__ tasks, double tol, int perturb,
                       int* __restrict__ perturbed) {
  small_front_body<T, KEEP, false>(jobs, tasks, tol, perturb, perturbed);
}
template <typename T, bool KEEP>
__global__ void __launch_bounds__(512, 2) small_front_wide_kernel(const JobDesc* __restrict__ jobs,
                                                                  const Task* __restrict__ tasks, double tol,
                                                                  int perturb, int* __restrict__ perturbed) {
  small_front_body<T, KEEP, true>(jobs, tasks, tol, perturb, perturbed);
}

// ---- large fronts -------------------------------------------------------------------------------
// Assembly into the arena, a tile of 32 columns per CTA.
// TC: precision of the children, T: of this front (the root may be wider than its children).
template <typename TC, typename T>
__global__ void __launch_bounds__(256) assemble_kernel(const JobDesc* __restrict__ jobs, const Task* __restrict__ tasks,
                                                       int is_root) {
  using V = typename Cx<T>::V;
  const Task t = tasks[blockIdx.y];
  const JobDesc& J = jobs[t.job];
  const FrontDesc& f = *t.fd;
  const int n = f.n;
  const int c0 = blockIdx.x * 32;
  if (c0 >= n) return;
  const int c1 = min(n, c0 + 32);
  V* F = is_root ? static_cast<V*>(J.root_arena) : static_cast<V*>(J.arena) + f.arena_off;
  const ChildBlocks<TC> kids(J, f);
  for (int j = c0 + (threadIdx.x >> 5); j < c1; j += blockDim.x >> 5) {
    int bj[2];
    kids.index(j, bj);
    for (int i = threadIdx.x & 31; i < n; i += 32) {
      int ai[2];
      kids.index(i, ai);
      V v = kids.template at<T>(ai, bj);
      if (i == j && J.own[f.own_off + i]) v.x += (T)J.energy;
      if (is_root) {
        int li = i - J.nd, lj = j - J.nd;
        if (li >= 0 && li < J.nl && lj >= 0 && lj < J.nl) v = csub(v, from64<V>(J.sigma_l[li + (int64_t)lj * J.nl]));
        li -= J.rpos;
        lj -= J.rpos;
        if (li >= 0 && li < J.nr && lj >= 0 && lj < J.nr) v = csub(v, from64<V>(J.sigma_r[li + (int64_t)lj * J.nr]));
      }
      F[i + (int64_t)j * n] = v;
    }
  }
  __syncthreads();
  apply_entries<T>(J, f, F, n, c0, c1);
}

// ---- root: Caroli trace -------------------------------------------------------------------------
// T = sum_ij Re[(Γ_L G)_ij conj((G Γ_R)_ij)] with G = G_LR inside the inverted root front
// (caroli-green/src/lib.rs:106-113). A CTA takes 8 columns of G; partial sums go to `part`.
template <typename T>
__global__ void __launch_bounds__(256) trace_kernel(const JobDesc* __restrict__ jobs, double* __restrict__ part,
                                                    int parts_per_job) {
  using V = typename Cx<T>::V;
  __shared__ double red[32];
  const JobDesc& J = jobs[blockIdx.y];
  const FrontDesc f = J.fronts[J.root];
  const int m = f.n, nl = J.nl, nr = J.nr;
  const V* Gfull = static_cast<const V*>(J.root_arena);
  // G(i, j) = Ginv(nd + i, nd + rpos + j).
  auto G = [&](int i, int j) -> double2 {
    V v = Gfull[(J.nd + i) + (int64_t)(J.nd + J.rpos + j) * m];
    return make_double2((double)v.x, (double)v.y);
  };
  double local = 0.0;
  const int j0 = blockIdx.x * 8;
  for (int jj = 0; jj < 8; ++jj) {
    const int j = j0 + jj;
    if (j >= nr) break;
    for (int i = threadIdx.x; i < nl; i += blockDim.x) {
      double2 a = make_double2(0.0, 0.0), b = make_double2(0.0, 0.0);
      for (int k = 0; k < nl; ++k) a = cfma(a, J.gamma_l[i + (int64_t)k * nl], G(k, j));
      for (int k = 0; k < nr; ++k) b = cfma(b, G(i, k), J.gamma_r[k + (int64_t)j * nr]);
      local += a.x * b.x + a.y * b.y;
    }
  }
  for (int o = 16; o > 0; o >>= 1) local += __shfl_xor_sync(0xffffffffu, local, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) red[w] = local;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) s += red[q];
    part[(int64_t)blockIdx.y * parts_per_job + blockIdx.x] = s;
  }
}

// ---- multi-terminal trace: T_pq = Tr[Γ_p G_pq Γ_q G_pq^†] for every pair of leads ------------
// (NestedMultiTerminal::block_transmissions, nested_multi.rs:337-364). The root inverse holds G on
// the kept orbitals (the union of the leads' orbitals); lead p occupies the kept positions
// lpos[lptr[p] .. lptr[p + 1]), in the order of its Γ_p (np x np, column-major).
struct MultiJob {
  const void* g;                // root inverse (m x m), in the precision of the root
  const int32_t* lpos;          // kept positions of every lead, concatenated
  const int32_t* lptr;          // P + 1 offsets into lpos
  const double2* const* gamma;  // Γ_p per lead (device pointers)
  double2* scratch;             // P * P blocks of `smax` elements: X = G_pq Γ_q
  double* out;                  // P * P transmissions, T[p * P + q]
  int32_t m, nd, P, pad;
};

// grid (P * P, jobs): one CTA per pair; X = G_pq Γ_q, then Σ_{a,d} (Γ_p X)[a,d] conj(G_pq[a,d]).
template <typename TR>
__global__ void __launch_bounds__(256) multi_trace_kernel(const MultiJob* __restrict__ jobs, int64_t smax) {
  using V = typename Cx<TR>::V;
  __shared__ double red[32];
  const MultiJob& J = jobs[blockIdx.y];
  if ((int)blockIdx.x >= J.P * J.P) return;
  const int p = blockIdx.x / J.P, q = blockIdx.x % J.P;
  const int np = J.lptr[p + 1] - J.lptr[p], nq = J.lptr[q + 1] - J.lptr[q];
  const int32_t* ip = J.lpos + J.lptr[p];
  const int32_t* iq = J.lpos + J.lptr[q];
  const double2* gp = J.gamma[p];
  const double2* gq = J.gamma[q];
  const V* Gfull = static_cast<const V*>(J.g);
  auto G = [&](int i, int j) -> double2 {
    const V v = Gfull[(J.nd + i) + (int64_t)(J.nd + j) * J.m];
    return make_double2((double)v.x, (double)v.y);
  };
  double2* X = J.scratch + (int64_t)blockIdx.x * smax;
  for (int64_t idx = threadIdx.x; idx < (int64_t)np * nq; idx += blockDim.x) {
    const int b = (int)(idx % np), d = (int)(idx / np);
    double2 acc = make_double2(0.0, 0.0);
    for (int c = 0; c < nq; ++c) acc = cfma(acc, G(ip[b], iq[c]), gq[c + (int64_t)d * nq]);
    X[idx] = acc;
  }
  __syncthreads();
  double local = 0.0;
  for (int64_t idx = threadIdx.x; idx < (int64_t)np * nq; idx += blockDim.x) {
    const int a = (int)(idx % np), d = (int)(idx / np);
    double2 y = make_double2(0.0, 0.0);
    for (int b = 0; b < np; ++b) y = cfma(y, gp[a + (int64_t)b * np], X[b + (int64_t)d * np]);
    const double2 g = G(ip[a], iq[d]);
    local += y.x * g.x + y.y * g.y;
  }
  for (int o = 16; o > 0; o >>= 1) local += __shfl_xor_sync(0xffffffffu, local, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) red[w] = local;
  __syncthreads();
  if (threadIdx.x == 0) {
    double sum = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) sum += red[k];
    J.out[blockIdx.x] = sum;
  }
}

__global__ void trace_finish_kernel(const double* __restrict__ part, int parts_per_job, int njobs,
                                    double* __restrict__ t_out, int32_t* __restrict__ status) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= njobs) return;
  double s = 0.0;
  for (int q = 0; q < parts_per_job; ++q) s += part[(int64_t)j * parts_per_job + q];
  t_out[j] = s;
  if (status[j] == ST_OK && !isfinite(s)) status[j] = ST_NONFINITE;
}

}  // namespace caroli
