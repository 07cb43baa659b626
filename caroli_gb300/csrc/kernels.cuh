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
  int64_t xoff;  // offset of the front's X block in the level's scratch (large fronts)
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
// Element (i, j) of a front before its H entries: the children's handed blocks through their
// index maps, plus z on the diagonal of the own separator, minus Σ on the root.
template <typename TC, typename T = TC>
__device__ __forceinline__ typename Cx<T>::V gather(const JobDesc& J, const FrontDesc& f, int i, int j,
                                                     bool is_root) {
  using V = typename Cx<T>::V;
  using VC = typename Cx<TC>::V;
  const VC* arena = static_cast<const VC*>(J.arena);
  V v = cx<V>(0.0, 0.0);
  for (int c = 0; c < f.nchild; ++c) {
    const int32_t* map = J.maps + f.map_off[c];
    int a = map[i], b = map[j];
    if (a >= 0 && b >= 0) {
      const FrontDesc& cf = J.fronts[f.child[c]];
      VC w = arena[cf.arena_off + f.child_off[c] + a + (int64_t)b * cf.n];
      v.x += (T)w.x;
      v.y += (T)w.y;
    }
  }
  if (i == j && J.own[f.own_off + i]) v.x += (T)J.energy;
  if (is_root) {
    int li = i - J.nd, lj = j - J.nd;
    if (li >= 0 && li < J.nl && lj >= 0 && lj < J.nl) v = csub(v, from64<V>(J.sigma_l[li + (int64_t)lj * J.nl]));
    li -= J.rpos; lj -= J.rpos;
    if (li >= 0 && li < J.nr && lj >= 0 && lj < J.nr) v = csub(v, from64<V>(J.sigma_r[li + (int64_t)lj * J.nr]));
  }
  return v;
}

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
// In-place sweep of the leading ne pivots of an n x n matrix F (column-major, leading dimension
// ld), pivot rows restricted to [k, ne). On exit (columns of the first block unpermuted)
//   F[0:ne, 0:ne] = F11^-1, F[0:ne, ne:n] = X = F11^-1 F12,
//   F[ne:n, 0:ne] = W = -F21 F11^-1, F[ne:n, ne:n] = S = F22 - F21 X.
// Returns false when a pivot is not above tol * max|F11| (uniform in the block).
// With `perturb`, a pivot below the threshold is replaced by tol * max|F11| in its own direction
// (static pivoting, counted in *perturbed) instead of refusing the block: the factors then only
// precondition an iterative refinement that removes the perturbation.
template <typename T>
__device__ bool gj_sweep(typename Cx<T>::V* F, int64_t ld, int n, int ne, double tol, typename Cx<T>::V* prow,
                         typename Cx<T>::V* colk, int* piv, double* redv, int* redi, bool perturb = false,
                         int* perturbed = nullptr) {
  using V = typename Cx<T>::V;
  const int tid = threadIdx.x, nt = blockDim.x;
  T local = 0;
  for (int64_t idx = tid; idx < (int64_t)ne * ne; idx += nt) {
    int i = (int)(idx % ne), j = (int)(idx / ne);
    local = fmax(local, cnorm(F[i + j * ld]));
  }
  const double scale2 = block_max((double)local, redv);
  const double thresh = tol * tol * scale2;
  for (int k = 0; k < ne; ++k) {
    T best = -1;
    int bi = 0x7fffffff;
    for (int i = k + tid; i < ne; i += nt) {
      const T m = cnorm(F[i + k * ld]);
      if (m > best) { best = m; bi = i; }
    }
    double big;
    int p = block_argmax((double)best, bi, redv, redi, &big);
    if (!(big > thresh) || p >= ne) {
      if (!perturb) return false;
      // NaN or an empty column: nothing sensible to perturb.
      if (!(big >= 0.0) || !(scale2 > 0.0) || p >= ne) return false;
      if (tid == 0) {
        V& d = F[p + k * ld];
        const double mag = sqrt(big), target = tol * sqrt(scale2);
        if (mag > 0.0) { d.x = (T)(d.x / mag * target); d.y = (T)(d.y / mag * target); }
        else { d.x = (T)target; d.y = (T)0; }
        if (perturbed) atomicAdd(perturbed, 1);
      }
      __syncthreads();
    }
    if (tid == 0) piv[k] = p;
    if (p != k)
      for (int j = tid; j < n; j += nt) {
        V a = F[k + j * ld];
        F[k + j * ld] = F[p + j * ld];
        F[p + j * ld] = a;
      }
    __syncthreads();
    const V inv = cinv(F[k + k * ld]);
    for (int j = tid; j < n; j += nt) prow[j] = (j == k) ? inv : cmul(F[k + j * ld], inv);
    for (int i = tid; i < n; i += nt) colk[i] = F[i + k * ld];
    __syncthreads();
    for (int64_t idx = tid; idx < (int64_t)n * n; idx += nt) {
      const int i = (int)(idx % n), j = (int)(idx / n);
      V* d = &F[i + j * ld];
      if (i == k) *d = prow[j];
      else if (j == k) *d = cmul(cx<V>(-colk[i].x, -colk[i].y), inv);
      else *d = cfms(*d, colk[i], prow[j]);
    }
    __syncthreads();
  }
  // Undo the row interchanges as column interchanges of the inverse, last first.
  for (int k = ne - 1; k >= 0; --k) {
    int p = piv[k];
    if (p != k)
      for (int i = tid; i < n; i += nt) {
        V a = F[i + k * ld];
        F[i + k * ld] = F[i + p * ld];
        F[i + p * ld] = a;
      }
    __syncthreads();
  }
  return true;
}

// ---- small fronts: assembly and elimination in shared memory, one CTA per front ---------------
template <typename T, bool KEEP>
__global__ void __launch_bounds__(256) small_front_kernel(const JobDesc* __restrict__ jobs,
                                                          const Task* __restrict__ tasks, double tol, int perturb,
                                                          int* __restrict__ perturbed) {
  using V = typename Cx<T>::V;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const Task t = tasks[blockIdx.x];
  const JobDesc& J = jobs[t.job];
  const FrontDesc f = J.fronts[t.front];
  const int n = f.n, ne = f.ne;
  const int ld = n | 1;
  V* F = reinterpret_cast<V*>(smem_raw);
  V* prow = F + (int64_t)ld * n;
  V* colk = prow + n;
  int* piv = reinterpret_cast<int*>(colk + n);
  double* redv = reinterpret_cast<double*>(piv + ((n + 1) & ~1));
  int* redi = reinterpret_cast<int*>(redv + 32);
  for (int idx = threadIdx.x; idx < n * n; idx += blockDim.x) {
    int i = idx % n, j = idx / n;
    F[i + j * ld] = gather<T>(J, f, i, j, false);
  }
  __syncthreads();
  apply_entries<T>(J, f, F, ld, 0, n);
  __syncthreads();
  V* out = static_cast<V*>(J.arena) + f.arena_off;
  if (ne == 0) {
    for (int idx = threadIdx.x; idx < n * n; idx += blockDim.x) out[idx] = F[idx % n + (idx / n) * ld];
    return;
  }
  bool ok = gj_sweep<T>(F, ld, n, ne, tol, prow, colk, piv, redv, redi, perturb != 0, perturbed ? perturbed + t.job : nullptr);
  if (!ok) {
    if (threadIdx.x == 0) J.fail[t.front] = 1;
    return;
  }
  for (int idx = threadIdx.x; idx < n * n; idx += blockDim.x) {
    int i = idx % n, j = idx / n;
    if (!KEEP && (i < ne || j < ne)) continue;
    out[i + (int64_t)j * n] = F[i + j * ld];
  }
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
  const FrontDesc f = J.fronts[t.front];
  const int n = f.n;
  const int c0 = blockIdx.x * 32;
  if (c0 >= n) return;
  const int c1 = min(n, c0 + 32);
  V* F = is_root ? static_cast<V*>(J.root_arena) : static_cast<V*>(J.arena) + f.arena_off;
  for (int64_t idx = threadIdx.x; idx < (int64_t)n * (c1 - c0); idx += blockDim.x) {
    int i = (int)(idx % n), j = c0 + (int)(idx / n);
    F[i + (int64_t)j * n] = gather<TC, T>(J, f, i, j, is_root != 0);
  }
  __syncthreads();
  apply_entries<T>(J, f, F, n, c0, c1);
}

// Sweep of the pivot block F11 of a large front (or the whole root front), one CTA per front.
// The block is staged in shared memory when it fits, else swept in place (L2-resident).
template <typename T>
__global__ void __launch_bounds__(1024) pivot_block_kernel(const JobDesc* __restrict__ jobs,
                                                           const Task* __restrict__ tasks, double tol,
                                                           int smem_bytes, int is_root,
                                                           int32_t* __restrict__ root_status, int perturb,
                                                           int* __restrict__ perturbed) {
  using V = typename Cx<T>::V;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const Task t = tasks[blockIdx.x];
  const JobDesc& J = jobs[t.job];
  const FrontDesc f = J.fronts[t.front];
  const int n = f.n;
  const int ne = is_root ? n : f.ne;
  if (ne == 0) return;
  V* G = is_root ? static_cast<V*>(J.root_arena) : static_cast<V*>(J.arena) + f.arena_off;
  // Stage the block in shared memory only when it fits in what this launch allocated.
  const int64_t extra = 2 * (int64_t)ne * sizeof(V) + ((ne + 1) & ~1) * 4 + 32 * 8 + 32 * 4 + 16;
  const bool staged = (int64_t)ne * (ne | 1) * (int64_t)sizeof(V) + extra <= smem_bytes;
  V* buf = reinterpret_cast<V*>(smem_raw);
  V* F = G;
  int64_t ld = n;
  int64_t off = staged ? (int64_t)ne * (ne | 1) : 0;
  if (staged) {
    ld = ne | 1;
    F = buf;
    for (int64_t idx = threadIdx.x; idx < (int64_t)ne * ne; idx += blockDim.x) {
      int i = (int)(idx % ne), j = (int)(idx / ne);
      F[i + j * ld] = G[i + (int64_t)j * n];
    }
    __syncthreads();
  }
  V* prow = buf + off;
  V* colk = prow + ne;
  int* piv = reinterpret_cast<int*>(colk + ne);
  double* redv = reinterpret_cast<double*>(piv + ((ne + 1) & ~1));
  int* redi = reinterpret_cast<int*>(redv + 32);
  bool ok = gj_sweep<T>(F, ld, ne, ne, tol, prow, colk, piv, redv, redi, perturb != 0, perturbed ? perturbed + t.job : nullptr);
  if (!ok) {
    if (threadIdx.x == 0) {
      if (is_root) root_status[t.job] = ST_SINGULAR;
      else J.fail[t.front] = 1;
    }
    return;
  }
  if (staged)
    for (int64_t idx = threadIdx.x; idx < (int64_t)ne * ne; idx += blockDim.x) {
      int i = (int)(idx % ne), j = (int)(idx / ne);
      G[i + (int64_t)j * n] = F[i + j * ld];
    }
}

// Batched complex GEMM on the fronts of a level:
//   mode 0: X = F11^-1 F12 into the level scratch (ld ne)
//   mode 1: F22 -= F21 X
// 64 x 64 tiles, 256 threads, 4 x 4 complex results per thread.
template <typename T>
__global__ void __launch_bounds__(256) front_gemm_kernel(const JobDesc* __restrict__ jobs, const Task* __restrict__ tasks,
                                                         typename Cx<T>::V* __restrict__ xs, int mode) {
  using V = typename Cx<T>::V;
  constexpr int BM = 64, BN = 64, BK = 16;
  __shared__ V As[BK][BM];
  __shared__ V Bs[BK][BN + 1];
  const Task t = tasks[blockIdx.z];
  const JobDesc& J = jobs[t.job];
  const FrontDesc f = J.fronts[t.front];
  const int n = f.n, ne = f.ne, nb = n - ne;
  if (ne == 0 || nb == 0) return;
  V* F = static_cast<V*>(J.arena) + f.arena_off;
  V* X = xs + t.xoff;
  const V *A, *B;
  V* C;
  int M, N, K;
  int64_t lda, ldb, ldc;
  if (mode == 0) { A = F; lda = n; B = F + (int64_t)ne * n; ldb = n; C = X; ldc = ne; M = ne; N = nb; K = ne; }
  else { A = F + ne; lda = n; B = X; ldb = ne; C = F + ne + (int64_t)ne * n; ldc = n; M = nb; N = nb; K = ne; }
  const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN;
  if (m0 >= M || n0 >= N) return;
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  V acc[4][4];
#pragma unroll
  for (int r = 0; r < 4; ++r)
#pragma unroll
    for (int c = 0; c < 4; ++c) acc[r][c] = cx<V>(0.0, 0.0);
  for (int k0 = 0; k0 < K; k0 += BK) {
    for (int idx = threadIdx.x; idx < BM * BK; idx += 256) {
      int i = idx % BM, k = idx / BM;
      int gi = m0 + i, gk = k0 + k;
      As[k][i] = (gi < M && gk < K) ? A[gi + (int64_t)gk * lda] : cx<V>(0.0, 0.0);
    }
    for (int idx = threadIdx.x; idx < BK * BN; idx += 256) {
      int k = idx % BK, j = idx / BK;
      int gk = k0 + k, gj = n0 + j;
      Bs[k][j] = (gk < K && gj < N) ? B[gk + (int64_t)gj * ldb] : cx<V>(0.0, 0.0);
    }
    __syncthreads();
#pragma unroll 4
    for (int k = 0; k < BK; ++k) {
      V a[4], b[4];
#pragma unroll
      for (int r = 0; r < 4; ++r) a[r] = As[k][tx + 16 * r];
#pragma unroll
      for (int c = 0; c < 4; ++c) b[c] = Bs[k][ty + 16 * c];
#pragma unroll
      for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int c = 0; c < 4; ++c) acc[r][c] = cfma(acc[r][c], a[r], b[c]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int r = 0; r < 4; ++r)
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      int gi = m0 + tx + 16 * r, gj = n0 + ty + 16 * c;
      if (gi < M && gj < N) {
        V* d = &C[gi + (int64_t)gj * ldc];
        if (mode == 0) *d = acc[r][c];
        else *d = csub(*d, acc[r][c]);
      }
    }
}

// X from the level scratch into its place in the front (F12).
template <typename T>
__global__ void __launch_bounds__(256) store_x_kernel(const JobDesc* __restrict__ jobs, const Task* __restrict__ tasks,
                                                      const typename Cx<T>::V* __restrict__ xs) {
  using V = typename Cx<T>::V;
  const Task t = tasks[blockIdx.y];
  const JobDesc& J = jobs[t.job];
  const FrontDesc f = J.fronts[t.front];
  const int n = f.n, ne = f.ne, nb = n - ne;
  V* F = static_cast<V*>(J.arena) + f.arena_off;
  const V* X = xs + t.xoff;
  for (int64_t idx = blockIdx.x * 256 + threadIdx.x; idx < (int64_t)ne * nb; idx += (int64_t)gridDim.x * 256) {
    int i = (int)(idx % ne), j = (int)(idx / ne);
    F[i + (int64_t)(ne + j) * n] = X[idx];
  }
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
