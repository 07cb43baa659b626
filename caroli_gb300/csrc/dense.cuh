// Batched in-place Gauss-Jordan sweep of dense complex fronts, blocked, with partial pivoting over
// the leading npiv rows: for a front [F11 F12; F21 F22] with npiv = ne it leaves
//     [ F11^-1          | X = F11^-1 F12 ]
//     [ W = -F21 F11^-1 | S = F22 - F21 X ]
// and with npiv = n (the root) the inverse. Rows below npiv are eliminated exactly as in
// right-looking LU, so S carries the accuracy of the reference's LU-based Schur step.
//
// A panel of kb columns is swept by one CTA per matrix (pivot search over the rows not pivoted
// yet, full-row interchanges, in-place Gauss-Jordan on the panel columns); the other columns
// then receive the panel's transformation as one rank-kb product, spread over many CTAs:
//     rows of the panel's pivots:  A_p,rest <- A_pc^-1 A_p,rest
//     other rows:                  A_o,rest <- A_o,rest - A_oc A_pc^-1 A_p,rest
// i.e. A[:, rest] = [0 on pivot rows; A_o,rest] + (swept panel) x Y with Y the pivot rows of the
// rest columns before the update (copied aside, so CTAs never read rows another CTA writes).
// After the last panel the row interchanges are undone as column interchanges, last first.
// The pivots are those of partial-pivoting LU, so the stability test |pivot| > tol max|A| of
// caroli-dense/src/field.rs:79-105 applies unchanged.
#pragma once
#include "kernels.cuh"

namespace caroli {

// One matrix of a batched inverse.
struct InvTask {
  void* a;          // column-major, leading dimension ld
  int64_t ld;
  int32_t n;        // rows and columns
  int32_t job;      // solve the matrix belongs to (status and fail flags)
  int32_t front;    // front index (-1: the root)
  int32_t npiv;     // pivots: the leading npiv rows and columns
  int32_t* piv;     // n entries
  void* y;          // kb x n scratch (pivot rows of the rest columns)
  double* scale2;   // max |a_ij|^2 of the input
  int32_t* bad;     // set when a pivot is refused
};

constexpr int GJ_KB = 32;

template <typename T>
__global__ void __launch_bounds__(256) inv_scale_kernel(const InvTask* __restrict__ tasks) {
  using V = typename Cx<T>::V;
  __shared__ double red[32];
  const InvTask t = tasks[blockIdx.x];
  const V* A = static_cast<const V*>(t.a);
  T mt = 0;
  for (int64_t idx = threadIdx.x; idx < (int64_t)t.npiv * t.npiv; idx += blockDim.x) {
    const int i = (int)(idx % t.npiv), j = (int)(idx / t.npiv);
    mt = fmax(mt, cnorm(A[i + (int64_t)j * t.ld]));
  }
  const double m = block_max((double)mt, red);
  if (threadIdx.x == 0) {
    *t.scale2 = m;
    *t.bad = 0;
  }
}

// Sweeps panel [k0, k0 + kb) of every matrix. Shared memory: the panel (n x kb) when it fits
// (`staged`), else it is swept in place in global memory.
template <typename T>
__global__ void __launch_bounds__(256) inv_panel_kernel(const InvTask* __restrict__ tasks, int k0, double tol,
                                                        int perturb, int smem_bytes) {
  using V = typename Cx<T>::V;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ double redv[32];
  __shared__ int redi[32];
  const InvTask t = tasks[blockIdx.x];
  const int n = t.n, np = t.npiv;
  if (k0 >= np) return;
  if (*t.bad) return;
  const int kb = min(GJ_KB, np - k0);
  V* A = static_cast<V*>(t.a);
  const int64_t ld = t.ld;
  const bool staged = (int64_t)n * kb * (int64_t)sizeof(V) + 2 * (int64_t)n * sizeof(V) <= smem_bytes;
  V* P;  // panel, column-major with leading dimension pld
  int64_t pld;
  V* work = reinterpret_cast<V*>(smem_raw);
  if (staged) {
    P = work;
    pld = n;
    work += (int64_t)n * kb;
    for (int64_t idx = threadIdx.x; idx < (int64_t)n * kb; idx += blockDim.x) {
      const int i = (int)(idx % n), c = (int)(idx / n);
      P[idx] = A[i + (int64_t)(k0 + c) * ld];
    }
  } else {
    P = A + (int64_t)k0 * ld;
    pld = ld;
  }
  V* prow = work;      // kb
  V* colk = work + kb; // n
  __syncthreads();
  const double scale2 = *t.scale2;
  const double thresh = tol * tol * scale2;
  for (int kk = 0; kk < kb; ++kk) {
    const int k = k0 + kk;
    T best = -1;
    int bi = 0x7fffffff;
    for (int i = k + threadIdx.x; i < np; i += blockDim.x) {
      const T m = cnorm(P[i + kk * pld]);
      if (m > best) { best = m; bi = i; }
    }
    double big;
    const int p = block_argmax((double)best, bi, redv, redi, &big);
    if (!(big > thresh) || p >= np) {
      if (!perturb || !(big >= 0.0) || !(scale2 > 0.0) || p >= np) {
        if (threadIdx.x == 0) *t.bad = 1;
        return;
      }
      if (threadIdx.x == 0) {
        V& d = P[p + kk * pld];
        const double mag = sqrt(big), target = tol * sqrt(scale2);
        if (mag > 0.0) { d.x = (T)(d.x / mag * target); d.y = (T)(d.y / mag * target); }
        else { d.x = (T)target; d.y = (T)0; }
      }
      __syncthreads();
    }
    if (threadIdx.x == 0) t.piv[k] = p;
    if (p != k) {
      // Full-row interchange: the panel (staged or not) and every column outside it.
      for (int c = threadIdx.x; c < kb; c += blockDim.x) {
        V tmp = P[k + c * pld];
        P[k + c * pld] = P[p + c * pld];
        P[p + c * pld] = tmp;
      }
      for (int j = threadIdx.x; j < n; j += blockDim.x) {
        if (j >= k0 && j < k0 + kb) continue;
        V tmp = A[k + (int64_t)j * ld];
        A[k + (int64_t)j * ld] = A[p + (int64_t)j * ld];
        A[p + (int64_t)j * ld] = tmp;
      }
    }
    __syncthreads();
    const V inv = cinv(P[k + kk * pld]);
    for (int c = threadIdx.x; c < kb; c += blockDim.x) prow[c] = (c == kk) ? inv : cmul(P[k + c * pld], inv);
    for (int i = threadIdx.x; i < n; i += blockDim.x) colk[i] = P[i + kk * pld];
    __syncthreads();
    for (int64_t idx = threadIdx.x; idx < (int64_t)n * kb; idx += blockDim.x) {
      const int i = (int)(idx % n), c = (int)(idx / n);
      V* d = &P[i + c * pld];
      if (i == k) *d = prow[c];
      else if (c == kk) *d = cmul(cx<V>(-colk[i].x, -colk[i].y), inv);
      else *d = cfms(*d, colk[i], prow[c]);
    }
    __syncthreads();
  }
  if (staged)
    for (int64_t idx = threadIdx.x; idx < (int64_t)n * kb; idx += blockDim.x) {
      const int i = (int)(idx % n), c = (int)(idx / n);
      A[i + (int64_t)(k0 + c) * ld] = P[idx];
    }
  // Pivot rows of the rest columns, before the update.
  V* Y = static_cast<V*>(t.y);
  for (int64_t idx = threadIdx.x; idx < (int64_t)kb * n; idx += blockDim.x) {
    const int r = (int)(idx % kb), j = (int)(idx / kb);
    if (j >= k0 && j < k0 + kb) continue;
    Y[r + (int64_t)j * kb] = A[(k0 + r) + (int64_t)j * ld];
  }
}

// Rank-kb update of the rest columns: grid (row tiles of 64, column tiles of 64, matrices).
template <typename T>
__global__ void __launch_bounds__(256) inv_update_kernel(const InvTask* __restrict__ tasks, int k0) {
  using V = typename Cx<T>::V;
  __shared__ V Ps[GJ_KB][64 + 1];  // panel rows of this tile, transposed: Ps[c][i]
  __shared__ V Ys[GJ_KB][64 + 1];  // Ys[c][j]
  const InvTask t = tasks[blockIdx.z];
  const int n = t.n;
  if (k0 >= t.npiv) return;
  if (*t.bad) return;
  const int kb = min(GJ_KB, t.npiv - k0);
  const int rest = n - kb;
  const int i0 = blockIdx.x * 64, r0 = blockIdx.y * 64;
  if (i0 >= n || r0 >= rest) return;
  V* A = static_cast<V*>(t.a);
  const V* Y = static_cast<const V*>(t.y);
  const int64_t ld = t.ld;
  auto col_of = [&](int r) { return r < k0 ? r : r + kb; };
  for (int idx = threadIdx.x; idx < 64 * GJ_KB; idx += 256) {
    const int i = idx % 64, c = idx / 64;
    const int gi = i0 + i;
    Ps[c][i] = (gi < n && c < kb) ? A[gi + (int64_t)(k0 + c) * ld] : cx<V>(0.0, 0.0);
  }
  for (int idx = threadIdx.x; idx < 64 * GJ_KB; idx += 256) {
    const int c = idx % GJ_KB, j = idx / GJ_KB;
    const int r = r0 + j;
    Ys[c][j] = (r < rest && c < kb) ? Y[c + (int64_t)col_of(r) * kb] : cx<V>(0.0, 0.0);
  }
  __syncthreads();
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  V acc[4][4];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      const int gi = i0 + tx + 16 * a, r = r0 + ty + 16 * b;
      const bool in = gi < n && r < rest;
      const bool pivot_row = gi >= k0 && gi < k0 + kb;
      acc[a][b] = (in && !pivot_row) ? A[gi + (int64_t)col_of(r) * ld] : cx<V>(0.0, 0.0);
    }
  for (int c = 0; c < kb; ++c) {
    V pa[4], yb[4];
#pragma unroll
    for (int a = 0; a < 4; ++a) pa[a] = Ps[c][tx + 16 * a];
#pragma unroll
    for (int b = 0; b < 4; ++b) yb[b] = Ys[c][ty + 16 * b];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
      for (int b = 0; b < 4; ++b) acc[a][b] = cfma(acc[a][b], pa[a], yb[b]);
  }
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      const int gi = i0 + tx + 16 * a, r = r0 + ty + 16 * b;
      if (gi < n && r < rest) A[gi + (int64_t)col_of(r) * ld] = acc[a][b];
    }
}

// Undo the row interchanges as column interchanges (last first); report refused pivots.
template <typename T>
__global__ void __launch_bounds__(256) inv_finish_kernel(const InvTask* __restrict__ tasks, const JobDesc* jobs,
                                                         int32_t* __restrict__ status) {
  using V = typename Cx<T>::V;
  const InvTask t = tasks[blockIdx.x];
  if (*t.bad) {
    if (threadIdx.x == 0) {
      if (t.front < 0) status[t.job] = ST_SINGULAR;
      else jobs[t.job].fail[t.front] = 1;
    }
    return;
  }
  V* A = static_cast<V*>(t.a);
  for (int k = t.npiv - 1; k >= 0; --k) {
    const int p = t.piv[k];
    if (p != k)
      for (int i = threadIdx.x; i < t.n; i += blockDim.x) {
        V a = A[i + (int64_t)k * t.ld];
        A[i + (int64_t)k * t.ld] = A[i + (int64_t)p * t.ld];
        A[i + (int64_t)p * t.ld] = a;
      }
    __syncthreads();
  }
}

}  // namespace caroli
