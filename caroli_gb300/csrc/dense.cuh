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
  for (int j = threadIdx.x >> 5; j < t.npiv; j += blockDim.x >> 5)
    for (int i = threadIdx.x & 31; i < t.npiv; i += 32) mt = fmax(mt, cnorm(A[i + (int64_t)j * t.ld]));
  const double m = block_max((double)mt, red);
  if (threadIdx.x == 0) {
    *t.scale2 = m;
    *t.bad = 0;
  }
}

// Shared memory of a panel launch: the candidate rows of the panel (m x kb) when they fit, the
// pivot rows of the steps (kb x kb), the column buffer (2m), pos (m) and the displaced rows (kb),
// 32 doubles.
__host__ __device__ inline int64_t panel_work_bytes(int m, int vbytes) {
  return ((int64_t)GJ_KB * GJ_KB + 2 * (int64_t)m) * vbytes + 32 * 8 + ((int64_t)m + GJ_KB) * 4 + 16;
}
__host__ __device__ inline int64_t panel_staged_bytes(int m, int vbytes) {
  return (int64_t)m * GJ_KB * vbytes + panel_work_bytes(m, vbytes);
}

// Sweeps panel [k0, k0 + kb) of every matrix, one CTA per matrix:
//  1. Gauss-Jordan sweep of the m = npiv - k0 candidate rows of the panel columns (in shared
//     memory when they fit), pivots from those rows: the pivot block P becomes P^-1 and the other
//     candidate rows -a P^-1;
//  2. the rows outside the candidates (the pivoted rows above k0, the rows below npiv) receive
//     their panel entries -a P^-1 by replaying the sweep's elimination steps from the recorded
//     pivot rows, a thread per row (the same operations, in the same order, as if they had been
//     swept with the candidates: an explicit P^-1 would lose accuracy on ill-conditioned blocks);
//  3. the row interchanges reach the other columns: the pivot rows of the rest columns are
//     copied to Y (the update's right factor) and the rows the interchanges displaced below the
//     pivot rows are moved; the pivot rows themselves are rewritten by the update.
template <typename T>
__global__ void __launch_bounds__(256) inv_panel_kernel(const InvTask* __restrict__ tasks, int k0, double tol,
                                                        int perturb, int smem_bytes) {
  using V = typename Cx<T>::V;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const InvTask t = tasks[blockIdx.x];
  const int n = t.n, np = t.npiv;
  if (k0 >= np) return;
  if (*t.bad) return;
  const int kb = min(GJ_KB, np - k0);
  const int m = np - k0;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  V* A = static_cast<V*>(t.a);
  const int64_t ld = t.ld;
  const bool staged = panel_staged_bytes(m, (int)sizeof(V)) <= smem_bytes;
  V* C;  // candidate rows of the panel, leading dimension ldc
  int64_t ldc;
  V* work = reinterpret_cast<V*>(smem_raw);
  if (staged) {
    C = work;
    ldc = m;
    work += (int64_t)m * kb;
    for (int c = w; c < kb; c += nw)
      for (int i = lane; i < m; i += 32) C[i + c * ldc] = A[(k0 + i) + (int64_t)(k0 + c) * ld];
    __syncthreads();
  } else {
    C = A + k0 + (int64_t)k0 * ld;
    ldc = ld;
  }
  V* prows = work;                                      // kb x kb
  V* cb = prows + GJ_KB * GJ_KB;                        // 2m
  double* red = reinterpret_cast<double*>(cb + 2 * m);  // 32
  int* pos = reinterpret_cast<int*>(red + 32);          // m
  int* disp = pos + m;                                  // kb
  __shared__ int piv[GJ_KB];
  __shared__ int ndisp;
  for (int i = threadIdx.x; i < m; i += blockDim.x) {
    cb[i] = C[i];
    pos[i] = i;
  }
  __syncthreads();
  const double scale2 = *t.scale2;
  if (!gj_sweep<T>(C, (int)ldc, m, kb, kb, m, scale2, tol, cb, piv, perturb != 0, nullptr, prows)) {
    if (threadIdx.x == 0) *t.bad = 1;
    return;
  }
  if (staged)
    for (int c = w; c < kb; c += nw)
      for (int i = lane; i < m; i += 32) A[(k0 + i) + (int64_t)(k0 + c) * ld] = C[i + c * ldc];
  if (threadIdx.x == 0)
    for (int k = 0; k < kb; ++k) {
      t.piv[k0 + k] = k0 + piv[k];
      const int a = pos[k];
      pos[k] = pos[piv[k]];
      pos[piv[k]] = a;
    }
  if (w == 0) {
    // Positions at or past kb that hold another row now: each is some piv[k] (they only ever
    // receive rows from the first kb positions, so there are at most kb), listed once.
    __syncwarp();
    const int p = lane < kb ? piv[lane] : -1;
    const bool moved = lane < kb && p >= kb && pos[p] != p;
    const unsigned same = __match_any_sync(0xffffffffu, moved ? p : -1 - lane);
    const bool leader = moved && (__ffs(same) - 1 == lane);
    const unsigned bal = __ballot_sync(0xffffffffu, leader);
    if (leader) disp[__popc(bal & ((1u << lane) - 1u))] = p;
    if (lane == 0) ndisp = __popc(bal);
  }
  // 2. Rows outside the candidates: the sweep's steps replayed on each row, a thread per row.
  const int nout = n - m;
  for (int r = threadIdx.x; r < nout; r += blockDim.x) {
    const int row = r < k0 ? r : r + m;
    V* Ar = A + row + (int64_t)k0 * ld;
    V a[GJ_KB];
#pragma unroll
    for (int c = 0; c < GJ_KB; ++c) a[c] = c < kb ? Ar[(int64_t)c * ld] : cx<V>(0.0, 0.0);
    for (int k = 0; k < kb; ++k) {
      const V* pk = prows + k * kb;
      V ak = a[0];
#pragma unroll
      for (int c = 1; c < GJ_KB; ++c)
        if (c == k) ak = a[c];
#pragma unroll
      for (int c = 0; c < GJ_KB; ++c) {
        if (c >= kb) continue;
        if (c == k) a[c] = cmul(cx<V>(-ak.x, -ak.y), pk[c]);
        else a[c] = cfms(a[c], ak, pk[c]);
      }
    }
#pragma unroll
    for (int c = 0; c < GJ_KB; ++c)
      if (c < kb) Ar[(int64_t)c * ld] = a[c];
  }
  __syncthreads();
  // 3. Pivot rows of the rest columns into Y; displaced rows into place. A warp per column.
  V* Y = static_cast<V*>(t.y);
  const int nd = ndisp;
  for (int j = w; j < n; j += nw) {
    if (j >= k0 && j < k0 + kb) continue;
    V* Aj = A + (int64_t)j * ld;
    V yv = cx<V>(0.0, 0.0), dv = cx<V>(0.0, 0.0);
    if (lane < kb) yv = Aj[k0 + pos[lane]];
    if (lane < nd) dv = Aj[k0 + pos[disp[lane]]];
    __syncwarp();
    if (lane < kb) Y[lane + (int64_t)j * kb] = yv;
    if (lane < nd) Aj[k0 + disp[lane]] = dv;
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

// Undo the row interchanges as column interchanges (last first), as cycles of the resulting column
// permutation: every thread moves its own rows, no barrier per interchange. Shared memory: cperm,
// the cycle list and a visited mark (3 x npiv ints). Reports refused pivots.
__host__ __device__ inline int64_t finish_bytes(int npiv) { return 3 * (int64_t)npiv * 4 + 16; }

template <typename T>
__global__ void __launch_bounds__(256) inv_finish_kernel(const InvTask* __restrict__ tasks, const JobDesc* jobs,
                                                         int32_t* __restrict__ status) {
  using V = typename Cx<T>::V;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const InvTask t = tasks[blockIdx.x];
  if (*t.bad) {
    if (threadIdx.x == 0) {
      if (t.front < 0) status[t.job] = ST_SINGULAR;
      else jobs[t.job].fail[t.front] = 1;
    }
    return;
  }
  const int np = t.npiv;
  int* cperm = reinterpret_cast<int*>(smem_raw);
  int* cyc = cperm + np;
  int* seen = cyc + np;
  __shared__ int ncyc;
  for (int j = threadIdx.x; j < np; j += blockDim.x) {
    cperm[j] = j;
    seen[j] = 0;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    column_order(t.piv, np, cperm);
    // Cycles of cperm, each closed by a marked (negative) last entry.
    int len = 0;
    for (int j = 0; j < np; ++j) {
      if (seen[j] || cperm[j] == j) continue;
      int c = j;
      do {
        seen[c] = 1;
        cyc[len++] = c;
        c = cperm[c];
      } while (c != j);
      cyc[len - 1] = -1 - cyc[len - 1];
    }
    ncyc = len;
  }
  __syncthreads();
  V* A = static_cast<V*>(t.a);
  const int len = ncyc;
  for (int i = threadIdx.x; i < t.n; i += blockDim.x) {
    int q = 0;
    while (q < len) {
      // Cycle c_0 .. c_L-1 with cperm[c_a] = c_a+1: column c_a takes column c_a+1, the last c_0.
      const int c0 = cyc[q];
      const V first = A[i + (int64_t)c0 * t.ld];
      int cur = c0;
      while (true) {
        const int nx = cyc[++q];
        const bool last = nx < 0;
        const int c = last ? -1 - nx : nx;
        A[i + (int64_t)cur * t.ld] = A[i + (int64_t)c * t.ld];
        cur = c;
        if (last) break;
      }
      A[i + (int64_t)cur * t.ld] = first;
      ++q;
    }
  }
}

}  // namespace caroli
