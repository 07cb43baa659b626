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
#include "tc.cuh"

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
  void* bt;         // f32 matrices: the same rows as the tensor-core operand B' (see tc_update_kernel)
  double* scale2;   // max |a_ij|^2 of the input
  int32_t* bad;     // set when a pivot is refused
  int32_t ncol;     // columns the sweep transforms (n; npiv when the rest columns are formed by one
                    // GEMM afterwards, see schur_split in the engine)
  int32_t pad;
};

constexpr int GJ_KB = 32;

// Tensor-core update tiles: 64 complex rows (M = 128 real rows) by 64 columns, K = 2 kb <= 64.
constexpr int TCU_ROWS = 64;
constexpr int TCU_COLS = 64;
constexpr int TCU_A_BYTES = 2 * TCU_ROWS * 2 * GJ_KB * 4;  // one of A' hi / lo: M x K f32
constexpr int TCU_B_BYTES = TCU_COLS * 2 * GJ_KB * 4;      // one of B' hi / lo: N x K f32
// B' of a matrix of n columns in global memory: per column tile of the rest columns, hi then lo,
// each in the shared-memory operand layout (copied by one bulk copy).
__host__ __device__ inline size_t tc_operand_bytes(int n) {
  return (size_t)((n + TCU_COLS - 1) / TCU_COLS) * 2 * TCU_B_BYTES;
}

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
//     pivot rows, two lanes per row (the same operations, in the same order, as if they had been
//     swept with the candidates: an explicit P^-1 would lose accuracy on ill-conditioned blocks);
//  3. the row interchanges reach the other columns: the pivot rows of the rest columns are
//     copied to Y (the update's right factor) and the rows the interchanges displaced below the
//     pivot rows are moved; the pivot rows themselves are rewritten by the update.
template <typename T>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? 3 : 2) inv_panel_kernel(const InvTask* __restrict__ tasks, int k0, double tol,
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
  // 2. Rows outside the candidates: the sweep's steps replayed on each row, two adjacent lanes
  // per row (16 panel columns each); the entry of step k's column comes from its owner by a shuffle.
  const int nout = n - m;
  for (int base = 0; base < 2 * nout; base += blockDim.x) {
    const int item = base + threadIdx.x;
    const bool act = item < 2 * nout;
    const int r = act ? item >> 1 : 0, h = item & 1;
    const int row = r < k0 ? r : r + m;
    V* Ar = A + row + (int64_t)(k0 + 16 * h) * ld;
    V a[16];
#pragma unroll
    for (int c = 0; c < 16; ++c) a[c] = (act && 16 * h + c < kb) ? Ar[(int64_t)c * ld] : cx<V>(0.0, 0.0);
#pragma unroll
    for (int k = 0; k < GJ_KB; ++k) {
      if (k >= kb) break;
      const V* pk = prows + k * kb;
      const V own = a[k & 15];
      const int src = (lane & ~1) | (k >> 4);
      const V ak = cx<V>(__shfl_sync(0xffffffffu, own.x, src), __shfl_sync(0xffffffffu, own.y, src));
#pragma unroll
      for (int c = 0; c < 16; ++c) {
        const int col = 16 * h + c;
        if (col >= kb) continue;
        if (col == k) a[c] = cmul(cx<V>(-ak.x, -ak.y), pk[col]);
        else a[c] = cfms_pk(a[c], ak, pk[col]);
      }
    }
    if (act)
#pragma unroll
      for (int c = 0; c < 16; ++c)
        if (16 * h + c < kb) Ar[(int64_t)c * ld] = a[c];
  }
  __syncthreads();
  // 3. Pivot rows of the rest columns into Y; displaced rows into place. A warp per column.
  V* Y = static_cast<V*>(t.y);
  const int nd = ndisp;
  for (int j = w; j < t.ncol; j += nw) {
    if (j >= k0 && j < k0 + kb) continue;
    V* Aj = A + (int64_t)j * ld;
    V yv = cx<V>(0.0, 0.0), dv = cx<V>(0.0, 0.0);
    if (lane < kb) yv = Aj[k0 + pos[lane]];
    if (lane < nd) dv = Aj[k0 + pos[disp[lane]]];
    __syncwarp();
    if (lane < kb) Y[lane + (int64_t)j * kb] = yv;
    if (lane < nd) Aj[k0 + disp[lane]] = dv;
    if (t.bt) {
      // The same row as B' of the tensor-core update: rest column r, K = 2 c (re), 2 c + 1 (im),
      // tf32 hi and lo; zero past kb.
      const int r = j < k0 ? j : j - kb;
      unsigned char* tile = static_cast<unsigned char*>(t.bt) + (size_t)(r / TCU_COLS) * 2 * TCU_B_BYTES;
      const uint32_t off = tc::kmajor_offset(r % TCU_COLS, 2 * lane, TCU_COLS);
      const float2 y = lane < kb ? make_float2((float)yv.x, (float)yv.y) : make_float2(0.f, 0.f);
      const float2 hi = make_float2(tc::to_tf32(y.x), tc::to_tf32(y.y));
      *reinterpret_cast<float2*>(tile + off) = hi;
      *reinterpret_cast<float2*>(tile + TCU_B_BYTES + off) =
          make_float2(tc::to_tf32(y.x - hi.x), tc::to_tf32(y.y - hi.y));
    }
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
  const int rest = t.ncol - kb;
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

// Rank-kb update of the rest columns on the tensor cores (f32 data, 3xTF32): the product of
// inv_update_kernel written as a real GEMM. With P (the swept panel, n x kb) and Y (the pivot rows
// of the rest columns, kb x rest) complex, the interleaved output rows (re, im) of 64 complex rows
// are the 128 rows of
//     D = A' B'^T,  A'[2i][2c] = Re P, A'[2i][2c+1] = -Im P, A'[2i+1][2c] = Im P, A'[2i+1][2c+1] = Re P,
//                   B'[j][2c] = Re Y[c, j], B'[j][2c+1] = Im Y[c, j],
// K = 2 kb. Both operands are split into tf32 hi + lo parts and D = lo hi + hi lo + hi hi
// accumulates in f32 in tensor memory (24 MMAs of 128 x 64 x 8 per 64-column tile), about the
// accuracy of an f32 product.
//
// A CTA takes 64 complex rows of one matrix: all warps stage A' from the panel columns, then
//   warp 0 (one thread) bulk-copies the B' tiles, written by the panel kernel, into shared memory;
//   warp 1 (one thread) issues the MMAs, alternating two 64-column accumulators in tensor memory;
//   warps 2-9 (two per 32-lane quarter of tensor memory, 32 columns each) add each finished tile to
//   the old values (zero on the pivot rows) while the next tile is copied and multiplied.
// Barriers: bfull (B' copied), bempty (its MMAs done), tfull[a] (accumulator a ready), tempty[a]
// (accumulator a drained). Every wait is bounded: the pipeline waits by `wait_limit` polls (TCU_WAIT
// unless the caller lowers it), the final drain by TCU_WAIT. A pipeline wait that runs out sets
// ST_TIMEOUT for the solve and stops the CTA after the copies and MMAs it issued have drained.
// grid (row tiles, matrices, column groups), 320 threads: a CTA walks TCU_GROUP column tiles,
// so a few very wide fronts still spread over many CTAs.
constexpr int TCU_EPI_WARPS = 16;
constexpr int TCU_THREADS = 32 * (2 + TCU_EPI_WARPS);
constexpr int TCU_GROUP = 8;
constexpr int TCU_SMEM = 2 * TCU_A_BYTES + 2 * TCU_B_BYTES + 1024;
constexpr uint32_t TCU_WAIT = 1u << 22;

__global__ void __launch_bounds__(TCU_THREADS, 2) tc_update_kernel(const InvTask* __restrict__ tasks, int k0,
                                                                int32_t* __restrict__ status, uint32_t wait_limit) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ uint32_t tslot;
  __shared__ __align__(8) uint64_t bfull, bempty, tfull[2], tempty[2];
  __shared__ int abort_flag;
  const InvTask t = tasks[blockIdx.y];
  const int n = t.n;
  if (k0 >= t.npiv || t.bt == nullptr) return;
  if (*t.bad) return;
  const int kb = min(GJ_KB, t.npiv - k0);
  const int rest = t.ncol - kb;
  const int i0 = blockIdx.x * TCU_ROWS;
  if (i0 >= n || rest <= 0) return;
  const int tid = threadIdx.x, w = tid >> 5, lane = tid & 31;
  constexpr int M = 2 * TCU_ROWS;
  unsigned char* base = reinterpret_cast<unsigned char*>(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  unsigned char* a_hi = base;
  unsigned char* a_lo = a_hi + TCU_A_BYTES;
  unsigned char* b_hi = a_lo + TCU_A_BYTES;
  unsigned char* b_lo = b_hi + TCU_B_BYTES;
  float2* A = static_cast<float2*>(t.a);
  const unsigned char* bt = static_cast<const unsigned char*>(t.bt);
  const int64_t ld = t.ld;
  const int tile0 = blockIdx.z * TCU_GROUP;
  const int tiles = min((rest + TCU_COLS - 1) / TCU_COLS - tile0, TCU_GROUP);
  if (tiles <= 0) return;
  if (w == 0) tc::tmem_alloc(&tslot, 2 * TCU_COLS);
  if (tid == 0) {
    tc::mbar_init(&bfull, 1);
    tc::mbar_init(&bempty, 1);
    tc::mbar_init(&tfull[0], 1);
    tc::mbar_init(&tfull[1], 1);
    tc::mbar_init(&tempty[0], TCU_EPI_WARPS);
    tc::mbar_init(&tempty[1], TCU_EPI_WARPS);
    abort_flag = 0;
  }
  // A' from the panel columns of this tile's rows (zero past n and past 2 kb): a complex row and
  // two complex columns per item, one 16-byte core-matrix row in each of real rows 2i, 2i + 1.
  for (int idx = tid; idx < TCU_ROWS * (GJ_KB / 2); idx += blockDim.x) {
    const int i = idx % TCU_ROWS, c = 2 * (idx / TCU_ROWS);
    float2 p0 = make_float2(0.f, 0.f), p1 = make_float2(0.f, 0.f);
    if (i0 + i < n) {
      if (c < kb) p0 = A[(i0 + i) + (int64_t)(k0 + c) * ld];
      if (c + 1 < kb) p1 = A[(i0 + i) + (int64_t)(k0 + c + 1) * ld];
    }
    const uint32_t o0 = tc::kmajor_offset(2 * i, 2 * c, M), o1 = tc::kmajor_offset(2 * i + 1, 2 * c, M);
    tc::store_split(a_hi + o0, a_lo + o0, make_float4(p0.x, -p0.y, p1.x, -p1.y));
    tc::store_split(a_hi + o1, a_lo + o1, make_float4(p0.y, p0.x, p1.y, p1.x));
  }
  tc::fence_smem_async();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tbase = tslot;
  volatile int* abort_v = &abort_flag;
  auto fail = [&]() {
    *abort_v = 1;
    status[t.job] = ST_TIMEOUT;
  };
  int copies = 0, mma_tiles = 0;  // issued by this thread (producer / MMA issuer)
  if (w == 0) {
    if (lane == 0)
      for (int ct = 0; ct < tiles && !*abort_v; ++ct) {
        if (ct >= 1 && !tc::mbar_wait(&bempty, (uint32_t)((ct - 1) & 1), wait_limit)) { fail(); break; }
        tc::mbar_arrive_expect_tx(&bfull, 2 * TCU_B_BYTES);
        const size_t tile = (size_t)(tile0 + ct) * 2 * TCU_B_BYTES;
        tc::bulk_copy_g2s(b_hi, bt + tile, TCU_B_BYTES, &bfull);
        tc::bulk_copy_g2s(b_lo, bt + tile + TCU_B_BYTES, TCU_B_BYTES, &bfull);
        ++copies;
      }
  } else if (w == 1) {
    if (lane == 0) {
      const uint32_t idesc = tc::idesc_tf32(M, TCU_COLS);
      const int slices = (2 * kb + 7) / 8;
      for (int ct = 0; ct < tiles && !*abort_v; ++ct) {
        const int a = ct & 1;
        if (!tc::mbar_wait(&bfull, (uint32_t)(ct & 1), wait_limit)) { fail(); break; }
        if (ct >= 2 && !tc::mbar_wait(&tempty[a], (uint32_t)(((ct >> 1) - 1) & 1), wait_limit)) { fail(); break; }
        tc::fence_after_sync();
        const uint32_t d = tbase + (uint32_t)(a * TCU_COLS);
        for (int sl = 0; sl < slices; ++sl) {
          const uint64_t ah = tc::smem_desc(tc::smem_addr(a_hi + sl * M * 32), 128, 256);
          const uint64_t al = tc::smem_desc(tc::smem_addr(a_lo + sl * M * 32), 128, 256);
          const uint64_t bh = tc::smem_desc(tc::smem_addr(b_hi + sl * TCU_COLS * 32), 128, 256);
          const uint64_t bl = tc::smem_desc(tc::smem_addr(b_lo + sl * TCU_COLS * 32), 128, 256);
          tc::mma_tf32(d, al, bh, idesc, sl > 0);
          tc::mma_tf32(d, ah, bl, idesc, true);
          tc::mma_tf32(d, ah, bh, idesc, true);
        }
        tc::mma_commit(&bempty);
        tc::mma_commit(&tfull[a]);
        ++mma_tiles;
      }
    }
  } else {
    // Epilogue: this warp's quarter of the 128 real rows (thread row r2, complex row i0 + r2 / 2)
    // and half of the 64 columns of each tile.
    constexpr int HC = TCU_COLS / (TCU_EPI_WARPS / 4);
    const int q = w & 3, h = (w - 2) >> 2;
    const int r2 = 32 * q + lane;
    const int gi = i0 + (r2 >> 1);
    const bool row_in = gi < n;
    const bool pivot_row = gi >= k0 && gi < k0 + kb;
    float* Af = reinterpret_cast<float*>(A) + (r2 & 1);
    for (int ct = 0; ct < tiles; ++ct) {
      const int a = ct & 1, r0 = (tile0 + ct) * TCU_COLS + h * HC;
      float old[HC];
#pragma unroll
      for (int j = 0; j < HC; ++j) {
        const int r = r0 + j;
        old[j] = 0.f;
        if (row_in && !pivot_row && r < rest) old[j] = Af[2 * (gi + (int64_t)(r < k0 ? r : r + kb) * ld)];
      }
      bool ok = !*abort_v && tc::mbar_wait(&tfull[a], (uint32_t)((ct >> 1) & 1), wait_limit);
      ok = __all_sync(0xffffffffu, ok);
      if (!ok) {
        if (lane == 0) fail();
        break;
      }
      tc::fence_after_sync();
      float v[HC];
#pragma unroll
      for (int c0 = 0; c0 < HC; c0 += 16) {
        float part[16];
        tc::tmem_ld16(tbase + ((uint32_t)(32 * q) << 16) + (uint32_t)(a * TCU_COLS + h * HC + c0), part);
#pragma unroll
        for (int i = 0; i < 16; ++i) v[c0 + i] = part[i];
      }
      tc::tmem_ld_wait();
      tc::fence_before_sync();
      __syncwarp();
      if (lane == 0) tc::mbar_arrive(&tempty[a]);
#pragma unroll
      for (int j = 0; j < HC; ++j) {
        const int r = r0 + j;
        if (row_in && r < rest) Af[2 * (gi + (int64_t)(r < k0 ? r : r + kb) * ld)] = old[j] + v[j];
      }
    }
  }
  // Drain what this thread issued before tensor memory and shared memory go away.
  if (*abort_v) {
    if (w == 0 && lane == 0 && copies > 0) tc::mbar_wait(&bfull, (uint32_t)((copies - 1) & 1), TCU_WAIT);
    if (w == 1 && lane == 0 && mma_tiles > 0) tc::mbar_wait(&bempty, (uint32_t)((mma_tiles - 1) & 1), TCU_WAIT);
  }
  tc::fence_before_sync();
  __syncthreads();
  if (w == 0) tc::tmem_dealloc(tbase, 2 * TCU_COLS);
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
