// Refinement sweeps through the f32 factors: M d = v, one level of fronts per launch.
//
//   forward  (bottom-up)  z = own v + Σ_children h_c,  t = F11^-1 z_e,  h = z_b + W z_e
//   root                  x = F_root^-1 z
//   backward (top-down)   x_e = t - X x_b
//
// The sweeps stream each front's factor columns once ([F11^-1; W] forward, X backward) against
// CB right-hand-side columns (the channels of W_R, mostly one or two), so they are bound by HBM
// bandwidth and by the latency of the gathers in front of the streams. Each front row finds its
// sources in one 16-byte SweepRow (built with the plan); fronts of at most 64 variables run one per
// warp with the right-hand side in registers (broadcast by shuffles), larger ones as row tiles of
// 64 with the inner dimension split four ways.
//
// Tasks come from lists compacted to the solves still iterating (compact_kernel), so a batch in
// which a few solves need more GMRES steps does not sweep the others' tasks again.
#pragma once
#include "refine.cuh"
#include "tiny.cuh"

namespace caroli {

constexpr int SW_ROWS = 64, SW_SLICES = 4;

// Right-hand side of front row `g` for columns [j0, j0 + CB) (zero past the job's c columns).
template <int CB>
__device__ __forceinline__ void load_z(const RefineDesc& R, const double2* __restrict__ rin, SweepRow g, int j0,
                                       float2 (&z)[CB]) {
#pragma unroll
  for (int j = 0; j < CB; ++j) {
    const int col = j0 + j;
    float2 v = make_float2(0.f, 0.f);
    if (col < R.c) {
      if (g.own >= 0) v = f2(rin[g.own + (int64_t)col * R.nblk]);
      if (g.h0 >= 0) { const float2 h = R.hb[g.h0 + (int64_t)col * R.sum_nb]; v.x += h.x; v.y += h.y; }
      if (g.h1 >= 0) { const float2 h = R.hb[g.h1 + (int64_t)col * R.sum_nb]; v.x += h.x; v.y += h.y; }
    }
    z[j] = v;
  }
}

__device__ __forceinline__ bool sweep_idle(const RefineDesc& R, int src) {
  return R.done || (src >= 0 && R.inner_done);
}

// ---- fronts of at most 32 RPL variables: a warp each --------------------------------------------
// Lane l owns rows l, l + 32, ... (RPL rows); the right-hand side of row k comes from lane k % 32 of
// register k / 32 by a shuffle, so a warp needs no shared memory and no barrier. RPL = 1 serves
// the tiny fronts (n <= 32), RPL = 2 the fronts up to 64 variables.
template <int RPL, int CB>
__device__ __forceinline__ float2 lane_value(const float2 (&v)[RPL][CB], int k, int j) {
  float2 src = v[0][j];
#pragma unroll
  for (int u = 1; u < RPL; ++u)
    if ((k >> 5) == u) src = v[u][j];
  return make_float2(__shfl_sync(0xffffffffu, src.x, k & 31), __shfl_sync(0xffffffffu, src.y, k & 31));
}

template <int CB, int RPL>
__global__ void __launch_bounds__(256) sweep_warp_fwd_kernel(const RefineDesc* __restrict__ rd,
                                                             const Task* __restrict__ tasks, int ntasks, int src) {
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int ti = blockIdx.y * TINY_WARPS + w;
  if (ti >= ntasks) return;
  const Task tk = tasks[ti];
  const RefineDesc& R = rd[tk.job];
  const int j0 = blockIdx.x * CB;
  if (sweep_idle(R, src) || j0 >= R.c) return;
  const FrontDesc& f = *tk.fd;
  const int n = f.n, ne = f.ne;
  const double2* rin = sweep_src(R, src);
  float2 z[RPL][CB], acc[RPL][CB];
#pragma unroll
  for (int u = 0; u < RPL; ++u) {
    const int r = lane + 32 * u;
    if (r < n) load_z<CB>(R, rin, R.srows[f.var_off + r], j0, z[u]);
    else
#pragma unroll
      for (int j = 0; j < CB; ++j) z[u][j] = make_float2(0.f, 0.f);
#pragma unroll
    for (int j = 0; j < CB; ++j) acc[u][j] = r < ne ? make_float2(0.f, 0.f) : z[u][j];
  }
  const float2* F = R.arena + f.arena_off + lane;  // rows lane + 32 u of [F11^-1; W]
#pragma unroll 4
  for (int k = 0; k < ne; ++k) {
    float2 a[RPL];
#pragma unroll
    for (int u = 0; u < RPL; ++u) a[u] = lane + 32 * u < n ? F[32 * u + (int64_t)k * n] : make_float2(0.f, 0.f);
#pragma unroll
    for (int j = 0; j < CB; ++j) {
      const float2 zk = lane_value<RPL, CB>(z, k, j);
#pragma unroll
      for (int u = 0; u < RPL; ++u) acc[u][j] = cfma(acc[u][j], a[u], zk);
    }
  }
#pragma unroll
  for (int u = 0; u < RPL; ++u) {
    const int r = lane + 32 * u;
    if (r >= n) continue;
#pragma unroll
    for (int j = 0; j < CB; ++j) {
      const int col = j0 + j;
      if (col >= R.c) break;
      if (r < ne) R.tb[(f.toff + r) + (int64_t)col * R.sum_ne] = acc[u][j];
      else R.hb[(f.hoff + r - ne) + (int64_t)col * R.sum_nb] = acc[u][j];
    }
  }
}

template <int CB, int RPL>
__global__ void __launch_bounds__(256) sweep_warp_bwd_kernel(const RefineDesc* __restrict__ rd,
                                                             const Task* __restrict__ tasks, int ntasks, int src,
                                                             int dst) {
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int ti = blockIdx.y * TINY_WARPS + w;
  if (ti >= ntasks) return;
  const Task tk = tasks[ti];
  const RefineDesc& R = rd[tk.job];
  const int j0 = blockIdx.x * CB;
  if (sweep_idle(R, src) || j0 >= R.c) return;
  const FrontDesc& f = *tk.fd;
  const int n = f.n, ne = f.ne, nb = n - ne;
  if (ne == 0) return;
  float2* dout = sweep_dst(R, dst);
  float2 xb[RPL][CB], acc[RPL][CB];
#pragma unroll
  for (int u = 0; u < RPL; ++u) {
    const int p = lane + 32 * u, r = lane + 32 * u;
    const int vb = p < nb ? R.srows[f.var_off + ne + p].var : 0;
#pragma unroll
    for (int j = 0; j < CB; ++j) {
      const int col = j0 + j;
      xb[u][j] = (p < nb && col < R.c) ? dout[vb + (int64_t)col * R.nblk] : make_float2(0.f, 0.f);
      acc[u][j] = (r < ne && col < R.c) ? R.tb[(f.toff + r) + (int64_t)col * R.sum_ne] : make_float2(0.f, 0.f);
    }
  }
  if (ne <= 16) {
    // Few eliminated rows: lane = r + ne2 s (ne2 = ne rounded up to a power of two, s < 32 / ne2)
    // sums X[r, p] x_b[p] over p = s (mod 32 / ne2); the slices meet by shuffles at the end.
    const int ne2 = ne <= 1 ? 1 : ne <= 2 ? 2 : ne <= 4 ? 4 : ne <= 8 ? 8 : 16;
    const int S = 32 / ne2, r = lane & (ne2 - 1), sl = lane / ne2;
    const float2* X = R.arena + f.arena_off + r + (int64_t)ne * n;  // row r of X
    float2 part[CB];
#pragma unroll
    for (int j = 0; j < CB; ++j) part[j] = make_float2(0.f, 0.f);
    for (int p0 = 0; p0 < nb; p0 += S) {
      const int p = p0 + sl;
      const float2 a = (r < ne && p < nb) ? X[(int64_t)p * n] : make_float2(0.f, 0.f);
      const int u = p0 >> 5;  // the same for the whole warp: S divides 32
#pragma unroll
      for (int j = 0; j < CB; ++j) {
        float2 src = xb[0][j];
#pragma unroll
        for (int q = 1; q < RPL; ++q)
          if (u == q) src = xb[q][j];
        const float2 xp = make_float2(__shfl_sync(0xffffffffu, src.x, p & 31), __shfl_sync(0xffffffffu, src.y, p & 31));
        part[j] = cfma(part[j], a, xp);
      }
    }
    for (int o = ne2; o < 32; o <<= 1)
#pragma unroll
      for (int j = 0; j < CB; ++j) {
        part[j].x += __shfl_xor_sync(0xffffffffu, part[j].x, o);
        part[j].y += __shfl_xor_sync(0xffffffffu, part[j].y, o);
      }
    // Lane r (slice 0) holds row r's sum: bring it to the lane that owns row r's output.
#pragma unroll
    for (int j = 0; j < CB; ++j) {
      const float2 sum = make_float2(__shfl_sync(0xffffffffu, part[j].x, lane & (ne2 - 1)),
                                     __shfl_sync(0xffffffffu, part[j].y, lane & (ne2 - 1)));
      if (lane < ne) { acc[0][j].x -= sum.x; acc[0][j].y -= sum.y; }
    }
  } else {
    const float2* F = R.arena + f.arena_off + lane + (int64_t)ne * n;  // rows lane + 32 u of X
#pragma unroll 4
    for (int p = 0; p < nb; ++p) {
      float2 a[RPL];
#pragma unroll
      for (int u = 0; u < RPL; ++u) a[u] = lane + 32 * u < ne ? F[32 * u + (int64_t)p * n] : make_float2(0.f, 0.f);
#pragma unroll
      for (int j = 0; j < CB; ++j) {
        const float2 xp = lane_value<RPL, CB>(xb, p, j);
#pragma unroll
        for (int u = 0; u < RPL; ++u) acc[u][j] = cfms(acc[u][j], a[u], xp);
      }
    }
  }
#pragma unroll
  for (int u = 0; u < RPL; ++u) {
    const int r = lane + 32 * u;
    if (r >= ne) continue;
    const int ve = R.srows[f.var_off + r].var;
#pragma unroll
    for (int j = 0; j < CB; ++j) {
      const int col = j0 + j;
      if (col >= R.c) break;
      dout[ve + (int64_t)col * R.nblk] = acc[u][j];
    }
  }
}

// ---- larger fronts: row tiles of 64, the inner dimension split four ways -----------------------
// Forward: grid (column chunks, row tiles, tasks), the chunks of a tile adjacent so that their
// re-reads of the same factor rows come from L2; dynamic shared memory z_e (max ne x CB).
template <int CB>
__global__ void __launch_bounds__(256) sweep_rows_fwd_kernel(const RefineDesc* __restrict__ rd,
                                                             const Task* __restrict__ tasks, int src) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ float2 part[SW_SLICES - 1][SW_ROWS][CB];
  const Task tk = tasks[blockIdx.z];
  const RefineDesc& R = rd[tk.job];
  const int j0 = blockIdx.x * CB;
  if (sweep_idle(R, src) || j0 >= R.c) return;
  const FrontDesc& f = *tk.fd;
  const int n = f.n, ne = f.ne;
  const int r0 = blockIdx.y * SW_ROWS;
  if (r0 >= n) return;
  const double2* rin = sweep_src(R, src);
  float2* ze = reinterpret_cast<float2*>(smem_raw);  // ne x CB, row-major
  for (int p = threadIdx.x; p < ne; p += blockDim.x) {
    float2 z[CB];
    load_z<CB>(R, rin, R.srows[f.var_off + p], j0, z);
#pragma unroll
    for (int j = 0; j < CB; ++j) ze[p * CB + j] = z[j];
  }
  const int lr = threadIdx.x % SW_ROWS, sl = threadIdx.x / SW_ROWS;
  const int r = r0 + lr;
  float2 zr[CB];
  if (sl == 0 && r < n && r >= ne) load_z<CB>(R, rin, R.srows[f.var_off + r], j0, zr);
  __syncthreads();
  float2 acc[CB];
#pragma unroll
  for (int j = 0; j < CB; ++j) acc[j] = make_float2(0.f, 0.f);
  if (r < n) {
    const int kper = (ne + SW_SLICES - 1) / SW_SLICES;
    const int k1 = min(ne, (sl + 1) * kper);
    const float2* F = R.arena + f.arena_off + r;
#pragma unroll 8
    for (int k = sl * kper; k < k1; ++k) {
      const float2 a = F[(int64_t)k * n];
#pragma unroll
      for (int j = 0; j < CB; ++j) acc[j] = cfma(acc[j], a, ze[k * CB + j]);
    }
  }
  if (sl > 0)
#pragma unroll
    for (int j = 0; j < CB; ++j) part[sl - 1][lr][j] = acc[j];
  __syncthreads();
  if (sl != 0 || r >= n) return;
#pragma unroll
  for (int j = 0; j < CB; ++j) {
#pragma unroll
    for (int q = 0; q < SW_SLICES - 1; ++q) { acc[j].x += part[q][lr][j].x; acc[j].y += part[q][lr][j].y; }
    const int col = j0 + j;
    if (col >= R.c) break;
    if (r < ne) {
      R.tb[(f.toff + r) + (int64_t)col * R.sum_ne] = acc[j];
    } else {
      R.hb[(f.hoff + r - ne) + (int64_t)col * R.sum_nb] = make_float2(acc[j].x + zr[j].x, acc[j].y + zr[j].y);
    }
  }
}

// Backward: grid (column chunks, row tiles of the ne rows, tasks); dynamic shared memory x_b
// (max nb x CB).
template <int CB>
__global__ void __launch_bounds__(256) sweep_rows_bwd_kernel(const RefineDesc* __restrict__ rd,
                                                             const Task* __restrict__ tasks, int src, int dst) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ float2 part[SW_SLICES - 1][SW_ROWS][CB];
  const Task tk = tasks[blockIdx.z];
  const RefineDesc& R = rd[tk.job];
  const int j0 = blockIdx.x * CB;
  if (sweep_idle(R, src) || j0 >= R.c) return;
  const FrontDesc& f = *tk.fd;
  const int n = f.n, ne = f.ne, nb = n - ne;
  const int r0 = blockIdx.y * SW_ROWS;
  if (r0 >= ne) return;
  float2* dout = sweep_dst(R, dst);
  float2* xb = reinterpret_cast<float2*>(smem_raw);  // nb x CB, row-major
  for (int p = threadIdx.x; p < nb; p += blockDim.x) {
    const int v = R.srows[f.var_off + ne + p].var;
#pragma unroll
    for (int j = 0; j < CB; ++j) {
      const int col = j0 + j;
      xb[p * CB + j] = col < R.c ? dout[v + (int64_t)col * R.nblk] : make_float2(0.f, 0.f);
    }
  }
  __syncthreads();
  const int lr = threadIdx.x % SW_ROWS, sl = threadIdx.x / SW_ROWS;
  const int r = r0 + lr;
  float2 acc[CB];
#pragma unroll
  for (int j = 0; j < CB; ++j) acc[j] = make_float2(0.f, 0.f);
  if (r < ne) {
    const int kper = (nb + SW_SLICES - 1) / SW_SLICES;
    const int k1 = min(nb, (sl + 1) * kper);
    const float2* F = R.arena + f.arena_off + r + (int64_t)ne * n;
#pragma unroll 8
    for (int k = sl * kper; k < k1; ++k) {
      const float2 a = F[(int64_t)k * n];
#pragma unroll
      for (int j = 0; j < CB; ++j) acc[j] = cfma(acc[j], a, xb[k * CB + j]);
    }
  }
  if (sl > 0)
#pragma unroll
    for (int j = 0; j < CB; ++j) part[sl - 1][lr][j] = acc[j];
  __syncthreads();
  if (sl != 0 || r >= ne) return;
  const int v = R.srows[f.var_off + r].var;
#pragma unroll
  for (int j = 0; j < CB; ++j) {
#pragma unroll
    for (int q = 0; q < SW_SLICES - 1; ++q) { acc[j].x += part[q][lr][j].x; acc[j].y += part[q][lr][j].y; }
    const int col = j0 + j;
    if (col >= R.c) break;
    const float2 tv = R.tb[(f.toff + r) + (int64_t)col * R.sum_ne];
    dout[v + (int64_t)col * R.nblk] = make_float2(tv.x - acc[j].x, tv.y - acc[j].y);
  }
}

// ---- root: x = F_root^-1 z (the conjugate transpose for the adjoint) ---------------------------
// grid (column chunks, jobs); dynamic shared memory z (m x CB).
template <int CB>
__global__ void __launch_bounds__(256) sweep_root_kernel(const RefineDesc* __restrict__ rd, const int32_t* __restrict__ jobs,
                                                         int src, int dst) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const RefineDesc& R = rd[jobs ? jobs[blockIdx.y] : blockIdx.y];
  const int j0 = blockIdx.x * CB;
  if (sweep_idle(R, src) || j0 >= R.c) return;
  const double2* rin = sweep_src(R, src);
  float2* dout = sweep_dst(R, dst);
  const FrontDesc& f = R.fronts[R.root_front];
  const int m = f.n;
  float2* z = reinterpret_cast<float2*>(smem_raw);
  for (int p = threadIdx.x; p < m; p += blockDim.x) {
    float2 zz[CB];
    load_z<CB>(R, rin, R.srows[f.var_off + p], j0, zz);
#pragma unroll
    for (int j = 0; j < CB; ++j) z[p * CB + j] = zz[j];
  }
  __syncthreads();
  for (int i = threadIdx.x; i < m; i += blockDim.x) {
    float2 acc[CB];
#pragma unroll
    for (int j = 0; j < CB; ++j) acc[j] = make_float2(0.f, 0.f);
    if (R.adjoint) {
      for (int k = 0; k < m; ++k) {
        float2 a = R.root[k + (int64_t)i * m];
        a.y = -a.y;
#pragma unroll
        for (int j = 0; j < CB; ++j) acc[j] = cfma(acc[j], a, z[k * CB + j]);
      }
    } else {
#pragma unroll 8
      for (int k = 0; k < m; ++k) {
        const float2 a = R.root[i + (int64_t)k * m];
#pragma unroll
        for (int j = 0; j < CB; ++j) acc[j] = cfma(acc[j], a, z[k * CB + j]);
      }
    }
    const int v = R.srows[f.var_off + i].var;
#pragma unroll
    for (int j = 0; j < CB; ++j) {
      const int col = j0 + j;
      if (col >= R.c) break;
      dout[v + (int64_t)col * R.nblk] = acc[j];
    }
  }
}

// ---- compaction of the tasks (and jobs) still iterating ----------------------------------------
// A segment is a contiguous range of the full task list (one level's tiny or row-tile tasks);
// active tasks are copied to the same range of `out`, in any order (a sweep's tasks are
// independent), and counted in counts[segment]. Segment `nseg` lists the active jobs.
// Active: not done and, with `inner`, the current GMRES not converged either.
struct TaskSeg {
  int64_t first;
  int64_t count;
};

__device__ __forceinline__ void append(bool act, int32_t* counter, int* pos) {
  const int lane = threadIdx.x & 31;
  const unsigned m = __ballot_sync(0xffffffffu, act);
  int base = 0;
  if (m) {
    const int lead = __ffs(m) - 1;
    if (lane == lead) base = atomicAdd(counter, __popc(m));
    base = __shfl_sync(0xffffffffu, base, lead);
  }
  *pos = base + __popc(m & ((1u << lane) - 1u));
}

__global__ void __launch_bounds__(256) compact_kernel(const RefineDesc* __restrict__ rd, int njobs,
                                                      const Task* __restrict__ tasks, const TaskSeg* __restrict__ segs,
                                                      int nseg, Task* __restrict__ out, int32_t* __restrict__ jobs_out,
                                                      int32_t* __restrict__ counts, int inner) {
  const int s = blockIdx.y;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  auto active = [&](int job) {
    const RefineDesc& R = rd[job];
    return !R.done && !(inner && R.inner_done);
  };
  if (s == nseg) {
    if ((int64_t)blockIdx.x * blockDim.x >= njobs) return;  // uniform in the block
    const bool act = i < njobs && active((int)i);
    int pos;
    append(act, counts + nseg, &pos);
    if (act) jobs_out[pos] = (int32_t)i;
    return;
  }
  const TaskSeg sg = segs[s];
  if ((int64_t)blockIdx.x * blockDim.x >= sg.count) return;  // uniform in the block
  Task t{};
  bool act = false;
  if (i < sg.count) {
    t = tasks[sg.first + i];
    act = active(t.job);
  }
  int pos;
  append(act, counts + s, &pos);
  if (act) out[sg.first + pos] = t;
}

}  // namespace caroli
