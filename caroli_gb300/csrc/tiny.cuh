// Fronts of at most 32 variables, one warp each (eight per CTA): three quarters of the fronts of a
// 2D nested-dissection tree are this small (leaves and the separators just above them) and carry
// about 2 % of the flops, so a block-wide synchronisation per pivot would dominate their cost.
// Lane i owns row i of the front; the warp synchronises with __syncwarp only.
//
// tiny_front_kernel is small_front_kernel (same assembly, same Gauss-Jordan sweep and pivot test,
// same factor layout [F11^-1 X; W S]).
#pragma once
#include "kernels.cuh"
#include "refine.cuh"

namespace caroli {

constexpr int TINY_MAX = 32;
constexpr int TINY_WARPS = 8;

// Dynamic shared memory of tiny_front_kernel for fronts of at most `nmax` variables: per warp the
// front (nmax x (nmax | 1)) and the pivot row.
template <typename T> size_t tiny_smem(int nmax) {
  return (size_t)TINY_WARPS * ((size_t)nmax * (nmax | 1) + nmax) * sizeof(typename Cx<T>::V);
}

// nmax: the launch's largest front (sizes each warp's shared-memory block, leading dimension nmax | 1).
template <typename T, bool KEEP>
__global__ void __launch_bounds__(256) tiny_front_kernel(const JobDesc* __restrict__ jobs, const Task* __restrict__ tasks,
                                                         int ntasks, double tol, int perturb, int* __restrict__ perturbed,
                                                         int nmax) {
  using V = typename Cx<T>::V;
  const int LD = nmax | 1;
  extern __shared__ __align__(16) unsigned char smem_raw[];  // per warp: front (nmax x LD) and pivot row
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int ti = blockIdx.x * TINY_WARPS + w;
  if (ti >= ntasks) return;
  const Task t = tasks[ti];
  const JobDesc& J = jobs[t.job];
  const FrontDesc f = *t.fd;  // copied at once: its fields load together, not on first use
  const int n = f.n, ne = f.ne;
  V* F = reinterpret_cast<V*>(smem_raw) + (size_t)w * ((size_t)nmax * LD + nmax);
  V* prow = F + (size_t)nmax * LD;
  // The front's first 32 H entries and their values are requested before the assembly, so that
  // their loads overlap its loads.
  const bool has0 = lane < f.ent_cnt;
  Entry en0{};
  double2 h0 = make_double2(0.0, 0.0);
  if (has0) {
    en0 = J.entries[f.ent_off + lane];
    h0 = J.vals[en0.q];
  }
  // Assembly: lane i builds row i. Column j's child positions are row j's, taken from lane j by a
  // shuffle, so the value loads of consecutive columns do not wait for index loads; eight columns
  // at a time keep sixteen loads in flight per lane.
  {
    const ChildBlocks<T> kids(J, f);
    int ai[2];
    kids.index(lane < n ? lane : 0, ai);
    const bool own = lane < n && J.own[f.own_off + lane];
#pragma unroll 8
    for (int j = 0; j < n; ++j) {
      const int bj[2] = {__shfl_sync(0xffffffffu, ai[0], j), __shfl_sync(0xffffffffu, ai[1], j)};
      V v = kids.template at<T>(ai, bj);
      if (j == lane && own) v.x += (T)J.energy;
      if (lane < n) F[lane + j * LD] = v;
    }
  }
  __syncwarp();
  if (has0) {
    if (en0.conj) h0.y = -h0.y;
    V& d = F[en0.a + en0.b * LD];
    d = csub(d, from64<V>(h0));
  }
  for (int64_t e = lane + 32; e < f.ent_cnt; e += 32) {
    const Entry en = J.entries[f.ent_off + e];
    double2 h = J.vals[en.q];
    if (en.conj) h.y = -h.y;
    V& d = F[en.a + en.b * LD];
    d = csub(d, from64<V>(h));
  }
  __syncwarp();
  V* out = static_cast<V*>(J.arena) + f.arena_off;
  if (ne > 0) {
    T s2 = 0;
    if (lane < ne)
      for (int j = 0; j < ne; ++j) s2 = fmax(s2, cnorm(F[lane + j * LD]));
    for (int o = 16; o > 0; o >>= 1) s2 = fmax(s2, __shfl_xor_sync(0xffffffffu, s2, o));
    const double scale2 = (double)s2;
    const double thresh = tol * tol * scale2;
    int mypiv = 0;  // lane k keeps piv[k]
    for (int k = 0; k < ne; ++k) {
      T bt = (T)-1;
      int bi = 0x7fffffff;
      if (lane >= k && lane < ne) {
        const T m = cnorm(F[lane + k * LD]);
        if (m > bt) { bt = m; bi = lane; }  // NaN is no candidate
      }
      warp_argmax(bt, bi);
      const double best = (double)bt;
      int p = bi;
      if (!(best > thresh) || p >= ne) {
        if (!perturb || !(best >= 0.0) || !(scale2 > 0.0) || p >= ne) {
          if (lane == 0) J.fail[t.front] = 1;
          return;
        }
        if (lane == 0) {
          V& d = F[p + k * LD];
          const double mag = sqrt(best), target = tol * sqrt(scale2);
          if (mag > 0.0) { d.x = (T)(d.x / mag * target); d.y = (T)(d.y / mag * target); }
          else { d.x = (T)target; d.y = (T)0; }
          if (perturbed) atomicAdd(perturbed + t.job, 1);
        }
        __syncwarp();
      }
      if (lane == k) mypiv = p;
      if (p != k && lane < n) {
        const V a = F[k + lane * LD];
        F[k + lane * LD] = F[p + lane * LD];
        F[p + lane * LD] = a;
      }
      __syncwarp();
      const V inv = cinv(F[k + k * LD]);
      if (lane < n) prow[lane] = (lane == k) ? inv : cmul(F[k + lane * LD], inv);
      __syncwarp();
      // Every lane runs the same loop: row i becomes row i - c_i prow with c_i its entry in column
      // k, which is cleared first so that column k receives -c_i / pivot (prow[k] = 1 / pivot).
      // Row k, the pivot row, is then overwritten with prow by the lanes of its columns.
      if (lane < n) {
        const V ck = F[lane + k * LD];
        F[lane + k * LD] = cx<V>(0.0, 0.0);
#pragma unroll 4
        for (int j = 0; j < n; ++j) F[lane + j * LD] = cfms(F[lane + j * LD], ck, prow[j]);
      }
      __syncwarp();
      if (lane < n) F[k + lane * LD] = prow[lane];
      __syncwarp();
    }
    // Undo the interchanges on the columns, last first (lane i moves its own row's entries).
    for (int k = ne - 1; k >= 0; --k) {
      const int p = __shfl_sync(0xffffffffu, mypiv, k);
      if (p != k && lane < n) {
        const V a = F[lane + k * LD];
        F[lane + k * LD] = F[lane + p * LD];
        F[lane + p * LD] = a;
      }
    }
    __syncwarp();
  }
  if (lane < n)
    for (int j = 0; j < n; ++j) {
      if (ne > 0 && !KEEP && (lane < ne || j < ne)) continue;
      out[lane + (int64_t)j * n] = F[lane + j * LD];
    }
}

}  // namespace caroli
