// Mixed precision: FP64 iterative refinement of the whole block solve, preconditioned by the
// complex-f32 multifrontal factors kept in the arena.
//
// For one block with A = z - H - Σ_L - Σ_R, the right-hand side is B = e_R W_R, where W_R W_R^† =
// Γ_R (a rank-revealing factor of the right lead's broadening, one column per channel). Then
// X = A^-1 B holds G W_R on every orbital, and T = Tr[Γ_L G_LR Γ_R G_LR^†] = Σ_j x_Lj^† Γ_L x_Lj,
// the Caroli trace of caroli-green/src/lib.rs:106-113 rewritten with Γ_R = W_R W_R^†.
//
// Each iteration: D = M^-1 R (f32 forward and backward sweeps through the tree and the f32 root
// inverse), X += D, R = B - A X with H, Σ in FP64 (CSR of the block), T and the correction norm
// in FP64. A front's factors are [F11^-1 | X; W | S] with W = -F21 F11^-1 (see kernels.cuh):
//   forward  z = own r + Σ_children h_c,  t = F11^-1 z_e,  h = z_b + W z_e  (handed to the parent)
//   root     x = F_root^-1 z
//   backward x_e = t - X x_b
#pragma once
#include "kernels.cuh"

namespace caroli {

struct RefineDesc {
  const FrontDesc* fronts;
  const int32_t* maps;
  const uint8_t* own;
  const int32_t* vidx;
  const SweepRow* srows;  // per front row: where the sweeps find its right-hand side
  const float2* arena;  // f32 factors
  const float2* root;   // f32 root inverse (m x m)
  const int32_t* csr_ptr;
  const int32_t* csr_col;
  const int64_t* csr_q;
  const double2* vals;
  const int32_t* slice_l;  // per block-local row: position in the left slice, or -1
  const int32_t* slice_r;
  const int32_t* left_local;
  const int32_t* right_local;
  const double2* sigma_l;
  const double2* sigma_r;
  const double2* gamma_l;
  const double2* w_r;  // nr x c, column-major
  double energy;
  int32_t nblk, nl, nr, c, root_front;
  int64_t sum_ne, sum_nb;
  double2* x;  // nblk x c
  double2* r;  // nblk x c
  float2* d;   // nblk x c
  float2* tb;  // sum_ne x c
  float2* hb;  // sum_nb x c
  double t_prev, t_cur, corr, err;
  int32_t done, iters, stalled, pad;
  // GMRES (right-preconditioned by the f32 factors) for the correction of each outer step.
  double2* V;   // (m + 1) Arnoldi vectors, each nblk x c
  float2* Z;    // m preconditioned vectors M^-1 V_k, each nblk x c
  double2* H;   // per column: (m + 1) x m Hessenberg, column-major
  double2* g;   // per column: m + 1 (rotated right-hand side)
  double* cs;   // per column: m cosines of the Givens rotations
  double2* sn;  // per column: m sines
  double2* y;   // per column: m solution coefficients
  double* beta; // per column: |r_j|
  int32_t* col_done;  // per column: the inner solve converged (or the column is empty)
  int32_t inner, inner_done;  // Arnoldi steps of the current outer step; all columns converged
  int32_t steps;              // preconditioner applications (Arnoldi steps) over all outer steps
  double inner_res;            // largest relative residual the last inner solve reached
  // The adjoint solve A^† z = b (gradient): Σ -> Σ^†, the root inverse conjugate-transposed, an
  // explicit right-hand side `rhs` (nblk x c), and convergence on the whole vector.
  const double2* rhs;
  int32_t adjoint;
  // Convergence on the whole vector instead of T (adjoint solves, scattering states).
  int32_t whole;
  // Scattering states: the first `cl` columns are sourced by W_L (nl x cl, column-major) on the
  // left slice, the others by W_R on the right slice; cl = 0 for a transmission.
  const double2* w_l;
  int32_t cl, pad2;
  // Γ_L x_L of the current x (nl x c, column-major), formed by slice_gemm_kernel for the check.
  double2* gx;
};

constexpr int GM_M = 12;  // Arnoldi steps per outer step

__device__ __forceinline__ float2 f2(double2 v) { return make_float2((float)v.x, (float)v.y); }

// Right-hand side B[i, j]: the explicit one, else W_L on the left slice (columns below cl) and
// W_R on the right slice.
__device__ __forceinline__ double2 rhs_at(const RefineDesc& R, int i, int j) {
  if (R.rhs) return R.rhs[i + (int64_t)j * R.nblk];
  if (j < R.cl) {
    const int li = R.slice_l[i];
    return li >= 0 ? R.w_l[li + (int64_t)j * R.nl] : make_double2(0.0, 0.0);
  }
  const int ri = R.slice_r[i];
  return ri >= 0 ? R.w_r[ri + (int64_t)(j - R.cl) * R.nr] : make_double2(0.0, 0.0);
}

// Forward sweep of the fronts of one level: grid (tasks, column chunks).
// The sweeps solve M d = v for v = the residual (src < 0) or the Arnoldi vector V_src, and write
// d to R.d (dst < 0) or to Z_dst.
__device__ __forceinline__ const double2* sweep_src(const RefineDesc& R, int src) {
  return src < 0 ? R.r : R.V + (int64_t)src * R.nblk * R.c;
}
__device__ __forceinline__ float2* sweep_dst(const RefineDesc& R, int dst) {
  return dst < 0 ? R.d : R.Z + (int64_t)dst * R.nblk * R.c;
}

// x += d, then the FP64 residual r = B - A x of every row: grid (jobs, row chunks of 256). The
// residual kernel applies B - (z - H) x; the slices' Σ x follow as slice_gemm_kernel launches.
__global__ void __launch_bounds__(256) refine_update_kernel(RefineDesc* __restrict__ rd) {
  RefineDesc& R = rd[blockIdx.x];
  if (R.done) return;
  const int i = blockIdx.y * 256 + threadIdx.x;
  if (i >= R.nblk) return;
  for (int j = 0; j < R.c; ++j) {
    const int64_t q = i + (int64_t)j * R.nblk;
    const float2 dv = R.d[q];
    R.x[q].x += (double)dv.x;
    R.x[q].y += (double)dv.y;
  }
}

__global__ void __launch_bounds__(256) refine_residual_kernel(RefineDesc* __restrict__ rd,
                                                              const int32_t* __restrict__ jl) {
  const RefineDesc& R = rd[jl[blockIdx.x]];
  if (R.done) return;
  const int i = blockIdx.y * 256 + threadIdx.x;
  if (i >= R.nblk) return;
  for (int j = 0; j < R.c; ++j) {
    const double2* xj = R.x + (int64_t)j * R.nblk;
    double2 acc = rhs_at(R, i, j);
    acc.x -= R.energy * xj[i].x;
    acc.y -= R.energy * xj[i].y;
    for (int q = R.csr_ptr[i]; q < R.csr_ptr[i + 1]; ++q) acc = cfma(acc, R.vals[R.csr_q[q]], xj[R.csr_col[q]]);
    R.r[i + (int64_t)j * R.nblk] = acc;  // + Σ_L x + Σ_R x on the slices: slice_gemm_kernel
  }
}

// T = Σ_j x_Lj^† Γ_L x_Lj and the relative size of the last correction on the left slice (the only
// rows T depends on); convergence decision. After a GMRES correction reaching inner relative
// residual rho, the remaining relative error of x_L is about corr * rho: converged when that is
// below `tol`; stalled when not finite, growing, or out of outer steps. Error estimate
// |T| * 2 * corr * rho.
__global__ void __launch_bounds__(256) refine_check_kernel(RefineDesc* __restrict__ rd, double tol, int max_iters,
                                                           double* __restrict__ t_out, double* __restrict__ err_out,
                                                           int32_t* __restrict__ done_out) {
  __shared__ double red[3][32];
  RefineDesc& R = rd[blockIdx.x];
  if (R.done) {
    if (threadIdx.x == 0) done_out[blockIdx.x] = R.stalled ? 2 : 1;
    return;
  }
  double tl = 0.0, dn = 0.0, xn = 0.0;
  if (R.whole)  // every orbital's value matters (dT/dV_a, ψ): the correction of the whole vector
    for (int64_t q = threadIdx.x; q < (int64_t)R.nblk * R.c; q += blockDim.x) {
      const float2 dv = R.d[q];
      const double2 xv = R.x[q];
      dn += (double)dv.x * dv.x + (double)dv.y * dv.y;
      xn += xv.x * xv.x + xv.y * xv.y;
    }
  for (int idx = threadIdx.x; idx < (R.whole ? 0 : R.nl * R.c); idx += blockDim.x) {
    const int a = idx % R.nl, j = idx / R.nl;
    const double2* xj = R.x + (int64_t)j * R.nblk;
    const int row = R.left_local[a];
    const double2 g = R.gx[a + (int64_t)j * R.nl];  // (Γ_L x_L)[a], from slice_gemm_kernel
    const double2 xa = xj[row];
    tl += xa.x * g.x + xa.y * g.y;
    const float2 dv = R.d[row + (int64_t)j * R.nblk];
    dn += (double)dv.x * dv.x + (double)dv.y * dv.y;
    xn += xa.x * xa.x + xa.y * xa.y;
  }
  double vals[3] = {tl, dn, xn};
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  for (int k = 0; k < 3; ++k) {
    double v = vals[k];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (l == 0) red[k][w] = v;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double sum[3] = {0.0, 0.0, 0.0};
    for (int k = 0; k < 3; ++k)
      for (int q = 0; q < (int)(blockDim.x >> 5); ++q) sum[k] += red[k][q];
    const double corr = sum[2] > 0.0 ? sqrt(sum[1] / sum[2]) : (sum[1] > 0.0 ? INFINITY : 0.0);
    const double prev = R.corr;
    R.iters += 1;
    R.t_prev = R.t_cur;
    R.t_cur = sum[0];
    const bool finite = isfinite(sum[0]) && isfinite(corr);
    // After a GMRES step the remaining error is about corr times the inner residual reached.
    const double rho = R.inner_res;
    const bool conv = finite && (corr == 0.0 || corr * rho <= tol);
    const bool stall = !finite || (!conv && R.iters >= max_iters) || (R.iters > 2 && corr > prev);
    R.corr = corr;
    R.err = fabs(sum[0]) * 2.0 * corr * rho;
    if (conv || stall) {
      R.done = 1;
      R.stalled = stall && !conv;
    }
    t_out[blockIdx.x] = sum[0];
    err_out[blockIdx.x] = R.err;
    done_out[blockIdx.x] = R.done ? (R.stalled ? 2 : 1) : 0;
  }
}

// Gives up the solves still iterating: marked stalled, they are recomputed in FP64 (a batch's
// last few slow solves, see refine in the engine).
__global__ void refine_giveup_kernel(RefineDesc* __restrict__ rd, int njobs) {
  const int job = blockIdx.x * blockDim.x + threadIdx.x;
  if (job >= njobs) return;
  RefineDesc& R = rd[job];
  if (R.done) return;
  R.done = 1;
  R.stalled = 1;
}

__global__ void refine_init_kernel(RefineDesc* __restrict__ rd, int njobs) {
  const int job = blockIdx.y;
  if (job >= njobs) return;
  RefineDesc& R = rd[job];
  const int64_t total = (int64_t)R.nblk * R.c;
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < total; q += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(q % R.nblk), j = (int)(q / R.nblk);
    R.x[q] = make_double2(0.0, 0.0);
    R.r[q] = rhs_at(R, i, j);
  }
}

}  // namespace caroli

namespace caroli {

// ---- GMRES for the correction of an outer step ---------------------------------------------------
// Right preconditioning: A M^-1 u = r, d = M^-1 (V y) = Z y. Arnoldi vectors in FP64, classical
// Gram-Schmidt (one pass), complex Givens rotations (c real), per right-hand-side column.

__device__ __forceinline__ double block_sum(double v, double* red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = (blockDim.x + 31) >> 5;
  __syncthreads();
  if (l == 0) red[w] = v;
  __syncthreads();
  if (w == 0) {
    v = l < nw ? red[l] : 0.0;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (l == 0) red[0] = v;
  }
  __syncthreads();
  const double r = red[0];
  __syncthreads();
  return r;
}

__device__ __forceinline__ double2 cconj_mul(double2 a, double2 b) {  // conj(a) b
  return make_double2(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x);
}

// The GMRES kernels run over a list of jobs `jl` (the solves still iterating, compacted on the
// device): grid x indexes the list, so finished solves cost no blocks.

// beta_j = |r_j|, V_0 = r / beta, g = (beta, 0, ...). grid (jobs, columns).
__global__ void __launch_bounds__(256) gm_start_kernel(RefineDesc* __restrict__ rd, const int32_t* __restrict__ jl) {
  __shared__ double red[32];
  RefineDesc& R = rd[jl[blockIdx.x]];
  const int j = blockIdx.y;
  if (R.done || j >= R.c) return;
  const double2* r = R.r + (int64_t)j * R.nblk;
  double ss = 0.0;
  for (int i = threadIdx.x; i < R.nblk; i += blockDim.x) ss += r[i].x * r[i].x + r[i].y * r[i].y;
  const double beta = sqrt(block_sum(ss, red));
  const double inv = beta > 0.0 ? 1.0 / beta : 0.0;
  double2* v0 = R.V + (int64_t)j * R.nblk;
  for (int i = threadIdx.x; i < R.nblk; i += blockDim.x) v0[i] = make_double2(r[i].x * inv, r[i].y * inv);
  if (threadIdx.x == 0) {
    R.beta[j] = beta;
    R.col_done[j] = beta > 0.0 ? 0 : -1;
    double2* g = R.g + (int64_t)j * (GM_M + 1);
    for (int i = 0; i <= GM_M; ++i) g[i] = make_double2(i == 0 ? beta : 0.0, 0.0);
    if (j == 0) {
      R.inner = 0;
      R.inner_done = 0;
    }
  }
}

// w = A z_k into V_{k+1}, A = z - H - Σ_L - Σ_R in FP64: z - H here, grid (jobs, row chunks of
// 256); the dense Σ blocks of the slices follow as slice_gemm_kernel launches.
__global__ void __launch_bounds__(256) gm_matvec_kernel(RefineDesc* __restrict__ rd, const int32_t* __restrict__ jl,
                                                        int k) {
  const RefineDesc& R = rd[jl[blockIdx.x]];
  if (R.done || R.inner_done) return;
  const int i = blockIdx.y * 256 + threadIdx.x;
  if (i >= R.nblk) return;
  const float2* Zk = R.Z + (int64_t)k * R.nblk * R.c;
  double2* W = R.V + (int64_t)(k + 1) * R.nblk * R.c;
  for (int j = 0; j < R.c; ++j) {
    const float2* zj = Zk + (int64_t)j * R.nblk;
    auto zd = [&](int q) { return make_double2((double)zj[q].x, (double)zj[q].y); };
    double2 acc = zd(i);
    acc.x *= R.energy;
    acc.y *= R.energy;
    for (int q = R.csr_ptr[i]; q < R.csr_ptr[i + 1]; ++q) acc = cfms(acc, R.vals[R.csr_q[q]], zd(R.csr_col[q]));
    W[i + (int64_t)j * R.nblk] = acc;  // - Σ_L z - Σ_R z on the slices: slice_gemm_kernel
  }
}

// Gram-Schmidt coefficients c_i = V_i^† w (i <= k) into y (pass 0 stores them in H, pass 1 adds).
// grid (jobs, columns, k + 1).
__global__ void __launch_bounds__(256) gm_dot_kernel(RefineDesc* __restrict__ rd, const int32_t* __restrict__ jl,
                                                     int k, int pass) {
  __shared__ double red[32];
  RefineDesc& R = rd[jl[blockIdx.x]];
  const int j = blockIdx.y, i = blockIdx.z;
  if (R.done || R.inner_done || j >= R.c || R.col_done[j] != 0) return;
  const double2* v = R.V + (int64_t)i * R.nblk * R.c + (int64_t)j * R.nblk;
  const double2* w = R.V + (int64_t)(k + 1) * R.nblk * R.c + (int64_t)j * R.nblk;
  double re = 0.0, im = 0.0;
  for (int q = threadIdx.x; q < R.nblk; q += blockDim.x) {
    const double2 p = cconj_mul(v[q], w[q]);
    re += p.x;
    im += p.y;
  }
  re = block_sum(re, red);
  im = block_sum(im, red);
  if (threadIdx.x == 0) {
    R.y[(int64_t)j * GM_M + i] = make_double2(re, im);
    double2* h = R.H + (int64_t)j * (GM_M + 1) * GM_M + i + (int64_t)k * (GM_M + 1);
    if (pass == 0) *h = make_double2(re, im);
    else { h->x += re; h->y += im; }
  }
}

// w -= Σ_i c_i V_i. grid (jobs, row chunks).
__global__ void __launch_bounds__(256) gm_axpy_kernel(RefineDesc* __restrict__ rd, const int32_t* __restrict__ jl,
                                                      int k) {
  const RefineDesc& R = rd[jl[blockIdx.x]];
  if (R.done || R.inner_done) return;
  const int q = blockIdx.y * 256 + threadIdx.x;
  if (q >= R.nblk) return;
  for (int j = 0; j < R.c; ++j) {
    if (R.col_done[j] != 0) continue;
    double2* w = R.V + (int64_t)(k + 1) * R.nblk * R.c + (int64_t)j * R.nblk;
    double2 acc = w[q];
    for (int i = 0; i <= k; ++i)
      acc = cfms(acc, R.y[(int64_t)j * GM_M + i], R.V[(int64_t)i * R.nblk * R.c + (int64_t)j * R.nblk + q]);
    w[q] = acc;
  }
}

// h_{k+1,k} = |w|, V_{k+1} = w / |w|, then the Givens rotations of column k and the residual
// estimate |g_{k+1}|; a column converges when it is below tol * beta. grid (jobs, columns).
__global__ void __launch_bounds__(256) gm_norm_kernel(RefineDesc* __restrict__ rd, const int32_t* __restrict__ jl,
                                                      int k, double tol) {
  __shared__ double red[32];
  RefineDesc& R = rd[jl[blockIdx.x]];
  const int j = blockIdx.y;
  if (R.done || R.inner_done || j >= R.c || R.col_done[j] != 0) return;
  double2* w = R.V + (int64_t)(k + 1) * R.nblk * R.c + (int64_t)j * R.nblk;
  double ss = 0.0;
  for (int q = threadIdx.x; q < R.nblk; q += blockDim.x) ss += w[q].x * w[q].x + w[q].y * w[q].y;
  const double nrm = sqrt(block_sum(ss, red));
  const double inv = nrm > 0.0 ? 1.0 / nrm : 0.0;
  for (int q = threadIdx.x; q < R.nblk; q += blockDim.x) w[q] = make_double2(w[q].x * inv, w[q].y * inv);
  if (threadIdx.x != 0) return;
  double2* H = R.H + (int64_t)j * (GM_M + 1) * GM_M + (int64_t)k * (GM_M + 1);
  double2* g = R.g + (int64_t)j * (GM_M + 1);
  double* cs = R.cs + (int64_t)j * GM_M;
  double2* sn = R.sn + (int64_t)j * GM_M;
  H[k + 1] = make_double2(nrm, 0.0);
  for (int i = 0; i < k; ++i) {
    // [h_i; h_{i+1}] <- [c s; -conj(s) c] [h_i; h_{i+1}]
    const double2 a = H[i], b = H[i + 1];
    const double2 sb = cmul(sn[i], b);
    const double2 sa = cconj_mul(sn[i], a);
    H[i] = make_double2(cs[i] * a.x + sb.x, cs[i] * a.y + sb.y);
    H[i + 1] = make_double2(cs[i] * b.x - sa.x, cs[i] * b.y - sa.y);
  }
  const double2 a = H[k], b = H[k + 1];
  const double na = sqrt(a.x * a.x + a.y * a.y), nb = sqrt(b.x * b.x + b.y * b.y);
  const double r = sqrt(na * na + nb * nb);
  double c;
  double2 sv;
  if (r == 0.0) { c = 1.0; sv = make_double2(0.0, 0.0); }
  else if (na == 0.0) { c = 0.0; sv = make_double2(b.x / nb, -b.y / nb); }  // s = conj(b)/|b|
  else {
    c = na / r;
    // s = (a / |a|) conj(b) / r
    const double2 ua = make_double2(a.x / na, a.y / na);
    sv = cmul(ua, make_double2(b.x / r, -b.y / r));
  }
  cs[k] = c;
  sn[k] = sv;
  H[k] = make_double2(c * a.x + (cmul(sv, b)).x, c * a.y + (cmul(sv, b)).y);
  H[k + 1] = make_double2(0.0, 0.0);
  const double2 gk = g[k];
  g[k] = make_double2(c * gk.x, c * gk.y);
  const double2 t = cconj_mul(sv, gk);
  g[k + 1] = make_double2(-t.x, -t.y);
  const double res = sqrt(g[k + 1].x * g[k + 1].x + g[k + 1].y * g[k + 1].y);
  if (!(res > tol * R.beta[j]) || nrm == 0.0) R.col_done[j] = k + 1;
}

// After step k: a job's inner solve ends when every column converged or after GM_M steps.
__global__ void gm_inner_check_kernel(RefineDesc* __restrict__ rd, int njobs, int k, int32_t* __restrict__ flags) {
  const int job = blockIdx.x * blockDim.x + threadIdx.x;
  if (job >= njobs) return;
  RefineDesc& R = rd[job];
  if (R.done) { flags[job] = 1; return; }
  if (R.inner_done) { flags[job] = 1; return; }
  R.inner = k + 1;
  R.steps += 1;
  bool all = true;
  for (int j = 0; j < R.c; ++j) all &= R.col_done[j] != 0;
  if (all || k + 1 >= GM_M) R.inner_done = 1;
  flags[job] = R.inner_done;
}

// y = H^-1 g on each column's steps (back substitution on the rotated Hessenberg matrix).
__device__ __forceinline__ void gm_solve_column(RefineDesc& R, int j) {
  const int kc = R.col_done[j] > 0 ? R.col_done[j] : (R.col_done[j] < 0 ? 0 : R.inner);
  const double2* H = R.H + (int64_t)j * (GM_M + 1) * GM_M;
  const double2* g = R.g + (int64_t)j * (GM_M + 1);
  double2* y = R.y + (int64_t)j * GM_M;
  for (int i = kc - 1; i >= 0; --i) {
    double2 acc = g[i];
    for (int t = i + 1; t < kc; ++t) acc = cfms(acc, H[i + (int64_t)t * (GM_M + 1)], y[t]);
    const double2 d = H[i + (int64_t)i * (GM_M + 1)];
    const double dd = d.x * d.x + d.y * d.y;
    y[i] = dd > 0.0 ? make_double2((acc.x * d.x + acc.y * d.y) / dd, (acc.y * d.x - acc.x * d.y) / dd)
                    : make_double2(0.0, 0.0);
  }
  for (int t = kc; t < GM_M; ++t) y[t] = make_double2(0.0, 0.0);
}

// The coefficients of every column of the listed jobs: grid (jobs), a thread per column.
__global__ void gm_solve_kernel(RefineDesc* __restrict__ rd, const int32_t* __restrict__ jl) {
  RefineDesc& R = rd[jl[blockIdx.x]];
  if (R.done) return;
  for (int j = threadIdx.x; j < R.c; j += blockDim.x) gm_solve_column(R, j);
}

__global__ void __launch_bounds__(256) gm_update_kernel(RefineDesc* __restrict__ rd, const int32_t* __restrict__ jl) {
  const RefineDesc& R = rd[jl[blockIdx.x]];
  if (R.done) return;
  const int q = blockIdx.y * 256 + threadIdx.x;
  if (q >= R.nblk) return;
  const int steps = R.inner;  // Arnoldi vectors of this outer step (coefficients past them are 0)
  for (int j = 0; j < R.c; ++j) {
    // The coefficients first, then every preconditioned vector's element at once.
    double2 yv[GM_M];
    float2 zv[GM_M];
#pragma unroll
    for (int t = 0; t < GM_M; ++t) yv[t] = t < steps ? R.y[(int64_t)j * GM_M + t] : make_double2(0.0, 0.0);
#pragma unroll
    for (int t = 0; t < GM_M; ++t)
      zv[t] = t < steps ? R.Z[(int64_t)t * R.nblk * R.c + (int64_t)j * R.nblk + q] : make_float2(0.f, 0.f);
    double2 acc = make_double2(0.0, 0.0);
#pragma unroll
    for (int t = 0; t < GM_M; ++t) acc = cfma(acc, yv[t], make_double2((double)zv[t].x, (double)zv[t].y));
    const int64_t o = q + (int64_t)j * R.nblk;
    R.x[o].x += acc.x;
    R.x[o].y += acc.y;
    R.d[o] = make_float2((float)acc.x, (float)acc.y);
  }
}

// Largest relative inner residual of each job's last outer step.
__global__ void gm_residual_kernel(RefineDesc* __restrict__ rd, int njobs) {
  const int job = blockIdx.x * blockDim.x + threadIdx.x;
  if (job >= njobs) return;
  RefineDesc& R = rd[job];
  if (R.done) return;
  double worst = 0.0;
  for (int j = 0; j < R.c; ++j) {
    if (R.col_done[j] < 0) continue;
    const int k = R.col_done[j] > 0 ? R.col_done[j] : R.inner;
    const double2 gk = R.g[(int64_t)j * (GM_M + 1) + k];
    const double res = sqrt(gk.x * gk.x + gk.y * gk.y) / fmax(R.beta[j], 1e-300);
    worst = fmax(worst, res);
  }
  R.inner_res = worst;
}

}  // namespace caroli

namespace caroli {

// ---- Dense slice products --------------------------------------------------------------------
// The lead blocks of A (Σ_L, Σ_R: m x m, dense, on the slices' orbitals) and Γ_L of the trace,
// applied to the c right-hand-side columns of a job at once: for i < m, j < c,
//     out[orow[i] + j ldo] = (accumulate ? out : 0) + sign Σ_a S(i, a) in[irow[a] + j ldi],
// S(i, a) = S[i + a m], or conj(S[a + i m]) for the adjoint solve. A batched complex FP64 GEMM:
// 64 x 32 output tiles, K in steps of 16 staged in shared memory, a 4 x 2 complex tile per thread;
// with hundreds of channels (a 32 x 32-site lead) these products carry most of the refinement's
// FP64 work.
struct SliceTask {
  const RefineDesc* rd;  // skipped once the job is done (mode 0: or its inner solve is done)
  const double2* s;
  const int32_t* irow;   // rows of the input (block-local), m entries
  const int32_t* orow;   // rows of the output, m entries; null: row i
  const void* in;        // double2, or float2 with in_f32
  double2* out;
  int64_t ldi, ldo;
  int32_t m, c, adj, in_f32, mode, accumulate;
  double sign;
};

constexpr int SG_ROWS = 64, SG_COLS = 32, SG_K = 16;

// Both slice kernels take the tasks of the jobs in `jl` (a job's task is tasks[job]).
__global__ void __launch_bounds__(256) slice_gemm_kernel(const SliceTask* __restrict__ tasks,
                                                         const int32_t* __restrict__ jl) {
  __shared__ double2 As[SG_K][SG_ROWS];
  __shared__ double2 Bs[SG_K][SG_COLS];
  const SliceTask t = tasks[jl[blockIdx.z]];
  const RefineDesc& R = *t.rd;
  if (R.done || (t.mode == 0 && R.inner_done)) return;
  const int i0 = blockIdx.x * SG_ROWS, j0 = blockIdx.y * SG_COLS;
  if (i0 >= t.m || j0 >= t.c) return;
  const int tid = threadIdx.x, ti = tid & 15, tj = tid >> 4;
  // Three real products per complex one (the 3M form): p1 = Σ ar br, p2 = Σ ai bi,
  // p3 = Σ (ar + ai)(br + bi); the product is (p1 - p2, p3 - p1 - p2). A quarter fewer FP64
  // multiply-adds than the four-product form on a part bound by the FP64 pipe.
  double p1[4][2], p2[4][2], p3[4][2];
#pragma unroll
  for (int r = 0; r < 4; ++r)
#pragma unroll
    for (int q = 0; q < 2; ++q) p1[r][q] = p2[r][q] = p3[r][q] = 0.0;
  for (int k0 = 0; k0 < t.m; k0 += SG_K) {
    // S tile: rows i0.., columns k0.. (coalesced along the stored dimension).
    for (int e = tid; e < SG_ROWS * SG_K; e += 256) {
      int ii, kk;
      if (t.adj) { kk = e % SG_K; ii = e / SG_K; }
      else { ii = e % SG_ROWS; kk = e / SG_ROWS; }
      const int i = i0 + ii, k = k0 + kk;
      double2 v = make_double2(0.0, 0.0);
      if (i < t.m && k < t.m) {
        if (t.adj) { v = t.s[k + (int64_t)i * t.m]; v.y = -v.y; }
        else v = t.s[i + (int64_t)k * t.m];
      }
      As[kk][ii] = v;
    }
    // Input tile: rows irow[k0..], columns j0.. (coalesced along the rows).
    for (int e = tid; e < SG_K * SG_COLS; e += 256) {
      const int kk = e % SG_K, jj = e / SG_K;
      const int k = k0 + kk, j = j0 + jj;
      double2 v = make_double2(0.0, 0.0);
      if (k < t.m && j < t.c) {
        const int64_t q = t.irow[k] + (int64_t)j * t.ldi;
        if (t.in_f32) {
          const float2 f = static_cast<const float2*>(t.in)[q];
          v = make_double2((double)f.x, (double)f.y);
        } else {
          v = static_cast<const double2*>(t.in)[q];
        }
      }
      Bs[kk][jj] = v;
    }
    __syncthreads();
#pragma unroll 4
    for (int kk = 0; kk < SG_K; ++kk) {
      double2 a[4], b[2];
#pragma unroll
      for (int r = 0; r < 4; ++r) a[r] = As[kk][ti + 16 * r];
#pragma unroll
      for (int q = 0; q < 2; ++q) b[q] = Bs[kk][tj + 16 * q];
      double as[4], bs[2];
#pragma unroll
      for (int r = 0; r < 4; ++r) as[r] = a[r].x + a[r].y;
#pragma unroll
      for (int q = 0; q < 2; ++q) bs[q] = b[q].x + b[q].y;
#pragma unroll
      for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int q = 0; q < 2; ++q) {
          p1[r][q] = fma(a[r].x, b[q].x, p1[r][q]);
          p2[r][q] = fma(a[r].y, b[q].y, p2[r][q]);
          p3[r][q] = fma(as[r], bs[q], p3[r][q]);
        }
    }
    __syncthreads();
  }
  double2 acc[4][2];
#pragma unroll
  for (int r = 0; r < 4; ++r)
#pragma unroll
    for (int q = 0; q < 2; ++q) acc[r][q] = make_double2(p1[r][q] - p2[r][q], p3[r][q] - p1[r][q] - p2[r][q]);
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const int i = i0 + ti + 16 * r;
    if (i >= t.m) continue;
    const int64_t orow = t.orow ? t.orow[i] : i;
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const int j = j0 + tj + 16 * q;
      if (j >= t.c) continue;
      double2& o = t.out[orow + (int64_t)j * t.ldo];
      const double2 v = make_double2(t.sign * acc[r][q].x, t.sign * acc[r][q].y);
      if (t.accumulate) { o.x += v.x; o.y += v.y; }
      else o = v;
    }
  }
}

// The same products for jobs with few columns (at most CB, the ribbons' few channels): a thread per
// output row holding its CB sums, the input rows of a K step staged in shared memory. A 64 x 32
// tile would leave most of its columns empty there. grid (row chunks of 128, tasks), 128 threads.
template <int CB>
__global__ void __launch_bounds__(128) slice_rows_kernel(const SliceTask* __restrict__ tasks,
                                                         const int32_t* __restrict__ jl) {
  constexpr int KS = 64;
  __shared__ double2 Xs[KS][CB];
  const SliceTask t = tasks[jl[blockIdx.y]];
  const RefineDesc& R = *t.rd;
  if (R.done || (t.mode == 0 && R.inner_done)) return;
  const int i0 = blockIdx.x * 128;
  if (i0 >= t.m) return;
  const int i = i0 + threadIdx.x;
  double2 acc[CB];
#pragma unroll
  for (int j = 0; j < CB; ++j) acc[j] = make_double2(0.0, 0.0);
  for (int k0 = 0; k0 < t.m; k0 += KS) {
    for (int e = threadIdx.x; e < KS * CB; e += 128) {
      const int kk = e % KS, j = e / KS, k = k0 + kk;
      double2 v = make_double2(0.0, 0.0);
      if (k < t.m && j < t.c) {
        const int64_t q = t.irow[k] + (int64_t)j * t.ldi;
        if (t.in_f32) {
          const float2 f = static_cast<const float2*>(t.in)[q];
          v = make_double2((double)f.x, (double)f.y);
        } else {
          v = static_cast<const double2*>(t.in)[q];
        }
      }
      Xs[kk][j] = v;
    }
    __syncthreads();
    if (i < t.m) {
      const int k1 = min(KS, t.m - k0);
      for (int kk = 0; kk < k1; ++kk) {
        double2 a;
        if (t.adj) { a = t.s[(k0 + kk) + (int64_t)i * t.m]; a.y = -a.y; }
        else a = t.s[i + (int64_t)(k0 + kk) * t.m];
#pragma unroll
        for (int j = 0; j < CB; ++j) acc[j] = cfma(acc[j], a, Xs[kk][j]);
      }
    }
    __syncthreads();
  }
  if (i >= t.m) return;
  const int64_t orow = t.orow ? t.orow[i] : i;
#pragma unroll
  for (int j = 0; j < CB; ++j) {
    if (j >= t.c) break;
    double2& o = t.out[orow + (int64_t)j * t.ldo];
    const double2 v = make_double2(t.sign * acc[j].x, t.sign * acc[j].y);
    if (t.accumulate) { o.x += v.x; o.y += v.y; }
    else o = v;
  }
}

// Transmission matrix t = W_L^† x_L of each job after its refinement (x = G W_R): t is
// cl x c column-major, W_L nl x cl. grid (jobs), threads over the entries of t.
__global__ void tmatrix_kernel(const RefineDesc* __restrict__ rd, const double2* const* __restrict__ wl,
                               const int32_t* __restrict__ cls, double2* const* __restrict__ tout) {
  const RefineDesc& R = rd[blockIdx.x];
  const int cl = cls[blockIdx.x];
  const double2* W = wl[blockIdx.x];
  double2* T = tout[blockIdx.x];
  for (int idx = threadIdx.x; idx < cl * R.c; idx += blockDim.x) {
    const int a = idx % cl, c = idx / cl;
    double2 acc = make_double2(0.0, 0.0);
    for (int i = 0; i < R.nl; ++i) {
      const double2 w = W[i + (int64_t)a * R.nl];
      const double2 x = R.x[R.left_local[i] + (int64_t)c * R.nblk];
      acc.x += w.x * x.x + w.y * x.y;  // conj(w) x
      acc.y += w.x * x.y - w.y * x.x;
    }
    T[idx] = acc;
  }
}

// Multi-terminal transmissions from the refined solution: for lead p and column c of job j,
// out[p * c_j + c] = x_c(p)^† Γ_p x_c(p), x_c(p) the rows of lead p's orbitals (block-local rows
// left_local[lpos[...]]). T_pq sums these over the columns sourced by lead q. grid (jobs, P, c).
__global__ void __launch_bounds__(256) multi_quadratic_kernel(const RefineDesc* __restrict__ rd,
                                                              const MultiJob* __restrict__ mj) {
  __shared__ double red[32];
  const RefineDesc& R = rd[blockIdx.x];
  const MultiJob& J = mj[blockIdx.x];
  const int p = blockIdx.y, c = blockIdx.z;
  if (p >= J.P || c >= R.c) return;
  const int np = J.lptr[p + 1] - J.lptr[p];
  const int32_t* pos = J.lpos + J.lptr[p];
  const double2* G = J.gamma[p];
  const double2* x = R.x + (int64_t)c * R.nblk;
  double local = 0.0;
  for (int a = threadIdx.x; a < np; a += blockDim.x) {
    double2 y = make_double2(0.0, 0.0);
    for (int b = 0; b < np; ++b) y = cfma(y, G[a + (int64_t)b * np], x[R.left_local[pos[b]]]);
    const double2 xa = x[R.left_local[pos[a]]];
    local += xa.x * y.x + xa.y * y.y;
  }
  for (int o = 16; o > 0; o >>= 1) local += __shfl_xor_sync(0xffffffffu, local, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) red[w] = local;
  __syncthreads();
  if (threadIdx.x == 0) {
    double sum = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) sum += red[k];
    J.out[p * R.c + c] = sum;
  }
}

// Multi-terminal sources: W_p (np x c, column-major) on the block-local rows of lead p's orbitals,
// rows[a] = left_local[pos[a]], into columns c0 .. c0 + c of B (nblk rows). grid: np x c elements.
__global__ void scatter_sources_kernel(double2* __restrict__ B, int nblk, int c0, const int32_t* __restrict__ left_local,
                                       const int32_t* __restrict__ pos, int np, const double2* __restrict__ W, int c) {
  const int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (idx >= (int64_t)np * c) return;
  const int a = (int)(idx % np), k = (int)(idx / np);
  const int row = left_local[pos[a]];
  const double2 w = W[idx];
  double2& dst = B[row + (int64_t)(c0 + k) * nblk];
  dst.x += w.x;
  dst.y += w.y;
}

// Right-hand side of the adjoint solve: Γ_L x_j on the left slice (x from the forward solve, Γ_L x
// from its last check).
// grid (jobs, row chunks).
__global__ void __launch_bounds__(256) grad_rhs_kernel(const RefineDesc* __restrict__ fwd, double2* const* rhs) {
  const RefineDesc& R = fwd[blockIdx.x];
  const int i = blockIdx.y * 256 + threadIdx.x;
  if (i >= R.nblk) return;
  const int li = R.slice_l[i];
  for (int j = 0; j < R.c; ++j) {
    // Γ_L x_L of the converged x: the last check's slice product (x does not change after it).
    const double2 acc = li >= 0 ? R.gx[li + (int64_t)j * R.nl] : make_double2(0.0, 0.0);
    rhs[blockIdx.x][i + (int64_t)j * R.nblk] = acc;
  }
}

// dT/dV_a = 2 Re Σ_j x_j[a] conj(z_j[a]) for every orbital a of the block.
__global__ void __launch_bounds__(256) grad_v_kernel(const RefineDesc* __restrict__ fwd, const RefineDesc* __restrict__ adj,
                                                     double* const* out) {
  const RefineDesc& X = fwd[blockIdx.x];
  const RefineDesc& Z = adj[blockIdx.x];
  const int i = blockIdx.y * 256 + threadIdx.x;
  if (i >= X.nblk) return;
  double s = 0.0;
  for (int j = 0; j < X.c; ++j) {
    const double2 x = X.x[i + (int64_t)j * X.nblk], z = Z.x[i + (int64_t)j * X.nblk];
    s += x.x * z.x + x.y * z.y;
  }
  out[blockIdx.x][i] = 2.0 * s;  // block-local order
}

// dT/dp = 2 Re Σ_j z_j^† (dH/dp) x_j for each parameter (dH given as values on the CSR pattern).
// grid (jobs, parameters); partial sums per CTA in `part`.
__global__ void __launch_bounds__(256) grad_p_kernel(const RefineDesc* __restrict__ fwd, const RefineDesc* __restrict__ adj,
                                                     const double2* const* dh, int64_t nnz, double* __restrict__ out,
                                                     int nparams) {
  __shared__ double red[32];
  const RefineDesc& X = fwd[blockIdx.x];
  const RefineDesc& Z = adj[blockIdx.x];
  const int k = blockIdx.y;
  const double2* d = dh[blockIdx.x] + (int64_t)k * nnz;
  double s = 0.0;
  for (int i = threadIdx.x; i < X.nblk; i += blockDim.x)
    for (int j = 0; j < X.c; ++j) {
      double2 hx = make_double2(0.0, 0.0);
      const double2* xj = X.x + (int64_t)j * X.nblk;
      for (int q = X.csr_ptr[i]; q < X.csr_ptr[i + 1]; ++q) hx = cfma(hx, d[X.csr_q[q]], xj[X.csr_col[q]]);
      const double2 z = Z.x[i + (int64_t)j * X.nblk];
      s += z.x * hx.x + z.y * hx.y;  // Re(conj(z) hx)
    }
  s = block_sum(s, red);
  if (threadIdx.x == 0) out[(int64_t)blockIdx.x * nparams + k] = 2.0 * s;
}

}  // namespace caroli
