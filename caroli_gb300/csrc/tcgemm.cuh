// Complex f32 GEMMs on the tcgen05 tensor cores: the refinement sweeps of solves with many
// right-hand-side columns, and the Schur complements of large fronts (schur_split in the engine).
//
// A solve whose right lead has hundreds of open channels (a 32 x 32-site cubic lead) carries one
// right-hand side per channel through every sweep, so each large front's sweep is a complex GEMM:
//   forward   [t; h - z_b] = [F11^-1; W] z_e        (n x ne times ne x c)
//   backward  x_e = t - X x_b                       (ne x nb times nb x c)
//   root      x = F_root^-1 z  (or its conjugate transpose for the adjoint)
// with the right-hand sides gathered into dense staging blocks first (gather kernels below); and
//   Schur     [X; S] = [F11^-1; W] F12 + [0; F22]    (n x ne times ne x nb, F12 staged aside)
// after the panel sweeps have formed the pivot columns [F11^-1; W]. The
// product runs as the real GEMM of the 2 x 2 expansion used by tc_update_kernel:
//     D = A' B'^T,  A'[2i][2k] = Re a, A'[2i][2k+1] = -Im a, A'[2i+1][2k] = Im a, A'[2i+1][2k+1] = Re a,
//                   B'[j][2k] = Re b[k, j], B'[j][2k+1] = Im b[k, j]
// (rows 2i, 2i+1 of D: real and imaginary parts of complex row i), both operands split into tf32
// hi + lo and D = lo hi + hi lo + hi hi accumulated in f32 in tensor memory (3xTF32, about the
// accuracy of an f32 product), K-major no-swizzle shared-memory operands (tc.cuh).
//
// A CTA computes a 64 x 64 complex tile of one task: K in chunks of 32 complex (64 real, 8 MMA
// slices), every warp stages the chunk's A' and B' (hi and lo) into shared memory from registers
// loaded one chunk ahead, one thread issues the 24 MMAs and commits them to an mbarrier that all
// threads wait on (bounded) before the next chunk reuses the buffers, while the next chunk's global
// loads are in flight; two CTAs per SM overlap each other's staging and MMAs. The
// epilogue reads the accumulator from tensor memory and writes C = add + sign A B, rows optionally
// scattered through the fronts' SweepRow table. A wait that runs out marks the solve stalled (the
// refinement then recomputes it in FP64) after the MMAs it issued have drained.
#pragma once
#include "sweep.cuh"
#include "tc.cuh"

namespace caroli {

constexpr int TG_ROWS = 64;                      // complex rows per tile (128 real rows: the MMA's M)
constexpr int TG_COLS = 64;                      // complex columns per tile (the MMA's N)
constexpr int TG_KC = 32;                        // complex K per chunk (64 real: 8 slices of 8)
constexpr int TG_A_BYTES = 2 * TG_ROWS * 2 * TG_KC * 4;  // one of A' hi / lo: 128 x 64 f32
constexpr int TG_B_BYTES = TG_COLS * 2 * TG_KC * 4;      // one of B' hi / lo: 64 x 64 f32
constexpr int TG_SMEM = 2 * TG_A_BYTES + 2 * TG_B_BYTES + 1024;
constexpr int TG_THREADS = 256;
constexpr int TG_MIN_COLS = 32;                  // jobs with at least this many columns use these sweeps

struct TGTask {
  const RefineDesc* rd;   // skipped once the solve is done (or, in an Arnoldi sweep, its GMRES is)
  const float2* a;        // A: m x k, column-major a[i + k lda] (adj: conj(a[k + i lda]))
  const float2* b;        // B: k x n, column-major b[k + j ldb]
  const float2* add;      // addend, m x n column-major (ldadd), or null
  float2* c;              // C: m x n column-major (ldc); null: the sweep's destination vector
  const SweepRow* crow;   // output row r goes to row crow[r].var of C (null: row r)
  int64_t lda, ldb, ldadd, ldc;
  int32_t m, n, k, adj;
  float sign;
  int32_t job;            // without rd (a factorization product): the solve whose status a timeout sets
  int32_t* status;
};

// grid (column tiles, row tiles, tasks), TG_THREADS threads, TG_SMEM dynamic shared memory.
__global__ void __launch_bounds__(TG_THREADS, 2) tc_sweep_gemm_kernel(const TGTask* __restrict__ tasks, int src,
                                                                   int dst, uint32_t wait_limit) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ uint32_t tslot;
  __shared__ __align__(8) uint64_t mma_done;
  __shared__ int abort_flag;
  const TGTask t = tasks[blockIdx.z];
  RefineDesc* Rp = const_cast<RefineDesc*>(t.rd);
  if (Rp && sweep_idle(*Rp, src)) return;
  const int i0 = blockIdx.y * TG_ROWS, j0 = blockIdx.x * TG_COLS;
  if (i0 >= t.m || j0 >= t.n) return;
  const int tid = threadIdx.x, w = tid >> 5, lane = tid & 31;
  constexpr int M = 2 * TG_ROWS;
  unsigned char* base = reinterpret_cast<unsigned char*>(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  unsigned char* a_hi = base;
  unsigned char* a_lo = a_hi + TG_A_BYTES;
  unsigned char* b_hi = a_lo + TG_A_BYTES;
  unsigned char* b_lo = b_hi + TG_B_BYTES;
  if (w == 0) tc::tmem_alloc(&tslot, TG_COLS);
  if (tid == 0) {
    tc::mbar_init(&mma_done, 1);
    abort_flag = 0;
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tbase = tslot;
  const uint32_t idesc = tc::idesc_tf32(M, TG_COLS);
  const int chunks = (t.k + TG_KC - 1) / TG_KC;
  int issued = 0;  // chunks whose MMAs were committed
  // The raw operands of a chunk are loaded into registers one chunk ahead: the next chunk's global
  // loads are in flight while the current chunk's MMAs run.
  constexpr int AI = TG_ROWS * (TG_KC / 2) / TG_THREADS, BI = TG_COLS * (TG_KC / 2) / TG_THREADS;
  float2 ra[AI][2], rb[BI][2];
  auto a_item = [&](int q, int& i, int& c) {
    const int idx = tid + q * TG_THREADS;
    if (t.adj) { c = 2 * (idx % (TG_KC / 2)); i = idx / (TG_KC / 2); }
    else { i = idx % TG_ROWS; c = 2 * (idx / TG_ROWS); }
  };
  auto b_item = [&](int q, int& j, int& c) {
    const int idx = tid + q * TG_THREADS;
    c = 2 * (idx % (TG_KC / 2));
    j = idx / (TG_KC / 2);
  };
  auto load_chunk = [&](int k0) {
#pragma unroll
    for (int q = 0; q < AI; ++q) {
      int i, c;
      a_item(q, i, c);
      float2 p0 = make_float2(0.f, 0.f), p1 = make_float2(0.f, 0.f);
      const int gi = i0 + i, gk = k0 + c;
      if (gi < t.m) {
        if (t.adj) {
          if (gk < t.k) { p0 = t.a[gk + (int64_t)gi * t.lda]; p0.y = -p0.y; }
          if (gk + 1 < t.k) { p1 = t.a[gk + 1 + (int64_t)gi * t.lda]; p1.y = -p1.y; }
        } else {
          if (gk < t.k) p0 = t.a[gi + (int64_t)gk * t.lda];
          if (gk + 1 < t.k) p1 = t.a[gi + (int64_t)(gk + 1) * t.lda];
        }
      }
      ra[q][0] = p0;
      ra[q][1] = p1;
    }
#pragma unroll
    for (int q = 0; q < BI; ++q) {
      int j, c;
      b_item(q, j, c);
      const int gk = k0 + c, gj = j0 + j;
      float2 q0 = make_float2(0.f, 0.f), q1 = make_float2(0.f, 0.f);
      if (gj < t.n) {
        if (gk < t.k) q0 = t.b[gk + (int64_t)gj * t.ldb];
        if (gk + 1 < t.k) q1 = t.b[gk + 1 + (int64_t)gj * t.ldb];
      }
      rb[q][0] = q0;
      rb[q][1] = q1;
    }
  };
  if (chunks > 0) load_chunk(0);
  for (int ch = 0; ch < chunks; ++ch) {
    // A' (two complex columns per item, the 2 x 2 expansion) and B' of this chunk into shared memory.
#pragma unroll
    for (int q = 0; q < AI; ++q) {
      int i, c;
      a_item(q, i, c);
      const float2 p0 = ra[q][0], p1 = ra[q][1];
      const uint32_t o0 = tc::kmajor_offset(2 * i, 2 * c, M), o1 = tc::kmajor_offset(2 * i + 1, 2 * c, M);
      tc::store_split(a_hi + o0, a_lo + o0, make_float4(p0.x, -p0.y, p1.x, -p1.y));
      tc::store_split(a_hi + o1, a_lo + o1, make_float4(p0.y, p0.x, p1.y, p1.x));
    }
#pragma unroll
    for (int q = 0; q < BI; ++q) {
      int j, c;
      b_item(q, j, c);
      const uint32_t o = tc::kmajor_offset(j, 2 * c, TG_COLS);
      tc::store_split(b_hi + o, b_lo + o, make_float4(rb[q][0].x, rb[q][0].y, rb[q][1].x, rb[q][1].y));
    }
    tc::fence_smem_async();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (tid == 0) {
      for (int sl = 0; sl < 2 * TG_KC / 8; ++sl) {
        const uint64_t ah = tc::smem_desc(tc::smem_addr(a_hi + sl * M * 32), 128, 256);
        const uint64_t al = tc::smem_desc(tc::smem_addr(a_lo + sl * M * 32), 128, 256);
        const uint64_t bh = tc::smem_desc(tc::smem_addr(b_hi + sl * TG_COLS * 32), 128, 256);
        const uint64_t bl = tc::smem_desc(tc::smem_addr(b_lo + sl * TG_COLS * 32), 128, 256);
        tc::mma_tf32(tbase, al, bh, idesc, ch > 0 || sl > 0);
        tc::mma_tf32(tbase, ah, bl, idesc, true);
        tc::mma_tf32(tbase, ah, bh, idesc, true);
      }
      tc::mma_commit(&mma_done);
    }
    issued = ch + 1;
    if (ch + 1 < chunks) load_chunk((ch + 1) * TG_KC);
    // The chunk's MMAs must finish before the operands are overwritten (and before the epilogue).
    const bool ok = tc::mbar_wait(&mma_done, (uint32_t)(ch & 1), wait_limit);
    if (!__all_sync(0xffffffffu, ok) && lane == 0) abort_flag = 1;
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (abort_flag) break;
  }
  if (abort_flag) {
    // Let the issued MMAs drain (bounded) before tensor memory is freed, and send the solve to
    // the FP64 recomputation.
    if (issued > 0) tc::mbar_wait(&mma_done, (uint32_t)((issued - 1) & 1), TCU_WAIT);
    if (tid == 0) {
      if (Rp) {
        Rp->stalled = 1;
        Rp->done = 1;
      } else if (t.status) {
        t.status[t.job] = ST_TIMEOUT;
      }
    }
  } else {
    // Epilogue: warp w reads TMEM lane quarter w & 3 (real rows 32 (w & 3) + lane) and column half
    // w >> 2 (32 columns).
    const int q = w & 3, h = w >> 2;
    const int r2 = 32 * q + lane;
    const int gi = i0 + (r2 >> 1), part = r2 & 1;
    float v[32];
#pragma unroll
    for (int c0 = 0; c0 < 32; c0 += 16) {
      float p16[16];
      tc::tmem_ld16(tbase + ((uint32_t)(32 * q) << 16) + (uint32_t)(32 * h + c0), p16);
#pragma unroll
      for (int e = 0; e < 16; ++e) v[c0 + e] = chunks > 0 ? p16[e] : 0.f;  // k = 0: C = add
    }
    tc::tmem_ld_wait();
    if (gi < t.m) {
      float* cbase = reinterpret_cast<float*>(t.c ? t.c : sweep_dst(*Rp, dst));
      const int64_t orow = t.crow ? t.crow[gi].var : gi;
      const float* abase = reinterpret_cast<const float*>(t.add);
#pragma unroll
      for (int e = 0; e < 32; ++e) {
        const int gj = j0 + 32 * h + e;
        if (gj < t.n) {
          float val = t.sign * v[e];
          if (abase) val += abase[2 * (gi + (int64_t)gj * t.ldadd) + part];
          cbase[2 * (orow + (int64_t)gj * t.ldc) + part] = val;
        }
      }
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (w == 0) tc::tmem_dealloc(tbase, TG_COLS);
}

// Forward gather of one level: z (n x c, column-major, ld n) of every front, the rows' own
// right-hand side plus the children's hand-ups. grid (element chunks, tasks).
struct TGFront {
  const RefineDesc* rd;
  const FrontDesc* fd;
  float2* stage;  // n x c (forward: z; backward: x_b, nb x c)
};

__global__ void __launch_bounds__(256) tg_gather_fwd_kernel(const TGFront* __restrict__ fr, int src) {
  const TGFront g = fr[blockIdx.y];
  const RefineDesc& R = *g.rd;
  if (sweep_idle(R, src)) return;
  const FrontDesc& f = *g.fd;
  const double2* rin = sweep_src(R, src);
  const int64_t total = (int64_t)f.n * R.c;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int p = (int)(e % f.n), j = (int)(e / f.n);
    float2 z[1];
    load_z<1>(R, rin, R.srows[f.var_off + p], j, z);
    g.stage[e] = z[0];
  }
}

// Backward gather of one level: x_b (nb x c, ld nb) of every front from the solution so far.
__global__ void __launch_bounds__(256) tg_gather_bwd_kernel(const TGFront* __restrict__ fr, int src, int dst) {
  const TGFront g = fr[blockIdx.y];
  const RefineDesc& R = *g.rd;
  if (sweep_idle(R, src)) return;
  const FrontDesc& f = *g.fd;
  const int nb = f.n - f.ne;
  const float2* dout = sweep_dst(R, dst);
  const int64_t total = (int64_t)nb * R.c;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int p = (int)(e % nb), j = (int)(e / nb);
    g.stage[e] = dout[R.srows[f.var_off + f.ne + p].var + (int64_t)j * R.nblk];
  }
}

// F12 (the rows of the pivot block, columns ne..n) of every front of a list copied aside, column-
// major ne x nb: the B operand of the Schur GEMM, whose output X overwrites F12. grid (element
// chunks, fronts).
struct F12Copy {
  const float2* a;  // the front, column-major n x n
  float2* stage;    // ne x nb
  int32_t n, ne;
  const int32_t* bad;  // the front's pivot block was refused: nothing to form
};

__global__ void __launch_bounds__(256) f12_copy_kernel(const F12Copy* __restrict__ list) {
  const F12Copy g = list[blockIdx.y];
  if (g.bad && *g.bad) return;
  const int nb = g.n - g.ne;
  const int64_t total = (int64_t)g.ne * nb;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(e % g.ne), j = (int)(e / g.ne);
    g.stage[e] = g.a[i + (int64_t)(g.ne + j) * g.n];
  }
}

}  // namespace caroli
