// Context, device memory and batch execution of the nested-dissection transmission, and the C ABI
// declared in include/caroli_gb300.h.
//
// A batch is a list of solves ("jobs": one block of one (energy, configuration) instance). Each
// job owns an arena holding all its fronts. Fronts run level by level (children before parents)
// across every job of the batch: one launch per kernel per level, so thousands of small fronts
// of many solves share each launch. Jobs whose fronts refused a pivot are re-run with those
// fronts delayed to their parents (nested.rs:356-373), alone, until none refuses.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cmath>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <numeric>
#include <string>
#include <type_traits>
#include <vector>

#include "../../include/caroli_gb300.h"
#include "kernels.cuh"
#include "plan.hpp"
#include "refine.cuh"
#include "dense.cuh"
#include "tiny.cuh"
#include "sweep.cuh"
#include "disorder.cuh"
#include "leadsig.cuh"
#include "tcgemm.cuh"

using namespace caroli;

namespace {

constexpr double PIVOT_TOL_F64 = 1e-11;  // caroli-dense/src/field.rs:61
constexpr double PIVOT_TOL_F32 = 1e-5;   // caroli-dense/src/field.rs:111
constexpr int SMALL_MAX_F64 = 64;        // fronts up to this size run in one CTA's shared memory
constexpr int SMALL_MAX_F32 = 96;
constexpr int SMEM_LIMIT = 220 * 1024;   // dynamic shared memory a kernel may request
constexpr int MIXED_MAX_CHANNELS = 96;    // CAROLI_MIXED block solves with more channels run in FP64

struct CudaError {
  cudaError_t e;
  const char* what;
};
// A failed call's error is also taken out of the runtime's last-error slot (it is not sticky
// unless the context is lost), so that the next call's launch checks do not report it again.
#define CK(x)                                             \
  do {                                                    \
    cudaError_t _e = (x);                                 \
    if (_e != cudaSuccess) {                              \
      (void)cudaGetLastError();                           \
      throw CudaError{_e, #x};                            \
    }                                                     \
  } while (0)

template <typename T> T* dalloc(size_t count) {
  void* p = nullptr;
  if (count == 0) return nullptr;
  cudaError_t e = cudaMalloc(&p, count * sizeof(T));
  if (e != cudaSuccess) throw CudaError{e, "cudaMalloc"};
  return static_cast<T*>(p);
}

// Source of plan identities (never reused, unlike addresses of freed plans).
uint64_t g_plan_generation = 0;

// Device copy of a front plan.
struct DevPlan {
  FrontPlan host;
  uint64_t id = ++g_plan_generation;
  FrontDesc* fronts = nullptr;
  int32_t* maps = nullptr;
  uint8_t* own = nullptr;
  Entry* entries = nullptr;
  int32_t* vidx = nullptr;
  SweepRow* srows = nullptr;
  void upload(cudaStream_t s) {
    fronts = dalloc<FrontDesc>(host.fronts.size());
    vidx = dalloc<int32_t>(std::max<size_t>(1, host.vidx.size()));
    if (!host.vidx.empty())
      CK(cudaMemcpyAsync(vidx, host.vidx.data(), host.vidx.size() * sizeof(int32_t), cudaMemcpyHostToDevice, s));
    srows = dalloc<SweepRow>(std::max<size_t>(1, host.srows.size()));
    if (!host.srows.empty())
      CK(cudaMemcpyAsync(srows, host.srows.data(), host.srows.size() * sizeof(SweepRow), cudaMemcpyHostToDevice, s));
    maps = dalloc<int32_t>(std::max<size_t>(1, host.maps.size()));
    own = dalloc<uint8_t>(std::max<size_t>(1, host.own.size()));
    entries = dalloc<Entry>(std::max<size_t>(1, host.entries.size()));
    CK(cudaMemcpyAsync(fronts, host.fronts.data(), host.fronts.size() * sizeof(FrontDesc), cudaMemcpyHostToDevice, s));
    if (!host.maps.empty())
      CK(cudaMemcpyAsync(maps, host.maps.data(), host.maps.size() * sizeof(int32_t), cudaMemcpyHostToDevice, s));
    if (!host.own.empty())
      CK(cudaMemcpyAsync(own, host.own.data(), host.own.size(), cudaMemcpyHostToDevice, s));
    if (!host.entries.empty())
      CK(cudaMemcpyAsync(entries, host.entries.data(), host.entries.size() * sizeof(Entry), cudaMemcpyHostToDevice, s));
    CK(cudaStreamSynchronize(s));
  }
  void release() {
    cudaFree(fronts); cudaFree(maps); cudaFree(own); cudaFree(entries); cudaFree(vidx); cudaFree(srows);
    fronts = nullptr; maps = nullptr; own = nullptr; entries = nullptr; vidx = nullptr; srows = nullptr;
  }
};

struct SigmaSlot {
  double energy = 0.0;
  bool set = false;
  std::vector<double2*> sl, sr, gl, gr, wr;  // per block, device
  std::vector<int> channels;                // columns of W_R per block
  // Multi-terminal systems: Γ_p of every (block, lead), and per block a device table of the P
  // pointers.
  std::vector<double2*> mgam;
  std::vector<double2**> mtab;
  std::vector<double2*> mw;  // W_p with W_p W_p^† = Γ_p per (block, lead): sources of the mixed path
  std::vector<int> mch;      // its columns
};

// Block data the refinement needs (block-local CSR of H, slice positions).
struct DevBlock {
  int32_t nblk = 0;
  int64_t nnz = 0;
  int32_t *csr_ptr = nullptr, *csr_col = nullptr, *slice_l = nullptr, *slice_r = nullptr, *left_local = nullptr,
          *right_local = nullptr;
  int64_t* csr_q = nullptr;
  void release() {
    for (int32_t* p : {csr_ptr, csr_col, slice_l, slice_r, left_local, right_local}) cudaFree(p);
    cudaFree(csr_q);
  }
};

template <typename T> T* upload_vec(const std::vector<T>& v, cudaStream_t s) {
  T* d = dalloc<T>(std::max<size_t>(1, v.size()));
  if (!v.empty()) CK(cudaMemcpyAsync(d, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s));
  return d;
}

struct System {
  // Owned copies of the description.
  std::vector<int64_t> row_ptr, cells, site_offsets, site_orbitals, interior, left_ptr, left, right_ptr, right;
  std::vector<uint32_t> cols;
  std::vector<int32_t> labels;
  SystemDesc desc{};
  std::vector<BlockTree> trees;
  std::vector<std::unique_ptr<DevPlan>> plans;  // static plan per block
  std::vector<DevBlock> blocks;
  double2* vals = nullptr;
  size_t vals_count = 0;  // elements allocated at vals
  int nconfigs = 0;
  double2* dvals = nullptr;  // dH/dp of every configuration: [config][param][nnz]
  int nparams = 0;
  std::vector<SigmaSlot> slots;
  // Multi-terminal systems (nleads > 0): the kept orbitals of each block are its "left" list;
  // lead p of block b occupies the kept positions mpos[b][mptr[b][p] .. mptr[b][p + 1]).
  int nleads = 0;
  std::vector<std::vector<int32_t>> mptr, mpos;
  std::vector<int32_t*> dmptr, dmpos;
  // On-device disorder: the site of every stored entry inside an on-site block (-1 otherwise) and
  // its (row, column) within the block.
  int32_t* os_site = nullptr;
  int16_t* os_ab = nullptr;
  // Lead modes for self-energies on the device: per side (left, right) and block, the
  // eigenvectors Y of the lead cell (slice x slice) and s c.
  std::vector<double2*> lead_y[2];
  std::vector<double> lead_sc[2];
  ~System() {
    for (auto& p : plans) p->release();
    for (auto& b : blocks) b.release();
    cudaFree(vals);
    cudaFree(dvals);
    for (auto& s : slots) {
      for (auto* v : {&s.sl, &s.sr, &s.gl, &s.gr, &s.wr, &s.mgam, &s.mw})
        for (auto* p : *v) cudaFree(p);
      for (auto* p : s.mtab) cudaFree(p);
    }
    for (auto* p : dmptr) cudaFree(p);
    for (auto* p : dmpos) cudaFree(p);
    cudaFree(os_site);
    cudaFree(os_ab);
    for (auto& v : lead_y)
      for (auto* p : v) cudaFree(p);
  }
};

// Grow-only device buffer.
struct Buf {
  void* p = nullptr;
  size_t bytes = 0;
  void* get(size_t need) {
    if (need > bytes) {
      cudaFree(p);
      p = nullptr;
      bytes = 0;
      CK(cudaMalloc(&p, need));
      bytes = need;
    }
    return p;
  }
  void release() {
    cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
  // As get, but also gives back most of an allocation far larger than needed (a batch in another
  // precision left it), so that buffers grown by different batches do not add up.
  void* fit(size_t need) {
    if (bytes > 2 * need + (size_t(64) << 20)) release();
    return get(need);
  }
  ~Buf() { cudaFree(p); }
};

// Kernel classes for per-kernel accounting: launches, algorithmic flops and bytes (computed on
// the host from the task lists), and device time when the class is probed.
enum KClass { K_SMALL = 0, K_ASSEMBLE, K_PANEL, K_UPDATE, K_ROOT_ASM, K_ROOT_INV, K_TRACE,
              K_REF_FWD, K_REF_ROOT, K_REF_BWD, K_REF_RES, K_REF_CHECK, K_REF_GMRES, K_COUNT };
const char* const kclass_names[K_COUNT] = {"small_front", "assemble", "large_front_panel", "large_front_update",
                                           "root_assemble", "root_inverse", "trace", "refine_forward",
                                           "refine_root", "refine_backward", "refine_residual", "refine_check",
                                           "refine_gmres"};
struct KStat {
  int64_t launches = 0;
  double flops = 0.0, bytes = 0.0, ms = 0.0;
};

// One block solve of a batch: the system it belongs to (a batch may mix systems), its block,
// energy slot, configuration and plan.
struct JobSpec {
  int block, slot, config;
  const DevPlan* plan;
  System* sys;
  int inst = -1;  // the caller's instance (sector transmissions)
};

// Sector transmissions of multi-terminal jobs: trace labels in place of the leads. Label k of a
// block sits at the positions of its lead (lptr/lpos per block, device and host copies); its Γ per
// (instance, block) in a device table of P pointers.
struct SectorRequest {
  int P = 0, nblocks = 0;
  std::vector<std::vector<int32_t>> hptr;
  std::vector<const int32_t*> lptr, lpos;       // per block
  std::vector<const double2* const*> gam;       // per (instance, block)
};

// Device state of one refinement (forward, or the adjoint of the gradient).
struct RefineBufs {
  Buf rdesc, rx, rr, rd, rtb, rhb, rt, rerr, rdone, rgx, stasks;
  Buf gV, gZ, gH, gg, gcs, gsn, gy, gbeta, gcol, gflags;
  Buf segs, ctasks, ccount, cjobs, ojobs;  // task and job lists compacted to the solves still iterating
  Buf tg_fr, tg_tasks, tg_stage;    // tensor-core sweeps of many-column solves (tcgemm.cuh)
  // The vectors (one column per channel; the bulk of a mixed batch's memory besides the fronts).
  void release_vectors() {
    for (Buf* b : {&rx, &rr, &rd, &rtb, &rhb, &rgx, &gV, &gZ, &tg_stage}) b->release();
  }
};

// A gradient request: d H / d p values of every configuration, and the per-job outputs.
struct GradRequest {
  const double2* dvals = nullptr;  // [config][param][nnz]
  int nparams = 0;
  int64_t nnz = 0;
};

// A scattering-states request: per job, the lead factors W_L (nl x cl) and W_R (nr x cr) on the
// device (column-major), and the host buffers of ψ (nblk x (cl + cr), block order).
struct StatesRequest {
  std::vector<const double2*> wl, wr;
  std::vector<int> cl, cr;
  std::vector<std::vector<double2>>* psi = nullptr;
  // Multi-terminal sources: an explicit right-hand side per job (nblk x (cl + cr)) instead of W_L, W_R.
  std::vector<const double2*> rhs;
  // Transmission matrices instead of ψ: t = W_L^† x_L with these W_L (nl x tcl, device) per job.
  std::vector<const double2*> twl;
  std::vector<int> tcl;
  // Multi-terminal transmissions instead of ψ: per job the leads' kept positions and Γ (MultiJob:
  // lpos, lptr, gamma, P); out receives x_c(p)^† Γ_p x_c(p) for every lead p and column c.
  std::vector<MultiJob> mtrace;
};

// One tree level of a batch: its fronts split by size class, and their algorithmic work.
struct TaskLevel {
  size_t tiny0 = 0, tiny_n = 0;
  size_t small0 = 0, small_n = 0, large0 = 0, large_n = 0;
  int max_small_n = 0, max_small_ne = 0, max_large_n = 0, max_large_ne = 0, max_n = 0;
  // Small fronts in size buckets (one launch each, shared memory sized to the bucket).
  size_t sb0[3] = {0, 0, 0}, sbn[3] = {0, 0, 0};
  int sb_n[3] = {0, 0, 0}, sb_ne[3] = {0, 0, 0};
  size_t inv0 = 0;
  double small_flops = 0, small_bytes = 0, inv_flops = 0, gemm0_flops = 0, gemm1_flops = 0, asm_bytes = 0;
  double tiny_flops = 0, tiny_bytes = 0;
  int max_tiny_n = 0;
  double upd_flops = 0, upd_bytes = 0;  // the rank-kb updates of the blocked sweep
  double pan_flops = 0;                 // its panel sweeps (kb steps over n rows of kb columns)
  // Split Schur update (f32 on the tensor cores): F12 copies and the [X; S] GEMM tasks of the level.
  size_t f12_0 = 0, f12_n = 0, sg0 = 0, sg_n = 0;
  int sg_max_m = 1, sg_max_cols = 1;
  double sg_flops = 0;
};

// The task lists of the last batch (see run_jobs).
struct TaskCache {
  bool valid = false;
  std::vector<uint64_t> plans;  // identities of the chunk's plans
  int tsize = 0, trsize = 0, max_levels = 0, small_max = 0;
  bool mixed = false, split = false;
  std::vector<F12Copy> f12;      // split Schur update: F12 copies, stage offsets (elements)
  std::vector<size_t> f12_off;
  std::vector<size_t> f12_inv;   // the InvTask (its bad flag) of each copy
  std::vector<TGTask> sgt;       // and the GEMM tasks (pointers into the arena and the stage)
  std::vector<std::pair<size_t, int>> sgt_stage;  // per task: copy index, 0 (X) or 1 (S)
  size_t f12_elems = 0;
  const void *f12_stage = nullptr, *f12_dev = nullptr, *sgt_dev = nullptr, *status_dev = nullptr;
  const void *arena = nullptr, *rarena = nullptr;
  std::vector<Task> tasks;
  std::vector<TaskLevel> levels;
  std::vector<InvTask> inv;
  std::vector<size_t> inv_piv_off, inv_y_off, inv_bt_off;
  size_t inv_piv = 0, inv_y = 0, inv_bt = 0, root0 = 0, rinv0 = 0;
  int max_root = 0;
  double root_flops = 0.0, trace_flops = 0.0;
  const void *piv = nullptr, *y = nullptr, *bt = nullptr, *scale = nullptr, *bad = nullptr, *dinv = nullptr,
             *dtasks = nullptr;
};

// The autotuner's choice for a plan set: the largest f32 front factored by one CTA in shared
// memory (fronts above it take the panel sweep and the rank-32 updates), whether those updates run
// on the tensor cores, whether the Schur complement of those fronts is one tensor-core GEMM after
// panels restricted to the pivot columns, and the factorization times the trials measured.
constexpr int TUNE_CANDIDATES = 9;
struct TuneChoice {
  int small_max = SMALL_MAX_F32;
  bool tensor_cores = true;
  bool split = false;
  bool tuned = false;
  // Per candidate: small_max 48 / 64 / 96 x (tensor cores with the split Schur GEMM, tensor cores
  // rank-32 updates only, CUDA cores).
  double ms[TUNE_CANDIDATES] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
};

// A captured factorization (every level's launches, the root assembly and inverse) and what it
// was captured with: a batch with the same key replays it with one graph launch.
struct FactorGraph {
  cudaGraphExec_t exec = nullptr;
  std::vector<uint64_t> key;
  std::vector<uint64_t> seen;  // the key of the previous batch: a key is captured on its second run
  int64_t launches = 0;
  KStat stats[K_COUNT];
  void reset() {
    if (exec) cudaGraphExecDestroy(exec);
    exec = nullptr;
    key.clear();
  }
};

}  // namespace

struct caroli_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr, evf = nullptr, evr = nullptr, reg0 = nullptr, reg1 = nullptr;
  int64_t region_launches = 0;
  KStat kstat[K_COUNT];
  int probe = -1;  // kernel class timed launch by launch (-1: none)
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> probe_events;
  size_t probe_used = 0;
  double factor_ms = 0.0, root_ms = 0.0, tail_ms = 0.0;
  std::string err;
  std::vector<std::unique_ptr<System>> systems;
  Buf arena, root_arena, jobs, tasks, fail, status, tout, part, pert;
  RefineBufs rb[2];  // forward and adjoint refinement state
  Buf inv, ipiv, iy, ibt, iscale, ibad;
  TaskCache tcache;
  Buf grhs, gptr, gdv, gdp;
  Buf states_w;  // lead factors W_L, W_R of a scattering-states call
  Buf states_rhs;  // multi-terminal sources
  Buf tm_out, tm_tab, tm_cls;  // transmission matrices
  const SectorRequest* sector = nullptr;  // set during caroli_multi_sector_transmissions
  // Set during caroli_root_green: the FP64 root Green's function on the kept orbitals of each
  // (instance, block) job, copied out after the root inverse.
  std::vector<std::vector<double2>>* green_out = nullptr;
  int green_blocks = 0;
  Buf sec_pos, sec_ptr, sec_gam, sec_tab;
  Buf mjobs, mscratch, mout;  // multi-terminal traces
  Buf dent, dspin, dscal, dcoef, dflag, dtab, dclean;  // on-device disorder
  Buf lead_d, lead_cols, lead_w;                       // self-energies from lead modes
  double inner_tol = 1e-10;
  bool tensor_cores = true;  // f32 rank-kb updates on tcgen05 (3xTF32); else on the CUDA cores
  int max_iters = 6;
  double refine_tol = 1e-10;
  double last_ms = 0.0;
  int64_t last_launches = 0;
  int64_t fallbacks = 0;
  int64_t refine_iters = 0;
  int64_t refine_job_steps = 0;    // Arnoldi steps summed over the solves
  int64_t refine_batch_steps = 0;  // Arnoldi steps launched for the batch (the slowest solve's)
  std::vector<int32_t> job_iters, job_perturbed, job_status, job_steps;
  std::vector<int32_t> steps_tmp;  // Arnoldi steps of each job of the last refinement
  size_t mem_budget = 0;
  int mixed_max_channels = MIXED_MAX_CHANNELS;  // CAROLI_MIXED block solves with more channels run in FP64
  uint32_t tc_wait_limit = TCU_WAIT;            // polls of a pipeline wait in tc_update_kernel
  unsigned char* noalloc_base = nullptr;        // device address of the allocation-free scratch array
  // Autotuner and graph replay (see run_jobs and tune_jobs).
  bool autotune = true;                         // pick the f32 factorization's schedule per plan set
  bool use_graphs = true;                       // replay a repeated batch's factorization as a CUDA graph
  int small_max_f32 = SMALL_MAX_F32;            // f32 fronts up to this size: one CTA each (else panel + update)
  bool tc_choice = true;                        // the autotuner's tensor-core choice (with tensor_cores set)
  bool split_choice = false;                    // f32 Schur complements as one tensor-core GEMM per front
  int fixed_small_max = SMALL_MAX_F32, fixed_mode = 1;  // the schedule without the autotuner
  int tg_min_cols = TG_MIN_COLS;  // batches with this many right-hand-side columns sweep on the tensor cores
  int small_threads = 512;        // threads of a CTA factoring a front of 64 to 96 variables
  Buf f12_stage, f12_list, sgt_list;            // its F12 copies and task lists
  bool factor_only = false;                     // run_jobs stops after the root inverse (tuning trials)
  std::map<std::vector<uint64_t>, TuneChoice> tuned;  // per plan set and precision
  TuneChoice last_tune;                               // the choice the last batch ran with
  FactorGraph fgraph;                                 // the factorization of the last repeated batch
  int64_t graph_replays = 0, graph_captures = 0;
  // Every entry point taking the context holds this for its whole call, so that threads sharing a
  // context are serialised (recursive: an entry point may reach another one's helpers).
  mutable std::recursive_mutex mu;
};

// Serialises the calls of threads sharing a context.
#define CTX_LOCK(ctx) \
  std::unique_lock<std::recursive_mutex> _ctx_lock = (ctx) ? std::unique_lock<std::recursive_mutex>((ctx)->mu) \
                                                           : std::unique_lock<std::recursive_mutex>()

namespace {

// Why the last caroli_ctx_create failed (caroli_last_error(NULL)).
std::string g_create_error = "no context";

int fail_with(caroli_ctx* ctx, int code, const std::string& msg) {
  if (ctx) ctx->err = msg;
  return code;
}

System* get_system(caroli_ctx* ctx, int id) {
  if (id < 0 || id >= (int)ctx->systems.size() || !ctx->systems[id]) return nullptr;
  return ctx->systems[id].get();
}

template <typename T> struct Prec {
  static constexpr double tol = sizeof(T) == 8 ? PIVOT_TOL_F64 : PIVOT_TOL_F32;
};

// Shared memory of a panel launch whose largest pivot count is pmax: the staged candidate rows
// when they fit under SMEM_LIMIT, else only the work vectors (the kernel then sweeps the panel in
// global memory); 0 when not even those fit.
size_t panel_smem(int pmax, size_t vbytes) {
  const int64_t staged = panel_staged_bytes(pmax, (int)vbytes), work = panel_work_bytes(pmax, (int)vbytes);
  if (staged <= SMEM_LIMIT) return (size_t)staged;
  return work <= SMEM_LIMIT ? (size_t)work : 0;
}

// Launches `fn(first, count)` over a task range in pieces of at most 65535 (grid y/z limit).
template <typename F> void in_pieces(size_t count, F fn) {
  for (size_t first = 0; first < count; first += 65535) fn(first, std::min<size_t>(65535, count - first));
}
template <typename F> void in_pieces_of(size_t count, size_t piece, F fn) {
  for (size_t first = 0; first < count; first += piece) fn(first, std::min<size_t>(piece, count - first));
}

struct LevelRange {
  size_t tiny0, tiny_n;  // fronts of at most TINY_MAX variables (one warp each)
  size_t mid0, mid_n;    // fronts of at most 96 variables (one warp each, three rows per lane)
  size_t first, count;   // the others
  int max_n;
  int max_ne;            // bound on the eliminated variables of the others
};

// FP64 iterative refinement of the jobs [begin, begin + cj) after their f32 factorization.
template <typename LaunchT>
RefineDesc* refine(caroli_ctx* ctx, System* sys, const std::vector<JobSpec>& specs, size_t begin, size_t cj,
                   const std::vector<LevelRange>& lr, int max_root, const Task* dtasks, const std::vector<JobDesc>& jd,
                   const float2* arena, const std::vector<size_t>& arena_off, const float2* rarena,
                   const std::vector<size_t>& root_off, LaunchT& launch, std::vector<double>& th,
                   std::vector<double>& eh, std::vector<int32_t>& sh, std::vector<int32_t>& ih, RefineBufs& rb,
                   int adjoint, const std::vector<const double2*>& rhs, const StatesRequest* states = nullptr,
                   bool allow_giveup = false) {
  cudaStream_t s = ctx->stream;
  std::vector<RefineDesc> rdh(cj);
  size_t xo = 0, to = 0, ho = 0;
  int cmax = 0, max_blk = 0;
  std::vector<size_t> xoffs(cj), toffs(cj), hoffs(cj), coffs(cj);
  size_t co = 0;
  double sweep_bytes = 0.0, resid_flops = 0.0;
  for (size_t j = 0; j < cj; ++j) {
    const JobSpec& sp = specs[begin + j];
    const FrontPlan& P = sp.plan->host;
    const DevBlock& B = sp.sys->blocks[sp.block];
    const int c = states ? states->cl[begin + j] + states->cr[begin + j] : sp.sys->slots[sp.slot].channels[sp.block];
    cmax = std::max(cmax, c);
    max_blk = std::max(max_blk, B.nblk);
    xoffs[j] = xo; xo += (size_t)B.nblk * c;
    coffs[j] = co; co += (size_t)c;
    toffs[j] = to; to += (size_t)P.sum_ne * c;
    hoffs[j] = ho; ho += (size_t)P.sum_nb * c;
    for (size_t k = 0; k + 1 < P.fronts.size(); ++k) {
      const double ne = P.fronts[k].ne, n = P.fronts[k].n;
      sweep_bytes += (ne * ne + 2 * ne * (n - ne)) * sizeof(float2);  // factors read per sweep pair
    }
    resid_flops += 8.0 * c * (double)B.nnz;  // the slices' dense Σ blocks: slice_products
  }
  double2* rx = static_cast<double2*>(rb.rx.get(std::max<size_t>(xo, 1) * sizeof(double2)));
  double2* rr = static_cast<double2*>(rb.rr.get(std::max<size_t>(xo, 1) * sizeof(double2)));
  float2* rdv = static_cast<float2*>(rb.rd.get(std::max<size_t>(xo, 1) * sizeof(float2)));
  float2* rtb = static_cast<float2*>(rb.rtb.get(std::max<size_t>(to, 1) * sizeof(float2)));
  float2* rhb = static_cast<float2*>(rb.rhb.get(std::max<size_t>(ho, 1) * sizeof(float2)));
  double* rt_out = static_cast<double*>(rb.rt.get(cj * sizeof(double)));
  double* rerr = static_cast<double*>(rb.rerr.get(cj * sizeof(double)));
  int32_t* rdone = static_cast<int32_t*>(rb.rdone.get(cj * sizeof(int32_t)));
  CK(cudaMemsetAsync(rt_out, 0, cj * sizeof(double), s));
  CK(cudaMemsetAsync(rerr, 0, cj * sizeof(double), s));
  const size_t M = GM_M;
  double2* gV = static_cast<double2*>(rb.gV.get(std::max<size_t>(xo, 1) * (M + 1) * sizeof(double2)));
  float2* gZ = static_cast<float2*>(rb.gZ.get(std::max<size_t>(xo, 1) * M * sizeof(float2)));
  double2* gH = static_cast<double2*>(rb.gH.get(std::max<size_t>(co, 1) * (M + 1) * M * sizeof(double2)));
  double2* gg = static_cast<double2*>(rb.gg.get(std::max<size_t>(co, 1) * (M + 1) * sizeof(double2)));
  double* gcs = static_cast<double*>(rb.gcs.get(std::max<size_t>(co, 1) * M * sizeof(double)));
  double2* gsn = static_cast<double2*>(rb.gsn.get(std::max<size_t>(co, 1) * M * sizeof(double2)));
  double2* gy = static_cast<double2*>(rb.gy.get(std::max<size_t>(co, 1) * M * sizeof(double2)));
  double* gbeta = static_cast<double*>(rb.gbeta.get(std::max<size_t>(co, 1) * sizeof(double)));
  int32_t* gcol = static_cast<int32_t*>(rb.gcol.get(std::max<size_t>(co, 1) * sizeof(int32_t)));
  int32_t* gflags = static_cast<int32_t*>(rb.gflags.get(cj * sizeof(int32_t)));
  std::vector<size_t> gxoffs(cj);
  size_t gxo = 0;
  for (size_t j = 0; j < cj; ++j) {
    const size_t cj_cols = (j + 1 < cj ? coffs[j + 1] : co) - coffs[j];
    gxoffs[j] = gxo;
    gxo += (size_t)specs[begin + j].plan->host.nl * cj_cols;
  }
  double2* rgx = static_cast<double2*>(rb.rgx.get(std::max<size_t>(gxo, 1) * sizeof(double2)));
  for (size_t j = 0; j < cj; ++j) {
    const JobSpec& sp = specs[begin + j];
    const DevPlan& P = *sp.plan;
    const DevBlock& B = sp.sys->blocks[sp.block];
    const SigmaSlot& sg = sp.sys->slots[sp.slot];
    RefineDesc& R = rdh[j];
    std::memset(&R, 0, sizeof(R));
    R.fronts = P.fronts; R.maps = P.maps; R.own = P.own; R.vidx = P.vidx; R.srows = P.srows;
    R.arena = arena + arena_off[j];
    R.root = rarena + root_off[j];
    R.csr_ptr = B.csr_ptr; R.csr_col = B.csr_col; R.csr_q = B.csr_q;
    R.vals = jd[j].vals;
    R.slice_l = B.slice_l; R.slice_r = B.slice_r; R.left_local = B.left_local; R.right_local = B.right_local;
    R.sigma_l = sg.sl[sp.block]; R.sigma_r = sg.sr[sp.block]; R.gamma_l = sg.gl[sp.block];
    R.w_r = sg.wr[sp.block];
    R.energy = sg.energy;
    R.nblk = B.nblk; R.nl = P.host.nl; R.nr = P.host.nr; R.c = sg.channels[sp.block]; R.root_front = P.host.root;
    R.sum_ne = P.host.sum_ne; R.sum_nb = P.host.sum_nb;
    R.x = rx + xoffs[j]; R.r = rr + xoffs[j]; R.d = rdv + xoffs[j];
    R.tb = rtb + toffs[j]; R.hb = rhb + hoffs[j];
    R.V = gV + xoffs[j] * (M + 1);
    R.Z = gZ + xoffs[j] * M;
    R.H = gH + coffs[j] * (M + 1) * M;
    R.g = gg + coffs[j] * (M + 1);
    R.cs = gcs + coffs[j] * M;
    R.sn = gsn + coffs[j] * M;
    R.y = gy + coffs[j] * M;
    R.beta = gbeta + coffs[j];
    R.col_done = gcol + coffs[j];
    R.adjoint = adjoint;
    R.whole = adjoint;
    R.rhs = adjoint ? rhs[j] : nullptr;
    if (states) {
      if (!states->rhs.empty()) {
        R.rhs = states->rhs[begin + j];
      } else {
        R.w_l = states->wl[begin + j];
        R.w_r = states->wr[begin + j];
      }
      R.cl = states->cl[begin + j];
      R.c = R.cl + states->cr[begin + j];
      R.whole = 1;
    }
    R.gx = rgx + gxoffs[j];
    R.done = R.c == 0 ? 1 : 0;  // no channel: T = 0
  }
  RefineDesc* drd = static_cast<RefineDesc*>(rb.rdesc.get(cj * sizeof(RefineDesc)));
  CK(cudaMemcpyAsync(drd, rdh.data(), cj * sizeof(RefineDesc), cudaMemcpyHostToDevice, s));
  // Dense slice products (Σ_L, Σ_R of A and Γ_L of the trace): one task per job and product,
  // built once. Matvec of step k: V_{k+1} -= Σ Z_k; residual: r += Σ x; check: gx = Γ_L x_L.
  // Left and right slices run as separate launches (they may share rows).
  const int nsides = 2;
  const size_t per_set = cj;  // tasks of one (product, side) set
  const size_t set_mv = 0, set_res = (size_t)GM_M * nsides, set_gam = set_res + nsides;
  const size_t nsets = set_gam + 1;
  std::vector<SliceTask> sth(nsets * per_set);
  int slice_m = 1;
  for (size_t j = 0; j < cj; ++j) {
    const RefineDesc& R = rdh[j];
    const RefineDesc* dR = drd + j;
    for (int side = 0; side < nsides; ++side) {
      const double2* sg = side == 0 ? R.sigma_l : R.sigma_r;
      const int m = side == 0 ? R.nl : R.nr;
      const int32_t* rows = side == 0 ? R.left_local : R.right_local;
      slice_m = std::max(slice_m, m);
      SliceTask base{};
      base.rd = dR; base.s = sg; base.irow = rows; base.orow = rows; base.ldi = base.ldo = R.nblk;
      base.m = (sg && m > 0) ? m : 0; base.c = R.c; base.adj = R.adjoint; base.accumulate = 1;
      for (int k = 0; k < GM_M; ++k) {
        SliceTask t = base;
        t.in = R.Z + (size_t)k * R.nblk * R.c; t.in_f32 = 1; t.out = R.V + (size_t)(k + 1) * R.nblk * R.c;
        t.mode = 0; t.sign = -1.0;
        sth[(set_mv + (size_t)k * nsides + side) * per_set + j] = t;
      }
      SliceTask t = base;
      t.in = R.x; t.in_f32 = 0; t.out = R.r; t.mode = 1; t.sign = 1.0;
      sth[(set_res + side) * per_set + j] = t;
    }
    SliceTask t{};
    t.rd = dR; t.s = R.gamma_l; t.irow = R.left_local; t.orow = nullptr; t.in = R.x; t.out = R.gx;
    t.ldi = R.nblk; t.ldo = R.nl; t.m = (R.gamma_l && !R.whole) ? R.nl : 0; t.c = R.c; t.mode = 1; t.sign = 1.0;
    sth[set_gam * per_set + j] = t;
  }
  SliceTask* dst_tasks = static_cast<SliceTask*>(rb.stasks.get(sth.size() * sizeof(SliceTask)));
  CK(cudaMemcpyAsync(dst_tasks, sth.data(), sth.size() * sizeof(SliceTask), cudaMemcpyHostToDevice, s));
  // Solves with many columns (TG_MIN_COLS or more channels) sweep their large fronts and the root
  // as tensor-core GEMMs (tcgemm.cuh): per level, the fronts' right-hand sides are gathered into a
  // staging block, then one GEMM task per output block. The lists hold every large front of every
  // such job; tasks of finished solves exit at once.
  const bool wide = cmax >= ctx->tg_min_cols;
  const int nlev_w = (int)lr.size();
  struct WideLevel { size_t fr0 = 0, nfr = 0, fw0 = 0, nfw = 0, bw0 = 0, nbw = 0; int max_m = 1; };
  std::vector<WideLevel> wl(nlev_w);
  TGFront* dtg_fr = nullptr;
  TGTask* dtg_tasks = nullptr;
  size_t root_fr0 = 0, root_nfr = 0, root_t0 = 0;
  int root_m = 1;
  if (wide) {
    const std::vector<Task>& htasks = ctx->tcache.tasks;
    std::vector<TGFront> frs;
    std::vector<TGTask> tgs;
    std::vector<size_t> stage_off_f, stage_off_b;  // per entry of frs (forward and backward stages)
    size_t stage_need = 1;
    // Fronts first (forward gathers, then backward gathers), then tasks (forward, backward, root).
        for (int L = 0; L < nlev_w; ++L) {
      size_t off = 0;
      WideLevel& W = wl[L];
      W.fr0 = frs.size();
      for (size_t q = lr[L].first; q < lr[L].first + lr[L].count; ++q) {
        const Task& tk = htasks[q];
        const RefineDesc& R = rdh[tk.job];
        if (R.c == 0) continue;
        const FrontDesc& f = specs[begin + tk.job].plan->host.fronts[tk.front];
        frs.push_back({drd + tk.job, tk.fd, nullptr});
        stage_off_f.push_back(off);
        off += (size_t)f.n * R.c;
        W.max_m = std::max(W.max_m, f.n);
      }
      W.nfr = frs.size() - W.fr0;
      stage_need = std::max(stage_need, off);
    }
    for (size_t j = 0; j < cj; ++j) {
      const RefineDesc& R = rdh[j];
      if (R.c == 0) continue;
      root_m = std::max(root_m, specs[begin + j].plan->host.fronts[R.root_front].n);
    }
    // Root gathers: one per wide job, stage m x c each.
    root_fr0 = frs.size();
    size_t roff = 0;
    for (size_t j = 0; j < cj; ++j) {
      const RefineDesc& R = rdh[j];
      if (R.c == 0) continue;
      const FrontPlan& P = specs[begin + j].plan->host;
      frs.push_back({drd + j, specs[begin + j].plan->fronts + P.root, nullptr});
      stage_off_f.push_back(roff);
      roff += (size_t)P.fronts[P.root].n * R.c;
    }
    root_nfr = frs.size() - root_fr0;
    stage_need = std::max(stage_need, roff);
    float2* stage = static_cast<float2*>(rb.tg_stage.get(stage_need * sizeof(float2)));
    for (size_t e = 0; e < frs.size(); ++e) frs[e].stage = stage + stage_off_f[e];
    for (int L = 0; L < nlev_w; ++L) {
      WideLevel& W = wl[L];
      W.fw0 = tgs.size();
      size_t e = W.fr0;
      for (size_t q = lr[L].first; q < lr[L].first + lr[L].count; ++q) {
        const Task& tk = htasks[q];
        const RefineDesc& R = rdh[tk.job];
        if (R.c == 0) continue;
        const FrontDesc& f = specs[begin + tk.job].plan->host.fronts[tk.front];
        const float2* F = R.arena + f.arena_off;
        const int ne = f.ne, nb = f.n - f.ne;
        TGTask a{};
        a.rd = drd + tk.job; a.b = frs[e].stage; a.ldb = f.n; a.n = R.c; a.k = ne; a.sign = 1.f;
        if (ne > 0) {  // t = F11^-1 z_e
          TGTask t1 = a;
          t1.a = F; t1.lda = f.n; t1.c = R.tb + f.toff; t1.ldc = R.sum_ne; t1.m = ne;
          tgs.push_back(t1);
        }
        if (nb > 0) {  // h = z_b + W z_e
          TGTask t2 = a;
          t2.a = F + ne; t2.lda = f.n; t2.add = frs[e].stage + ne; t2.ldadd = f.n;
          t2.c = R.hb + f.hoff; t2.ldc = R.sum_nb; t2.m = nb;
          tgs.push_back(t2);
        }
        ++e;
      }
      W.nfw = tgs.size() - W.fw0;
      W.bw0 = tgs.size();
      e = W.fr0;
      for (size_t q = lr[L].first; q < lr[L].first + lr[L].count; ++q) {
        const Task& tk = htasks[q];
        const RefineDesc& R = rdh[tk.job];
        if (R.c == 0) continue;
        const FrontDesc& f = specs[begin + tk.job].plan->host.fronts[tk.front];
        const int ne = f.ne, nb = f.n - f.ne;
        if (ne > 0) {  // x_e = t - X x_b (x_b staged with leading dimension nb)
          TGTask t3{};
          t3.rd = drd + tk.job; t3.a = R.arena + f.arena_off + (size_t)ne * f.n; t3.lda = f.n;
          t3.b = frs[e].stage; t3.ldb = std::max(nb, 1); t3.add = R.tb + f.toff; t3.ldadd = R.sum_ne;
          t3.c = nullptr; t3.crow = R.srows + f.var_off; t3.ldc = R.nblk; t3.m = ne; t3.n = R.c; t3.k = nb;
          t3.sign = -1.f;
          tgs.push_back(t3);
        }
        ++e;
      }
      W.nbw = tgs.size() - W.bw0;
    }
    root_t0 = tgs.size();
    for (size_t e = root_fr0; e < root_fr0 + root_nfr; ++e) {
      const size_t j = (size_t)(frs[e].rd - drd);
      const RefineDesc& R = rdh[j];
      const FrontPlan& P = specs[begin + j].plan->host;
      const int m = P.fronts[P.root].n;
      TGTask t4{};
      t4.rd = drd + j; t4.a = R.root; t4.lda = m; t4.adj = R.adjoint; t4.b = frs[e].stage; t4.ldb = m;
      t4.c = nullptr; t4.crow = R.srows + P.fronts[P.root].var_off; t4.ldc = R.nblk; t4.m = m; t4.n = R.c; t4.k = m;
      t4.sign = 1.f;
      tgs.push_back(t4);
    }
    dtg_fr = static_cast<TGFront*>(rb.tg_fr.get(std::max<size_t>(frs.size(), 1) * sizeof(TGFront)));
    dtg_tasks = static_cast<TGTask*>(rb.tg_tasks.get(std::max<size_t>(tgs.size(), 1) * sizeof(TGTask)));
    if (!frs.empty()) CK(cudaMemcpyAsync(dtg_fr, frs.data(), frs.size() * sizeof(TGFront), cudaMemcpyHostToDevice, s));
    if (!tgs.empty()) CK(cudaMemcpyAsync(dtg_tasks, tgs.data(), tgs.size() * sizeof(TGTask), cudaMemcpyHostToDevice, s));
  }
  // GEMM launches of a task range: grid (column tiles, row tiles of the largest m, tasks).
  auto tg_gemm = [&](size_t t0, size_t nt, int max_m, int src, int dst, KClass cls) {
    const unsigned gx = (unsigned)((cmax + TG_COLS - 1) / TG_COLS), gy = (unsigned)((max_m + TG_ROWS - 1) / TG_ROWS);
    in_pieces(nt, [&](size_t f0, size_t c) {
      launch(cls, 0.0, 0.0, [&] {
        tc_sweep_gemm_kernel<<<dim3(gx, gy, (unsigned)c), TG_THREADS, TG_SMEM, s>>>(dtg_tasks + t0 + f0, src, dst,
                                                                                   ctx->tc_wait_limit);
      });
    });
  };
  auto tg_gather = [&](bool fwd, size_t f0r, size_t nf, int src, int dst, KClass cls) {
    in_pieces(nf, [&](size_t f0, size_t c) {
      launch(cls, 0.0, 0.0, [&] {
        if (fwd) tg_gather_fwd_kernel<<<dim3(64, (unsigned)c), 256, 0, s>>>(dtg_fr + f0r + f0, src);
        else tg_gather_bwd_kernel<<<dim3(64, (unsigned)c), 256, 0, s>>>(dtg_fr + f0r + f0, src, dst);
      });
    });
  };
  // Launches the slice products of one set for the `nl` jobs listed in `jl`; flops for the
  // accounting (the set's flops over all jobs, in proportion to the jobs listed).
  auto slice_products = [&](size_t set, KClass cls, const int32_t* jl, size_t nl) {
    double fl = 0.0;
    for (size_t j = 0; j < cj; ++j) fl += 8.0 * sth[set * per_set + j].m * (double)sth[set * per_set + j].m * sth[set * per_set + j].c;
    if (fl == 0.0 || nl == 0) return;
    const dim3 grid((unsigned)((slice_m + SG_ROWS - 1) / SG_ROWS), (unsigned)((std::max(1, cmax) + SG_COLS - 1) / SG_COLS));
    const unsigned rchunks = (unsigned)((slice_m + 127) / 128);
    in_pieces(nl, [&](size_t f0, size_t c) {
      launch(cls, fl * c / cj, 0.0, [&] {
        const SliceTask* tk = dst_tasks + set * per_set;
        if (cmax <= 1) slice_rows_kernel<1><<<dim3(rchunks, (unsigned)c), 128, 0, s>>>(tk, jl + f0);
        else if (cmax <= 2) slice_rows_kernel<2><<<dim3(rchunks, (unsigned)c), 128, 0, s>>>(tk, jl + f0);
        else if (cmax <= 4) slice_rows_kernel<4><<<dim3(rchunks, (unsigned)c), 128, 0, s>>>(tk, jl + f0);
        else if (cmax <= 8) slice_rows_kernel<8><<<dim3(rchunks, (unsigned)c), 128, 0, s>>>(tk, jl + f0);
        else slice_gemm_kernel<<<dim3(grid.x, grid.y, (unsigned)c), 256, 0, s>>>(tk, jl + f0);
      });
    });
  };
  // Right-hand-side columns per CTA: the batch's largest channel count, rounded up to 1, 2, 4, 8.
  const int cbw = cmax <= 1 ? 1 : cmax <= 2 ? 2 : cmax <= 4 ? 4 : 8;
  const unsigned cchunks = (unsigned)std::max(1, (cmax + cbw - 1) / cbw);
  in_pieces(cj, [&](size_t f0, size_t c) {
    launch(K_REF_RES, 0.0, 0.0, [&] { refine_init_kernel<<<dim3(16, (unsigned)c), 256, 0, s>>>(drd + f0, (int)c); });
  });
  std::vector<int32_t> dh(cj, 0);
  const int nlev = (int)lr.size();
  const unsigned rows = (unsigned)((max_blk + 255) / 256);
  const unsigned cols = (unsigned)std::max(1, cmax);
  // Task segments (per level: tiny fronts, then the others) and their compacted copies.
  const int nseg = 3 * nlev;
  std::vector<TaskSeg> segs(nseg);
  int64_t seg_max = 0;
  for (int L = 0; L < nlev; ++L) {
    segs[3 * L] = {(int64_t)lr[L].tiny0, (int64_t)lr[L].tiny_n};
    segs[3 * L + 1] = {(int64_t)lr[L].mid0, (int64_t)lr[L].mid_n};
    segs[3 * L + 2] = {(int64_t)lr[L].first, (int64_t)lr[L].count};
    seg_max = std::max<int64_t>(seg_max, std::max(std::max(lr[L].tiny_n, lr[L].mid_n), lr[L].count));
  }
  size_t ntask_all = 0;
  for (const auto& sg : segs) ntask_all = std::max<size_t>(ntask_all, (size_t)(sg.first + sg.count));
  TaskSeg* dsegs = static_cast<TaskSeg*>(rb.segs.get(nseg * sizeof(TaskSeg)));
  Task* ctasks = static_cast<Task*>(rb.ctasks.get(std::max<size_t>(ntask_all, 1) * sizeof(Task)));
  int32_t* ccount = static_cast<int32_t*>(rb.ccount.get((nseg + 1) * sizeof(int32_t)));
  int32_t* cjobs = static_cast<int32_t*>(rb.cjobs.get(cj * sizeof(int32_t)));
  int32_t* ojobs = static_cast<int32_t*>(rb.ojobs.get(cj * sizeof(int32_t)));
  CK(cudaMemcpyAsync(dsegs, segs.data(), nseg * sizeof(TaskSeg), cudaMemcpyHostToDevice, s));
  std::vector<int32_t> hcount(nseg + 1, 0);
  // Compacts the lists to the solves still iterating; the counts reach the host with the next
  // synchronisation. The jobs not done go to `ojobs` (outer steps), those whose GMRES still runs
  // to `cjobs` (inner steps); `jobs` is the list of the last compaction, `njobs_l` its length
  // once synchronised.
  const int32_t* jobs = ojobs;
  auto compact = [&](int inner) {
    CK(cudaMemsetAsync(ccount, 0, (nseg + 1) * sizeof(int32_t), s));
    const unsigned gx = (unsigned)std::max<int64_t>(1, (std::max<int64_t>(seg_max, (int64_t)cj) + 255) / 256);
    int32_t* out = inner ? cjobs : ojobs;
    launch(K_REF_GMRES, 0.0, 0.0, [&] {
      compact_kernel<<<dim3(gx, (unsigned)(nseg + 1)), 256, 0, s>>>(drd, (int)cj, dtasks, dsegs, nseg, ctasks, out,
                                                                  ccount, inner);
    });
    CK(cudaMemcpyAsync(hcount.data(), ccount, (nseg + 1) * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    jobs = out;
  };
  compact(0);
  CK(cudaStreamSynchronize(s));
  size_t njobs_l = (size_t)hcount[nseg], nouter = njobs_l;
  // Algorithmic bytes of the Arnoldi vectors of all jobs (one pass over every column); a GMRES
  // step k reads and writes 3 k + 8 such passes (k + 1 Gram-Schmidt dot products, the axpy, the
  // norm and the scaling), accounted in proportion to the jobs listed.
  double vec_pass = 0.0;
  for (size_t j = 0; j < cj; ++j) vec_pass += 16.0 * (double)rdh[j].nblk * rdh[j].c;
  auto sweep_cb = [&](auto cbt, int src, int dst) {
    constexpr int CB = decltype(cbt)::value;
    // Warp-per-front launches over a segment, at most 65535 blocks of TINY_WARPS (grid y).
    auto warp_fwd = [&](auto rplt, size_t seg0, int cnt) {
      constexpr int RPL = decltype(rplt)::value;
      in_pieces_of((size_t)cnt, (size_t)65535 * TINY_WARPS, [&](size_t f0, size_t c) {
        launch(K_REF_FWD, 0.0, 0.0, [&] {
          sweep_warp_fwd_kernel<CB, RPL><<<dim3(cchunks, (unsigned)((c + TINY_WARPS - 1) / TINY_WARPS)), 256, 0, s>>>(
              drd, ctasks + seg0 + f0, (int)c, src);
        });
      });
    };
    auto warp_bwd = [&](auto rplt, size_t seg0, int cnt) {
      constexpr int RPL = decltype(rplt)::value;
      in_pieces_of((size_t)cnt, (size_t)65535 * TINY_WARPS, [&](size_t f0, size_t c) {
        launch(K_REF_BWD, 0.0, 0.0, [&] {
          sweep_warp_bwd_kernel<CB, RPL><<<dim3(cchunks, (unsigned)((c + TINY_WARPS - 1) / TINY_WARPS)), 256, 0, s>>>(
              drd, ctasks + seg0 + f0, (int)c, src, dst);
        });
      });
    };
    for (int L = 0; L < nlev; ++L) {
      const int nt = hcount[3 * L], nm = hcount[3 * L + 1], nr = hcount[3 * L + 2];
      if (nt) warp_fwd(std::integral_constant<int, 1>{}, lr[L].tiny0, nt);
      if (nm) warp_fwd(std::integral_constant<int, 3>{}, lr[L].mid0, nm);
      if (wide) {
        if (wl[L].nfr) {
          tg_gather(true, wl[L].fr0, wl[L].nfr, src, dst, K_REF_FWD);
          tg_gemm(wl[L].fw0, wl[L].nfw, wl[L].max_m, src, dst, K_REF_FWD);
        }
        continue;
      }
      if (!nr) continue;
      const size_t sm = (size_t)std::max(1, lr[L].max_ne) * CB * sizeof(float2);
      const unsigned tiles = (unsigned)((lr[L].max_n + SW_ROWS - 1) / SW_ROWS);
      in_pieces((size_t)nr, [&](size_t f0, size_t c) {
        launch(K_REF_FWD, 0.0, sweep_bytes * 0.5 / nlev, [&] {
          sweep_rows_fwd_kernel<CB><<<dim3(cchunks, tiles, (unsigned)c), 256, sm, s>>>(drd, ctasks + lr[L].first + f0,
                                                                                     src);
        });
      });
    }
    const int nj = hcount[nseg];
    if (wide) {
      tg_gather(true, root_fr0, root_nfr, src, dst, K_REF_ROOT);
      tg_gemm(root_t0, root_nfr, root_m, src, dst, K_REF_ROOT);
    } else {
      in_pieces((size_t)nj, [&](size_t f0, size_t c) {
        launch(K_REF_ROOT, 0.0, 0.0, [&] {
          sweep_root_kernel<CB><<<dim3(cchunks, (unsigned)c), 256, (size_t)max_root * CB * sizeof(float2), s>>>(
              drd, jobs + f0, src, dst);
        });
      });
    }
    for (int L = nlev - 1; L >= 0; --L) {
      const int nt = hcount[3 * L], nm = hcount[3 * L + 1], nr = hcount[3 * L + 2];
      if (nt) warp_bwd(std::integral_constant<int, 1>{}, lr[L].tiny0, nt);
      if (nm) warp_bwd(std::integral_constant<int, 3>{}, lr[L].mid0, nm);
      if (wide) {
        if (wl[L].nfr) {
          tg_gather(false, wl[L].fr0, wl[L].nfr, src, dst, K_REF_BWD);
          tg_gemm(wl[L].bw0, wl[L].nbw, wl[L].max_m, src, dst, K_REF_BWD);
        }
        continue;
      }
      if (!nr) continue;
      const size_t sm = (size_t)std::max(1, lr[L].max_n) * CB * sizeof(float2);
      const unsigned tiles = (unsigned)((std::max(1, lr[L].max_ne) + SW_ROWS - 1) / SW_ROWS);
      in_pieces((size_t)nr, [&](size_t f0, size_t c) {
        launch(K_REF_BWD, 0.0, sweep_bytes * 0.5 / nlev, [&] {
          sweep_rows_bwd_kernel<CB><<<dim3(cchunks, tiles, (unsigned)c), 256, sm, s>>>(drd, ctasks + lr[L].first + f0,
                                                                                     src, dst);
        });
      });
    }
  };
  auto sweep = [&](int src, int dst) {
    switch (cbw) {
      case 1: sweep_cb(std::integral_constant<int, 1>{}, src, dst); break;
      case 2: sweep_cb(std::integral_constant<int, 2>{}, src, dst); break;
      case 4: sweep_cb(std::integral_constant<int, 4>{}, src, dst); break;
      default: sweep_cb(std::integral_constant<int, 8>{}, src, dst); break;
    }
  };
  for (int it = 0; it < ctx->max_iters; ++it) {
    // The outer step's jobs: those not done (the list of the last outer compaction).
    const size_t no = nouter;
    in_pieces(no, [&](size_t f0, size_t c) {
      launch(K_REF_GMRES, 0.0, vec_pass * 2.0 * c / cj,
             [&] { gm_start_kernel<<<dim3((unsigned)c, cols), 256, 0, s>>>(drd, ojobs + f0); });
    });
    for (int k = 0; k < GM_M; ++k) {
      sweep(k, k);
      ctx->refine_batch_steps += 1;
      // This inner step's jobs: the outer list at k = 0, else those whose GMRES still runs.
      const int32_t* jl = k == 0 ? ojobs : cjobs;
      const size_t nl = k == 0 ? no : njobs_l;
      in_pieces(nl, [&](size_t f0, size_t c) {
        launch(K_REF_RES, resid_flops * c / cj, 0.0,
               [&] { gm_matvec_kernel<<<dim3((unsigned)c, rows), 256, 0, s>>>(drd, jl + f0, k); });
      });
      for (int side = 0; side < nsides; ++side) slice_products(set_mv + (size_t)k * nsides + side, K_REF_RES, jl, nl);
      // Classical Gram-Schmidt, one pass (gm_dot_kernel pass 0): right-preconditioned by the f32
      // factors, A M^-1 is close to the identity and its few Krylov vectors stay orthogonal to
      // working accuracy; the outer step checks the true FP64 residual either way.
      in_pieces(nl, [&](size_t f0, size_t c) {
        launch(K_REF_GMRES, 0.0, vec_pass * 2.0 * (k + 1) * c / cj, [&] {
          gm_dot_kernel<<<dim3((unsigned)c, cols, (unsigned)(k + 1)), 256, 0, s>>>(drd, jl + f0, k, 0);
        });
        launch(K_REF_GMRES, 0.0, vec_pass * (k + 3.0) * c / cj,
               [&] { gm_axpy_kernel<<<dim3((unsigned)c, rows), 256, 0, s>>>(drd, jl + f0, k); });
      });
      in_pieces(nl, [&](size_t f0, size_t c) {
        launch(K_REF_GMRES, 0.0, vec_pass * 3.0 * c / cj,
               [&] { gm_norm_kernel<<<dim3((unsigned)c, cols), 256, 0, s>>>(drd, jl + f0, k, ctx->inner_tol); });
      });
      launch(K_REF_GMRES, 0.0, 0.0, [&] {
        gm_inner_check_kernel<<<(unsigned)((cj + 127) / 128), 128, 0, s>>>(drd, (int)cj, k, gflags);
      });
      compact(1);
      CK(cudaMemcpyAsync(dh.data(), gflags, cj * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
      CK(cudaStreamSynchronize(s));
      njobs_l = (size_t)hcount[nseg];
      bool all = true;
      for (size_t j = 0; j < cj; ++j) all &= dh[j] != 0;
      if (all) break;
    }
    // The correction and the new residual of every job of the outer step.
    in_pieces(no, [&](size_t f0, size_t c) {
      launch(K_REF_GMRES, 0.0, 0.0, [&] {
        gm_solve_kernel<<<(unsigned)c, std::min(1024, std::max(32, ((cmax + 31) / 32) * 32)), 0, s>>>(drd, ojobs + f0);
      });
    });
    in_pieces(no, [&](size_t f0, size_t c) {
      launch(K_REF_GMRES, 0.0, 0.0,
             [&] { gm_update_kernel<<<dim3((unsigned)c, rows), 256, 0, s>>>(drd, ojobs + f0); });
    });
    launch(K_REF_GMRES, 0.0, 0.0, [&] {
      gm_residual_kernel<<<(unsigned)((cj + 127) / 128), 128, 0, s>>>(drd, (int)cj);
    });
    in_pieces(no, [&](size_t f0, size_t c) {
      launch(K_REF_RES, resid_flops * c / cj, 0.0,
             [&] { refine_residual_kernel<<<dim3((unsigned)c, rows), 256, 0, s>>>(drd, ojobs + f0); });
    });
    for (int side = 0; side < nsides; ++side) slice_products(set_res + side, K_REF_RES, ojobs, no);
    slice_products(set_gam, K_REF_CHECK, ojobs, no);
    launch(K_REF_CHECK, 0.0, 0.0, [&] {
      refine_check_kernel<<<(unsigned)cj, 256, 0, s>>>(drd, ctx->refine_tol, ctx->max_iters, rt_out, rerr, rdone);
    });
    compact(0);
    CK(cudaMemcpyAsync(dh.data(), rdone, cj * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    njobs_l = nouter = (size_t)hcount[nseg];
    size_t active = 0;
    for (size_t j = 0; j < cj; ++j) active += (dh[j] == 0 && rdh[j].c != 0) ? 1 : 0;
    if (active == 0) break;
    // The batch's tail: after two outer steps, when at most 1/32 of the solves still iterate, every
    // further step would run the whole launch sequence for those few; they are recomputed in FP64
    // instead (as failed points, precision.rs:102-115).
    if (allow_giveup && it >= 1 && it + 1 < ctx->max_iters && active * 32 <= cj) {
      launch(K_REF_CHECK, 0.0, 0.0, [&] {
        refine_giveup_kernel<<<(unsigned)((cj + 127) / 128), 128, 0, s>>>(drd, (int)cj);
      });
      break;
    }
  }
  CK(cudaEventRecord(ctx->ev1, s));
  if (!adjoint && !states) {
    CK(cudaMemcpyAsync(th.data(), rt_out, cj * sizeof(double), cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(eh.data(), rerr, cj * sizeof(double), cudaMemcpyDeviceToHost, s));
  }
  if (states && !states->mtrace.empty()) {
    // x_c(p)^† Γ_p x_c(p) per (job, lead, column) into the ψ buffers (P x c each).
    size_t to = 0;
    std::vector<size_t> toffs(cj);
    int pmax = 1;
    for (size_t j = 0; j < cj; ++j) {
      toffs[j] = to;
      to += (size_t)states->mtrace[begin + j].P * rdh[j].c;
      pmax = std::max(pmax, states->mtrace[begin + j].P);
    }
    double* qdev = static_cast<double*>(ctx->tm_out.get(std::max<size_t>(to, 1) * sizeof(double)));
    std::vector<MultiJob> mj(cj);
    for (size_t j = 0; j < cj; ++j) {
      mj[j] = states->mtrace[begin + j];
      mj[j].out = qdev + toffs[j];
    }
    MultiJob* dmj = static_cast<MultiJob*>(ctx->tm_tab.get(cj * sizeof(MultiJob)));
    CK(cudaMemcpyAsync(dmj, mj.data(), cj * sizeof(MultiJob), cudaMemcpyHostToDevice, s));
    in_pieces(cj, [&](size_t f0, size_t c) {
      launch(K_REF_CHECK, 0.0, 0.0, [&] {
        multi_quadratic_kernel<<<dim3((unsigned)c, (unsigned)pmax, (unsigned)std::max(1, cmax)), 256, 0, s>>>(
            drd + f0, dmj + f0);
      });
    });
    for (size_t j = 0; j < cj; ++j) {
      std::vector<double2>& t = (*states->psi)[begin + j];
      const size_t cnt = (size_t)mj[j].P * rdh[j].c;
      std::vector<double> tmp(cnt);
      if (cnt) CK(cudaMemcpyAsync(tmp.data(), qdev + toffs[j], cnt * sizeof(double), cudaMemcpyDeviceToHost, s));
      CK(cudaStreamSynchronize(s));
      t.resize(cnt);
      for (size_t e = 0; e < cnt; ++e) t[e] = make_double2(tmp[e], 0.0);
    }
  } else if (states && !states->twl.empty()) {
    // t = W_L^† x_L per job into the ψ buffers (tcl x c each).
    size_t to = 0;
    std::vector<size_t> toffs(cj);
    for (size_t j = 0; j < cj; ++j) {
      toffs[j] = to;
      to += (size_t)states->tcl[begin + j] * rdh[j].c;
    }
    double2* tdev = static_cast<double2*>(ctx->tm_out.get(std::max<size_t>(to, 1) * sizeof(double2)));
    std::vector<const void*> tabs(3 * cj);
    std::vector<int32_t> cls(cj);
    for (size_t j = 0; j < cj; ++j) {
      tabs[j] = states->twl[begin + j];
      tabs[cj + j] = tdev + toffs[j];
      cls[j] = states->tcl[begin + j];
    }
    void** dtabs = static_cast<void**>(ctx->tm_tab.get(3 * cj * sizeof(void*)));
    int32_t* dcls = static_cast<int32_t*>(ctx->tm_cls.get(cj * sizeof(int32_t)));
    CK(cudaMemcpyAsync(dtabs, tabs.data(), 2 * cj * sizeof(void*), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(dcls, cls.data(), cj * sizeof(int32_t), cudaMemcpyHostToDevice, s));
    launch(K_REF_CHECK, 0.0, 0.0, [&] {
      tmatrix_kernel<<<(unsigned)cj, 256, 0, s>>>(drd, reinterpret_cast<const double2* const*>(dtabs), dcls,
                                                   reinterpret_cast<double2* const*>(dtabs + cj));
    });
    for (size_t j = 0; j < cj; ++j) {
      std::vector<double2>& t = (*states->psi)[begin + j];
      t.resize((size_t)states->tcl[begin + j] * rdh[j].c);
      if (!t.empty())
        CK(cudaMemcpyAsync(t.data(), tdev + toffs[j], t.size() * sizeof(double2), cudaMemcpyDeviceToHost, s));
    }
  } else if (states) {
    for (size_t j = 0; j < cj; ++j) {
      std::vector<double2>& psi = (*states->psi)[begin + j];
      psi.resize((size_t)rdh[j].nblk * rdh[j].c);
      if (!psi.empty())
        CK(cudaMemcpyAsync(psi.data(), rx + xoffs[j], psi.size() * sizeof(double2), cudaMemcpyDeviceToHost, s));
    }
  }
  std::vector<RefineDesc> fin(cj);
  CK(cudaMemcpyAsync(fin.data(), drd, cj * sizeof(RefineDesc), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  for (size_t j = 0; j < cj; ++j) {
    ih[j] = std::max(ih[j], fin[j].iters);
    if (j == 0) ctx->steps_tmp.assign(cj, 0);
    ctx->steps_tmp[j] = fin[j].steps;
    ctx->refine_job_steps += fin[j].steps;
    if (rdh[j].c == 0 || states) {
      if (!adjoint) { th[j] = 0.0; eh[j] = 0.0; }
      if (rdh[j].c == 0) continue;
    }
    if (!fin[j].done || fin[j].stalled) sh[j] = ST_REFINE_STALLED;
  }
  return drd;
}

enum Mode { MODE_DOUBLE = 0, MODE_SINGLE = 1, MODE_MIXED = 2 };

struct JobOut {
  double t = 0.0, err = 0.0;
  int32_t status = ST_OK;
  int32_t iters = 0;
  int32_t steps = 0;  // Arnoldi steps of the mixed refinement
  int32_t perturbed = 0;
  std::vector<double> dv, dp;  // gradient: dT/dV of the block's orbitals (block order), dT/dp
  std::vector<double> tm;      // multi-terminal: T[p * P + q] of the block
  std::vector<uint8_t> fail;
};

// Launch bookkeeping: counts, algorithmic work per kernel class, and launch-by-launch device time
// of the probed class.
struct Launcher {
  caroli_ctx* ctx;
  cudaStream_t s;
  int64_t launches = 0;
  std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> timed;
  template <typename F> void operator()(KClass k, double flops, double bytes, F fn) {
    const bool probe = ctx->probe == (int)k;
    std::pair<cudaEvent_t, cudaEvent_t> ev{};
    if (probe) {
      if (ctx->probe_used == ctx->probe_events.size()) {
        cudaEvent_t a, b;
        CK(cudaEventCreate(&a));
        CK(cudaEventCreate(&b));
        ctx->probe_events.push_back({a, b});
      }
      ev = ctx->probe_events[ctx->probe_used++];
      CK(cudaEventRecord(ev.first, s));
    }
    fn();
    CK(cudaGetLastError());
    if (probe) {
      CK(cudaEventRecord(ev.second, s));
      timed.push_back({(int)k, ev});
    }
    KStat& st = ctx->kstat[k];
    st.launches += 1;
    st.flops += flops;
    st.bytes += bytes;
    ++launches;
  }
  // After a stream synchronisation: device time of the probed launches.
  void collect() {
    for (auto& t : timed) {
      float ms = 0.f;
      CK(cudaEventElapsedTime(&ms, t.second.first, t.second.second));
      ctx->kstat[t.first].ms += ms;
    }
    timed.clear();
    ctx->probe_used = 0;
  }
};

// Adjoint solve and gradient of the jobs [begin, begin + cj) after their forward refinement:
// A^† z_j = Γ_L x_j on the left slice, then dT/dV_a = 2 Re Σ_j x_j[a] conj(z_j[a]) and
// dT/dp = 2 Re Σ_j z_j^† (dH/dp) x_j. The tree fronts are Hermitian (only the root carries Σ), so
// the same f32 factors precondition the adjoint with the root inverse conjugate-transposed.
template <typename LaunchT>
void gradient(caroli_ctx* ctx, System* sys, const std::vector<JobSpec>& specs, size_t begin, size_t cj,
              const std::vector<LevelRange>& lr, int max_root, const Task* dtasks, const std::vector<JobDesc>& jd,
              const float2* arena, const std::vector<size_t>& arena_off, const float2* rarena,
              const std::vector<size_t>& root_off, LaunchT& launch, std::vector<double>& th, std::vector<double>& eh,
              std::vector<int32_t>& sh, std::vector<int32_t>& ih, RefineDesc* fwd, const GradRequest& grad,
              std::vector<JobOut>& out) {
  cudaStream_t s = ctx->stream;
  std::vector<size_t> roff(cj), doff(cj);
  size_t ro = 0, dvo = 0;
  int max_blk = 0;
  for (size_t j = 0; j < cj; ++j) {
    const JobSpec& sp = specs[begin + j];
    const int nblk = sp.sys->blocks[sp.block].nblk;
    const int c = sp.sys->slots[sp.slot].channels[sp.block];
    roff[j] = ro;
    ro += (size_t)nblk * c;
    doff[j] = dvo;
    dvo += (size_t)nblk;
    max_blk = std::max(max_blk, nblk);
  }
  double2* rhs = static_cast<double2*>(ctx->grhs.get(std::max<size_t>(ro, 1) * sizeof(double2)));
  double* dv = static_cast<double*>(ctx->gdv.get(std::max<size_t>(dvo, 1) * sizeof(double)));
  double* dp = static_cast<double*>(ctx->gdp.get(std::max<size_t>(cj * std::max(grad.nparams, 1), 1) * sizeof(double)));
  // Pointer tables: rhs per job, dv per job, dH per job.
  std::vector<const void*> ptrs(3 * cj);
  std::vector<const double2*> rhs_ptr(cj);
  for (size_t j = 0; j < cj; ++j) {
    const JobSpec& sp = specs[begin + j];
    rhs_ptr[j] = rhs + roff[j];
    ptrs[j] = rhs + roff[j];
    ptrs[cj + j] = dv + doff[j];
    ptrs[2 * cj + j] = grad.dvals ? grad.dvals + (size_t)sp.config * grad.nparams * grad.nnz : nullptr;
  }
  void** dptrs = static_cast<void**>(ctx->gptr.get(3 * cj * sizeof(void*)));
  CK(cudaMemcpyAsync(dptrs, ptrs.data(), 3 * cj * sizeof(void*), cudaMemcpyHostToDevice, s));
  const unsigned rows = (unsigned)((max_blk + 255) / 256);
  in_pieces(cj, [&](size_t f0, size_t c) {
    launch(K_REF_RES, 0.0, 0.0, [&] {
      grad_rhs_kernel<<<dim3((unsigned)c, rows), 256, 0, s>>>(fwd + f0, reinterpret_cast<double2* const*>(dptrs) + f0);
    });
  });
  std::vector<double> tz(cj), ez(cj);
  RefineDesc* adj = refine(ctx, sys, specs, begin, cj, lr, max_root, dtasks, jd, arena, arena_off, rarena, root_off,
                           launch, tz, ez, sh, ih, ctx->rb[1], 1, rhs_ptr);
  in_pieces(cj, [&](size_t f0, size_t c) {
    launch(K_REF_RES, 0.0, 0.0, [&] {
      grad_v_kernel<<<dim3((unsigned)c, rows), 256, 0, s>>>(fwd + f0, adj + f0,
                                                            reinterpret_cast<double* const*>(dptrs + cj) + f0);
    });
  });
  if (grad.nparams > 0 && grad.dvals)
    in_pieces(cj, [&](size_t f0, size_t c) {
      launch(K_REF_RES, 0.0, 0.0, [&] {
        grad_p_kernel<<<dim3((unsigned)c, (unsigned)grad.nparams), 256, 0, s>>>(
            fwd + f0, adj + f0, reinterpret_cast<const double2* const*>(dptrs + 2 * cj) + f0, grad.nnz,
            dp + f0 * grad.nparams, grad.nparams);
      });
    });
  std::vector<double> dvh(dvo), dph(cj * std::max(grad.nparams, 1));
  CK(cudaMemcpyAsync(dvh.data(), dv, dvo * sizeof(double), cudaMemcpyDeviceToHost, s));
  if (grad.nparams > 0 && grad.dvals)
    CK(cudaMemcpyAsync(dph.data(), dp, cj * grad.nparams * sizeof(double), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  for (size_t j = 0; j < cj; ++j) {
    JobOut& o = out[begin + j];
    const int nblk = specs[begin + j].sys->blocks[specs[begin + j].block].nblk;
    o.dv.assign(dvh.begin() + doff[j], dvh.begin() + doff[j] + nblk);
    o.dp.assign(grad.nparams, 0.0);
    if (grad.dvals)
      for (int k = 0; k < grad.nparams; ++k) o.dp[k] = dph[j * grad.nparams + k];
  }
  (void)th;
  (void)eh;
}

// Runs `specs` in `mode`: complex f64 fronts (DOUBLE), complex f32 fronts under an f64 root
// (SINGLE), or complex f32 factors refined in FP64 (MIXED). T: front precision, TR: root precision.
template <typename T, typename TR>
void run_jobs(caroli_ctx* ctx, System* sys, const std::vector<JobSpec>& specs, Mode mode, std::vector<JobOut>& out,
              const GradRequest* grad = nullptr, const StatesRequest* states = nullptr) {
  using V = typename Cx<T>::V;
  using VR = typename Cx<TR>::V;
  cudaStream_t s = ctx->stream;
  const size_t vb = sizeof(V), vr = sizeof(VR);
  const size_t nj = specs.size();
  const bool mixed = mode == MODE_MIXED;
  out.assign(nj, JobOut{});
  Launcher launch{ctx, s};
  // The memory budget of a batch covers its fronts and, in mixed precision, its refinement vectors;
  // a batch without refinement gives the idle vectors of an earlier mixed batch back first.
  if (!mixed)
    for (RefineBufs& b : ctx->rb) b.release_vectors();
  size_t begin = 0;
  while (begin < nj) {
    // Chunk of jobs within the memory budget: the fronts and, in mixed precision, the refinement's
    // vectors (one column per channel: x, r, d, the FP64 Arnoldi basis and the f32 preconditioned
    // vectors, the sweeps' buffers; twice with the adjoint solve of a gradient).
    size_t end = begin, bytes = 0;
    while (end < nj) {
      const FrontPlan& P = specs[end].plan->host;
      size_t b = (size_t)P.arena_elems * vb + (size_t)P.fronts[P.root].n * P.fronts[P.root].n * vr;
      if (mixed) {
        const SigmaSlot& sg = specs[end].sys->slots[specs[end].slot];
        const size_t c = states ? (size_t)(states->cl[end] + states->cr[end]) : (size_t)sg.channels[specs[end].block];
        const size_t nblk = (size_t)specs[end].sys->blocks[specs[end].block].nblk;
        const size_t per = c * (nblk * (16 * (GM_M + 1) + 8 * GM_M + 16 + 16 + 8) +
                                (size_t)(P.sum_ne + P.sum_nb) * 8 + (size_t)P.nl * 16);
        b += per * (grad ? 2 : 1);
      }
      if (end > begin && bytes + b > ctx->mem_budget) break;
      bytes += b;
      ++end;
    }
    const size_t cj = end - begin;
    std::vector<JobDesc> jd(cj);
    std::vector<size_t> arena_off(cj), root_off(cj), fail_off(cj);
    size_t aoff = 0, roff = 0, foff = 0;
    int max_levels = 0;
    size_t parts_per_job = 1;
    for (size_t j = 0; j < cj; ++j) {
      const FrontPlan& P = specs[begin + j].plan->host;
      arena_off[j] = aoff;
      aoff += (size_t)P.arena_elems;
      root_off[j] = roff;
      roff += (size_t)P.fronts[P.root].n * P.fronts[P.root].n;
      fail_off[j] = foff;
      foff += P.fronts.size();
      max_levels = std::max(max_levels, P.levels);
      parts_per_job = std::max(parts_per_job, (size_t)(P.nr + 7) / 8);
    }
    V* arena = static_cast<V*>(ctx->arena.fit(std::max<size_t>(aoff, 1) * vb));
    VR* rarena = static_cast<VR*>(ctx->root_arena.fit(std::max<size_t>(roff, 1) * vr));
    uint8_t* fail = static_cast<uint8_t*>(ctx->fail.get(std::max<size_t>(foff, 1)));
    int32_t* status = static_cast<int32_t*>(ctx->status.get(cj * sizeof(int32_t)));
    int* pert = static_cast<int*>(ctx->pert.get(cj * sizeof(int)));
    double* tdev = static_cast<double*>(ctx->tout.get(cj * sizeof(double)));
    double* part = static_cast<double*>(ctx->part.get(cj * parts_per_job * sizeof(double)));
    CK(cudaMemsetAsync(fail, 0, foff, s));
    CK(cudaMemsetAsync(status, 0, cj * sizeof(int32_t), s));
    CK(cudaMemsetAsync(pert, 0, cj * sizeof(int), s));
    for (size_t j = 0; j < cj; ++j) {
      const JobSpec& sp = specs[begin + j];
      const DevPlan& P = *sp.plan;
      const SigmaSlot& sg = sp.sys->slots[sp.slot];
      JobDesc& d = jd[j];
      d.fronts = P.fronts; d.maps = P.maps; d.own = P.own; d.entries = P.entries;
      d.arena = arena + arena_off[j];
      d.root_arena = rarena + root_off[j];
      d.vals = sp.sys->vals + (size_t)sp.config * sp.sys->desc.row_ptr[sp.sys->desc.n];
      d.sigma_l = sg.sl[sp.block]; d.sigma_r = sg.sr[sp.block];
      d.gamma_l = sg.gl[sp.block]; d.gamma_r = sg.gr[sp.block];
      d.fail = fail + fail_off[j];
      d.energy = sg.energy;
      d.root = P.host.root; d.nl = P.host.nl; d.nr = P.host.nr; d.rpos = P.host.rpos; d.nd = P.host.nd;
      d.nfronts = (int32_t)P.host.fronts.size();
    }
    JobDesc* djobs = static_cast<JobDesc*>(ctx->jobs.get(cj * sizeof(JobDesc)));
    CK(cudaMemcpyAsync(djobs, jd.data(), cj * sizeof(JobDesc), cudaMemcpyHostToDevice, s));

    // Task lists: per level the small fronts then the large ones (contiguous), then the roots.
    // Built once per distinct batch (the plans of the chunk, precisions and arena addresses) and
    // kept with its device copies: a repeated batch reuses them without host work.
    using Level = TaskLevel;
    TaskCache& tc = ctx->tcache;
    const int small_max = sizeof(T) == 8 ? SMALL_MAX_F64 : ctx->small_max_f32;
    // Split Schur update: the panel sweeps transform only the pivot columns, then one tensor-core
    // GEMM per front forms [X; S] = [F11^-1; W] F12 + [0; F22] (f32 fronts below the root).
    const bool split = std::is_same<T, float>::value && ctx->tensor_cores && ctx->tc_choice && ctx->split_choice;
    std::vector<uint64_t> key_plans(cj);
    for (size_t j = 0; j < cj; ++j) key_plans[j] = specs[begin + j].plan->id;
    const bool hit = tc.valid && tc.plans == key_plans && tc.tsize == (int)sizeof(T) && tc.trsize == (int)sizeof(TR) &&
                     tc.mixed == mixed && tc.arena == (const void*)arena && tc.rarena == (const void*)rarena &&
                     tc.max_levels == max_levels && tc.small_max == small_max && tc.split == split;
    std::vector<Task>& tasks = tc.tasks;
    std::vector<Level>& levels = tc.levels;
    std::vector<InvTask>& inv = tc.inv;  // large fronts' pivot blocks per level, then the roots
    size_t& inv_piv = tc.inv_piv;  // scratch sizes: pivots (entries) and Y blocks (bytes)
    size_t& inv_y = tc.inv_y;
    size_t& inv_bt = tc.inv_bt;
    std::vector<size_t>& inv_bt_off = tc.inv_bt_off;
    std::vector<size_t>& inv_piv_off = tc.inv_piv_off;
    std::vector<size_t>& inv_y_off = tc.inv_y_off;
    size_t& root0 = tc.root0;
    size_t& rinv0 = tc.rinv0;
    int& max_root = tc.max_root;
    double& root_flops = tc.root_flops;
    double& trace_flops = tc.trace_flops;
    if (!hit) {
    tc.valid = false;
    tc.f12.clear(); tc.f12_off.clear(); tc.f12_inv.clear(); tc.sgt.clear(); tc.sgt_stage.clear();
    tc.f12_elems = 0;
    tasks.clear();
    levels.assign(max_levels, Level{});
    inv.clear();
    inv_piv = inv_y = inv_bt = 0;
    inv_bt_off.clear();
    inv_piv_off.clear();
    inv_y_off.clear();
    for (int L = 0; L < max_levels; ++L) {
      Level& lv = levels[L];
      lv = Level{};
      lv.tiny0 = tasks.size();
      for (size_t j = 0; j < cj; ++j) {
        const auto& fr = specs[begin + j].plan->host.fronts;
        const FrontDesc* dfr = specs[begin + j].plan->fronts;
        for (size_t k = 0; k + 1 < fr.size(); ++k)
          if (fr[k].level == L && fr[k].n <= TINY_MAX) {
            tasks.push_back({(int32_t)j, (int32_t)k, dfr + k});
            const double ne = fr[k].ne, nb = fr[k].n - fr[k].ne;
            lv.tiny_flops += 8.0 / 3 * ne * ne * ne + 8 * ne * ne * nb + 8 * nb * nb * ne;
            lv.max_tiny_n = std::max(lv.max_tiny_n, fr[k].n);
            lv.tiny_bytes += ((double)fr[k].n * fr[k].n + (mixed ? (double)fr[k].n * fr[k].n : nb * nb)) * vb;
          }
      }
      lv.tiny_n = tasks.size() - lv.tiny0;
      // Largest fronts first: the eight warps of a tiny-front CTA get fronts of about one size (a
      // CTA lasts as long as its largest front), and the longest CTAs start first.
      auto by_size = [&](size_t a0, size_t a1) {
        std::stable_sort(tasks.begin() + a0, tasks.begin() + a1, [&](const Task& x, const Task& y) {
          return specs[begin + x.job].plan->host.fronts[x.front].n > specs[begin + y.job].plan->host.fronts[y.front].n;
        });
      };
      by_size(lv.tiny0, tasks.size());
      lv.small0 = tasks.size();
      const int bucket_hi[3] = {48, 64, small_max};
      for (int b = 0; b < 3; ++b) {
        const int lo = b == 0 ? TINY_MAX : bucket_hi[b - 1], hi = bucket_hi[b];
        lv.sb0[b] = tasks.size();
        for (size_t j = 0; j < cj; ++j) {
          const auto& fr = specs[begin + j].plan->host.fronts;
          const FrontDesc* dfr = specs[begin + j].plan->fronts;
          for (size_t k = 0; k + 1 < fr.size(); ++k)
            if (fr[k].level == L && fr[k].n > lo && fr[k].n <= hi) {
              tasks.push_back({(int32_t)j, (int32_t)k, dfr + k});
              const double ne = fr[k].ne, nb = fr[k].n - fr[k].ne;
              lv.max_small_n = std::max(lv.max_small_n, fr[k].n);
              lv.max_small_ne = std::max(lv.max_small_ne, fr[k].ne);
              lv.sb_n[b] = std::max(lv.sb_n[b], fr[k].n);
              lv.sb_ne[b] = std::max(lv.sb_ne[b], fr[k].ne);
              lv.small_flops += 8.0 / 3 * ne * ne * ne + 8 * ne * ne * nb + 8 * nb * nb * ne;
              // The front written (mixed keeps all of it, else S) and the children's blocks read.
              lv.small_bytes += ((double)fr[k].n * fr[k].n + (mixed ? (double)fr[k].n * fr[k].n : nb * nb)) * vb;
            }
        }
        lv.sbn[b] = tasks.size() - lv.sb0[b];
        by_size(lv.sb0[b], tasks.size());
        if (hi >= small_max) break;
      }
      lv.small_n = tasks.size() - lv.small0;
      lv.large0 = tasks.size();
      lv.inv0 = inv.size();
      lv.f12_0 = tc.f12.size();
      lv.sg0 = tc.sgt.size();
      for (size_t j = 0; j < cj; ++j) {
        const auto& fr = specs[begin + j].plan->host.fronts;
        const FrontDesc* dfr = specs[begin + j].plan->fronts;
        for (size_t k = 0; k + 1 < fr.size(); ++k)
          if (fr[k].level == L && fr[k].n > small_max) {
            tasks.push_back({(int32_t)j, (int32_t)k, dfr + k});
            const double ne = fr[k].ne, nb = fr[k].n - fr[k].ne;
            lv.max_large_n = std::max(lv.max_large_n, fr[k].n);
            lv.max_large_ne = std::max(lv.max_large_ne, fr[k].ne);
            lv.inv_flops += 8.0 / 3 * ne * ne * ne;
            lv.gemm0_flops += 8 * ne * ne * nb;
            lv.gemm1_flops += 8 * nb * nb * ne;
            const double ncol = split ? ne : (double)fr[k].n;  // columns the sweep transforms
            for (int k0 = 0; k0 < fr[k].ne; k0 += GJ_KB) {
              const double kb = std::min(GJ_KB, fr[k].ne - k0), nn = fr[k].n;
              lv.upd_flops += 8.0 * nn * (ncol - kb) * kb;  // complex n x kb times kb x (ncol - kb)
              lv.upd_bytes += 2.0 * nn * (ncol - kb) * vb;  // the rest columns read and written
              lv.pan_flops += 8.0 * nn * kb * kb;
            }
            if (split) {
              lv.upd_flops += 8.0 * fr[k].n * ne * nb;                           // [X; S] = [F11^-1; W] F12
              lv.upd_bytes += ((double)fr[k].n * ne + 3.0 * ne * nb + 2.0 * nb * nb) * vb;  // A, F12 twice, X, F22
            }
            lv.asm_bytes += (double)fr[k].n * fr[k].n * vb;
            if (fr[k].ne > 0) {
              InvTask it{};
              it.a = arena + arena_off[j] + fr[k].arena_off;
              it.ld = fr[k].n;
              it.n = fr[k].n;
              it.npiv = fr[k].ne;
              it.ncol = split ? fr[k].ne : fr[k].n;
              it.job = (int32_t)j;
              it.front = (int32_t)k;
              if (split && fr[k].n > fr[k].ne) {
                const int fne = fr[k].ne, fnb = fr[k].n - fr[k].ne;
                float2* fa = reinterpret_cast<float2*>(arena + arena_off[j] + fr[k].arena_off);
                const size_t ci = tc.f12.size();
                tc.f12.push_back({fa, nullptr, fr[k].n, fne, nullptr});
                tc.f12_off.push_back(tc.f12_elems);
                tc.f12_inv.push_back(inv.size());
                tc.f12_elems += (size_t)fne * fnb;
                TGTask tx{};
                tx.a = fa; tx.lda = fr[k].n; tx.ldb = fne; tx.c = fa + (size_t)fne * fr[k].n; tx.ldc = fr[k].n;
                tx.m = fne; tx.n = fnb; tx.k = fne; tx.sign = 1.f; tx.job = (int32_t)j;
                TGTask ts = tx;
                ts.a = fa + fne; ts.add = fa + fne + (size_t)fne * fr[k].n; ts.ldadd = fr[k].n;
                ts.c = fa + fne + (size_t)fne * fr[k].n; ts.m = fnb;
                tc.sgt.push_back(tx);
                tc.sgt_stage.push_back({ci, 0});
                tc.sgt.push_back(ts);
                tc.sgt_stage.push_back({ci, 1});
                lv.sg_max_m = std::max(lv.sg_max_m, std::max(fne, fnb));
                lv.sg_max_cols = std::max(lv.sg_max_cols, fnb);
                lv.sg_flops += 8.0 * fr[k].n * (double)fne * fnb;
              }
              inv_piv_off.push_back(inv_piv);
              inv_y_off.push_back(inv_y);
              inv_bt_off.push_back(vb == sizeof(float2) ? inv_bt : SIZE_MAX);
              inv_piv += fr[k].ne;
              inv_y += (size_t)GJ_KB * fr[k].n * vb;
              if (vb == sizeof(float2)) inv_bt += tc_operand_bytes(fr[k].n);
              inv.push_back(it);
            }
          }
      }
      lv.large_n = tasks.size() - lv.large0;
      lv.f12_n = tc.f12.size() - lv.f12_0;
      lv.sg_n = tc.sgt.size() - lv.sg0;
      lv.max_n = std::max(std::max(lv.max_small_n, lv.max_large_n), lv.tiny_n ? TINY_MAX : 0);
    }
    root0 = tasks.size();
    rinv0 = inv.size();
    max_root = 0;
    root_flops = trace_flops = 0.0;
    for (size_t j = 0; j < cj; ++j) {
      const auto& P = specs[begin + j].plan->host;
      tasks.push_back({(int32_t)j, P.root, specs[begin + j].plan->fronts + P.root});
      const int m = P.fronts[P.root].n;
      max_root = std::max(max_root, m);
      root_flops += 8.0 / 3 * m * (double)m * m + 8.0 * m * (double)m * P.nr;
      trace_flops += 16.0 * P.nl * (double)P.nl * P.nr;
      InvTask it{};
      it.a = rarena + root_off[j];
      it.ld = m;
      it.n = m;
      it.npiv = m;
      it.ncol = m;
      it.job = (int32_t)j;
      it.front = -1;
      inv_piv_off.push_back(inv_piv);
      inv_y_off.push_back(inv_y);
      inv_bt_off.push_back(vr == sizeof(float2) ? inv_bt : SIZE_MAX);
      inv_piv += m;
      inv_y += (size_t)GJ_KB * m * vr;
      if (vr == sizeof(float2)) inv_bt += tc_operand_bytes(m);
      inv.push_back(it);
    }
    }  // !hit
    // Inverse scratch: pivots, the Y blocks (sized for the wider type), scale and flags.
    int32_t* dpiv = static_cast<int32_t*>(ctx->ipiv.get(std::max<size_t>(inv_piv, 1) * sizeof(int32_t)));
    unsigned char* dy = static_cast<unsigned char*>(ctx->iy.get(std::max<size_t>(inv_y, 16)));
    unsigned char* dbt = static_cast<unsigned char*>(ctx->ibt.get(std::max<size_t>(inv_bt, 16)));
    double* dscale = static_cast<double*>(ctx->iscale.get(std::max<size_t>(inv.size(), 1) * sizeof(double)));
    int32_t* dbad = static_cast<int32_t*>(ctx->ibad.get(std::max<size_t>(inv.size(), 1) * sizeof(int32_t)));
    InvTask* dinv = static_cast<InvTask*>(ctx->inv.get(std::max<size_t>(inv.size(), 1) * sizeof(InvTask)));
    Task* dtasks = static_cast<Task*>(ctx->tasks.get(tasks.size() * sizeof(Task)));
    float2* f12_stage = static_cast<float2*>(ctx->f12_stage.get(std::max<size_t>(tc.f12_elems, 1) * sizeof(float2)));
    F12Copy* df12 = static_cast<F12Copy*>(ctx->f12_list.get(std::max<size_t>(tc.f12.size(), 1) * sizeof(F12Copy)));
    TGTask* dsgt = static_cast<TGTask*>(ctx->sgt_list.get(std::max<size_t>(tc.sgt.size(), 1) * sizeof(TGTask)));
    const bool same_scratch = hit && tc.piv == dpiv && tc.y == dy && tc.bt == dbt && tc.scale == dscale &&
                              tc.bad == dbad && tc.dinv == dinv && tc.dtasks == dtasks && tc.f12_stage == f12_stage &&
                              tc.f12_dev == df12 && tc.sgt_dev == dsgt && tc.status_dev == status;
    if (!same_scratch) {
      for (size_t q = 0; q < inv.size(); ++q) {
        inv[q].piv = dpiv + inv_piv_off[q];
        inv[q].y = dy + inv_y_off[q];
        inv[q].bt = inv_bt_off[q] == SIZE_MAX ? nullptr : dbt + inv_bt_off[q];
        inv[q].scale2 = dscale + q;
        inv[q].bad = dbad + q;
      }
      if (!inv.empty())
        CK(cudaMemcpyAsync(dinv, inv.data(), inv.size() * sizeof(InvTask), cudaMemcpyHostToDevice, s));
      CK(cudaMemcpyAsync(dtasks, tasks.data(), tasks.size() * sizeof(Task), cudaMemcpyHostToDevice, s));
      for (size_t q = 0; q < tc.f12.size(); ++q) {
        tc.f12[q].stage = f12_stage + tc.f12_off[q];
        tc.f12[q].bad = dbad + tc.f12_inv[q];
      }
      for (size_t q = 0; q < tc.sgt.size(); ++q) {
        tc.sgt[q].b = f12_stage + tc.f12_off[tc.sgt_stage[q].first];
        tc.sgt[q].status = status;
      }
      if (!tc.f12.empty())
        CK(cudaMemcpyAsync(df12, tc.f12.data(), tc.f12.size() * sizeof(F12Copy), cudaMemcpyHostToDevice, s));
      if (!tc.sgt.empty())
        CK(cudaMemcpyAsync(dsgt, tc.sgt.data(), tc.sgt.size() * sizeof(TGTask), cudaMemcpyHostToDevice, s));
      tc.piv = dpiv; tc.y = dy; tc.bt = dbt; tc.scale = dscale; tc.bad = dbad; tc.dinv = dinv; tc.dtasks = dtasks;
      tc.f12_stage = f12_stage; tc.f12_dev = df12; tc.sgt_dev = dsgt; tc.status_dev = status;
    }
    tc.plans = key_plans;
    tc.tsize = (int)sizeof(T);
    tc.trsize = (int)sizeof(TR);
    tc.mixed = mixed;
    tc.arena = arena;
    tc.rarena = rarena;
    tc.max_levels = max_levels;
    tc.small_max = small_max;
    tc.split = split;
    tc.valid = true;

    // Batched blocked inverse of `count` matrices starting at dinv + first, largest n.
    // Batched blocked sweep of `count` fronts starting at dinv + first: largest size nmax, largest
    // pivot count pmax.
    // Work attribution (kernel-class accounting): the panel sweeps to `cls` with `flops`, the
    // rank-kb updates to `ucls` with their flops and bytes.
    auto inverse = [&](auto tag, size_t first, size_t count, int nmax, int pmax, double tol, int perturb, KClass cls,
                       double flops, KClass ucls, double uflops, double ubytes) {
      using TT = decltype(tag);
      using VV = typename Cx<TT>::V;
      if (!count || nmax <= 0 || pmax <= 0) return;
      const size_t sm = panel_smem(pmax, sizeof(VV));
      const size_t smf = (size_t)finish_bytes(pmax);
      if (!sm || smf > (size_t)SMEM_LIMIT) throw CudaError{cudaErrorInvalidValue, "front too large for a panel sweep"};
      const int panels = (pmax + GJ_KB - 1) / GJ_KB;
      const double per = flops / panels;
      const double uper = uflops / panels, ubper = ubytes / panels;
      launch(cls, 0.0, 0.0, [&] { inv_scale_kernel<TT><<<(unsigned)count, 256, 0, s>>>(dinv + first); });
      for (int k0 = 0; k0 < pmax; k0 += GJ_KB) {
        launch(cls, per, 0.0, [&] {
          inv_panel_kernel<TT><<<(unsigned)count, 256, sm, s>>>(dinv + first, k0, tol, perturb, (int)sm);
        });
        const unsigned rt = (unsigned)((nmax + 63) / 64);
        in_pieces(count, [&](size_t f0, size_t c) {
          launch(ucls, uper * c / count, ubper * c / count, [&] {
            if (std::is_same<TT, float>::value && ctx->tensor_cores && ctx->tc_choice)
              tc_update_kernel<<<dim3((unsigned)((nmax + TCU_ROWS - 1) / TCU_ROWS), (unsigned)c,
                                      (unsigned)((nmax + TCU_COLS * TCU_GROUP - 1) / (TCU_COLS * TCU_GROUP))),
                                 TCU_THREADS, TCU_SMEM, s>>>(
                  dinv + first + f0, k0, status, ctx->tc_wait_limit);
            else
              inv_update_kernel<TT><<<dim3(rt, rt, (unsigned)c), 256, 0, s>>>(dinv + first + f0, k0);
          });
        });
      }
      launch(cls, 0.0, 0.0, [&] { inv_finish_kernel<TT><<<(unsigned)count, 256, smf, s>>>(dinv + first, djobs, status); });
    };

    const int perturb = mixed ? 1 : 0;
    // Factorization level by level, then the root front and its inverse: a fixed launch sequence
    // for a given batch (task lists, scratch, schedule).
    // Phase events: recorded as event nodes when the factorization is captured into a graph (the
    // external flag is only valid during a capture), so that every replay records them.
    bool capturing = false;
    auto record = [&](cudaEvent_t ev) {
      if (capturing) CK(cudaEventRecordWithFlags(ev, s, cudaEventRecordExternal));
      else CK(cudaEventRecord(ev, s));
    };
    cudaEvent_t ev0 = ctx->ev0, evf = ctx->evf, evr = ctx->evr;
    auto factor_all = [&]() {
      record(ev0);
      // Factorization, level by level.
      for (int L = 0; L < max_levels; ++L) {
        const Level& lv = levels[L];
        if (lv.tiny_n) {
          const unsigned blocks = (unsigned)((lv.tiny_n + TINY_WARPS - 1) / TINY_WARPS);
          launch(K_SMALL, lv.tiny_flops, lv.tiny_bytes, [&] {
            if (mixed)
              tiny_front_kernel<T, true><<<blocks, 256, tiny_smem<T>(lv.max_tiny_n), s>>>(
                  djobs, dtasks + lv.tiny0, (int)lv.tiny_n, Prec<T>::tol, perturb, pert, lv.max_tiny_n);
            else
              tiny_front_kernel<T, false><<<blocks, 256, tiny_smem<T>(lv.max_tiny_n), s>>>(
                  djobs, dtasks + lv.tiny0, (int)lv.tiny_n, Prec<T>::tol, perturb, pert, lv.max_tiny_n);
          });
        }
        for (int b = 0; b < 3; ++b) {
          if (!lv.sbn[b]) continue;
          const size_t sm = small_smem_bytes(lv.sb_n[b], lv.sb_ne[b], vb);
          const unsigned nblk = (unsigned)lv.sbn[b];
          const Task* st = dtasks + lv.sb0[b];
          const double share = (double)lv.sbn[b] / (double)lv.small_n;
          const bool wide_cta = ctx->small_threads == 512 && lv.sb_n[b] > 64;
          launch(K_SMALL, lv.small_flops * share, lv.small_bytes * share, [&] {
            if (mixed && wide_cta)
              small_front_wide_kernel<T, true><<<nblk, 512, sm, s>>>(djobs, st, Prec<T>::tol, perturb, pert);
            else if (mixed)
              small_front_kernel<T, true><<<nblk, 256, sm, s>>>(djobs, st, Prec<T>::tol, perturb, pert);
            else if (wide_cta)
              small_front_wide_kernel<T, false><<<nblk, 512, sm, s>>>(djobs, st, Prec<T>::tol, perturb, pert);
            else
              small_front_kernel<T, false><<<nblk, 256, sm, s>>>(djobs, st, Prec<T>::tol, perturb, pert);
          });
        }
        if (lv.large_n) {
          const Task* lt = dtasks + lv.large0;
          const int mt = (lv.max_large_n + 63) / 64;
          in_pieces(lv.large_n, [&](size_t f0, size_t c) {
            launch(K_ASSEMBLE, 0.0, lv.asm_bytes * c / lv.large_n, [&] {
              assemble_kernel<T, T><<<dim3((lv.max_large_n + 31) / 32, (unsigned)c), 256, 0, s>>>(djobs, lt + f0, 0);
            });
          });
          const size_t ninv = (L + 1 < max_levels ? levels[L + 1].inv0 : rinv0) - lv.inv0;
          inverse(T{}, lv.inv0, ninv, lv.max_large_n, lv.max_large_ne, Prec<T>::tol, perturb, K_PANEL, lv.pan_flops,
                  K_UPDATE, lv.upd_flops, lv.upd_bytes);
          if (split && lv.f12_n) {
            // [X; S] = [F11^-1; W] F12 + [0; F22] of every front of the level on the tensor cores
            // (its flops and bytes are counted with the level's updates above).
            in_pieces(lv.f12_n, [&](size_t f0, size_t c) {
              launch(K_UPDATE, 0.0, 0.0, [&] {
                f12_copy_kernel<<<dim3(32, (unsigned)c), 256, 0, s>>>(df12 + lv.f12_0 + f0);
              });
            });
            in_pieces(lv.sg_n, [&](size_t f0, size_t c) {
              launch(K_UPDATE, 0.0, 0.0, [&] {
                tc_sweep_gemm_kernel<<<dim3((unsigned)((lv.sg_max_cols + TG_COLS - 1) / TG_COLS),
                                            (unsigned)((lv.sg_max_m + TG_ROWS - 1) / TG_ROWS), (unsigned)c),
                                       TG_THREADS, TG_SMEM, s>>>(dsgt + lv.sg0 + f0, 0, 0, ctx->tc_wait_limit);
              });
            });
          }
          (void)mt;
        }
      }
      record(evf);
      // Root front in TR, then its inverse. The reference's root LU has no stability test (a zero
      // pivot means a singular root); in mixed precision tiny root pivots are perturbed like the
      // fronts' (the refinement corrects).
      const Task* rt = dtasks + root0;
      in_pieces(cj, [&](size_t f0, size_t c) {
        launch(K_ROOT_ASM, 0.0, 0.0, [&] {
          assemble_kernel<T, TR><<<dim3((max_root + 31) / 32, (unsigned)c), 256, 0, s>>>(djobs, rt + f0, 1);
        });
      });
      inverse(TR{}, rinv0, cj, max_root, max_root, mixed ? Prec<T>::tol * 1e-2 : 0.0, perturb, K_ROOT_INV, root_flops,
              K_ROOT_INV, 0.0, 0.0);
      record(evr);
    };
    // A batch seen twice in a row (same plans, schedule and scratch) is captured as a CUDA graph
    // on its second run and replayed afterwards: one launch in place of the level-by-level
    // sequence. Probed runs (per-launch events) always launch directly.
    std::vector<uint64_t> gkey(key_plans);
    for (uint64_t v : {(uint64_t)sizeof(T), (uint64_t)sizeof(TR), (uint64_t)mixed, (uint64_t)small_max,
                       (uint64_t)(ctx->tensor_cores && ctx->tc_choice), (uint64_t)ctx->tc_wait_limit, (uint64_t)cj,
                       (uint64_t)(uintptr_t)djobs,
                       (uint64_t)(uintptr_t)dtasks, (uint64_t)(uintptr_t)dinv, (uint64_t)(uintptr_t)pert,
                       (uint64_t)(uintptr_t)status, (uint64_t)(uintptr_t)arena, (uint64_t)(uintptr_t)rarena,
                       (uint64_t)split, (uint64_t)ctx->small_threads, (uint64_t)(uintptr_t)df12,
                       (uint64_t)(uintptr_t)dsgt,
                       (uint64_t)(uintptr_t)f12_stage})
      gkey.push_back(v);
    FactorGraph& fg = ctx->fgraph;
    if (!ctx->use_graphs || ctx->probe >= 0) {
      factor_all();
    } else if (fg.exec && fg.key == gkey) {
      CK(cudaGraphLaunch(fg.exec, s));
      for (int k = 0; k < K_COUNT; ++k) {
        ctx->kstat[k].launches += fg.stats[k].launches;
        ctx->kstat[k].flops += fg.stats[k].flops;
        ctx->kstat[k].bytes += fg.stats[k].bytes;
      }
      launch.launches += fg.launches;
      ctx->graph_replays += 1;
    } else if (fg.seen == gkey) {
      fg.reset();
      KStat before[K_COUNT];
      for (int k = 0; k < K_COUNT; ++k) before[k] = ctx->kstat[k];
      const int64_t l0 = launch.launches;
      cudaGraph_t graph = nullptr;
      CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
      capturing = true;
      try {
        factor_all();
      } catch (...) {
        capturing = false;
        cudaStreamEndCapture(s, &graph);
        if (graph) cudaGraphDestroy(graph);
        (void)cudaGetLastError();
        throw;
      }
      capturing = false;
      CK(cudaStreamEndCapture(s, &graph));
      const cudaError_t ie = cudaGraphInstantiate(&fg.exec, graph, 0);
      cudaGraphDestroy(graph);
      CK(ie);
      fg.key = gkey;
      fg.launches = launch.launches - l0;
      for (int k = 0; k < K_COUNT; ++k) {
        fg.stats[k].launches = ctx->kstat[k].launches - before[k].launches;
        fg.stats[k].flops = ctx->kstat[k].flops - before[k].flops;
        fg.stats[k].bytes = ctx->kstat[k].bytes - before[k].bytes;
      }
      CK(cudaGraphLaunch(fg.exec, s));
      ctx->graph_captures += 1;
    } else {
      factor_all();
    }
    fg.seen = gkey;
    if (ctx->factor_only) {  // a tuning trial: the factorization time is all it needs
      CK(cudaStreamSynchronize(s));
      float mf = 0.f, mr = 0.f;
      CK(cudaEventElapsedTime(&mf, ctx->ev0, ctx->evf));
      CK(cudaEventElapsedTime(&mr, ctx->evf, ctx->evr));
      ctx->factor_ms += mf;
      ctx->root_ms += mr;
      launch.collect();
      begin = end;
      continue;
    }
    std::vector<double> th(cj), eh(cj, 0.0);
    std::vector<int32_t> sh(cj, ST_OK), ih(cj, 0);
    if (!mixed) {
      in_pieces(cj, [&](size_t f0, size_t c) {
        launch(K_TRACE, trace_flops * c / cj, 0.0, [&] {
          trace_kernel<TR><<<dim3((unsigned)parts_per_job, (unsigned)c), 256, 0, s>>>(djobs + f0, part + f0 * parts_per_job,
                                                                                    (int)parts_per_job);
        });
      });
      launch(K_TRACE, 0.0, 0.0, [&] {
        trace_finish_kernel<<<(unsigned)((cj + 127) / 128), 128, 0, s>>>(part, (int)parts_per_job, (int)cj, tdev, status);
      });
      if constexpr (std::is_same<TR, double>::value) {
        if (ctx->green_out)
          for (size_t j = 0; j < cj; ++j) {
            const JobSpec& sp = specs[begin + j];
            if (sp.inst < 0) continue;
            const FrontPlan& P = sp.plan->host;
            const int m = P.fronts[P.root].n, nd = P.nd, k = m - nd;
            std::vector<double2>& g = (*ctx->green_out)[(size_t)sp.inst * ctx->green_blocks + sp.block];
            g.resize((size_t)k * k);
            if (k)
              CK(cudaMemcpy2DAsync(g.data(), (size_t)k * sizeof(double2), rarena + root_off[j] + nd + (size_t)nd * m,
                                   (size_t)m * sizeof(double2), (size_t)k * sizeof(double2), (size_t)k,
                                   cudaMemcpyDeviceToHost, s));
          }
      }
      // Multi-terminal blocks: every T_pq from the root inverse.
      std::vector<MultiJob> mj;
      std::vector<size_t> midx;
      int64_t smax = 1;
      int pmax = 0;
      const SectorRequest* sec = ctx->sector;
      for (size_t j = 0; j < cj; ++j) {
        const JobSpec& sp = specs[begin + j];
        if (sp.sys->nleads <= 0) continue;
        const bool labels = sec && sp.inst >= 0;
        const int P = labels ? sec->P : sp.sys->nleads;
        const std::vector<int32_t>& lp = labels ? sec->hptr[sp.block] : sp.sys->mptr[sp.block];
        for (int a = 0; a < P; ++a)
          for (int b = 0; b < P; ++b)
            smax = std::max<int64_t>(smax, (int64_t)(lp[a + 1] - lp[a]) * (lp[b + 1] - lp[b]));
        pmax = std::max(pmax, P);
        MultiJob m{};
        m.g = rarena + root_off[j];
        if (labels) {
          m.lpos = sec->lpos[sp.block];
          m.lptr = sec->lptr[sp.block];
          m.gamma = sec->gam[(size_t)sp.inst * sec->nblocks + sp.block];
        } else {
          m.lpos = sp.sys->dmpos[sp.block];
          m.lptr = sp.sys->dmptr[sp.block];
          m.gamma = sp.sys->slots[sp.slot].mtab[sp.block];
        }
        m.m = sp.plan->host.fronts[sp.plan->host.root].n;
        m.nd = sp.plan->host.nd;
        m.P = P;
        mj.push_back(m);
        midx.push_back(j);
      }
      std::vector<double> mh;
      if (!mj.empty()) {
        const size_t pairs = (size_t)pmax * pmax;
        double2* scratch = static_cast<double2*>(ctx->mscratch.get(mj.size() * pairs * smax * sizeof(double2)));
        double* mout = static_cast<double*>(ctx->mout.get(mj.size() * pairs * sizeof(double)));
        for (size_t k = 0; k < mj.size(); ++k) {
          mj[k].scratch = scratch + k * pairs * smax;
          mj[k].out = mout + k * pairs;
        }
        MultiJob* dmj = static_cast<MultiJob*>(ctx->mjobs.get(mj.size() * sizeof(MultiJob)));
        CK(cudaMemcpyAsync(dmj, mj.data(), mj.size() * sizeof(MultiJob), cudaMemcpyHostToDevice, s));
        in_pieces(mj.size(), [&](size_t f0, size_t c) {
          launch(K_TRACE, 0.0, 0.0, [&] {
            multi_trace_kernel<TR><<<dim3((unsigned)pairs, (unsigned)c), 256, 0, s>>>(dmj + f0, smax);
          });
        });
        mh.resize(mj.size() * pairs);
        CK(cudaMemcpyAsync(mh.data(), mout, mh.size() * sizeof(double), cudaMemcpyDeviceToHost, s));
        for (size_t k = 0; k < mj.size(); ++k) {
          JobOut& o = out[begin + midx[k]];
          o.tm.clear();
          o.tm.resize((size_t)mj[k].P * mj[k].P);  // filled after the synchronisation below
        }
      }
      CK(cudaEventRecord(ctx->ev1, s));
      CK(cudaMemcpyAsync(th.data(), tdev, cj * sizeof(double), cudaMemcpyDeviceToHost, s));
      if (!mj.empty()) {
        CK(cudaStreamSynchronize(s));
        const size_t pairs = (size_t)pmax * pmax;
        for (size_t k = 0; k < mj.size(); ++k) {
          JobOut& o = out[begin + midx[k]];
          for (size_t q = 0; q < o.tm.size(); ++q) o.tm[q] = mh[k * pairs + q];
        }
      }
    } else {
      if constexpr (std::is_same<T, float>::value && std::is_same<TR, float>::value) {
        std::vector<LevelRange> lr;
        for (const Level& lv : levels) {
          // Every small bucket (at most 96 variables) sweeps a warp per front; the large fronts follow.
          const size_t mid = lv.small_n;
          lr.push_back({lv.tiny0, lv.tiny_n, lv.small0, mid, lv.small0 + mid, lv.small_n - mid + lv.large_n, lv.max_n,
                        std::max(lv.max_large_ne, lv.max_small_n)});
        }
        // Transmissions only: a stalled solve is recomputed in FP64 there (not so for gradients and
        // states, whose callers receive the stalled status).
        RefineDesc* fwd = refine(ctx, sys, specs, begin, cj, lr, max_root, dtasks, jd, arena, arena_off, rarena,
                                 root_off, launch, th, eh, sh, ih, ctx->rb[0], 0, {}, states, !grad && !states);
        for (size_t j = 0; j < cj && j < ctx->steps_tmp.size(); ++j) out[begin + j].steps = ctx->steps_tmp[j];
        if (grad) gradient(ctx, sys, specs, begin, cj, lr, max_root, dtasks, jd, arena, arena_off, rarena, root_off,
                           launch, th, eh, sh, ih, fwd, *grad, out);
      }
    }
    std::vector<int32_t> sdev(cj);
    std::vector<uint8_t> fh(foff);
    CK(cudaMemcpyAsync(sdev.data(), status, cj * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(fh.data(), fail, foff, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    launch.collect();
    float ms = 0.f, mf = 0.f, mr = 0.f;
    CK(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
    CK(cudaEventElapsedTime(&mf, ctx->ev0, ctx->evf));
    CK(cudaEventElapsedTime(&mr, ctx->evf, ctx->evr));
    ctx->last_ms += ms;
    ctx->factor_ms += mf;
    ctx->root_ms += mr;
    ctx->tail_ms += ms - mf - mr;
    std::vector<int> ph(cj, 0);
    CK(cudaMemcpy(ph.data(), pert, cj * sizeof(int), cudaMemcpyDeviceToHost));
    for (size_t j = 0; j < cj; ++j) ctx->refine_iters = std::max<int64_t>(ctx->refine_iters, ih[j]);
    for (size_t j = 0; j < cj; ++j) {
      JobOut& o = out[begin + j];
      o.t = th[j];
      o.err = eh[j];
      o.iters = ih[j];
      int32_t st = sdev[j] != ST_OK ? sdev[j] : sh[j];
      if (st == ST_OK && !std::isfinite(o.t)) st = ST_NONFINITE;
      for (double v : o.tm)
        if (st == ST_OK && !std::isfinite(v)) st = ST_NONFINITE;
      const size_t nf = specs[begin + j].plan->host.fronts.size();
      bool delayed = false;
      for (size_t k = 0; k < nf; ++k) delayed |= fh[fail_off[j] + k] != 0;
      // A timed-out solve keeps its status: its fronts hold garbage that re-planning cannot fix.
      if (delayed && st != ST_TIMEOUT) {
        if (!mixed) {
          st = ST_PIVOT_DELAYED;
          o.fail.assign(fh.begin() + fail_off[j], fh.begin() + fail_off[j] + nf);
        } else {
          st = ST_REFINE_STALLED;
        }
      }
      o.status = st;
      o.perturbed = ph[j];
    }
    begin = end;
  }
  ctx->last_launches += launch.launches;
  ctx->region_launches += launch.launches;
}

// Runs jobs; those with refused pivots are re-planned with the refusing fronts delayed to their
// parents and re-run together, round after round, until none refuses (nested.rs:356-373).
template <typename T, typename TR>
void solve_with_delays(caroli_ctx* ctx, System* sys, const std::vector<JobSpec>& specs, Mode mode,
                       std::vector<JobOut>& out) {
  run_jobs<T, TR>(ctx, sys, specs, mode, out);
  std::vector<size_t> pending;
  std::vector<std::vector<uint8_t>> delayed(specs.size());
  for (size_t j = 0; j < specs.size(); ++j)
    if (out[j].status == ST_PIVOT_DELAYED) {
      pending.push_back(j);
      delayed[j].assign(specs[j].sys->trees[specs[j].block].nodes.size(), 0);
    }
  for (int round = 0; !pending.empty() && round < 64; ++round) {
    std::vector<std::unique_ptr<DevPlan>> plans;
    std::vector<JobSpec> again;
    for (size_t j : pending) {
      const BlockTree& tree = specs[j].sys->trees[specs[j].block];
      for (size_t k = 0; k < tree.nodes.size(); ++k)
        if (k < out[j].fail.size() && out[j].fail[k]) delayed[j][k] = 1;
      auto dp = std::make_unique<DevPlan>();
      dp->host = make_plan(specs[j].sys->desc, tree, delayed[j]);
      dp->upload(ctx->stream);
      again.push_back({specs[j].block, specs[j].slot, specs[j].config, dp.get(), specs[j].sys, specs[j].inst});
      plans.push_back(std::move(dp));
    }
    std::vector<JobOut> res;
    run_jobs<T, TR>(ctx, sys, again, mode, res);
    for (auto& p : plans) p->release();
    std::vector<size_t> next;
    for (size_t q = 0; q < pending.size(); ++q) {
      const size_t j = pending[q];
      bool grew = false;
      if (res[q].status == ST_PIVOT_DELAYED)
        for (size_t k = 0; k < res[q].fail.size() && k < delayed[j].size(); ++k)
          if (res[q].fail[k] && !delayed[j][k]) grew = true;
      out[j] = res[q];
      if (res[q].status == ST_PIVOT_DELAYED) {
        if (grew) next.push_back(j);
        else out[j].status = ST_SINGULAR;
      }
    }
    pending.swap(next);
  }
}

// The autotuner of the f32 factorization: for a plan set not seen before, the factorization (tree
// and root, device time between CUDA events) of up to 256 of its block solves is run under each
// candidate schedule, and the fastest is kept for that plan set and precision. Candidates: the
// largest front factored by one CTA in shared memory (48, 64 or 96 variables; larger fronts take
// the panel sweep and rank-32 updates) x those updates on the tensor cores or on the CUDA cores.
// The trials leave the results and the accounting of the call untouched.
template <typename TR>
void apply_tuning(caroli_ctx* ctx, System* sys, const std::vector<JobSpec>& specs, Mode mode) {
  ctx->small_max_f32 = SMALL_MAX_F32;
  ctx->tc_choice = true;
  ctx->split_choice = false;
  if (specs.empty()) return;
  std::vector<uint64_t> key;
  for (const JobSpec& sp : specs) key.push_back(sp.plan->id);
  std::sort(key.begin(), key.end());
  key.erase(std::unique(key.begin(), key.end()), key.end());
  key.push_back(0xC0FFEE00u + (uint64_t)mode);
  key.push_back(ctx->tensor_cores ? 1 : 0);
  auto it = ctx->tuned.find(key);
  if (it == ctx->tuned.end()) {
    if (!ctx->autotune || ctx->probe >= 0) {
      // The fixed schedule (caroli_set_schedule; by default the tuner's default).
      ctx->small_max_f32 = ctx->fixed_small_max;
      ctx->tc_choice = ctx->fixed_mode >= 1;
      ctx->split_choice = ctx->fixed_mode == 2;
      ctx->last_tune = TuneChoice{};
      ctx->last_tune.small_max = ctx->fixed_small_max;
      ctx->last_tune.tensor_cores = ctx->tensor_cores && ctx->fixed_mode >= 1;
      ctx->last_tune.split = ctx->fixed_mode == 2;
      return;
    }
    // Saved accounting of the call (the trials must not show in it).
    KStat saved[K_COUNT];
    for (int k = 0; k < K_COUNT; ++k) saved[k] = ctx->kstat[k];
    const double s_last = ctx->last_ms, s_f = ctx->factor_ms, s_r = ctx->root_ms, s_t = ctx->tail_ms;
    const int64_t s_ll = ctx->last_launches, s_rl = ctx->region_launches;
    std::vector<JobSpec> sample(specs.begin(), specs.begin() + std::min<size_t>(specs.size(), 256));
    // The default schedule (fronts up to 96 variables in one CTA, rank-32 updates on the tensor
    // cores, or the CUDA cores when they are off) is kept unless a candidate is more than 5 %
    // faster: the schedule also shapes the refinement's preconditioner, which the trials do not
    // time, so a difference within the trials' noise is not worth a change.
    TuneChoice best;
    best.tuned = true;
    best.split = false;
    best.tensor_cores = ctx->tensor_cores;
    double best_ms = INFINITY, default_ms = INFINITY;
    const int cand_small[3] = {48, 64, 96};
    const bool use_graphs = ctx->use_graphs;
    ctx->use_graphs = false;
    ctx->factor_only = true;
    try {
      for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) {
          const bool tcv = b < 2, spl = b == 0;
          if (tcv && !ctx->tensor_cores) { best.ms[a * 3 + b] = NAN; continue; }
          ctx->small_max_f32 = cand_small[a];
          ctx->tc_choice = tcv;
          ctx->split_choice = spl;
          ctx->factor_ms = ctx->root_ms = 0.0;
          std::vector<JobOut> tmp;
          run_jobs<float, TR>(ctx, sys, sample, mode, tmp);
          const double ms = ctx->factor_ms + ctx->root_ms;
          best.ms[a * 3 + b] = ms;
          if (cand_small[a] == SMALL_MAX_F32 && !spl && tcv == ctx->tensor_cores) default_ms = ms;
          if (ms < best_ms) {
            best_ms = ms;
            best.small_max = cand_small[a];
            best.tensor_cores = tcv;
            best.split = spl;
          }
        }
      if (!(best_ms < 0.95 * default_ms)) {
        best.small_max = SMALL_MAX_F32;
        best.tensor_cores = ctx->tensor_cores;
        best.split = false;
      }
    } catch (...) {
      ctx->factor_only = false;
      ctx->use_graphs = use_graphs;
      throw;
    }
    ctx->factor_only = false;
    ctx->use_graphs = use_graphs;
    for (int k = 0; k < K_COUNT; ++k) ctx->kstat[k] = saved[k];
    ctx->last_ms = s_last; ctx->factor_ms = s_f; ctx->root_ms = s_r; ctx->tail_ms = s_t;
    ctx->last_launches = s_ll; ctx->region_launches = s_rl;
    it = ctx->tuned.emplace(key, best).first;
  }
  ctx->small_max_f32 = it->second.small_max;
  ctx->tc_choice = it->second.tensor_cores;
  ctx->split_choice = it->second.split;
  ctx->last_tune = it->second;
}

void solve_jobs(caroli_ctx* ctx, System* sys, const std::vector<JobSpec>& specs, Mode mode, std::vector<JobOut>& out) {
  if (mode == MODE_DOUBLE) {
    solve_with_delays<double, double>(ctx, sys, specs, mode, out);
  } else if (mode == MODE_SINGLE) {
    apply_tuning<double>(ctx, sys, specs, mode);
    solve_with_delays<float, double>(ctx, sys, specs, mode, out);
  } else {
    // Block solves with many right-lead channels go to the FP64 path directly: the refinement
    // carries one right-hand side per channel through every sweep, and past ctx->mixed_max_channels
    // that costs more than the FP64 factorization it replaces (a 32 x 32-site cubic lead has
    // hundreds of open channels; the two-dimensional ribbons have a few).
    std::vector<JobSpec> few;
    std::vector<size_t> few_idx, many_idx;
    for (size_t j = 0; j < specs.size(); ++j) {
      const int c = specs[j].sys->slots[specs[j].slot].channels[specs[j].block];
      if (c > ctx->mixed_max_channels) many_idx.push_back(j);
      else { few.push_back(specs[j]); few_idx.push_back(j); }
    }
    out.assign(specs.size(), JobOut{});
    if (!few.empty()) {
      std::vector<JobOut> fo;
      apply_tuning<float>(ctx, sys, few, mode);
      run_jobs<float, float>(ctx, sys, few, mode, fo);
      for (size_t q = 0; q < few_idx.size(); ++q) out[few_idx[q]] = std::move(fo[q]);
    }
    if (!many_idx.empty()) {
      std::vector<JobSpec> many;
      for (size_t j : many_idx) many.push_back(specs[j]);
      std::vector<JobOut> mo;
      solve_with_delays<double, double>(ctx, sys, many, MODE_DOUBLE, mo);
      for (size_t q = 0; q < many_idx.size(); ++q) out[many_idx[q]] = std::move(mo[q]);
    }
    // Points the reduced precision could not resolve are computed in double precision
    // (precision.rs:102-115 does the same for failed points).
    std::vector<JobSpec> again;
    std::vector<size_t> idx;
    for (size_t j : few_idx)
      if (out[j].status != ST_OK) {
        again.push_back(specs[j]);
        idx.push_back(j);
      }
    if (!again.empty()) {
      const double ms = ctx->last_ms;
      std::vector<JobOut> res;
      solve_with_delays<double, double>(ctx, sys, again, MODE_DOUBLE, res);
      ctx->fallbacks += (int64_t)again.size();
      (void)ms;
      for (size_t q = 0; q < idx.size(); ++q) {
        const int32_t it = out[idx[q]].iters, pt = out[idx[q]].perturbed, st = out[idx[q]].status;
        out[idx[q]] = res[q];
        out[idx[q]].err = 0.0;
        out[idx[q]].iters = it;
        out[idx[q]].perturbed = pt;
        if (out[idx[q]].status == ST_OK) out[idx[q]].status = 100 + st;  // recomputed in double
      }
    }
  }
}

// W with W W^† = Γ for a Hermitian positive semi-definite Γ (m x m, column-major interleaved):
// pivoted Cholesky, stopped when the largest remaining diagonal is below 1e-15 of the largest
// diagonal, just above the rounding noise of Γ = i(Σ - Σ^†). (gamma_root, nested.rs:1036-1047,
// cuts eigenvalues at 1e-12; a Cholesky residual is not aligned with small eigenvalues, so its
// cut must be tighter for T = Tr[Γ_L G W W^† G^†] to keep the reference's full-Γ trace to 1e-12.)
// Returns the number of columns (channels); w is m x columns.
int gamma_factor(const std::vector<double>& g, size_t m, std::vector<double>& w) {
  std::vector<double> dres(m);
  double top = 0.0;
  for (size_t i = 0; i < m; ++i) {
    dres[i] = g[2 * (i + i * m)];
    top = std::max(top, dres[i]);
  }
  std::vector<uint8_t> used(m, 0);
  std::vector<double> cols;  // interleaved, m per column
  const double tol = 1e-15 * top;
  for (size_t k = 0; k < m; ++k) {
    size_t p = m;
    double best = tol;
    for (size_t i = 0; i < m; ++i)
      if (!used[i] && dres[i] > best) { best = dres[i]; p = i; }
    if (p == m) break;
    used[p] = 1;
    const double piv = std::sqrt(dres[p]);
    std::vector<double> col(2 * m);
    for (size_t i = 0; i < m; ++i) {
      double re = g[2 * (i + p * m)], im = g[2 * (i + p * m) + 1];
      for (size_t t = 0; t < k; ++t) {
        const double* c = &cols[2 * m * t];
        // L[i,t] conj(L[p,t])
        re -= c[2 * i] * c[2 * p] + c[2 * i + 1] * c[2 * p + 1];
        im -= c[2 * i + 1] * c[2 * p] - c[2 * i] * c[2 * p + 1];
      }
      col[2 * i] = used[i] && i != p ? 0.0 : re / piv;
      col[2 * i + 1] = used[i] && i != p ? 0.0 : im / piv;
    }
    col[2 * p + 1] = 0.0;
    for (size_t i = 0; i < m; ++i)
      if (!used[i]) dres[i] -= col[2 * i] * col[2 * i] + col[2 * i + 1] * col[2 * i + 1];
    cols.insert(cols.end(), col.begin(), col.end());
  }
  w = cols;
  return (int)(cols.size() / (2 * m));
}

double2* upload_c64(const double* host, size_t count, cudaStream_t s) {
  double2* d = dalloc<double2>(std::max<size_t>(count, 1));
  if (count) CK(cudaMemcpyAsync(d, host, count * sizeof(double2), cudaMemcpyHostToDevice, s));
  return d;
}

}  // namespace

// Defined beside caroli_solve_batch_noalloc, which uses it.
cudaError_t noalloc_lookup(unsigned char** out);

extern "C" {

int caroli_ctx_create(int device_ordinal, caroli_ctx** out) {
  if (!out) return CAROLI_EINVAL;
  *out = nullptr;
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) return CAROLI_EUNAVAILABLE;
  if (device_ordinal < 0 || device_ordinal >= count) return CAROLI_EINVAL;
  auto ctx = std::make_unique<caroli_ctx>();
  ctx->device = device_ordinal;
  try {
    CK(cudaSetDevice(device_ordinal));
    CK(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
    CK(cudaEventCreate(&ctx->ev0));
    CK(cudaEventCreate(&ctx->ev1));
    CK(cudaEventCreate(&ctx->evf));
    CK(cudaEventCreate(&ctx->evr));
    CK(cudaEventCreate(&ctx->reg0));
    CK(cudaEventCreate(&ctx->reg1));
    size_t free_b = 0, total_b = 0;
    CK(cudaMemGetInfo(&free_b, &total_b));
    ctx->mem_budget = free_b / 2;
    int optin = 0;
    CK(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device_ordinal));
    for (auto* k : {(const void*)tc_update_kernel, (const void*)tc_sweep_gemm_kernel,
                    (const void*)small_front_kernel<double, false>, (const void*)small_front_kernel<float, false>,
                    (const void*)small_front_kernel<double, true>, (const void*)small_front_kernel<float, true>,
                    (const void*)small_front_wide_kernel<double, false>, (const void*)small_front_wide_kernel<float, false>,
                    (const void*)small_front_wide_kernel<double, true>, (const void*)small_front_wide_kernel<float, true>,
                    (const void*)inv_finish_kernel<double>, (const void*)inv_finish_kernel<float>,
                    (const void*)inv_panel_kernel<double>, (const void*)inv_panel_kernel<float>,
                    (const void*)tiny_front_kernel<double, false>, (const void*)tiny_front_kernel<double, true>,
                    (const void*)tiny_front_kernel<float, false>, (const void*)tiny_front_kernel<float, true>,
                    (const void*)sweep_rows_fwd_kernel<1>, (const void*)sweep_rows_fwd_kernel<2>,
                    (const void*)sweep_rows_fwd_kernel<4>, (const void*)sweep_rows_fwd_kernel<8>,
                    (const void*)sweep_rows_bwd_kernel<1>, (const void*)sweep_rows_bwd_kernel<2>,
                    (const void*)sweep_rows_bwd_kernel<4>, (const void*)sweep_rows_bwd_kernel<8>,
                    (const void*)sweep_root_kernel<1>, (const void*)sweep_root_kernel<2>,
                    (const void*)sweep_root_kernel<4>, (const void*)sweep_root_kernel<8>}) {
      // Dynamic shared memory up to SMEM_LIMIT, less what the kernel declares statically.
      cudaFuncAttributes fa;
      CK(cudaFuncGetAttributes(&fa, k));
      const int room = std::min<int>(SMEM_LIMIT, optin - (int)fa.sharedSizeBytes);
      CK(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, room));
    }
    // The allocation-free entry point's static scratch: its device address on this device, once,
    // so that caroli_solve_batch_noalloc itself only launches kernels and copies.
    CK(noalloc_lookup(&ctx->noalloc_base));
  } catch (const CudaError& e) {
    g_create_error = std::string(e.what) + ": " + cudaGetErrorString(e.e);
    return CAROLI_ECUDA;
  }
  *out = ctx.release();
  return CAROLI_OK;
}

void caroli_ctx_destroy(caroli_ctx* ctx) {
  if (!ctx) return;
  // Waits for a call of another thread still inside the context (none may start after this).
  { std::lock_guard<std::recursive_mutex> wait(ctx->mu); }
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  ctx->systems.clear();
  if (ctx->ev0) cudaEventDestroy(ctx->ev0);
  if (ctx->ev1) cudaEventDestroy(ctx->ev1);
  if (ctx->evf) cudaEventDestroy(ctx->evf);
  if (ctx->evr) cudaEventDestroy(ctx->evr);
  if (ctx->reg0) cudaEventDestroy(ctx->reg0);
  if (ctx->reg1) cudaEventDestroy(ctx->reg1);
  for (auto& e : ctx->probe_events) {
    cudaEventDestroy(e.first);
    cudaEventDestroy(e.second);
  }
  ctx->fgraph.reset();
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
}

const char* caroli_last_error(const caroli_ctx* ctx) { return ctx ? ctx->err.c_str() : g_create_error.c_str(); }

int caroli_plan_upload(caroli_ctx* ctx, int64_t n, const int64_t* row_ptr, const uint32_t* cols, int64_t nsites,
                       int dim, const int64_t* cells, const int64_t* site_offsets, const int64_t* site_orbitals,
                       const int64_t* range, int64_t n_interior, const int64_t* interior, int nblocks,
                       const int32_t* labels, const int64_t* left_ptr, const int64_t* left,
                       const int64_t* right_ptr, const int64_t* right, int* plan_id) {
  CTX_LOCK(ctx);
  if (!ctx || !plan_id || n < 0 || !row_ptr || (n > 0 && !cols) || dim < 1 || dim > 3 || nblocks < 0)
    return fail_with(ctx, CAROLI_EINVAL, "caroli_plan_upload: bad arguments");
  try {
    CK(cudaSetDevice(ctx->device));
    auto sys = std::make_unique<System>();
    const int64_t nnz = row_ptr[n];
    for (int64_t r = 0; r < n; ++r)
      if (row_ptr[r + 1] < row_ptr[r]) return fail_with(ctx, CAROLI_EINVAL, "row_ptr is not monotone");
    for (int64_t q = 0; q < nnz; ++q)
      if ((int64_t)cols[q] >= n) return fail_with(ctx, CAROLI_EINVAL, "column index out of range");
    for (int64_t i = 0; i < n_interior; ++i)
      if (interior[i] < 0 || interior[i] >= nsites) return fail_with(ctx, CAROLI_EINVAL, "interior site out of range");
    for (int64_t i = 0; i < nsites; ++i)
      if (site_offsets[i] < 0 || site_offsets[i] + site_orbitals[i] > n)
        return fail_with(ctx, CAROLI_EINVAL, "site orbitals outside the matrix");
    for (int b = 0; b < nblocks; ++b)
      for (const int64_t* lst : {left, right})
        for (int64_t q = (lst == left ? left_ptr : right_ptr)[b]; q < (lst == left ? left_ptr : right_ptr)[b + 1]; ++q)
          if (lst[q] < 0 || lst[q] >= n || labels[lst[q]] != b)
            return fail_with(ctx, CAROLI_EINVAL, "lead orbital outside its block");
    sys->row_ptr.assign(row_ptr, row_ptr + n + 1);
    sys->cols.assign(cols, cols + nnz);
    sys->cells.assign(cells, cells + 3 * nsites);
    sys->site_offsets.assign(site_offsets, site_offsets + nsites);
    sys->site_orbitals.assign(site_orbitals, site_orbitals + nsites);
    sys->interior.assign(interior, interior + n_interior);
    sys->labels.assign(labels, labels + n);
    sys->left_ptr.assign(left_ptr, left_ptr + nblocks + 1);
    sys->right_ptr.assign(right_ptr, right_ptr + nblocks + 1);
    sys->left.assign(left, left + left_ptr[nblocks]);
    sys->right.assign(right, right + right_ptr[nblocks]);
    SystemDesc& d = sys->desc;
    d.n = n; d.row_ptr = sys->row_ptr.data(); d.cols = sys->cols.data();
    d.nsites = nsites; d.dim = dim; d.cells = sys->cells.data();
    d.site_offsets = sys->site_offsets.data(); d.site_orbitals = sys->site_orbitals.data();
    for (int a = 0; a < 3; ++a) d.range[a] = std::max<int64_t>(1, range[a]);
    d.n_interior = n_interior; d.interior = sys->interior.data();
    d.nblocks = nblocks; d.labels = sys->labels.data();
    d.left_ptr = sys->left_ptr.data(); d.left = sys->left.data();
    d.right_ptr = sys->right_ptr.data(); d.right = sys->right.data();
    sys->trees = build_trees(d);
    for (int b = 0; b < nblocks; ++b) {
      auto dp = std::make_unique<DevPlan>();
      dp->host = make_plan(d, sys->trees[b], {});
      dp->upload(ctx->stream);
      sys->plans.push_back(std::move(dp));
      const BlockTree& t = sys->trees[b];
      DevBlock B;
      B.nblk = (int32_t)t.orbitals.size();
      B.nnz = (int64_t)t.csr_col.size();
      std::vector<int32_t> sl(B.nblk, -1), sr(B.nblk, -1);
      for (size_t a = 0; a < t.left_local.size(); ++a) sl[t.left_local[a]] = (int32_t)a;
      for (size_t a = 0; a < t.right_local.size(); ++a) sr[t.right_local[a]] = (int32_t)a;
      B.csr_ptr = upload_vec(t.csr_ptr, ctx->stream);
      B.csr_col = upload_vec(t.csr_col, ctx->stream);
      B.csr_q = upload_vec(t.csr_q, ctx->stream);
      B.slice_l = upload_vec(sl, ctx->stream);
      B.slice_r = upload_vec(sr, ctx->stream);
      B.left_local = upload_vec(t.left_local, ctx->stream);
      B.right_local = upload_vec(t.right_local, ctx->stream);
      CK(cudaStreamSynchronize(ctx->stream));
      sys->blocks.push_back(B);
    }
    ctx->systems.push_back(std::move(sys));
    *plan_id = (int)ctx->systems.size() - 1;
    return CAROLI_OK;
  } catch (const CudaError& e) {
    return fail_with(ctx, e.e == cudaErrorMemoryAllocation ? CAROLI_ENOMEM : CAROLI_ECUDA,
                     std::string(e.what) + ": " + cudaGetErrorString(e.e));
  } catch (const std::exception& e) {
    return fail_with(ctx, CAROLI_EINVAL, e.what());
  }
}

int caroli_plan_info(caroli_ctx* ctx, int plan_id, int block, int64_t* fronts, int64_t* max_n, int64_t* max_ne,
                     int64_t* root_n, int64_t* arena_elems) {
  CTX_LOCK(ctx);
  System* sys = ctx ? get_system(ctx, plan_id) : nullptr;
  if (!sys) return fail_with(ctx, CAROLI_EINVAL, "unknown plan");
  if (block < 0 || block >= (int)sys->plans.size()) {
    if (fronts) *fronts = (int64_t)sys->plans.size();
    return CAROLI_OK;
  }
  const FrontPlan& p = sys->plans[block]->host;
  if (fronts) *fronts = (int64_t)p.fronts.size() - 1;
  if (max_n) *max_n = p.max_n;
  if (max_ne) *max_ne = p.max_ne;
  if (root_n) *root_n = p.fronts[p.root].n;
  if (arena_elems) *arena_elems = p.arena_elems;
  return CAROLI_OK;
}

int caroli_plan_fronts(caroli_ctx* ctx, int plan_id, int block, int64_t capacity, int32_t* n, int32_t* ne,
                       int32_t* level, int64_t* count) {
  CTX_LOCK(ctx);
  System* sys = ctx ? get_system(ctx, plan_id) : nullptr;
  if (!sys || block < 0 || block >= (int)sys->plans.size()) return fail_with(ctx, CAROLI_EINVAL, "unknown plan or block");
  const auto& fr = sys->plans[block]->host.fronts;
  const int64_t m = (int64_t)fr.size() - 1;  // tree fronts, without the root
  if (count) *count = m;
  for (int64_t k = 0; k < std::min(m, capacity); ++k) {
    if (n) n[k] = fr[k].n;
    if (ne) ne[k] = fr[k].ne;
    if (level) level[k] = fr[k].level;
  }
  return CAROLI_OK;
}

int caroli_values_upload(caroli_ctx* ctx, int plan_id, int nconfigs, const double* values) {
  CTX_LOCK(ctx);
  System* sys = ctx ? get_system(ctx, plan_id) : nullptr;
  if (!sys || nconfigs <= 0 || !values) return fail_with(ctx, CAROLI_EINVAL, "caroli_values_upload: bad arguments");
  try {
    CK(cudaSetDevice(ctx->device));
    const size_t nnz = (size_t)sys->desc.row_ptr[sys->desc.n];
    const size_t count = nnz * (size_t)nconfigs;
    if (!sys->vals || sys->vals_count != count) {  // the same size re-uses the buffer
      cudaFree(sys->vals);
      sys->vals = nullptr;
      sys->vals_count = 0;
      sys->vals = dalloc<double2>(std::max<size_t>(count, 1));
      sys->vals_count = count;
    }
    if (count) CK(cudaMemcpyAsync(sys->vals, values, count * sizeof(double2), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    sys->nconfigs = nconfigs;
    return CAROLI_OK;
  } catch (const CudaError& e) {
    return fail_with(ctx, e.e == cudaErrorMemoryAllocation ? CAROLI_ENOMEM : CAROLI_ECUDA, cudaGetErrorString(e.e));
  }
}

int caroli_values_generate(caroli_ctx* ctx, int plan_id, const double* clean_values, int nentries,
                           const caroli_disorder* entries, int nconfigs, int first_config) {
  CTX_LOCK(ctx);
  System* sys = ctx ? get_system(ctx, plan_id) : nullptr;
  if (!sys || !clean_values || nentries < 0 || (nentries > 0 && !entries) || nconfigs <= 0 || first_config < 0)
    return fail_with(ctx, CAROLI_EINVAL, "caroli_values_generate: bad arguments");
  const SystemDesc& d = sys->desc;
  const int64_t n = d.n, nnz = d.row_ptr[n], nsites = d.nsites;
  // Site of every orbital, and the stored entries of each site's on-site block.
  std::vector<int32_t> site_of(n, -1);
  for (int64_t i = 0; i < nsites; ++i)
    for (int64_t o = d.site_offsets[i]; o < d.site_offsets[i] + d.site_orbitals[i]; ++o) site_of[o] = (int32_t)i;
  std::vector<int32_t> os_site(std::max<int64_t>(nnz, 1), -1);
  std::vector<int16_t> os_ab(2 * std::max<int64_t>(nnz, 1), 0);
  std::vector<std::vector<uint8_t>> present(nsites);
  for (int64_t r = 0; r < n; ++r)
    for (int64_t q = d.row_ptr[r]; q < d.row_ptr[r + 1]; ++q) {
      const int64_t c = d.cols[q];
      const int32_t si = site_of[r];
      if (si < 0 || site_of[c] != si) continue;
      const int64_t k = d.site_orbitals[si];
      const int a = (int)(r - d.site_offsets[si]), b = (int)(c - d.site_offsets[si]);
      os_site[q] = si;
      os_ab[2 * q] = (int16_t)a;
      os_ab[2 * q + 1] = (int16_t)b;
      if (present[si].empty()) present[si].assign(k * k, 0);
      present[si][a + b * k] = 1;
    }
  // Entries: the pattern must hold every on-site entry a term can make non-zero.
  std::vector<DisorderDev> ent(nentries);
  std::vector<double2> spin;
  std::vector<size_t> spin_off(nentries, 0);
  for (int e = 0; e < nentries; ++e) {
    const caroli_disorder& x = entries[e];
    DisorderDev& y = ent[e];
    y.kind = x.kind;
    y.moments = x.moments;
    y.seed = x.seed;
    y.strength = x.strength;
    y.exchange = x.exchange;
    y.mparam = x.moment_param;
    y.orb = x.orbitals;
    if (x.kind == CAROLI_ANDERSON) {
      for (int64_t i = 0; i < nsites; ++i)
        for (int64_t a = 0; a < d.site_orbitals[i]; ++a)
          if (present[i].empty() || !present[i][a + a * d.site_orbitals[i]])
            return fail_with(ctx, CAROLI_EINVAL, "caroli_values_generate: the pattern lacks an on-site diagonal entry");
    } else if (x.kind == CAROLI_MAGNETIC) {
      if (!x.spin || x.orbitals <= 0 || x.orbitals > 32 || x.concentration < 0.0 || x.concentration > 1.0 ||
          x.moments < CAROLI_MOMENTS_ISOTROPIC || x.moments > CAROLI_MOMENTS_CONE)
        return fail_with(ctx, CAROLI_EINVAL, "caroli_values_generate: bad magnetic entry");
      y.n_imp = (int32_t)(x.concentration * (double)nsites);
      const int64_t k = x.orbitals;
      spin_off[e] = spin.size();
      for (int64_t m = 0; m < 3 * k * k; ++m) spin.push_back(make_double2(x.spin[2 * m], x.spin[2 * m + 1]));
      for (int64_t i = 0; i < nsites; ++i) {
        if (d.site_orbitals[i] != k)
          return fail_with(ctx, CAROLI_EINVAL, "caroli_values_generate: spin matrices of another orbital count");
        // n = z exactly (m_z = 1, or a cone of zero angle): S_x and S_y get exact zeros.
        const bool only_z = (x.moments == CAROLI_MOMENTS_POLARIZED && x.moment_param == 1.0) ||
                            (x.moments == CAROLI_MOMENTS_CONE && x.moment_param == 0.0);
        for (int64_t m = 0; m < k * k; ++m) {
          bool nz = false;
          for (int sidx = only_z ? 2 : 0; sidx < 3; ++sidx)
            nz |= x.spin[2 * (sidx * k * k + m)] != 0.0 || x.spin[2 * (sidx * k * k + m) + 1] != 0.0;
          if (nz && (present[i].empty() || !present[i][m]))
            return fail_with(ctx, CAROLI_EINVAL, "caroli_values_generate: the pattern lacks an on-site entry of the spin");
        }
      }
    } else {
      return fail_with(ctx, CAROLI_EINVAL, "caroli_values_generate: unknown disorder kind");
    }
  }
  try {
    CK(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    if (!sys->os_site) {
      sys->os_site = upload_vec(os_site, s);
      sys->os_ab = upload_vec(os_ab, s);
    }
    double2* dspin = static_cast<double2*>(ctx->dspin.get(std::max<size_t>(spin.size(), 1) * sizeof(double2)));
    if (!spin.empty()) CK(cudaMemcpyAsync(dspin, spin.data(), spin.size() * sizeof(double2), cudaMemcpyHostToDevice, s));
    for (int e = 0; e < nentries; ++e) ent[e].spin = dspin + spin_off[e];
    DisorderDev* dent = static_cast<DisorderDev*>(ctx->dent.get(std::max<size_t>(nentries, 1) * sizeof(DisorderDev)));
    if (nentries) CK(cudaMemcpyAsync(dent, ent.data(), nentries * sizeof(DisorderDev), cudaMemcpyHostToDevice, s));
    const size_t per = (size_t)std::max(nentries, 1) * nconfigs * (size_t)std::max<int64_t>(nsites, 1);
    double* scal = static_cast<double*>(ctx->dscal.get(per * sizeof(double)));
    double* coef = static_cast<double*>(ctx->dcoef.get(per * 3 * sizeof(double)));
    uint8_t* flag = static_cast<uint8_t*>(ctx->dflag.get(per));
    int32_t* tab = static_cast<int32_t*>(ctx->dtab.get(per * sizeof(int32_t)));
    double2* clean = static_cast<double2*>(ctx->dclean.get(std::max<int64_t>(nnz, 1) * sizeof(double2)));
    if (nnz) CK(cudaMemcpyAsync(clean, clean_values, nnz * sizeof(double2), cudaMemcpyHostToDevice, s));
    const size_t count = (size_t)nnz * nconfigs;
    if (!sys->vals || sys->vals_count != count) {
      cudaFree(sys->vals);
      sys->vals = nullptr;
      sys->vals_count = 0;
      sys->vals = dalloc<double2>(std::max<size_t>(count, 1));
      sys->vals_count = count;
    }
    int64_t launches = 0;
    const int threads = nentries * nconfigs;
    if (threads > 0) {
      disorder_draw_kernel<<<(threads + 31) / 32, 32, 0, s>>>(dent, nentries, nconfigs, first_config, (int)nsites, scal,
                                                                coef, flag, tab);
      CK(cudaGetLastError());
      ++launches;
    }
    if (nnz > 0)
      in_pieces((size_t)nconfigs, [&](size_t c0, size_t c) {
        disorder_apply_kernel<<<dim3((unsigned)((nnz + 255) / 256), (unsigned)c), 256, 0, s>>>(
            dent, nentries, nconfigs, (int)nsites, nnz, clean, sys->os_site, sys->os_ab, scal + c0 * nsites,
            coef + c0 * nsites * 3, flag + c0 * nsites, sys->vals + c0 * nnz);
        CK(cudaGetLastError());
        ++launches;
      });
    CK(cudaStreamSynchronize(s));
    ctx->last_launches = launches;
    ctx->region_launches += launches;
    sys->nconfigs = nconfigs;
    return CAROLI_OK;
  } catch (const CudaError& e) {
    return fail_with(ctx, e.e == cudaErrorMemoryAllocation ? CAROLI_ENOMEM : CAROLI_ECUDA,
                     std::string(e.what) + ": " + cudaGetErrorString(e.e));
  }
}

int caroli_values_download(caroli_ctx* ctx, int plan_id, int config, double* values) {
  CTX_LOCK(ctx);
  System* sys = ctx ? get_system(ctx, plan_id) : nullptr;
  if (!sys || !values || !sys->vals || config < 0 || config >= sys->nconfigs)
    return fail_with(ctx, CAROLI_EINVAL, "caroli_values_download: bad arguments");
  try {
    CK(cudaSetDevice(ctx->device));
    const size_t nnz = (size_t)sys->desc.row_ptr[sys->desc.n];
    if (nnz)
      CK(cudaMemcpyAsync(values, sys->vals + (size_t)config * nnz, nnz * sizeof(double2), cudaMemcpyDeviceToHost,
                         ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return CAROLI_OK;
  } catch (const CudaError& e) {
    return fail_with(ctx, CAROLI_ECUDA, cudaGetErrorString(e.e));
  }
}

int caroli_derivs_upload(caroli_ctx* ctx, int plan_id, int nparams, const double* values) {
  CTX_LOCK(ctx);
  System* sys = ctx ? get_system(ctx, plan_id) : nullptr;
  if (!sys || nparams < 0 || (nparams > 0 && !values) || sys->nconfigs <= 0)
    return fail_with(ctx, CAROLI_EINVAL, "caroli_derivs_upload: bad arguments (upload the values first)");
  try {
    CK(cudaSetDevice(ctx->device));
    cudaFree(sys->dvals);
    sys->dvals = nullptr;
    const size_t nnz = (size_t)sys->desc.row_ptr[sys->desc.n];
    if (nparams > 0) sys->dvals = upload_c64(values, nnz * (size_t)nparams * sys->nconfigs, ctx->stream);
    CK(cudaStreamSynchronize(ctx->stream));
    sys->nparams = nparams;
    return CAROLI_OK;
  } catch (const CudaError& e) {
    return fail_with(ctx, e.e == cudaErrorMemoryAllocation ? CAROLI_ENOMEM : CAROLI_ECUDA, cudaGetErrorString(e.e));
  }
}

int caroli_transmission_with_grad(caroli_ctx* ctx, int plan_id, int count, const int32_t* slots,
                                  const int32_t* configs, double* t, int32_t* status, double* dt_dv, double* dt_dp) {
  CTX_LOCK(ctx);
  System* sys = ctx ? get_system(ctx, plan_id) : nullptr;
  if (!sys || count < 0 || (count > 0 && (!slots || !configs || !t || !status || !dt_dv)))
    return fail_with(ctx, CAROLI_EINVAL, "caroli_transmission_with_grad: bad arguments");
  if (sys->nleads > 0) return fail_with(ctx, CAROLI_EINVAL, "caroli_transmission_with_grad: a multi-terminal plan");
  if (!sys->vals) return fail_with(ctx, CAROLI_EINVAL, "no H values uploaded");
  for (int i = 0; i < count; ++i) {
    if (slots[i] < 0 || slots[i] >= (int)sys->slots.size() || !sys->slots[slots[i]].set)
      return fail_with(ctx, CAROLI_EINVAL, "energy slot without self-energies");
    if (configs[i] < 0 || configs[i] >= sys->nconfigs) return fail_with(ctx, CAROLI_EINVAL, "configuration out of range");
  }
  try {
    CK(cudaSetDevice(ctx->device));
    ctx->last_ms = 0.0;
    ctx->last_launches = 0;
    ctx->factor_ms = ctx->root_ms = ctx->tail_ms = 0.0;
    ctx->refine_iters = 0;
    ctx->fallbacks = 0;
    ctx->refine_job_steps = ctx->refine_batch_steps = 0;
    const int nb = (int)sys->plans.size();
    std::vector<JobSpec> specs;
    for (int i = 0; i < count; ++i)
      for (int b = 0; b < nb; ++b) specs.push_back({b, slots[i], configs[i], sys->plans[b].get(), sys});
    GradRequest g;
    g.dvals = sys->dvals;
    g.nparams = sys->dvals ? sys->nparams : 0;
    g.nnz = sys->desc.row_ptr[sys->desc.n];
    std::vector<JobOut> jo;
    apply_tuning<float>(ctx, sys, specs, MODE_MIXED);
    run_jobs<float, float>(ctx, sys, specs, MODE_MIXED, jo, &g);
    const int64_t n = sys->desc.n;
    for (int i = 0; i < count; ++i) {
      double sum = 0.0;
      int32_t st = ST_OK;
      double* dv = dt_dv + (size_t)i * n;
      std::fill(dv, dv + n, 0.0);
      if (dt_dp) std::fill(dt_dp + (size_t)i * g.nparams, dt_dp + (size_t)(i + 1) * g.nparams, 0.0);
      for (int b = 0; b < nb; ++b) {
        const JobOut& o = jo[(size_t)i * nb + b];
        sum += o.t;
        if (st == ST_OK) st = o.status;
        const auto& orbs = sys->trees[b].orbitals;
        for (size_t a = 0; a < o.dv.size() && a < orbs.size(); ++a) dv[orbs[a]] = o.dv[a];
        if (dt_dp)
          for (int k = 0; k < g.nparams && k < (int)o.dp.size(); ++k) dt_dp[(size_t)i * g.nparams + k] += o.dp[k];
      }
      t[i] = sum;
      status[i] = st;
    }
    return CAROLI_OK;
  } catch (const CudaError& e) {
    return fail_with(ctx, e.e == cudaErrorMemoryAllocation ? CAROLI_ENOMEM : CAROLI_ECUDA,
                     std::string(e.what) + ": " + cudaGetErrorString(e.e));
  }
}

int caroli_scattering_states(caroli_ctx* ctx, int plan_id, int count, const int32_t* slots, const int32_t* configs,
                             const double* const* w_left, const int32_t* left_channels, const double* const* w_right,
                             const int32_t* right_channels, double* const* psi_left, double* const* psi_right,
                             int32_t* status) {
  CTX_LOCK(ctx);
  System* sys = ctx ? get_system(ctx, plan_id) : nullptr;
  if (!sys || count < 0 ||
      (count > 0 && (!slots || !configs || !w_left || !left_channels || !w_right || !right_channels || !psi_left ||
                     !psi_right || !status)))
    return fail_with(ctx, CAROLI_EINVAL, "caroli_scattering_states: bad arguments");
  if (sys->nleads > 0) return fail_with(ctx, CAROLI_EINVAL, "caroli_scattering_states: a multi-terminal plan");
  if (!sys->vals) return fail_with(ctx, CAROLI_EINVAL, "no H values uploaded");
  const int nb = (int)sys->plans.size();
  for (int i = 0; i < count; ++i) {
    if (slots[i] < 0 || slots[i] >= (int)sys->slots.size() || !sys->slots[slots[i]].set)
      return fail_with(ctx, CAROLI_EINVAL, "energy slot without self-energies");
    if (configs[i] < 0 || configs[i] >= sys->nconfigs) return fail_with(ctx, CAROLI_EINVAL, "configuration out of range");
    int64_t cl = 0, cr = 0;
    for (int b = 0; b < nb; ++b) {
      const size_t q = (size_t)i * nb + b;
      const int l = left_channels[q], r = right_channels[q];
      if (l < 0 || l > sys->plans[b]->host.nl || r < 0 || r > sys->plans[b]->host.nr || (l && !w_left[q]) ||
          (r && !w_right[q]))
        return fail_with(ctx, CAROLI_EINVAL, "caroli_scattering_states: bad lead factor");
      cl += l;
      cr += r;
    }
    if ((cl && !psi_left[i]) || (cr && !psi_right[i]))
      return fail_with(ctx, CAROLI_EINVAL, "caroli_scattering_states: missing output");
  }
  try {
    CK(cudaSetDevice(ctx->device));
    ctx->last_ms = 0.0;
    ctx->last_launches = 0;
    ctx->factor_ms = ctx->root_ms = ctx->tail_ms = 0.0;
    ctx->refine_iters = 0;
    ctx->fallbacks = 0;
    ctx->refine_job_steps = ctx->refine_batch_steps = 0;
    std::vector<JobSpec> specs;
    StatesRequest rq;
    size_t welems = 0;
    std::vector<size_t> woff;
    for (int i = 0; i < count; ++i)
      for (int b = 0; b < nb; ++b) {
        const size_t q = (size_t)i * nb + b;
        specs.push_back({b, slots[i], configs[i], sys->plans[b].get(), sys});
        rq.cl.push_back(left_channels[q]);
        rq.cr.push_back(right_channels[q]);
        woff.push_back(welems);
        welems += (size_t)sys->plans[b]->host.nl * left_channels[q] + (size_t)sys->plans[b]->host.nr * right_channels[q];
      }
    double2* w = static_cast<double2*>(ctx->states_w.get(std::max<size_t>(welems, 1) * sizeof(double2)));
    for (size_t q = 0; q < specs.size(); ++q) {
      const FrontPlan& P = specs[q].plan->host;
      const size_t nl = (size_t)P.nl * rq.cl[q], nr = (size_t)P.nr * rq.cr[q];
      rq.wl.push_back(w + woff[q]);
      rq.wr.push_back(w + woff[q] + nl);
      if (nl) CK(cudaMemcpyAsync(w + woff[q], w_left[q], nl * sizeof(double2), cudaMemcpyHostToDevice, ctx->stream));
      if (nr) CK(cudaMemcpyAsync(w + woff[q] + nl, w_right[q], nr * sizeof(double2), cudaMemcpyHostToDevice, ctx->stream));
    }
    std::vector<std::vector<double2>> psi(specs.size());
    rq.psi = &psi;
    std::vector<JobOut> jo;
    apply_tuning<float>(ctx, sys, specs, MODE_MIXED);
    run_jobs<float, float>(ctx, sys, specs, MODE_MIXED, jo, nullptr, &rq);
    // Block-local columns to the caller's layout: ψ_L of instance i is n x Σ_b cl_b, block b's
    // columns after those of the blocks before it, zero outside the block's orbitals.
    const int64_t n = sys->desc.n;
    for (int i = 0; i < count; ++i) {
      int64_t cl = 0, cr = 0;
      for (int b = 0; b < nb; ++b) {
        cl += left_channels[(size_t)i * nb + b];
        cr += right_channels[(size_t)i * nb + b];
      }
      if (cl) std::fill(psi_left[i], psi_left[i] + 2 * (size_t)n * cl, 0.0);
      if (cr) std::fill(psi_right[i], psi_right[i] + 2 * (size_t)n * cr, 0.0);
      int32_t st = ST_OK;
      int64_t c0l = 0, c0r = 0;
      for (int b = 0; b < nb; ++b) {
        const size_t q = (size_t)i * nb + b;
        const JobOut& o = jo[q];
        if (st == ST_OK) st = o.status;
        const auto& orbs = sys->trees[b].orbitals;
        const size_t nblk = orbs.size();
        const int l = rq.cl[q], r = rq.cr[q];
        const std::vector<double2>& x = psi[q];
        if (x.size() < nblk * (size_t)(l + r)) {
          if (st == ST_OK) st = ST_NONFINITE;
          continue;
        }
        for (int c = 0; c < l + r; ++c) {
          double* dst = c < l ? psi_left[i] + 2 * (size_t)n * (c0l + c) : psi_right[i] + 2 * (size_t)n * (c0r + c - l);
          for (size_t a = 0; a < nblk; ++a) {
            const double2 v = x[a + c * nblk];
            if (st == ST_OK && !(std::isfinite(v.x) && std::isfinite(v.y))) st = ST_NONFINITE;
            dst[2 * orbs[a]] = v.x;
            dst[2 * orbs[a] + 1] = v.y;
          }
        }
        c0l += l;
        c0r += r;
      }
      status[i] = st;
    }
    return CAROLI_OK;
  } catch (const CudaError& e) {
    return fail_with(ctx, e.e == cudaErrorMemoryAllocation ? CAROLI_ENOMEM : CAROLI_ECUDA,
                     std::string(e.what) + ": " + cudaGetErrorString(e.e));
  }
}

}  // extern "C"

namespace {

// Multi-terminal T_pq in mixed precision: X = A^-1 [W_1 ... W_P] (every lead's sources,
// W_p W_p^† = Γ_p) refined in FP64 from the f32 factors, then T_pq = Σ over lead q's columns of
// x^†(p) Γ_p x(p). Block solves with more than ctx->mixed_max_channels sources, and those the
// refinement cannot resolve, take the FP64 path.
void multi_mixed(caroli_ctx* ctx, System* sys, const std::vector<JobSpec>& specs, std::vector<JobOut>& out) {
  cudaStream_t s = ctx->stream;
  const int P = sys->nleads;
  out.assign(specs.size(), JobOut{});
  std::vector<size_t> few, many;
  for (size_t j = 0; j < specs.size(); ++j) {
    const SigmaSlot& sg = sys->slots[specs[j].slot];
    int c = 0;
    for (int p = 0; p < P; ++p) c += sg.mch[(size_t)specs[j].block * P + p];
    (c > ctx->mixed_max_channels ? many : few).push_back(j);
  }
  std::vector<size_t> again = many;
  if (!few.empty()) {
    std::vector<JobSpec> fs;
    StatesRequest rq;
    std::vector<size_t> roff;
    size_t relems = 0;
    for (size_t j : few) {
      const JobSpec& sp = specs[j];
      fs.push_back(sp);
      int c = 0;
      for (int p = 0; p < P; ++p) c += sys->slots[sp.slot].mch[(size_t)sp.block * P + p];
      rq.cl.push_back(c);
      rq.cr.push_back(0);
      rq.wl.push_back(nullptr);
      rq.wr.push_back(nullptr);
      roff.push_back(relems);
      relems += (size_t)sys->blocks[sp.block].nblk * c;
    }
    double2* rhs = static_cast<double2*>(ctx->states_rhs.get(std::max<size_t>(relems, 1) * sizeof(double2)));
    CK(cudaMemsetAsync(rhs, 0, std::max<size_t>(relems, 1) * sizeof(double2), s));
    for (size_t k = 0; k < fs.size(); ++k) {
      const JobSpec& sp = fs[k];
      const SigmaSlot& sg = sys->slots[sp.slot];
      const int b = sp.block;
      int c0 = 0;
      for (int p = 0; p < P; ++p) {
        const int np = sys->mptr[b][p + 1] - sys->mptr[b][p], c = sg.mch[(size_t)b * P + p];
        if (np && c) {
          scatter_sources_kernel<<<(unsigned)(((int64_t)np * c + 255) / 256), 256, 0, s>>>(
              rhs + roff[k], sys->blocks[b].nblk, c0, sys->blocks[b].left_local, sys->dmpos[b] + sys->mptr[b][p], np,
              sg.mw[(size_t)b * P + p], c);
          CK(cudaGetLastError());
        }
        c0 += c;
      }
      rq.rhs.push_back(rhs + roff[k]);
      MultiJob m{};
      m.lpos = sys->dmpos[b];
      m.lptr = sys->dmptr[b];
      m.gamma = sg.mtab[b];
      m.P = P;
      rq.mtrace.push_back(m);
    }
    std::vector<std::vector<double2>> q(fs.size());
    rq.psi = &q;
    std::vector<JobOut> fo;
    apply_tuning<float>(ctx, sys, fs, MODE_MIXED);
    run_jobs<float, float>(ctx, sys, fs, MODE_MIXED, fo, nullptr, &rq);
    for (size_t k = 0; k < fs.size(); ++k) {
      const size_t j = few[k];
      JobOut& o = out[j];
      o = fo[k];
      o.tm.assign((size_t)P * P, 0.0);
      const SigmaSlot& sg = sys->slots[fs[k].slot];
      const int b = fs[k].block, c = rq.cl[k];
      if (o.status != ST_OK || q[k].size() < (size_t)P * c) {
        again.push_back(j);
        continue;
      }
      int c0 = 0;
      for (int lq = 0; lq < P; ++lq) {
        const int cq = sg.mch[(size_t)b * P + lq];
        for (int p = 0; p < P; ++p)
          for (int cc = c0; cc < c0 + cq; ++cc) o.tm[(size_t)p * P + lq] += q[k][(size_t)p * c + cc].x;
        c0 += cq;
      }
    }
  }
  if (!again.empty()) {
    std::vector<JobSpec> as;
    for (size_t j : again) as.push_back(specs[j]);
    std::vector<JobOut> ao;
    solve_jobs(ctx, sys, as, MODE_DOUBLE, ao);
    for (size_t k = 0; k < again.size(); ++k) out[again[k]] = std::move(ao[k]);
    ctx->fallbacks += (int64_t)(again.size() - many.size());  // the refinement's failures, not the routing
  }
}

}  // namespace

extern "C" {

int caroli_multi_leads(caroli_ctx* ctx, int plan_id, int nleads, const int64_t* lead_ptr, const int64_t* lead_orbitals) {
  CTX_LOCK(ctx);
  System* sys = ctx ? get_system(ctx, plan_id) : nullptr;
  if (!sys || nleads <= 0 || !lead_ptr || !lead_orbitals)
    return fail_with(ctx, CAROLI_EINVAL, "caroli_multi_leads: bad arguments");
  const int nb = (int)sys->plans.size();
  for (int b = 0; b < nb; ++b)
    if (sys->plans[b]->host.nr != 0)
      return fail_with(ctx, CAROLI_EINVAL, "caroli_multi_leads: a multi-terminal plan has no right slice");
  if (lead_ptr[0] != 0) return fail_with(ctx, CAROLI_EINVAL, "caroli_multi_leads: lead_ptr[0] must be 0");
  std::vector<std::vector<int32_t>> mptr(nb), mpos(nb);
  for (int b = 0; b < nb; ++b) {
    // Kept orbitals of the block (its left list) and their positions.
    std::vector<std::pair<int64_t, int32_t>> kept;
    for (int64_t q = sys->left_ptr[b]; q < sys->left_ptr[b + 1]; ++q)
      kept.push_back({sys->left[q], (int32_t)(q - sys->left_ptr[b])});
    std::sort(kept.begin(), kept.end());
    mptr[b].push_back(0);
    for (int p = 0; p < nleads; ++p) {
      const int64_t lo = lead_ptr[(size_t)b * nleads + p], hi = lead_ptr[(size_t)b * nleads + p + 1];
      if (hi < lo) return fail_with(ctx, CAROLI_EINVAL, "caroli_multi_leads: lead_ptr not increasing");
      for (int64_t q = lo; q < hi; ++q) {
        auto it = std::lower_bound(kept.begin(), kept.end(), std::make_pair(lead_orbitals[q], (int32_t)-1));
        if (it == kept.end() || it->first != lead_orbitals[q])
          return fail_with(ctx, CAROLI_EINVAL, "caroli_multi_leads: a lead orbital is not kept in its block");
        mpos[b].push_back(it->second);
      }
      mptr[b].push_back((int32_t)mpos[b].size());
    }
  }
  try {
    CK(cudaSetDevice(ctx->device));
    for (auto* p : sys->dmptr) cudaFree(p);
    for (auto* p : sys->dmpos) cudaFree(p);
    sys->dmptr.clear();
    sys->dmpos.clear();
    for (int b = 0; b < nb; ++b) {
      sys->dmptr.push_back(upload_vec(mptr[b], ctx->stream));
      sys->dmpos.push_back(upload_vec(mpos[b], ctx->stream));
    }
    CK(cudaStreamSynchronize(ctx->stream));
    sys->mptr = std::move(mptr);
    sys->mpos = std::move(mpos);
    sys->nleads = nleads;
    for (auto& sg : sys->slots) sg.set = false;  // self-energies of the old leads
    return CAROLI_OK;
  } catch (const CudaError& e) {
    return fail_with(ctx, e.e == cudaErrorMemoryAllocation ? CAROLI_ENOMEM : CAROLI_ECUDA, cudaGetErrorString(e.e));
  }
}

int caroli_multi_sigma_upload(caroli_ctx* ctx, int plan_id, int slot, double energy, const double* const* sigma) {
  CTX_LOCK(ctx);
  System* sys = ctx ? get_system(ctx, plan_id) : nullptr;
  if (!sys || slot < 0 || !sigma) return fail_with(ctx, CAROLI_EINVAL, "caroli_multi_sigma_upload: bad arguments");
  if (sys->nleads <= 0) return fail_with(ctx, CAROLI_EINVAL, "caroli_multi_sigma_upload: no leads (caroli_multi_leads)");
  const int nb = (int)sys->plans.size(), P = sys->nleads;
  for (int b = 0; b < nb; ++b)
    for (int p = 0; p < P; ++p)
      if (sys->mptr[b][p + 1] > sys->mptr[b][p] && !sigma[(size_t)b * P + p])
        return fail_with(ctx, CAROLI_EINVAL, "caroli_multi_sigma_upload: missing self-energy");
  // Σ of the kept orbitals: every lead's Σ_p added at its positions (nested_multi.rs:309-318).
  std::vector<std::vector<double>> comb(nb), empty(nb);
  std::vector<const double*> pl(nb), pr(nb);
  for (int b = 0; b < nb; ++b) {
    const size_t nl = (size_t)sys->plans[b]->host.nl;
    comb[b].assign(2 * nl * nl, 0.0);
    for (int p = 0; p < P; ++p) {
      const int32_t* pos = sys->mpos[b].data() + sys->mptr[b][p];
      const int np = sys->mptr[b][p + 1] - sys->mptr[b][p];
      const double* sp = sigma[(size_t)b * P + p];
      for (int j = 0; j < np; ++j)
        for (int i = 0; i < np; ++i) {
          comb[b][2 * (pos[i] + pos[j] * nl)] += sp[2 * (i + (size_t)j * np)];
          comb[b][2 * (pos[i] + pos[j] * nl) + 1] += sp[2 * (i + (size_t)j * np) + 1];
        }
    }
    empty[b].assign(2, 0.0);
    pl[b] = comb[b].data();
    pr[b] = empty[b].data();
  }
  int rc = caroli_sigma_upload(ctx, plan_id, slot, energy, pl.data(), pr.data(), nullptr, nullptr);
  if (rc != CAROLI_OK) return rc;
  try {
    SigmaSlot& sg = sys->slots[slot];
    sg.set = false;
    if (sg.mgam.size() != (size_t)nb * P) {
      for (auto* p : sg.mgam) cudaFree(p);
      for (auto* p : sg.mtab) cudaFree(p);
      for (auto* p : sg.mw) cudaFree(p);
      sg.mgam.clear();
      sg.mtab.clear();
      sg.mw.clear();
      for (int b = 0; b < nb; ++b) {
        for (int p = 0; p < P; ++p) {
          const size_t np = (size_t)(sys->mptr[b][p + 1] - sys->mptr[b][p]);
          sg.mgam.push_back(dalloc<double2>(std::max<size_t>(np * np, 1)));
          sg.mw.push_back(dalloc<double2>(std::max<size_t>(np * np, 1)));
        }
        sg.mtab.push_back(dalloc<double2*>((size_t)P));
        CK(cudaMemcpyAsync(sg.mtab[b], sg.mgam.data() + (size_t)b * P, P * sizeof(double2*), cudaMemcpyHostToDevice,
                           ctx->stream));
      }
    }
    std::vector<std::vector<double>> keep;
    sg.mch.assign((size_t)nb * P, 0);
    for (int b = 0; b < nb; ++b)
      for (int p = 0; p < P; ++p) {
        const size_t np = (size_t)(sys->mptr[b][p + 1] - sys->mptr[b][p]);
        if (!np) continue;
        // Γ_p = i (Σ_p - Σ_p^†) (caroli-green/src/lib.rs:67-71).
        const double* sp = sigma[(size_t)b * P + p];
        std::vector<double> g(2 * np * np);
        for (size_t j = 0; j < np; ++j)
          for (size_t i = 0; i < np; ++i) {
            const double dr = sp[2 * (i + j * np)] - sp[2 * (j + i * np)];
            const double di = sp[2 * (i + j * np) + 1] + sp[2 * (j + i * np) + 1];
            g[2 * (i + j * np)] = -di;
            g[2 * (i + j * np) + 1] = dr;
          }
        CK(cudaMemcpyAsync(sg.mgam[(size_t)b * P + p], g.data(), np * np * sizeof(double2), cudaMemcpyHostToDevice,
                           ctx->stream));
        std::vector<double> w;
        sg.mch[(size_t)b * P + p] = gamma_factor(g, np, w);
        if (!w.empty())
          CK(cudaMemcpyAsync(sg.mw[(size_t)b * P + p], w.data(), w.size() / 2 * sizeof(double2), cudaMemcpyHostToDevice,
                             ctx->stream));
        keep.push_back(std::move(g));
        keep.push_back(std::move(w));
      }
    CK(cudaStreamSynchronize(ctx->stream));
    sg.set = true;
    return CAROLI_OK;
  } catch (const CudaError& e) {
    return fail_with(ctx, e.e == cudaErrorMemoryAllocation ? CAROLI_ENOMEM : CAROLI_ECUDA, cudaGetErrorString(e.e));
  }
}

int caroli_multi_transmissions(caroli_ctx* ctx, int plan_id, int count, const int32_t* slots, const int32_t* configs,
                               int precision, double* t, int32_t* status) {
  CTX_LOCK(ctx);
  System* sys = ctx ? get_system(ctx, plan_id) : nullptr;
  if (!sys || count < 0 || (count > 0 && (!slots || !configs || !t || !status)))
    return fail_with(ctx, CAROLI_EINVAL, "caroli_multi_transmissions: bad arguments");
  if (sys->nleads <= 0) return fail_with(ctx, CAROLI_EINVAL, "caroli_multi_transmissions: no leads (caroli_multi_leads)");
  if (precision != CAROLI_DOUBLE && precision != CAROLI_SINGLE && precision != CAROLI_MIXED)
    return fail_with(ctx, CAROLI_EINVAL, "caroli_multi_transmissions: unknown precision");
  if (!sys->vals) return fail_with(ctx, CAROLI_EINVAL, "no H values uploaded");
  for (int i = 0; i < count; ++i) {
    if (slots[i] < 0 || slots[i] >= (int)sys->slots.size() || !sys->slots[slots[i]].set ||
        sys->slots[slots[i]].mtab.empty())
      return fail_with(ctx, CAROLI_EINVAL, "energy slot without multi-terminal self-energies");
    if (configs[i] < 0 || configs[i] >= sys->nconfigs) return fail_with(ctx, CAROLI_EINVAL, "configuration out of range");
  }
  try {
    CK(cudaSetDevice(ctx->device));
    ctx->last_ms = 0.0;
    ctx->last_launches = 0;
    ctx->factor_ms = ctx->root_ms = ctx->tail_ms = 0.0;
    ctx->fallbacks = 0;
    ctx->refine_iters = 0;
    ctx->refine_job_steps = ctx->refine_batch_steps = 0;
    const int nb = (int)sys->plans.size(), P = sys->nleads;
    std::vector<JobSpec> specs;
    for (int i = 0; i < count; ++i)
      for (int b = 0; b < nb; ++b) specs.push_back({b, slots[i], configs[i], sys->plans[b].get(), sys});
    std::vector<JobOut> jo;
    if (precision == CAROLI_MIXED) multi_mixed(ctx, sys, specs, jo);
    else solve_jobs(ctx, sys, specs, (Mode)precision, jo);
    for (int i = 0; i < count; ++i) {
      double* ti = t + (size_t)i * P * P;
      std::fill(ti, ti + (size_t)P * P, 0.0);
      int32_t st = ST_OK;
      for (int b = 0; b < nb; ++b) {
        const JobOut& o = jo[(size_t)i * nb + b];
        if (st == ST_OK) st = o.status;
        for (size_t q = 0; q < o.tm.size() && q < (size_t)P * P; ++q) ti[q] += o.tm[q];
      }
      status[i] = st;
    }
    return CAROLI_OK;
  } catch (const CudaError& e) {
    return fail_with(ctx, e.e == cudaErrorMemoryAllocation ? CAROLI_ENOMEM : CAROLI_ECUDA,
                     std::string(e.what) + ": " + cudaGetErrorString(e.e));
  }
}

}  // extern "C"

namespace {

// The device buffers of energy slot `slot` (sized by the blocks' lead slices, W_R for up to nr
// channels), allocated on first use: uploading the next energy into a slot only copies. The slot
// is marked unset until its caller has filled it.
SigmaSlot& slot_buffers(System* sys, int slot) {
  if ((int)sys->slots.size() <= slot) sys->slots.resize(slot + 1);
  SigmaSlot& sg = sys->slots[slot];
  const size_t nblocks = sys->plans.size();
  if (sg.sl.size() != nblocks) {
    for (auto* v : {&sg.sl, &sg.sr, &sg.gl, &sg.gr, &sg.wr}) {
      for (auto* p : *v) cudaFree(p);
      v->clear();
    }
    for (size_t b = 0; b < nblocks; ++b) {
      const size_t nl = sys->plans[b]->host.nl, nr = sys->plans[b]->host.nr;
      sg.sl.push_back(dalloc<double2>(std::max<size_t>(nl * nl, 1)));
      sg.sr.push_back(dalloc<double2>(std::max<size_t>(nr * nr, 1)));
      sg.gl.push_back(dalloc<double2>(std::max<size_t>(nl * nl, 1)));
      sg.gr.push_back(dalloc<double2>(std::max<size_t>(nr * nr, 1)));
      sg.wr.push_back(dalloc<double2>(std::max<size_t>(nr * nr, 1)));
    }
  }
  sg.channels.assign(nblocks, 0);
  sg.set = false;
  return sg;
}

}  // namespace

extern "C" {

int caroli_root_green(caroli_ctx* ctx, int plan_id, int count, const int32_t* slots, const int32_t* configs,
                      double* const* g, int32_t* kept, int32_t* status) {
  CTX_LOCK(ctx);
  System* sys = ctx ? get_system(ctx, plan_id) : nullptr;
  if (!sys || count < 0 || (count > 0 && (!slots || !configs || !g || !kept || !status)))
    return fail_with(ctx, CAROLI_EINVAL, "caroli_root_green: bad arguments");
  if (!sys->vals) return fail_with(ctx, CAROLI_EINVAL, "no H values uploaded");
  const int nb = (int)sys->plans.size();
  for (int i = 0; i < count; ++i) {
    if (slots[i] < 0 || slots[i] >= (int)sys->slots.size() || !sys->slots[slots[i]].set)
      return fail_with(ctx, CAROLI_EINVAL, "energy slot without self-energies");
    if (configs[i] < 0 || configs[i] >= sys->nconfigs) return fail_with(ctx, CAROLI_EINVAL, "configuration out of range");
    for (int b = 0; b < nb; ++b)
      if (!g[(size_t)i * nb + b]) return fail_with(ctx, CAROLI_EINVAL, "caroli_root_green: missing output");
  }
  try {
    CK(cudaSetDevice(ctx->device));
    ctx->last_ms = 0.0;
    ctx->last_launches = 0;
    ctx->factor_ms = ctx->root_ms = ctx->tail_ms = 0.0;
    ctx->fallbacks = 0;
    ctx->refine_iters = 0;
    ctx->refine_job_steps = ctx->refine_batch_steps = 0;
    std::vector<JobSpec> specs;
    for (int i = 0; i < count; ++i)
      for (int b = 0; b < nb; ++b) specs.push_back({b, slots[i], configs[i], sys->plans[b].get(), sys, i});
    std::vector<std::vector<double2>> out((size_t)count * nb);
    std::vector<JobOut> jo;
    ctx->green_out = &out;
    ctx->green_blocks = nb;
    try {
      solve_jobs(ctx, sys, specs, MODE_DOUBLE, jo);
    } catch (...) {
      ctx->green_out = nullptr;
      throw;
    }
    ctx->green_out = nullptr;
    for (int i = 0; i < count; ++i) {
      int32_t st = ST_OK;
      for (int b = 0; b < nb; ++b) {
        const size_t q = (size_t)i * nb + b;
        if (st == ST_OK) st = jo[q].status;
        const FrontPlan& P = sys->plans[b]->host;
        const int k = P.nl + (P.rpos == 0 && P.nr ? 0 : P.nr);
        kept[q] = k;
        for (size_t e = 0; e < out[q].size() && e < (size_t)k * k; ++e) {
          g[q][2 * e] = out[q][e].x;
          g[q][2 * e + 1] = out[q][e].y;
        }
      }
      status[i] = st;
    }
    return CAROLI_OK;
  } catch (const CudaError& e) {
    ctx->green_out = nullptr;
    return fail_with(ctx, e.e == cudaErrorMemoryAllocation ? CAROLI_ENOMEM : CAROLI_ECUDA,
                     std::string(e.what) + ": " + cudaGetErrorString(e.e));
  }
}

int caroli_transmission_matrix(caroli_ctx* ctx, int plan_id, int count, const int32_t* slots, const int32_t* configs,
                               const double* const* w_left, const int32_t* left_channels, double* const* t,
                               int32_t* right_channels, int32_t* status) {
  CTX_LOCK(ctx);
  System* sys = ctx ? get_system(ctx, plan_id) : nullptr;
  if (!sys || count < 0 ||
      (count > 0 && (!slots || !configs || !w_left || !left_channels || !t || !right_channels || !status)))
    return fail_with(ctx, CAROLI_EINVAL, "caroli_transmission_matrix: bad arguments");
  if (sys->nleads > 0) return fail_with(ctx, CAROLI_EINVAL, "caroli_transmission_matrix: a multi-terminal plan");
  if (!sys->vals) return fail_with(ctx, CAROLI_EINVAL, "no H values uploaded");
  const int nb = (int)sys->plans.size();
  for (int i = 0; i < count; ++i) {
    if (slots[i] < 0 || slots[i] >= (int)sys->slots.size() || !sys->slots[slots[i]].set)
      return fail_with(ctx, CAROLI_EINVAL, "energy slot without self-energies");
    if (configs[i] < 0 || configs[i] >= sys->nconfigs) return fail_with(ctx, CAROLI_EINVAL, "configuration out of range");
    for (int b = 0; b < nb; ++b) {
      const size_t q = (size_t)i * nb + b;
      if (left_channels[q] < 0 || left_channels[q] > sys->plans[b]->host.nl || (left_channels[q] && !w_left[q]) ||
          !t[q])
        return fail_with(ctx, CAROLI_EINVAL, "caroli_transmission_matrix: bad lead factor or output");
    }
  }
  try {
    CK(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    ctx->last_ms = 0.0;
    ctx->last_launches = 0;
    ctx->factor_ms = ctx->root_ms = ctx->tail_ms = 0.0;
    ctx->refine_iters = 0;
    ctx->fallbacks = 0;
    ctx->refine_job_steps = ctx->refine_batch_steps = 0;
    std::vector<JobSpec> specs;
    StatesRequest rq;
    size_t welems = 0;
    std::vector<size_t> woff;
    for (int i = 0; i < count; ++i)
      for (int b = 0; b < nb; ++b) {
        const size_t q = (size_t)i * nb + b;
        const SigmaSlot& sg = sys->slots[slots[i]];
        specs.push_back({b, slots[i], configs[i], sys->plans[b].get(), sys, i});
        rq.wl.push_back(nullptr);
        rq.wr.push_back(sg.wr[b]);
        rq.cl.push_back(0);
        rq.cr.push_back(sg.channels[b]);
        rq.tcl.push_back(left_channels[q]);
        woff.push_back(welems);
        welems += (size_t)sys->plans[b]->host.nl * left_channels[q];
      }
    double2* wd = static_cast<double2*>(ctx->states_w.get(std::max<size_t>(welems, 1) * sizeof(double2)));
    for (size_t q = 0; q < specs.size(); ++q) {
      const size_t nl = (size_t)specs[q].plan->host.nl * rq.tcl[q];
      if (nl) CK(cudaMemcpyAsync(wd + woff[q], w_left[q], nl * sizeof(double2), cudaMemcpyHostToDevice, s));
      rq.twl.push_back(wd + woff[q]);
    }
    CK(cudaStreamSynchronize(s));
    std::vector<std::vector<double2>> tm(specs.size());
    rq.psi = &tm;
    std::vector<JobOut> jo;
    apply_tuning<float>(ctx, sys, specs, MODE_MIXED);
    run_jobs<float, float>(ctx, sys, specs, MODE_MIXED, jo, nullptr, &rq);
    for (int i = 0; i < count; ++i) {
      int32_t st = ST_OK;
      for (int b = 0; b < nb; ++b) {
        const size_t q = (size_t)i * nb + b;
        if (st == ST_OK) st = jo[q].status;
        right_channels[q] = rq.cr[q];
        const size_t cnt = (size_t)rq.tcl[q] * rq.cr[q];
        for (size_t e = 0; e < cnt && e < tm[q].size(); ++e) {
          t[q][2 * e] = tm[q][e].x;
          t[q][2 * e + 1] = tm[q][e].y;
          if (st == ST_OK && !(std::isfinite(tm[q][e].x) && std::isfinite(tm[q][e].y))) st = ST_NONFINITE;
        }
      }
      status[i] = st;
    }
    return CAROLI_OK;
  } catch (const CudaError& e) {
    return fail_with(ctx, e.e == cudaErrorMemoryAllocation ? CAROLI_ENOMEM : CAROLI_ECUDA,
                     std::string(e.what) + ": " + cudaGetErrorString(e.e));
  }
}

int caroli_multi_sector_transmissions(caroli_ctx* ctx, int plan_id, int count, const int32_t* slots,
                                      const int32_t* configs, int precision, int nlabels, const int32_t* label_lead,
                                      const double* const* gammas, double* t, int32_t* status) {
  CTX_LOCK(ctx);
  System* sys = ctx ? get_system(ctx, plan_id) : nullptr;
  if (!sys || count < 0 || nlabels <= 0 || !label_lead ||
      (count > 0 && (!slots || !configs || !gammas || !t || !status)))
    return fail_with(ctx, CAROLI_EINVAL, "caroli_multi_sector_transmissions: bad arguments");
  if (sys->nleads <= 0) return fail_with(ctx, CAROLI_EINVAL, "caroli_multi_sector_transmissions: no leads");
  if (precision != CAROLI_DOUBLE && precision != CAROLI_SINGLE)
    return fail_with(ctx, CAROLI_EINVAL, "caroli_multi_sector_transmissions: CAROLI_DOUBLE or CAROLI_SINGLE");
  if (!sys->vals) return fail_with(ctx, CAROLI_EINVAL, "no H values uploaded");
  const int nb = (int)sys->plans.size(), P = nlabels;
  for (int k = 0; k < P; ++k)
    if (label_lead[k] < 0 || label_lead[k] >= sys->nleads)
      return fail_with(ctx, CAROLI_EINVAL, "caroli_multi_sector_transmissions: label of an unknown lead");
  for (int i = 0; i < count; ++i) {
    if (slots[i] < 0 || slots[i] >= (int)sys->slots.size() || !sys->slots[slots[i]].set ||
        sys->slots[slots[i]].mtab.empty())
      return fail_with(ctx, CAROLI_EINVAL, "energy slot without multi-terminal self-energies");
    if (configs[i] < 0 || configs[i] >= sys->nconfigs) return fail_with(ctx, CAROLI_EINVAL, "configuration out of range");
    for (int b = 0; b < nb; ++b)
      for (int k = 0; k < P; ++k) {
        const int p = label_lead[k];
        if (sys->mptr[b][p + 1] > sys->mptr[b][p] && !gammas[((size_t)i * nb + b) * P + k])
          return fail_with(ctx, CAROLI_EINVAL, "caroli_multi_sector_transmissions: missing Γ");
      }
  }
  try {
    CK(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    ctx->last_ms = 0.0;
    ctx->last_launches = 0;
    ctx->factor_ms = ctx->root_ms = ctx->tail_ms = 0.0;
    ctx->fallbacks = 0;
    ctx->refine_iters = 0;
    ctx->refine_job_steps = ctx->refine_batch_steps = 0;
    SectorRequest rq;
    rq.P = P;
    rq.nblocks = nb;
    // Label positions per block: those of the label's lead.
    std::vector<int32_t> hpos, hptr;
    std::vector<size_t> pos_off(nb), ptr_off(nb);
    for (int b = 0; b < nb; ++b) {
      std::vector<int32_t> lp(1, 0);
      pos_off[b] = hpos.size();
      for (int k = 0; k < P; ++k) {
        const int p = label_lead[k];
        for (int32_t q = sys->mptr[b][p]; q < sys->mptr[b][p + 1]; ++q) hpos.push_back(sys->mpos[b][q]);
        lp.push_back((int32_t)(hpos.size() - pos_off[b]));
      }
      ptr_off[b] = hptr.size();
      hptr.insert(hptr.end(), lp.begin(), lp.end());
      rq.hptr.push_back(lp);
    }
    int32_t* dpos = static_cast<int32_t*>(ctx->sec_pos.get(std::max<size_t>(hpos.size(), 1) * sizeof(int32_t)));
    int32_t* dptr = static_cast<int32_t*>(ctx->sec_ptr.get(std::max<size_t>(hptr.size(), 1) * sizeof(int32_t)));
    if (!hpos.empty()) CK(cudaMemcpyAsync(dpos, hpos.data(), hpos.size() * sizeof(int32_t), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(dptr, hptr.data(), hptr.size() * sizeof(int32_t), cudaMemcpyHostToDevice, s));
    for (int b = 0; b < nb; ++b) {
      rq.lpos.push_back(dpos + pos_off[b]);
      rq.lptr.push_back(dptr + ptr_off[b]);
    }
    // Γ of every (instance, block, label), and per (instance, block) a table of P pointers.
    size_t gel = 0;
    std::vector<size_t> goff((size_t)count * nb * P);
    for (int i = 0; i < count; ++i)
      for (int b = 0; b < nb; ++b)
        for (int k = 0; k < P; ++k) {
          const size_t np = (size_t)(rq.hptr[b][k + 1] - rq.hptr[b][k]);
          goff[((size_t)i * nb + b) * P + k] = gel;
          gel += np * np;
        }
    double2* dg = static_cast<double2*>(ctx->sec_gam.get(std::max<size_t>(gel, 1) * sizeof(double2)));
    const double2** dtab =
        static_cast<const double2**>(ctx->sec_tab.get(std::max<size_t>((size_t)count * nb * P, 1) * sizeof(double2*)));
    std::vector<const double2*> htab((size_t)count * nb * P);
    for (int i = 0; i < count; ++i)
      for (int b = 0; b < nb; ++b)
        for (int k = 0; k < P; ++k) {
          const size_t q = ((size_t)i * nb + b) * P + k;
          const size_t np = (size_t)(rq.hptr[b][k + 1] - rq.hptr[b][k]);
          htab[q] = dg + goff[q];
          if (np) CK(cudaMemcpyAsync(dg + goff[q], gammas[q], np * np * sizeof(double2), cudaMemcpyHostToDevice, s));
        }
    if (!htab.empty())
      CK(cudaMemcpyAsync(dtab, htab.data(), htab.size() * sizeof(double2*), cudaMemcpyHostToDevice, s));
    for (int i = 0; i < count; ++i)
      for (int b = 0; b < nb; ++b) rq.gam.push_back(dtab + ((size_t)i * nb + b) * P);
    CK(cudaStreamSynchronize(s));
    std::vector<JobSpec> specs;
    for (int i = 0; i < count; ++i)
      for (int b = 0; b < nb; ++b) specs.push_back({b, slots[i], configs[i], sys->plans[b].get(), sys, i});
    std::vector<JobOut> jo;
    ctx->sector = &rq;
    try {
      solve_jobs(ctx, sys, specs, (Mode)precision, jo);
    } catch (...) {
      ctx->sector = nullptr;
      throw;
    }
    ctx->sector = nullptr;
    for (int i = 0; i < count; ++i) {
      double* ti = t + (size_t)i * P * P;
      std::fill(ti, ti + (size_t)P * P, 0.0);
      int32_t st = ST_OK;
      for (int b = 0; b < nb; ++b) {
        const JobOut& o = jo[(size_t)i * nb + b];
        if (st == ST_OK) st = o.status;
        for (size_t q = 0; q < o.tm.size() && q < (size_t)P * P; ++q) ti[q] += o.tm[q];
      }
      status[i] = st;
    }
    return CAROLI_OK;
  } catch (const CudaError& e) {
    ctx->sector = nullptr;
    return fail_with(ctx, e.e == cudaErrorMemoryAllocation ? CAROLI_ENOMEM : CAROLI_ECUDA,
                     std::string(e.what) + ": " + cudaGetErrorString(e.e));
  }
}

int caroli_multi_scattering_states(caroli_ctx* ctx, int plan_id, int count, const int32_t* slots,
                                   const int32_t* configs, const double* const* w, const int32_t* channels,
                                   double* const* psi, int32_t* status) {
  CTX_LOCK(ctx);
  System* sys = ctx ? get_system(ctx, plan_id) : nullptr;
  if (!sys || count < 0 || (count > 0 && (!slots || !configs || !w || !channels || !psi || !status)))
    return fail_with(ctx, CAROLI_EINVAL, "caroli_multi_scattering_states: bad arguments");
  if (sys->nleads <= 0) return fail_with(ctx, CAROLI_EINVAL, "caroli_multi_scattering_states: no leads");
  if (!sys->vals) return fail_with(ctx, CAROLI_EINVAL, "no H values uploaded");
  const int nb = (int)sys->plans.size(), P = sys->nleads;
  for (int i = 0; i < count; ++i) {
    if (slots[i] < 0 || slots[i] >= (int)sys->slots.size() || !sys->slots[slots[i]].set ||
        sys->slots[slots[i]].mtab.empty())
      return fail_with(ctx, CAROLI_EINVAL, "energy slot without multi-terminal self-energies");
    if (configs[i] < 0 || configs[i] >= sys->nconfigs) return fail_with(ctx, CAROLI_EINVAL, "configuration out of range");
    for (int p = 0; p < P; ++p) {
      int64_t cols = 0;
      for (int b = 0; b < nb; ++b) {
        const size_t q = ((size_t)i * nb + b) * P + p;
        const int np = sys->mptr[b][p + 1] - sys->mptr[b][p];
        if (channels[q] < 0 || channels[q] > np || (channels[q] && !w[q]))
          return fail_with(ctx, CAROLI_EINVAL, "caroli_multi_scattering_states: bad lead factor");
        cols += channels[q];
      }
      if (cols && !psi[(size_t)i * P + p]) return fail_with(ctx, CAROLI_EINVAL, "caroli_multi_scattering_states: missing output");
    }
  }
  try {
    CK(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    ctx->last_ms = 0.0;
    ctx->last_launches = 0;
    ctx->factor_ms = ctx->root_ms = ctx->tail_ms = 0.0;
    ctx->refine_iters = 0;
    ctx->fallbacks = 0;
    ctx->refine_job_steps = ctx->refine_batch_steps = 0;
    std::vector<JobSpec> specs;
    StatesRequest rq;
    std::vector<size_t> roff, woff;
    size_t relems = 0, welems = 0;
    for (int i = 0; i < count; ++i)
      for (int b = 0; b < nb; ++b) {
        specs.push_back({b, slots[i], configs[i], sys->plans[b].get(), sys});
        int c = 0;
        for (int p = 0; p < P; ++p) {
          const size_t q = ((size_t)i * nb + b) * P + p;
          woff.push_back(welems);
          welems += (size_t)(sys->mptr[b][p + 1] - sys->mptr[b][p]) * channels[q];
          c += channels[q];
        }
        rq.cl.push_back(c);
        rq.cr.push_back(0);
        roff.push_back(relems);
        relems += (size_t)sys->blocks[b].nblk * c;
      }
    double2* rhs = static_cast<double2*>(ctx->states_rhs.get(std::max<size_t>(relems, 1) * sizeof(double2)));
    double2* wd = static_cast<double2*>(ctx->states_w.get(std::max<size_t>(welems, 1) * sizeof(double2)));
    CK(cudaMemsetAsync(rhs, 0, std::max<size_t>(relems, 1) * sizeof(double2), s));
    for (size_t j = 0; j < specs.size(); ++j) {
      const int b = specs[j].block;
      int c0 = 0;
      for (int p = 0; p < P; ++p) {
        const size_t q = j * P + p;
        const int np = sys->mptr[b][p + 1] - sys->mptr[b][p], c = channels[q];
        if (np && c) {
          CK(cudaMemcpyAsync(wd + woff[q], w[q], (size_t)np * c * sizeof(double2), cudaMemcpyHostToDevice, s));
          scatter_sources_kernel<<<(unsigned)(((int64_t)np * c + 255) / 256), 256, 0, s>>>(
              rhs + roff[j], sys->blocks[b].nblk, c0, sys->blocks[b].left_local, sys->dmpos[b] + sys->mptr[b][p], np,
              wd + woff[q], c);
          CK(cudaGetLastError());
        }
        c0 += c;
      }
      rq.rhs.push_back(rhs + roff[j]);
      rq.wl.push_back(nullptr);
      rq.wr.push_back(nullptr);
    }
    CK(cudaStreamSynchronize(s));
    std::vector<std::vector<double2>> x(specs.size());
    rq.psi = &x;
    std::vector<JobOut> jo;
    apply_tuning<float>(ctx, sys, specs, MODE_MIXED);
    run_jobs<float, float>(ctx, sys, specs, MODE_MIXED, jo, nullptr, &rq);
    const int64_t n = sys->desc.n;
    for (int i = 0; i < count; ++i) {
      int32_t st = ST_OK;
      for (int p = 0; p < P; ++p) {
        int64_t cols = 0;
        for (int b = 0; b < nb; ++b) cols += channels[((size_t)i * nb + b) * P + p];
        if (cols) std::fill(psi[(size_t)i * P + p], psi[(size_t)i * P + p] + 2 * (size_t)n * cols, 0.0);
      }
      std::vector<int64_t> c0p(P, 0);  // next output column of each lead
      for (int b = 0; b < nb; ++b) {
        const size_t j = (size_t)i * nb + b;
        if (st == ST_OK) st = jo[j].status;
        const auto& orbs = sys->trees[b].orbitals;
        const size_t nblk = orbs.size();
        int c0 = 0;
        for (int p = 0; p < P; ++p) {
          const int c = channels[j * P + p];
          for (int k = 0; k < c; ++k) {
            if (x[j].size() < nblk * (size_t)(c0 + k + 1)) {
              if (st == ST_OK) st = ST_NONFINITE;
              continue;
            }
            double* dst = psi[(size_t)i * P + p] + 2 * (size_t)n * (c0p[p] + k);
            for (size_t a = 0; a < nblk; ++a) {
              const double2 v = x[j][a + (size_t)(c0 + k) * nblk];
              if (st == ST_OK && !(std::isfinite(v.x) && std::isfinite(v.y))) st = ST_NONFINITE;
              dst[2 * orbs[a]] = v.x;
              dst[2 * orbs[a] + 1] = v.y;
            }
          }
          c0 += c;
          c0p[p] += c;
        }
      }
      status[i] = st;
    }
    return CAROLI_OK;
  } catch (const CudaError& e) {
    return fail_with(ctx, e.e == cudaErrorMemoryAllocation ? CAROLI_ENOMEM : CAROLI_ECUDA,
                     std::string(e.what) + ": " + cudaGetErrorString(e.e));
  }
}

int caroli_gamma_override(caroli_ctx* ctx, int plan_id, int slot, const double* const* gamma_l,
                          const double* const* gamma_r) {
  CTX_LOCK(ctx);
  System* sys = ctx ? get_system(ctx, plan_id) : nullptr;
  if (!sys || slot < 0 || slot >= (int)sys->slots.size() || !sys->slots[slot].set || !gamma_l || !gamma_r)
    return fail_with(ctx, CAROLI_EINVAL, "caroli_gamma_override: bad arguments");
  try {
    CK(cudaSetDevice(ctx->device));
    SigmaSlot& sg = sys->slots[slot];
    for (size_t b = 0; b < sys->plans.size(); ++b) {
      const size_t nl = sys->plans[b]->host.nl, nr = sys->plans[b]->host.nr;
      if (nl && gamma_l[b])
        CK(cudaMemcpyAsync(sg.gl[b], gamma_l[b], nl * nl * sizeof(double2), cudaMemcpyHostToDevice, ctx->stream));
      if (nr && gamma_r[b])
        CK(cudaMemcpyAsync(sg.gr[b], gamma_r[b], nr * nr * sizeof(double2), cudaMemcpyHostToDevice, ctx->stream));
    }
    CK(cudaStreamSynchronize(ctx->stream));
    return CAROLI_OK;
  } catch (const CudaError& e) {
    return fail_with(ctx, CAROLI_ECUDA, cudaGetErrorString(e.e));
  }
}

int caroli_lead_modes(caroli_ctx* ctx, int plan_id, int block, int side, int n, const double* y, double sc) {
  CTX_LOCK(ctx);
  System* sys = ctx ? get_system(ctx, plan_id) : nullptr;
  if (!sys || block < 0 || block >= (int)sys->plans.size() || (side != 0 && side != 1) || !y)
    return fail_with(ctx, CAROLI_EINVAL, "caroli_lead_modes: bad arguments");
  const FrontPlan& P = sys->plans[block]->host;
  if (n != (side == 0 ? P.nl : P.nr)) return fail_with(ctx, CAROLI_EINVAL, "caroli_lead_modes: n is not the slice size");
  try {
    CK(cudaSetDevice(ctx->device));
    const size_t nb = sys->plans.size();
    if (sys->lead_y[side].size() != nb) {
      sys->lead_y[side].assign(nb, nullptr);
      sys->lead_sc[side].assign(nb, 0.0);
    }
    cudaFree(sys->lead_y[side][block]);
    sys->lead_y[side][block] = dalloc<double2>(std::max<size_t>((size_t)n * n, 1));
    if (n) CK(cudaMemcpyAsync(sys->lead_y[side][block], y, (size_t)n * n * sizeof(double2), cudaMemcpyHostToDevice,
                              ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    sys->lead_sc[side][block] = sc;
    return CAROLI_OK;
  } catch (const CudaError& e) {
    return fail_with(ctx, e.e == cudaErrorMemoryAllocation ? CAROLI_ENOMEM : CAROLI_ECUDA, cudaGetErrorString(e.e));
  }
}

int caroli_sigma_from_modes(caroli_ctx* ctx, int plan_id, int slot, double energy, const double* const* d_left,
                            const double* const* d_right, const int32_t* channels, const int32_t* const* channel_modes,
                            const double* const* channel_weights) {
  CTX_LOCK(ctx);
  System* sys = ctx ? get_system(ctx, plan_id) : nullptr;
  if (!sys || slot < 0 || !d_left || !d_right || !channels || !channel_modes || !channel_weights)
    return fail_with(ctx, CAROLI_EINVAL, "caroli_sigma_from_modes: bad arguments");
  const int nb = (int)sys->plans.size();
  for (int side = 0; side < 2; ++side)
    if ((int)sys->lead_y[side].size() != nb) return fail_with(ctx, CAROLI_EINVAL, "caroli_sigma_from_modes: no lead modes");
  for (int b = 0; b < nb; ++b) {
    const FrontPlan& P = sys->plans[b]->host;
    if (!sys->lead_y[0][b] || !sys->lead_y[1][b] || !d_left[b] || !d_right[b])
      return fail_with(ctx, CAROLI_EINVAL, "caroli_sigma_from_modes: missing lead modes of a block");
    if (channels[b] < 0 || channels[b] > P.nr || (channels[b] && (!channel_modes[b] || !channel_weights[b])))
      return fail_with(ctx, CAROLI_EINVAL, "caroli_sigma_from_modes: bad channels");
    for (int c = 0; c < channels[b]; ++c)
      if (channel_modes[b][c] < 0 || channel_modes[b][c] >= P.nr)
        return fail_with(ctx, CAROLI_EINVAL, "caroli_sigma_from_modes: channel mode out of range");
  }
  try {
    CK(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    SigmaSlot& sg = slot_buffers(sys, slot);
    int nmax = 1;
    for (int b = 0; b < nb; ++b) nmax = std::max(nmax, std::max(sys->plans[b]->host.nl, sys->plans[b]->host.nr));
    double2* dd = static_cast<double2*>(ctx->lead_d.get(2 * (size_t)nmax * sizeof(double2)));
    int32_t* dcols = static_cast<int32_t*>(ctx->lead_cols.get((size_t)nmax * sizeof(int32_t)));
    double* dw = static_cast<double*>(ctx->lead_w.get((size_t)nmax * sizeof(double)));
    for (int b = 0; b < nb; ++b) {
      const FrontPlan& P = sys->plans[b]->host;
      for (int side = 0; side < 2; ++side) {
        const int n = side == 0 ? P.nl : P.nr;
        if (!n) continue;
        double2* d = dd + (size_t)side * nmax;
        CK(cudaMemcpyAsync(d, side == 0 ? d_left[b] : d_right[b], (size_t)n * sizeof(double2), cudaMemcpyHostToDevice, s));
        double2* S = side == 0 ? sg.sl[b] : sg.sr[b];
        double2* G = side == 0 ? sg.gl[b] : sg.gr[b];
        const unsigned t = (unsigned)((n + LS_TILE - 1) / LS_TILE);
        lead_sigma_kernel<<<dim3(t, t), 256, 0, s>>>(sys->lead_y[side][b], n, d, sys->lead_sc[side][b], S);
        CK(cudaGetLastError());
        lead_gamma_kernel<<<(unsigned)(((int64_t)n * n + 255) / 256), 256, 0, s>>>(S, n, G);
        CK(cudaGetLastError());
      }
      const int nc = channels[b];
      if (nc) {
        CK(cudaMemcpyAsync(dcols, channel_modes[b], nc * sizeof(int32_t), cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(dw, channel_weights[b], nc * sizeof(double), cudaMemcpyHostToDevice, s));
        lead_channels_kernel<<<(unsigned)(((int64_t)P.nr * nc + 255) / 256), 256, 0, s>>>(sys->lead_y[1][b], P.nr, dcols,
                                                                                        dw, nc, sg.wr[b]);
        CK(cudaGetLastError());
      }
      sg.channels[b] = nc;
      // The host vectors of this block must outlive the copies: synchronise per block.
      CK(cudaStreamSynchronize(s));
    }
    sg.energy = energy;
    sg.set = true;
    return CAROLI_OK;
  } catch (const CudaError& e) {
    return fail_with(ctx, e.e == cudaErrorMemoryAllocation ? CAROLI_ENOMEM : CAROLI_ECUDA, cudaGetErrorString(e.e));
  }
}

int caroli_sigma_upload(caroli_ctx* ctx, int plan_id, int slot, double energy, const double* const* sigma_l,
                        const double* const* sigma_r, const double* const* w_right, const int32_t* channels) {
  CTX_LOCK(ctx);
  System* sys = ctx ? get_system(ctx, plan_id) : nullptr;
  if (!sys || slot < 0 || !sigma_l || !sigma_r) return fail_with(ctx, CAROLI_EINVAL, "caroli_sigma_upload: bad arguments");
  try {
    CK(cudaSetDevice(ctx->device));
    SigmaSlot& sg = slot_buffers(sys, slot);
    const size_t nblocks = sys->plans.size();
    std::vector<std::vector<double>> keep;  // host data of the asynchronous copies
    auto put = [&](double2* d, const double* h, size_t count) {
      if (count) CK(cudaMemcpyAsync(d, h, count * sizeof(double2), cudaMemcpyHostToDevice, ctx->stream));
    };
    for (size_t b = 0; b < nblocks; ++b) {
      const FrontPlan& p = sys->plans[b]->host;
      const size_t nl = p.nl, nr = p.nr;
      put(sg.sl[b], sigma_l[b], nl * nl);
      put(sg.sr[b], sigma_r[b], nr * nr);
      // Γ = i (Σ - Σ^†) (caroli-green/src/lib.rs:67-71), formed on the device.
      if (nl) {
        lead_gamma_kernel<<<(unsigned)((nl * nl + 255) / 256), 256, 0, ctx->stream>>>(sg.sl[b], (int)nl, sg.gl[b]);
        CK(cudaGetLastError());
      }
      if (nr) {
        lead_gamma_kernel<<<(unsigned)((nr * nr + 255) / 256), 256, 0, ctx->stream>>>(sg.sr[b], (int)nr, sg.gr[b]);
        CK(cudaGetLastError());
      }
      int ch;
      if (w_right && channels) {
        ch = channels[b];
        if (ch < 0 || (size_t)ch > nr) return fail_with(ctx, CAROLI_EINVAL, "caroli_sigma_upload: bad channel count");
        if (ch && !w_right[b]) return fail_with(ctx, CAROLI_EINVAL, "caroli_sigma_upload: missing W_R");
        put(sg.wr[b], w_right[b], nr * (size_t)ch);
      } else {
        // W_R by pivoted Cholesky of the host's Γ_R.
        std::vector<double> gr(2 * nr * nr), wr;
        const double* sr = sigma_r[b];
        for (size_t j = 0; j < nr; ++j)
          for (size_t i = 0; i < nr; ++i) {
            gr[2 * (i + j * nr)] = -(sr[2 * (i + j * nr) + 1] + sr[2 * (j + i * nr) + 1]);
            gr[2 * (i + j * nr) + 1] = sr[2 * (i + j * nr)] - sr[2 * (j + i * nr)];
          }
        ch = gamma_factor(gr, nr, wr);
        put(sg.wr[b], wr.data(), nr * (size_t)ch);
        keep.push_back(std::move(wr));
      }
      sg.channels[b] = ch;
    }
    CK(cudaStreamSynchronize(ctx->stream));
    sg.energy = energy;
    sg.set = true;
    return CAROLI_OK;
  } catch (const CudaError& e) {
    return fail_with(ctx, e.e == cudaErrorMemoryAllocation ? CAROLI_ENOMEM : CAROLI_ECUDA, cudaGetErrorString(e.e));
  }
}

}  // extern "C"

namespace {

// T of `count` instances (system isys[i], energy slot, configuration) in one batch: the instances
// may belong to different systems (different sizes and trees); every block solve of every instance
// goes into the same level-synchronous launches.
int solve_instances(caroli_ctx* ctx, const std::vector<System*>& isys, int count, const int32_t* slots,
                    const int32_t* configs, int precision, double* t, int32_t* status, double* err, const char* who) {
  if (count < 0 || (count > 0 && (!slots || !configs || !t || !status)))
    return fail_with(ctx, CAROLI_EINVAL, std::string(who) + ": bad arguments");
  if (precision != CAROLI_DOUBLE && precision != CAROLI_SINGLE && precision != CAROLI_MIXED)
    return fail_with(ctx, CAROLI_EINVAL, "unknown precision");
  for (int i = 0; i < count; ++i) {
    System* sys = isys[i];
    if (!sys) return fail_with(ctx, CAROLI_EINVAL, std::string(who) + ": unknown plan");
    if (sys->nleads > 0)
      return fail_with(ctx, CAROLI_EINVAL, std::string(who) + ": a multi-terminal plan (caroli_multi_transmissions)");
    if (!sys->vals) return fail_with(ctx, CAROLI_EINVAL, "no H values uploaded");
    if (slots[i] < 0 || slots[i] >= (int)sys->slots.size() || !sys->slots[slots[i]].set)
      return fail_with(ctx, CAROLI_EINVAL, "energy slot without self-energies");
    if (configs[i] < 0 || configs[i] >= sys->nconfigs) return fail_with(ctx, CAROLI_EINVAL, "configuration out of range");
  }
  try {
    CK(cudaSetDevice(ctx->device));
    ctx->last_ms = 0.0;
    ctx->last_launches = 0;
    ctx->factor_ms = ctx->root_ms = ctx->tail_ms = 0.0;
    std::vector<JobSpec> specs;
    std::vector<size_t> first(count + 1, 0);
    for (int i = 0; i < count; ++i) {
      System* sys = isys[i];
      first[i] = specs.size();
      for (int b = 0; b < (int)sys->plans.size(); ++b)
        specs.push_back({b, slots[i], configs[i], sys->plans[b].get(), sys});
    }
    first[count] = specs.size();
    std::vector<JobOut> jo;
    ctx->fallbacks = 0;
    ctx->refine_iters = 0;
    ctx->refine_job_steps = ctx->refine_batch_steps = 0;
    solve_jobs(ctx, count ? isys[0] : nullptr, specs, (Mode)precision, jo);
    ctx->job_iters.clear();
    ctx->job_steps.clear();
    ctx->job_perturbed.clear();
    ctx->job_status.clear();
    for (const JobOut& o : jo) {
      ctx->job_iters.push_back(o.iters);
      ctx->job_steps.push_back(o.steps);
      ctx->job_perturbed.push_back(o.perturbed);
      ctx->job_status.push_back(o.status);
    }
    for (int i = 0; i < count; ++i) {
      double sum = 0.0, e = 0.0;
      int32_t st = ST_OK;
      for (size_t q = first[i]; q < first[i + 1]; ++q) {
        const JobOut& o = jo[q];
        sum += o.t;
        e += o.err;
        if (st == ST_OK) st = o.status >= 100 ? ST_OK : o.status;
      }
      t[i] = sum;
      status[i] = st;
      if (err) err[i] = e;
    }
    return CAROLI_OK;
  } catch (const CudaError& e) {
    return fail_with(ctx, e.e == cudaErrorMemoryAllocation ? CAROLI_ENOMEM : CAROLI_ECUDA,
                     std::string(e.what) + ": " + cudaGetErrorString(e.e));
  } catch (const std::exception& e) {
    return fail_with(ctx, CAROLI_EINVAL, e.what());
  }
}

}  // namespace

extern "C" {

int caroli_solve_batch(caroli_ctx* ctx, int plan_id, int count, const int32_t* slots, const int32_t* configs,
                       int precision, double* t, int32_t* status, double* err) {
  CTX_LOCK(ctx);
  System* sys = ctx ? get_system(ctx, plan_id) : nullptr;
  if (!sys) return fail_with(ctx, CAROLI_EINVAL, "caroli_solve_batch: bad arguments");
  std::vector<System*> isys(std::max(count, 0), sys);
  return solve_instances(ctx, isys, count, slots, configs, precision, t, status, err, "caroli_solve_batch");
}

int caroli_solve_multi(caroli_ctx* ctx, int count, const int32_t* plan_ids, const int32_t* slots,
                       const int32_t* configs, int precision, double* t, int32_t* status, double* err) {
  CTX_LOCK(ctx);
  if (!ctx || count < 0 || (count > 0 && !plan_ids)) return fail_with(ctx, CAROLI_EINVAL, "caroli_solve_multi: bad arguments");
  std::vector<System*> isys(count);
  for (int i = 0; i < count; ++i) isys[i] = get_system(ctx, plan_ids[i]);
  return solve_instances(ctx, isys, count, slots, configs, precision, t, status, err, "caroli_solve_multi");
}

int caroli_last_phases(const caroli_ctx* ctx, double* factor_ms, double* root_ms, double* tail_ms) {
  CTX_LOCK(ctx);
  if (!ctx) return CAROLI_EINVAL;
  if (factor_ms) *factor_ms = ctx->factor_ms;
  if (root_ms) *root_ms = ctx->root_ms;
  if (tail_ms) *tail_ms = ctx->tail_ms;
  return CAROLI_OK;
}

int caroli_last_job_steps(const caroli_ctx* ctx, int64_t capacity, int32_t* steps, int64_t* count) {
  CTX_LOCK(ctx);
  if (!ctx || !count) return CAROLI_EINVAL;
  const int64_t n = (int64_t)ctx->job_steps.size();
  for (int64_t j = 0; j < n && j < capacity; ++j)
    if (steps) steps[j] = ctx->job_steps[j];
  *count = n;
  return CAROLI_OK;
}

int caroli_last_job_info(const caroli_ctx* ctx, int64_t capacity, int32_t* iters, int32_t* perturbed,
                         int32_t* status, int64_t* count) {
  CTX_LOCK(ctx);
  if (!ctx) return CAROLI_EINVAL;
  const int64_t n = (int64_t)ctx->job_iters.size();
  if (count) *count = n;
  for (int64_t j = 0; j < std::min(n, capacity); ++j) {
    if (iters) iters[j] = ctx->job_iters[j];
    if (perturbed) perturbed[j] = ctx->job_perturbed[j];
    if (status) status[j] = ctx->job_status[j];
  }
  return CAROLI_OK;
}

int caroli_last_stats(const caroli_ctx* ctx, int64_t* fallbacks, int64_t* max_refine_iters) {
  CTX_LOCK(ctx);
  if (!ctx) return CAROLI_EINVAL;
  if (fallbacks) *fallbacks = ctx->fallbacks;
  if (max_refine_iters) *max_refine_iters = ctx->refine_iters;
  return CAROLI_OK;
}

int caroli_last_refine_steps(const caroli_ctx* ctx, int64_t* job_steps, int64_t* batch_steps) {
  CTX_LOCK(ctx);
  if (!ctx) return CAROLI_EINVAL;
  if (job_steps) *job_steps = ctx->refine_job_steps;
  if (batch_steps) *batch_steps = ctx->refine_batch_steps;
  return CAROLI_OK;
}

int caroli_set_refine_options(caroli_ctx* ctx, int max_iters, double tol, double inner_tol) {
  CTX_LOCK(ctx);
  if (!ctx) return CAROLI_EINVAL;
  if (max_iters < 1 || max_iters > 64 || !(tol > 0.0 && tol < 1.0) || !(inner_tol > 0.0 && inner_tol < 1.0))
    return fail_with(ctx, CAROLI_EINVAL, "refinement options out of range (1 <= max_iters <= 64, 0 < tol < 1)");
  ctx->max_iters = max_iters;
  ctx->refine_tol = tol;
  ctx->inner_tol = inner_tol;
  return CAROLI_OK;
}

int caroli_set_tensor_cores(caroli_ctx* ctx, int enable) {
  CTX_LOCK(ctx);
  if (!ctx) return CAROLI_EINVAL;
  ctx->tensor_cores = enable != 0;
  return CAROLI_OK;
}

int caroli_set_mixed_max_channels(caroli_ctx* ctx, int channels) {
  CTX_LOCK(ctx);
  if (!ctx) return CAROLI_EINVAL;
  if (channels < 0) return fail_with(ctx, CAROLI_EINVAL, "caroli_set_mixed_max_channels: negative channel count");
  ctx->mixed_max_channels = channels;
  return CAROLI_OK;
}

int caroli_set_autotune(caroli_ctx* ctx, int enable) {
  CTX_LOCK(ctx);
  if (!ctx) return CAROLI_EINVAL;
  ctx->autotune = enable != 0;
  ctx->tuned.clear();
  return CAROLI_OK;
}

int caroli_set_schedule(caroli_ctx* ctx, int small_max, int update_mode) {
  CTX_LOCK(ctx);
  if (!ctx) return CAROLI_EINVAL;
  if ((small_max != 48 && small_max != 64 && small_max != 96) || update_mode < 0 || update_mode > 2)
    return fail_with(ctx, CAROLI_EINVAL, "caroli_set_schedule: small_max 48, 64 or 96 and update_mode 0, 1 or 2");
  ctx->fixed_small_max = small_max;
  ctx->fixed_mode = update_mode;
  return CAROLI_OK;
}

int caroli_set_small_threads(caroli_ctx* ctx, int threads) {
  CTX_LOCK(ctx);
  if (!ctx) return CAROLI_EINVAL;
  if (threads != 256 && threads != 512) return fail_with(ctx, CAROLI_EINVAL, "caroli_set_small_threads: 256 or 512");
  ctx->small_threads = threads;
  return CAROLI_OK;
}

int caroli_set_sweep_columns(caroli_ctx* ctx, int min_columns) {
  CTX_LOCK(ctx);
  if (!ctx) return CAROLI_EINVAL;
  if (min_columns < 1) return fail_with(ctx, CAROLI_EINVAL, "caroli_set_sweep_columns: at least 1 column");
  ctx->tg_min_cols = min_columns;
  return CAROLI_OK;
}

int caroli_set_graphs(caroli_ctx* ctx, int enable) {
  CTX_LOCK(ctx);
  if (!ctx) return CAROLI_EINVAL;
  ctx->use_graphs = enable != 0;
  ctx->fgraph.reset();
  ctx->fgraph.seen.clear();
  return CAROLI_OK;
}

int caroli_last_schedule(const caroli_ctx* ctx, int32_t* small_max, int32_t* tensor_cores, int32_t* tuned,
                         double* trial_ms, int64_t* graph_replays, int64_t* graph_captures) {
  CTX_LOCK(ctx);
  if (!ctx) return CAROLI_EINVAL;
  const TuneChoice& t = ctx->last_tune;
  if (small_max) *small_max = t.small_max;
  if (tensor_cores) *tensor_cores = !t.tensor_cores ? 0 : (t.split ? 2 : 1);
  if (tuned) *tuned = t.tuned ? 1 : 0;
  if (trial_ms)
    for (int k = 0; k < TUNE_CANDIDATES; ++k) trial_ms[k] = t.ms[k];
  if (graph_replays) *graph_replays = ctx->graph_replays;
  if (graph_captures) *graph_captures = ctx->graph_captures;
  return CAROLI_OK;
}

int caroli_set_wait_limit(caroli_ctx* ctx, int64_t polls) {
  CTX_LOCK(ctx);
  if (!ctx) return CAROLI_EINVAL;
  ctx->tc_wait_limit = polls < 0 ? TCU_WAIT : (uint32_t)std::min<int64_t>(polls, TCU_WAIT);
  return CAROLI_OK;
}

int caroli_kernel_classes(void) { return K_COUNT; }

const char* caroli_kernel_class_name(int k) { return (k >= 0 && k < K_COUNT) ? kclass_names[k] : ""; }

int caroli_probe_kernel(caroli_ctx* ctx, int kclass) {
  CTX_LOCK(ctx);
  if (!ctx || kclass < -1 || kclass >= K_COUNT) return CAROLI_EINVAL;
  ctx->probe = kclass;
  return CAROLI_OK;
}

int caroli_kernel_stats(caroli_ctx* ctx, int kclass, int64_t* launches, double* flops, double* bytes, double* ms,
                        int reset) {
  CTX_LOCK(ctx);
  if (!ctx || kclass < 0 || kclass >= K_COUNT) return CAROLI_EINVAL;
  KStat& st = ctx->kstat[kclass];
  if (launches) *launches = st.launches;
  if (flops) *flops = st.flops;
  if (bytes) *bytes = st.bytes;
  if (ms) *ms = st.ms;
  if (reset) st = KStat{};
  return CAROLI_OK;
}

int caroli_region_begin(caroli_ctx* ctx) {
  CTX_LOCK(ctx);
  if (!ctx) return CAROLI_EINVAL;
  cudaSetDevice(ctx->device);
  ctx->region_launches = 0;
  return cudaEventRecord(ctx->reg0, ctx->stream) == cudaSuccess ? CAROLI_OK : CAROLI_ECUDA;
}

int caroli_region_end(caroli_ctx* ctx, double* device_ms, int64_t* launches) {
  CTX_LOCK(ctx);
  if (!ctx) return CAROLI_EINVAL;
  cudaSetDevice(ctx->device);
  if (cudaEventRecord(ctx->reg1, ctx->stream) != cudaSuccess || cudaEventSynchronize(ctx->reg1) != cudaSuccess)
    return CAROLI_ECUDA;
  float ms = 0.f;
  if (cudaEventElapsedTime(&ms, ctx->reg0, ctx->reg1) != cudaSuccess) return CAROLI_ECUDA;
  if (device_ms) *device_ms = ms;
  if (launches) *launches = ctx->region_launches;
  return CAROLI_OK;
}

int caroli_last_timing(const caroli_ctx* ctx, double* device_ms, int64_t* launches) {
  CTX_LOCK(ctx);
  if (!ctx) return CAROLI_EINVAL;
  if (device_ms) *device_ms = ctx->last_ms;
  if (launches) *launches = ctx->last_launches;
  return CAROLI_OK;
}

}  // extern "C"

// ---- Transmission without device allocation -------------------------------------------------------
// caroli_solve_batch grows device buffers with cudaMalloc as batches grow. Some callers cannot
// allocate device memory when they solve: a host program whose device memory is entirely
// reserved by another allocator (a framework's caching pool that has claimed the GPU), or a
// latency-critical loop that forbids allocation. For them caroli_solve_batch_noalloc runs the
// double-precision path on scratch carved from one file-scope device array of fixed size,
// NOALLOC_BYTES, which every GPU that loads this library holds until the process exits.
namespace {

constexpr size_t NOALLOC_BYTES = size_t(64) << 20;  // 64 MiB
static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_BYTES];

}  // namespace

// The device address of the scratch array on the current device, looked up once per context by
// caroli_ctx_create (with the context's device current). Host code cannot use the symbol itself:
// its name stands for a host-side shadow, not device memory.
cudaError_t noalloc_lookup(unsigned char** out) {
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e == cudaSuccess) *out = static_cast<unsigned char*>(p);
  return e;
}

namespace {

// Bump allocation inside the scratch array (256-byte aligned pieces).
struct Carve {
  unsigned char* base;
  size_t used = 0;
  size_t need(size_t bytes) {
    size_t at = (used + 255) & ~size_t(255);
    used = at + std::max<size_t>(bytes, 1);
    return at;
  }
};

}  // namespace

extern "C" int caroli_solve_batch_noalloc(caroli_ctx* ctx, int plan_id, int count, const int32_t* slots,
                                          const int32_t* configs, double* t, int32_t* status) {
  CTX_LOCK(ctx);
  System* sys = ctx ? get_system(ctx, plan_id) : nullptr;
  if (!sys || count < 0 || (count > 0 && (!slots || !configs || !t || !status)))
    return fail_with(ctx, CAROLI_EINVAL, "caroli_solve_batch_noalloc: bad arguments");
  if (sys->nleads > 0) return fail_with(ctx, CAROLI_EINVAL, "caroli_solve_batch_noalloc: a multi-terminal plan");
  if (!sys->vals) return fail_with(ctx, CAROLI_EINVAL, "no H values uploaded");
  for (int i = 0; i < count; ++i) {
    if (slots[i] < 0 || slots[i] >= (int)sys->slots.size() || !sys->slots[slots[i]].set)
      return fail_with(ctx, CAROLI_EINVAL, "energy slot without self-energies");
    if (configs[i] < 0 || configs[i] >= sys->nconfigs) return fail_with(ctx, CAROLI_EINVAL, "configuration out of range");
  }
  if (count == 0) return CAROLI_OK;
  try {
    CK(cudaSetDevice(ctx->device));
    unsigned char* base = ctx->noalloc_base;
    if (!base) return fail_with(ctx, CAROLI_ECUDA, "caroli_solve_batch_noalloc: the scratch array has no device address");
    cudaStream_t s = ctx->stream;
    const int nb = (int)sys->plans.size();
    const size_t nj = (size_t)count * nb;
    const size_t vb = sizeof(double2);
    // Layout of the scratch, with every size checked before anything runs.
    std::vector<size_t> arena_off(nj), root_off(nj), fail_off(nj);
    size_t aoff = 0, roff = 0, foff = 0, ntask = 0, ninv = 0, npiv = 0, ny = 0;
    int max_levels = 0, max_root = 0;
    size_t parts = 1;
    for (size_t j = 0; j < nj; ++j) {
      const FrontPlan& P = sys->plans[j % nb]->host;
      arena_off[j] = aoff;
      aoff += (size_t)P.arena_elems;
      const int m = P.fronts[P.root].n;
      root_off[j] = roff;
      roff += (size_t)m * m;
      fail_off[j] = foff;
      foff += P.fronts.size();
      ntask += P.fronts.size();
      max_levels = std::max(max_levels, P.levels);
      max_root = std::max(max_root, m);
      parts = std::max(parts, (size_t)(P.nr + 7) / 8);
      for (size_t k = 0; k + 1 < P.fronts.size(); ++k)
        if (P.fronts[k].n > SMALL_MAX_F64 && P.fronts[k].ne > 0) {
          ++ninv;
          npiv += P.fronts[k].ne;
          ny += (size_t)GJ_KB * P.fronts[k].n;
        }
      ++ninv;
      npiv += m;
      ny += (size_t)GJ_KB * m;
    }
    Carve cv{base};
    const size_t o_arena = cv.need(aoff * vb), o_root = cv.need(roff * vb), o_fail = cv.need(foff);
    const size_t o_status = cv.need(nj * 4), o_t = cv.need(nj * 8), o_part = cv.need(nj * parts * 8);
    const size_t o_jobs = cv.need(nj * sizeof(JobDesc)), o_tasks = cv.need(ntask * sizeof(Task));
    const size_t o_inv = cv.need(ninv * sizeof(InvTask)), o_piv = cv.need(npiv * 4), o_y = cv.need(ny * vb);
    const size_t o_scale = cv.need(ninv * 8), o_bad = cv.need(ninv * 4);
    if (cv.used > NOALLOC_BYTES)
      return fail_with(ctx, CAROLI_EINVAL,
                       "caroli_solve_batch_noalloc: the batch needs " + std::to_string(cv.used) +
                           " bytes of scratch; the static scratch holds " + std::to_string(NOALLOC_BYTES) +
                           " (solve fewer instances per call)");
    double2* arena = reinterpret_cast<double2*>(base + o_arena);
    double2* rarena = reinterpret_cast<double2*>(base + o_root);
    uint8_t* fail = base + o_fail;
    int32_t* dstatus = reinterpret_cast<int32_t*>(base + o_status);
    double* tdev = reinterpret_cast<double*>(base + o_t);
    double* part = reinterpret_cast<double*>(base + o_part);
    JobDesc* djobs = reinterpret_cast<JobDesc*>(base + o_jobs);
    Task* dtasks = reinterpret_cast<Task*>(base + o_tasks);
    InvTask* dinv = reinterpret_cast<InvTask*>(base + o_inv);
    // The flags and statuses the kernels only set must start at zero: the array keeps the
    // contents of the previous call.
    CK(cudaMemsetAsync(fail, 0, std::max<size_t>(foff, 1), s));
    CK(cudaMemsetAsync(dstatus, 0, nj * 4, s));
    std::vector<JobDesc> jd(nj);
    for (size_t j = 0; j < nj; ++j) {
      const int b = (int)(j % nb);
      const size_t i = j / nb;
      const DevPlan& P = *sys->plans[b];
      const SigmaSlot& sg = sys->slots[slots[i]];
      JobDesc& d = jd[j];
      d.fronts = P.fronts; d.maps = P.maps; d.own = P.own; d.entries = P.entries;
      d.arena = arena + arena_off[j];
      d.root_arena = rarena + root_off[j];
      d.vals = sys->vals + (size_t)configs[i] * sys->desc.row_ptr[sys->desc.n];
      d.sigma_l = sg.sl[b]; d.sigma_r = sg.sr[b]; d.gamma_l = sg.gl[b]; d.gamma_r = sg.gr[b];
      d.fail = fail + fail_off[j];
      d.energy = sg.energy;
      d.root = P.host.root; d.nl = P.host.nl; d.nr = P.host.nr; d.rpos = P.host.rpos; d.nd = P.host.nd;
      d.nfronts = (int32_t)P.host.fronts.size();
    }
    // Tasks level by level: small fronts, then large ones with their sweeps; roots last.
    std::vector<Task> tasks;
    std::vector<InvTask> inv;
    struct Lv { size_t s0, sn, l0, ln, i0, in; int smax, lmax, lne; };
    std::vector<Lv> lv(max_levels);
    size_t po = 0, yo = 0;
    auto add_inv = [&](void* a, int n, int np, int32_t job, int32_t front) {
      InvTask it{};
      it.a = a; it.ld = n; it.n = n; it.npiv = np; it.ncol = n; it.job = job; it.front = front;
      it.piv = reinterpret_cast<int32_t*>(base + o_piv) + po;
      it.y = reinterpret_cast<double2*>(base + o_y) + yo;
      it.scale2 = reinterpret_cast<double*>(base + o_scale) + inv.size();
      it.bad = reinterpret_cast<int32_t*>(base + o_bad) + inv.size();
      po += np;
      yo += (size_t)GJ_KB * n;
      inv.push_back(it);
    };
    for (int L = 0; L < max_levels; ++L) {
      Lv& v = lv[L];
      v = Lv{tasks.size(), 0, 0, 0, 0, 0, 0, 0, 0};
      for (size_t j = 0; j < nj; ++j) {
        const auto& fr = sys->plans[j % nb]->host.fronts;
        const FrontDesc* dfr = sys->plans[j % nb]->fronts;
        for (size_t k = 0; k + 1 < fr.size(); ++k)
          if (fr[k].level == L && fr[k].n <= SMALL_MAX_F64) {
            tasks.push_back({(int32_t)j, (int32_t)k, dfr + k});
            v.smax = std::max(v.smax, fr[k].n);
          }
      }
      v.sn = tasks.size() - v.s0;
      v.l0 = tasks.size();
      v.i0 = inv.size();
      for (size_t j = 0; j < nj; ++j) {
        const auto& fr = sys->plans[j % nb]->host.fronts;
        const FrontDesc* dfr = sys->plans[j % nb]->fronts;
        for (size_t k = 0; k + 1 < fr.size(); ++k)
          if (fr[k].level == L && fr[k].n > SMALL_MAX_F64) {
            tasks.push_back({(int32_t)j, (int32_t)k, dfr + k});
            v.lmax = std::max(v.lmax, fr[k].n);
            v.lne = std::max(v.lne, fr[k].ne);
            if (fr[k].ne > 0) add_inv(arena + arena_off[j] + fr[k].arena_off, fr[k].n, fr[k].ne, (int32_t)j, (int32_t)k);
          }
      }
      v.ln = tasks.size() - v.l0;
      v.in = inv.size() - v.i0;
    }
    const size_t root0 = tasks.size(), rinv0 = inv.size();
    for (size_t j = 0; j < nj; ++j) {
      const FrontPlan& P = sys->plans[j % nb]->host;
      tasks.push_back({(int32_t)j, P.root, sys->plans[j % nb]->fronts + P.root});
      const int m = P.fronts[P.root].n;
      add_inv(rarena + root_off[j], m, m, (int32_t)j, -1);
    }
    CK(cudaMemcpyAsync(djobs, jd.data(), nj * sizeof(JobDesc), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(dtasks, tasks.data(), tasks.size() * sizeof(Task), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(dinv, inv.data(), inv.size() * sizeof(InvTask), cudaMemcpyHostToDevice, s));
    auto sweep = [&](size_t first, size_t cnt, int nmax, int pmax, double tol) {
      if (!cnt) return;
      const size_t sm = panel_smem(pmax, vb), smf = (size_t)finish_bytes(pmax);
      if (!sm || smf > (size_t)SMEM_LIMIT) throw CudaError{cudaErrorInvalidValue, "front too large for a panel sweep"};
      inv_scale_kernel<double><<<(unsigned)cnt, 256, 0, s>>>(dinv + first);
      for (int k0 = 0; k0 < pmax; k0 += GJ_KB) {
        inv_panel_kernel<double><<<(unsigned)cnt, 256, sm, s>>>(dinv + first, k0, tol, 0, (int)sm);
        const unsigned rt = (unsigned)((nmax + 63) / 64);
        in_pieces(cnt, [&](size_t f0, size_t c) {
          inv_update_kernel<double><<<dim3(rt, rt, (unsigned)c), 256, 0, s>>>(dinv + first + f0, k0);
        });
      }
      inv_finish_kernel<double><<<(unsigned)cnt, 256, smf, s>>>(dinv + first, djobs, dstatus);
    };
    for (int L = 0; L < max_levels; ++L) {
      const Lv& v = lv[L];
      if (v.sn)
        small_front_kernel<double, false><<<(unsigned)v.sn, 256, small_smem_bytes(v.smax, v.smax, vb), s>>>(djobs, dtasks + v.s0,
                                                                                              PIVOT_TOL_F64, 0, nullptr);
      if (v.ln) {
        in_pieces(v.ln, [&](size_t f0, size_t c) {
          assemble_kernel<double, double><<<dim3((v.lmax + 31) / 32, (unsigned)c), 256, 0, s>>>(djobs,
                                                                                                dtasks + v.l0 + f0, 0);
        });
        sweep(v.i0, v.in, v.lmax, v.lne, PIVOT_TOL_F64);
      }
      CK(cudaGetLastError());
    }
    in_pieces(nj, [&](size_t f0, size_t c) {
      assemble_kernel<double, double><<<dim3((max_root + 31) / 32, (unsigned)c), 256, 0, s>>>(djobs, dtasks + root0 + f0, 1);
    });
    sweep(rinv0, nj, max_root, max_root, 0.0);
    in_pieces(nj, [&](size_t f0, size_t c) {
      trace_kernel<double><<<dim3((unsigned)parts, (unsigned)c), 256, 0, s>>>(djobs + f0, part + f0 * parts, (int)parts);
    });
    trace_finish_kernel<<<(unsigned)((nj + 127) / 128), 128, 0, s>>>(part, (int)parts, (int)nj, tdev, dstatus);
    CK(cudaGetLastError());
    std::vector<double> th(nj);
    std::vector<int32_t> sh(nj);
    std::vector<uint8_t> fh(std::max<size_t>(foff, 1));
    CK(cudaMemcpyAsync(th.data(), tdev, nj * 8, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(sh.data(), dstatus, nj * 4, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(fh.data(), fail, std::max<size_t>(foff, 1), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    for (int i = 0; i < count; ++i) {
      double sum = 0.0;
      int32_t st = ST_OK;
      for (int b = 0; b < nb; ++b) {
        const size_t j = (size_t)i * nb + b;
        bool delayed = false;
        for (size_t k = 0; k < sys->plans[b]->host.fronts.size(); ++k) delayed |= fh[fail_off[j] + k] != 0;
        int32_t sj = sh[j] != ST_OK ? sh[j] : (delayed ? ST_PIVOT_DELAYED : (std::isfinite(th[j]) ? ST_OK : ST_NONFINITE));
        sum += th[j];
        if (st == ST_OK) st = sj;
      }
      t[i] = sum;
      status[i] = st;
    }
    return CAROLI_OK;
  } catch (const CudaError& e) {
    return fail_with(ctx, CAROLI_ECUDA, std::string(e.what) + ": " + cudaGetErrorString(e.e));
  }
}
