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
#include <cstring>
#include <memory>
#include <numeric>
#include <string>
#include <vector>

#include "../../include/caroli_gb300.h"
#include "kernels.cuh"
#include "plan.hpp"

using namespace caroli;

namespace {

constexpr double PIVOT_TOL_F64 = 1e-11;  // caroli-dense/src/field.rs:61
constexpr double PIVOT_TOL_F32 = 1e-5;   // caroli-dense/src/field.rs:111
constexpr int SMALL_MAX_F64 = 64;        // fronts up to this size run in one CTA's shared memory
constexpr int SMALL_MAX_F32 = 96;
constexpr int SMEM_LIMIT = 220 * 1024;   // dynamic shared memory a kernel may request

struct CudaError {
  cudaError_t e;
  const char* what;
};
#define CK(x)                                             \
  do {                                                    \
    cudaError_t _e = (x);                                 \
    if (_e != cudaSuccess) throw CudaError{_e, #x};       \
  } while (0)

template <typename T> T* dalloc(size_t count) {
  void* p = nullptr;
  if (count == 0) return nullptr;
  cudaError_t e = cudaMalloc(&p, count * sizeof(T));
  if (e != cudaSuccess) throw CudaError{e, "cudaMalloc"};
  return static_cast<T*>(p);
}

// Device copy of a front plan.
struct DevPlan {
  FrontPlan host;
  FrontDesc* fronts = nullptr;
  int32_t* maps = nullptr;
  uint8_t* own = nullptr;
  Entry* entries = nullptr;
  void upload(cudaStream_t s) {
    fronts = dalloc<FrontDesc>(host.fronts.size());
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
    cudaFree(fronts); cudaFree(maps); cudaFree(own); cudaFree(entries);
    fronts = nullptr; maps = nullptr; own = nullptr; entries = nullptr;
  }
};

struct SigmaSlot {
  double energy = 0.0;
  bool set = false;
  std::vector<double2*> sl, sr, gl, gr;  // per block, device
};

struct System {
  // Owned copies of the description.
  std::vector<int64_t> row_ptr, cells, site_offsets, site_orbitals, interior, left_ptr, left, right_ptr, right;
  std::vector<uint32_t> cols;
  std::vector<int32_t> labels;
  SystemDesc desc{};
  std::vector<BlockTree> trees;
  std::vector<std::unique_ptr<DevPlan>> plans;  // static plan per block
  double2* vals = nullptr;
  int nconfigs = 0;
  std::vector<SigmaSlot> slots;
  ~System() {
    for (auto& p : plans) p->release();
    cudaFree(vals);
    for (auto& s : slots)
      for (auto* v : {&s.sl, &s.sr, &s.gl, &s.gr})
        for (auto* p : *v) cudaFree(p);
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
  ~Buf() { cudaFree(p); }
};

struct JobSpec {
  int block, slot, config;
  const DevPlan* plan;
};

}  // namespace

struct caroli_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  std::string err;
  std::vector<std::unique_ptr<System>> systems;
  Buf arena, xs, jobs, tasks, fail, status, tout, part;
  double last_ms = 0.0;
  int64_t last_launches = 0;
  size_t mem_budget = 0;
};

namespace {

int fail_with(caroli_ctx* ctx, int code, const std::string& msg) {
  if (ctx) ctx->err = msg;
  return code;
}

System* get_system(caroli_ctx* ctx, int id) {
  if (id < 0 || id >= (int)ctx->systems.size() || !ctx->systems[id]) return nullptr;
  return ctx->systems[id].get();
}

template <typename T> struct Prec {
  static constexpr int small_max = sizeof(T) == 8 ? SMALL_MAX_F64 : SMALL_MAX_F32;
  static constexpr double tol = sizeof(T) == 8 ? PIVOT_TOL_F64 : PIVOT_TOL_F32;
};

size_t small_smem(int n, size_t vbytes) {
  int ld = n | 1;
  return (size_t)ld * n * vbytes + 2 * (size_t)n * vbytes + (size_t)((n + 1) & ~1) * 4 + 32 * 8 + 32 * 4 + 16;
}
// Shared memory of a pivot-block launch whose largest block is ne: the staged block when it fits
// under SMEM_LIMIT, else only the work vectors (the kernel then sweeps in global memory).
size_t pivot_smem(int ne, size_t vbytes) {
  size_t work = 2 * (size_t)ne * vbytes + (size_t)((ne + 1) & ~1) * 4 + 32 * 8 + 32 * 4 + 16;
  size_t staged = (size_t)ne * (ne | 1) * vbytes + work;
  return staged <= (size_t)SMEM_LIMIT ? staged : work;
}

// Launches `fn(first, count)` over a task range in pieces of at most 65535 (grid y/z limit).
template <typename F> void in_pieces(size_t count, F fn) {
  for (size_t first = 0; first < count; first += 65535) fn(first, std::min<size_t>(65535, count - first));
}

// Runs `specs` (all of precision T); fills per-job T, status and (optionally) fail flags.
template <typename T>
void run_jobs(caroli_ctx* ctx, System* sys, const std::vector<JobSpec>& specs, std::vector<double>& t_out,
              std::vector<int32_t>& st_out, std::vector<std::vector<uint8_t>>* fails) {
  using V = typename Cx<T>::V;
  cudaStream_t s = ctx->stream;
  const size_t vb = sizeof(V);
  const size_t nj = specs.size();
  t_out.assign(nj, 0.0);
  st_out.assign(nj, ST_OK);
  if (fails) fails->assign(nj, {});
  // Chunks of jobs that fit the memory budget.
  size_t begin = 0;
  while (begin < nj) {
    size_t end = begin, bytes = 0;
    while (end < nj) {
      size_t b = (size_t)specs[end].plan->host.arena_elems * vb;
      if (end > begin && bytes + b > ctx->mem_budget) break;
      bytes += b;
      ++end;
    }
    const size_t cj = end - begin;
    // Arena offsets, job descriptors, fail-flag offsets.
    std::vector<JobDesc> jd(cj);
    std::vector<size_t> arena_off(cj), fail_off(cj);
    size_t aoff = 0, foff = 0;
    int max_levels = 0;
    size_t parts_per_job = 1;
    for (size_t j = 0; j < cj; ++j) {
      const JobSpec& sp = specs[begin + j];
      arena_off[j] = aoff;
      aoff += (size_t)sp.plan->host.arena_elems;
      fail_off[j] = foff;
      foff += sp.plan->host.fronts.size();
      max_levels = std::max(max_levels, sp.plan->host.levels);
      parts_per_job = std::max(parts_per_job, (size_t)(sp.plan->host.nr + 7) / 8);
    }
    V* arena = static_cast<V*>(ctx->arena.get(std::max<size_t>(aoff, 1) * vb));
    uint8_t* fail = static_cast<uint8_t*>(ctx->fail.get(std::max<size_t>(foff, 1)));
    int32_t* status = static_cast<int32_t*>(ctx->status.get(cj * sizeof(int32_t)));
    double* tdev = static_cast<double*>(ctx->tout.get(cj * sizeof(double)));
    double* part = static_cast<double*>(ctx->part.get(cj * parts_per_job * sizeof(double)));
    CK(cudaMemsetAsync(fail, 0, foff, s));
    CK(cudaMemsetAsync(status, 0, cj * sizeof(int32_t), s));
    for (size_t j = 0; j < cj; ++j) {
      const JobSpec& sp = specs[begin + j];
      const DevPlan& P = *sp.plan;
      const SigmaSlot& sg = sys->slots[sp.slot];
      JobDesc& d = jd[j];
      d.fronts = P.fronts; d.maps = P.maps; d.own = P.own; d.entries = P.entries;
      d.arena = arena + arena_off[j];
      d.vals = sys->vals + (size_t)sp.config * sys->desc.row_ptr[sys->desc.n];
      d.sigma_l = sg.sl[sp.block]; d.sigma_r = sg.sr[sp.block];
      d.gamma_l = sg.gl[sp.block]; d.gamma_r = sg.gr[sp.block];
      d.fail = fail + fail_off[j];
      d.energy = sg.energy;
      d.root = P.host.root; d.nl = P.host.nl; d.nr = P.host.nr; d.rpos = P.host.rpos; d.nd = P.host.nd;
      d.nfronts = (int32_t)P.host.fronts.size();
    }
    JobDesc* djobs = static_cast<JobDesc*>(ctx->jobs.get(cj * sizeof(JobDesc)));
    CK(cudaMemcpyAsync(djobs, jd.data(), cj * sizeof(JobDesc), cudaMemcpyHostToDevice, s));
    // Task lists: per level, small and large tree fronts; then the roots.
    struct Level { size_t small0, small_n, large0, large_n; int max_small_n, max_large_n, max_large_ne; size_t xs_elems; };
    std::vector<Task> tasks;
    std::vector<Level> levels(max_levels);
    const int small_max = Prec<T>::small_max;
    for (int L = 0; L < max_levels; ++L) {
      Level& lv = levels[L];
      lv = Level{tasks.size(), 0, 0, 0, 0, 0, 0, 0};
      for (size_t j = 0; j < cj; ++j) {
        const auto& fr = specs[begin + j].plan->host.fronts;
        for (size_t k = 0; k + 1 < fr.size(); ++k)
          if (fr[k].level == L && fr[k].n <= small_max) {
            tasks.push_back({(int32_t)j, (int32_t)k, 0});
            lv.max_small_n = std::max(lv.max_small_n, fr[k].n);
          }
      }
      lv.small_n = tasks.size() - lv.small0;
      lv.large0 = tasks.size();
      size_t xo = 0;
      for (size_t j = 0; j < cj; ++j) {
        const auto& fr = specs[begin + j].plan->host.fronts;
        for (size_t k = 0; k + 1 < fr.size(); ++k)
          if (fr[k].level == L && fr[k].n > small_max) {
            tasks.push_back({(int32_t)j, (int32_t)k, (int64_t)xo});
            xo += (size_t)fr[k].ne * (fr[k].n - fr[k].ne);
            lv.max_large_n = std::max(lv.max_large_n, fr[k].n);
            lv.max_large_ne = std::max(lv.max_large_ne, fr[k].ne);
          }
      }
      lv.large_n = tasks.size() - lv.large0;
      lv.xs_elems = xo;
    }
    const size_t root0 = tasks.size();
    int max_root = 0;
    for (size_t j = 0; j < cj; ++j) {
      const auto& P = specs[begin + j].plan->host;
      tasks.push_back({(int32_t)j, P.root, 0});
      max_root = std::max(max_root, P.fronts[P.root].n);
    }
    Task* dtasks = static_cast<Task*>(ctx->tasks.get(tasks.size() * sizeof(Task)));
    CK(cudaMemcpyAsync(dtasks, tasks.data(), tasks.size() * sizeof(Task), cudaMemcpyHostToDevice, s));
    size_t xs_max = 1;
    for (auto& lv : levels) xs_max = std::max(xs_max, lv.xs_elems);
    V* xs = static_cast<V*>(ctx->xs.get(xs_max * vb));

    CK(cudaEventRecord(ctx->ev0, s));
    int64_t launches = 0;
    for (int L = 0; L < max_levels; ++L) {
      const Level& lv = levels[L];
      if (lv.small_n) {
        size_t sm = small_smem(lv.max_small_n, vb);
        small_front_kernel<T, false><<<(unsigned)lv.small_n, 256, sm, s>>>(djobs, dtasks + lv.small0, Prec<T>::tol);
        ++launches;
      }
      if (lv.large_n) {
        const Task* lt = dtasks + lv.large0;
        const int mt = (lv.max_large_n + 63) / 64;
        const size_t sm = pivot_smem(lv.max_large_ne, vb);
        in_pieces(lv.large_n, [&](size_t f0, size_t c) {
          assemble_kernel<T><<<dim3((lv.max_large_n + 31) / 32, (unsigned)c), 256, 0, s>>>(djobs, lt + f0, 0);
          ++launches;
        });
        pivot_block_kernel<T><<<(unsigned)lv.large_n, 1024, sm, s>>>(djobs, lt, Prec<T>::tol, (int)sm, 0, status);
        ++launches;
        for (int mode = 0; mode < 2; ++mode)
          in_pieces(lv.large_n, [&](size_t f0, size_t c) {
            front_gemm_kernel<T><<<dim3(mt, mt, (unsigned)c), 256, 0, s>>>(djobs, lt + f0, xs, mode);
            ++launches;
          });
        in_pieces(lv.large_n, [&](size_t f0, size_t c) {
          store_x_kernel<T><<<dim3(8, (unsigned)c), 256, 0, s>>>(djobs, lt + f0, xs);
          ++launches;
        });
      }
      CK(cudaGetLastError());
    }
    // Roots: always complex f64 for DOUBLE; the fronts' precision otherwise.
    {
      const Task* rt = dtasks + root0;
      in_pieces(cj, [&](size_t f0, size_t c) {
        assemble_kernel<T><<<dim3((max_root + 31) / 32, (unsigned)c), 256, 0, s>>>(djobs, rt + f0, 1);
        ++launches;
      });
      const size_t sm = pivot_smem(max_root, vb);
      pivot_block_kernel<T><<<(unsigned)cj, 1024, sm, s>>>(djobs, rt, 0.0, (int)sm, 1, status);
      ++launches;
      in_pieces(cj, [&](size_t f0, size_t c) {
        trace_kernel<T><<<dim3((unsigned)parts_per_job, (unsigned)c), 256, 0, s>>>(djobs + f0, part + f0 * parts_per_job,
                                                                                 (int)parts_per_job);
        ++launches;
      });
      trace_finish_kernel<<<(unsigned)((cj + 127) / 128), 128, 0, s>>>(part, (int)parts_per_job, (int)cj, tdev, status);
      ++launches;
      CK(cudaGetLastError());
    }
    CK(cudaEventRecord(ctx->ev1, s));
    std::vector<double> th(cj);
    std::vector<int32_t> sh(cj);
    std::vector<uint8_t> fh(foff);
    CK(cudaMemcpyAsync(th.data(), tdev, cj * sizeof(double), cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(sh.data(), status, cj * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(fh.data(), fail, foff, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
    ctx->last_ms += ms;
    ctx->last_launches += launches;
    for (size_t j = 0; j < cj; ++j) {
      t_out[begin + j] = th[j];
      int32_t st = sh[j];
      const size_t nf = specs[begin + j].plan->host.fronts.size();
      bool delayed = false;
      for (size_t k = 0; k < nf; ++k) delayed |= fh[fail_off[j] + k] != 0;
      if (delayed) st = ST_PIVOT_DELAYED;
      st_out[begin + j] = st;
      if (fails && delayed) (*fails)[begin + j].assign(fh.begin() + fail_off[j], fh.begin() + fail_off[j] + nf);
    }
    begin = end;
  }
}

template <typename T>
void solve_jobs(caroli_ctx* ctx, System* sys, std::vector<JobSpec>& specs, std::vector<double>& t,
                std::vector<int32_t>& st) {
  std::vector<std::vector<uint8_t>> fails;
  run_jobs<T>(ctx, sys, specs, t, st, &fails);
  // Jobs with refused pivots: re-plan with those fronts delayed and run them again, one by one.
  for (size_t j = 0; j < specs.size(); ++j) {
    if (st[j] != ST_PIVOT_DELAYED) continue;
    const BlockTree& tree = sys->trees[specs[j].block];
    std::vector<uint8_t> delayed(tree.nodes.size(), 0);
    for (size_t k = 0; k < tree.nodes.size(); ++k) delayed[k] = fails[j][k];
    for (size_t round = 0; round <= tree.nodes.size(); ++round) {
      DevPlan dp;
      dp.host = make_plan(sys->desc, tree, delayed);
      dp.upload(ctx->stream);
      std::vector<JobSpec> one{{specs[j].block, specs[j].slot, specs[j].config, &dp}};
      std::vector<double> t1;
      std::vector<int32_t> s1;
      std::vector<std::vector<uint8_t>> f1;
      run_jobs<T>(ctx, sys, one, t1, s1, &f1);
      dp.release();
      t[j] = t1[0];
      st[j] = s1[0];
      if (s1[0] != ST_PIVOT_DELAYED) break;
      bool grew = false;
      for (size_t k = 0; k < tree.nodes.size(); ++k)
        if (f1[0][k] && !delayed[k]) { delayed[k] = 1; grew = true; }
      if (!grew) { st[j] = ST_SINGULAR; break; }
    }
  }
}

double2* upload_c64(const double* host, size_t count, cudaStream_t s) {
  double2* d = dalloc<double2>(std::max<size_t>(count, 1));
  if (count) CK(cudaMemcpyAsync(d, host, count * sizeof(double2), cudaMemcpyHostToDevice, s));
  return d;
}

}  // namespace

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
    size_t free_b = 0, total_b = 0;
    CK(cudaMemGetInfo(&free_b, &total_b));
    ctx->mem_budget = free_b / 2;
    for (auto* k : {(const void*)small_front_kernel<double, false>, (const void*)small_front_kernel<float, false>,
                    (const void*)pivot_block_kernel<double>, (const void*)pivot_block_kernel<float>})
      CK(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_LIMIT));
  } catch (const CudaError& e) {
    return CAROLI_ECUDA;
  }
  *out = ctx.release();
  return CAROLI_OK;
}

void caroli_ctx_destroy(caroli_ctx* ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  ctx->systems.clear();
  if (ctx->ev0) cudaEventDestroy(ctx->ev0);
  if (ctx->ev1) cudaEventDestroy(ctx->ev1);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
}

const char* caroli_last_error(const caroli_ctx* ctx) { return ctx ? ctx->err.c_str() : "no context"; }

int caroli_plan_upload(caroli_ctx* ctx, int64_t n, const int64_t* row_ptr, const uint32_t* cols, int64_t nsites,
                       int dim, const int64_t* cells, const int64_t* site_offsets, const int64_t* site_orbitals,
                       const int64_t* range, int64_t n_interior, const int64_t* interior, int nblocks,
                       const int32_t* labels, const int64_t* left_ptr, const int64_t* left,
                       const int64_t* right_ptr, const int64_t* right, int* plan_id) {
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

int caroli_values_upload(caroli_ctx* ctx, int plan_id, int nconfigs, const double* values) {
  System* sys = ctx ? get_system(ctx, plan_id) : nullptr;
  if (!sys || nconfigs <= 0 || !values) return fail_with(ctx, CAROLI_EINVAL, "caroli_values_upload: bad arguments");
  try {
    CK(cudaSetDevice(ctx->device));
    cudaFree(sys->vals);
    sys->vals = nullptr;
    const size_t nnz = (size_t)sys->desc.row_ptr[sys->desc.n];
    sys->vals = upload_c64(values, nnz * (size_t)nconfigs, ctx->stream);
    CK(cudaStreamSynchronize(ctx->stream));
    sys->nconfigs = nconfigs;
    return CAROLI_OK;
  } catch (const CudaError& e) {
    return fail_with(ctx, e.e == cudaErrorMemoryAllocation ? CAROLI_ENOMEM : CAROLI_ECUDA, cudaGetErrorString(e.e));
  }
}

int caroli_sigma_upload(caroli_ctx* ctx, int plan_id, int slot, double energy, const double* const* sigma_l,
                        const double* const* sigma_r) {
  System* sys = ctx ? get_system(ctx, plan_id) : nullptr;
  if (!sys || slot < 0 || !sigma_l || !sigma_r) return fail_with(ctx, CAROLI_EINVAL, "caroli_sigma_upload: bad arguments");
  try {
    CK(cudaSetDevice(ctx->device));
    if ((int)sys->slots.size() <= slot) sys->slots.resize(slot + 1);
    SigmaSlot& sg = sys->slots[slot];
    for (auto* v : {&sg.sl, &sg.sr, &sg.gl, &sg.gr}) {
      for (auto* p : *v) cudaFree(p);
      v->clear();
    }
    for (size_t b = 0; b < sys->plans.size(); ++b) {
      const FrontPlan& p = sys->plans[b]->host;
      const size_t nl = p.nl, nr = p.nr;
      // Γ = i (Σ - Σ^†) (caroli-green/src/lib.rs:67-71).
      std::vector<double> gl(2 * nl * nl), gr(2 * nr * nr);
      auto gamma = [](const double* s, size_t m, std::vector<double>& g) {
        for (size_t j = 0; j < m; ++j)
          for (size_t i = 0; i < m; ++i) {
            double dr = s[2 * (i + j * m)] - s[2 * (j + i * m)];
            double di = s[2 * (i + j * m) + 1] + s[2 * (j + i * m) + 1];
            g[2 * (i + j * m)] = -di;
            g[2 * (i + j * m) + 1] = dr;
          }
      };
      gamma(sigma_l[b], nl, gl);
      gamma(sigma_r[b], nr, gr);
      sg.sl.push_back(upload_c64(sigma_l[b], nl * nl, ctx->stream));
      sg.sr.push_back(upload_c64(sigma_r[b], nr * nr, ctx->stream));
      sg.gl.push_back(upload_c64(gl.data(), nl * nl, ctx->stream));
      sg.gr.push_back(upload_c64(gr.data(), nr * nr, ctx->stream));
      CK(cudaStreamSynchronize(ctx->stream));
    }
    sg.energy = energy;
    sg.set = true;
    return CAROLI_OK;
  } catch (const CudaError& e) {
    return fail_with(ctx, e.e == cudaErrorMemoryAllocation ? CAROLI_ENOMEM : CAROLI_ECUDA, cudaGetErrorString(e.e));
  }
}

int caroli_solve_batch(caroli_ctx* ctx, int plan_id, int count, const int32_t* slots, const int32_t* configs,
                       int precision, double* t, int32_t* status, double* err) {
  System* sys = ctx ? get_system(ctx, plan_id) : nullptr;
  if (!sys || count < 0 || (count > 0 && (!slots || !configs || !t || !status)))
    return fail_with(ctx, CAROLI_EINVAL, "caroli_solve_batch: bad arguments");
  if (precision != CAROLI_DOUBLE && precision != CAROLI_SINGLE && precision != CAROLI_MIXED)
    return fail_with(ctx, CAROLI_EINVAL, "unknown precision");
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
    const int nb = (int)sys->plans.size();
    std::vector<JobSpec> specs;
    specs.reserve((size_t)count * nb);
    for (int i = 0; i < count; ++i)
      for (int b = 0; b < nb; ++b) specs.push_back({b, slots[i], configs[i], sys->plans[b].get()});
    std::vector<double> tj;
    std::vector<int32_t> sj;
    if (precision == CAROLI_DOUBLE) solve_jobs<double>(ctx, sys, specs, tj, sj);
    else solve_jobs<float>(ctx, sys, specs, tj, sj);
    for (int i = 0; i < count; ++i) {
      double sum = 0.0;
      int32_t st = ST_OK;
      for (int b = 0; b < nb; ++b) {
        sum += tj[(size_t)i * nb + b];
        if (st == ST_OK) st = sj[(size_t)i * nb + b];
      }
      t[i] = sum;
      status[i] = st;
      if (err) err[i] = 0.0;
    }
    return CAROLI_OK;
  } catch (const CudaError& e) {
    return fail_with(ctx, e.e == cudaErrorMemoryAllocation ? CAROLI_ENOMEM : CAROLI_ECUDA,
                     std::string(e.what) + ": " + cudaGetErrorString(e.e));
  } catch (const std::exception& e) {
    return fail_with(ctx, CAROLI_EINVAL, e.what());
  }
}

int caroli_last_timing(const caroli_ctx* ctx, double* device_ms, int64_t* launches) {
  if (!ctx) return CAROLI_EINVAL;
  if (device_ms) *device_ms = ctx->last_ms;
  if (launches) *launches = ctx->last_launches;
  return CAROLI_OK;
}

}  // extern "C"
