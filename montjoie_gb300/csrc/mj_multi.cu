// Heterogeneous batch: leap-frog runs on many meshes of different size and
// order (FP32 chosen form), advanced by ONE cooperative persistent kernel per
// time step.
//
// Every run is an mj_lf on its own MJ_FP32 operator, so the per-mesh data
// (element-major Nodle, factors and contribution slots, the dof-ordered CSR
// of R, dt^2/D, the pulse and the step counters) are the operator's and the
// integrator's own buffers; the batch only adds a table of device pointers
// per mesh (a kernel parameter), work lists and the grid-barrier state.
//
// One step of the batch = one launch of k_mesh_batch_step:
//   phase 1  element tiles of all meshes, sorted by decreasing cost (high
//            order first) and dealt round-robin to the CTAs.  One tile = E
//            elements of one mesh, E*n*n of the CTA's threads each owning a
//            z-line (the compact single-RHS element product).  The factors
//            and Nodle of the next tile arrive by 1-D bulk copy (TMA) into
//            the other of two shared-memory stages, and the next tile's u is
//            gathered while the current tile's divergence runs;
//   barrier  grid-wide, bounded (a cooperative launch guarantees that every
//            CTA is resident, and every wait gives up after a time limit,
//            reporting through the error flag);
//   phase 2  dof chunks of all meshes, walked by each warp on its own with
//            two buffers of its own: the chunk's u^{n+1}, u^n, dt^2/D, CSR
//            offsets and its contiguous range of R arrive by bulk copy (the
//            next chunk's during this one), then each dof's sum, leap-frog
//            update and source term (a per-dof bit mask marks source dofs).
// Two launch configurations are compiled (256 threads with large tiles, 128
// threads with small tiles and more CTAs per SM); the first advance times
// both on the batch itself and keeps the faster.  A batch whose meshes all
// have one order runs that order's instance of the kernel
// (mj_multi_one.cu), which holds that order's code alone.
// The reference runs one ModifiedEquationIterator per problem, one after the
// other (MONTJOIE/src/Instationary/ModifiedEquation.cxx:290-345).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <memory>
#include <numeric>
#include <vector>

#include "mj_internal.cuh"
#include "mj_multi_kernel.cuh"


using namespace mj;

namespace mj {

// Per-run source state of a union group (kernel parameter): each run keeps
// its own pulse, step counters and dt; qc_par is the run's counter parity at
// the uploaded table (step k of the batch reads ctr[(k + qc_par) & 1]).
struct UnionRun {
  int* ctr;
  const double* pulse;
  double dt2;
  int n_pulse, qc_par;
};
struct UnionRuns {
  UnionRun r[kMaxRuns];
  int n;
};

// Sources of a union group's step k, after its streaming gather: every run's
// entries with that run's pulse, in the arithmetic of the source term of the
// run's own streaming gather (u = u + dt^2 (1/D) p f in FP64, rounded once),
// so the union steps bitwise like the runs' own kernels.  Block 0 advances
// every run's counters as the run's own gather does.
static __global__ void k_union_sources(const __grid_constant__ UnionRuns runs, int k, const int* __restrict__ sdof,
                                const int* __restrict__ srun, const float* __restrict__ sval, int n_src,
                                const double* __restrict__ inv_mass, float* __restrict__ u) {
  if (blockIdx.x == 0 && threadIdx.x < runs.n) {
    const UnionRun& q = runs.r[threadIdx.x];
    const int qc = (k + q.qc_par) & 1;
    q.ctr[1 - qc] = q.ctr[qc] + 1;
  }
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n_src; e += gridDim.x * blockDim.x) {
    const UnionRun& q = runs.r[srun[e]];
    const int step = q.ctr[(k + q.qc_par) & 1];
    const float f = sval[e];
    if (step >= q.n_pulse || f == 0.f) continue;
    const int d = sdof[e];
    u[d] = float(double(u[d]) + q.dt2 * inv_mass[d] * q.pulse[step] * double(f));
  }
}

// A group's runs stepped as one union operator (lf_union_create).
struct UnionGroup {
  std::unique_ptr<mj_op> op;
  std::unique_ptr<mj_lf> lf;
  std::vector<int> dof_off, elt_off, fac_version;
  DevBuf sdof, srun, sval;
  int n_src = 0;
  UnionRuns table{};
};

}  // namespace mj

struct mj_mb {
  std::vector<mj_lf*> runs;
  DevBuf sync, err;
  MeshTable table;  // kernel parameter
  std::vector<std::unique_ptr<DevBuf>> keep;  // per-run source masks and sorted sources
  std::vector<MeshDev> h_mesh;
  MbLists cfg[2];   // 0: 256 threads, 1: 128 threads
  int only = 0;     // the order n of every mesh (single-order kernels), or 0
  int use = -1;     // configuration in use (-1: not tuned yet)
  double tune_ms[4] = {0, 0, 0, 0};  // one kernel (256, 128 threads), grouped by order, union
  // launch parity of the uploaded table: per run (cur_is_a, step & 1) at upload
  std::vector<int> base_cur, base_qc;
  cudaGraphExec_t graph[2] = {nullptr, nullptr};  // 20 steps starting at k = 0 or k = 1
  bool last_graph = false;
  DevBuf stamps;        // per-CTA phase time stamps when profiling (plain launches only)
  bool profile = false;
  cudaStream_t stream = nullptr;
  // Mixed orders: one sub-batch per order (each runs its single-order
  // instance), the alternative to the all-orders kernel.  use == 2 selects it:
  // a step is then one cooperative launch per order, in a fixed order.
  std::vector<std::unique_ptr<mj_mb>> groups;
  // A group may instead step its runs with their own kernels, one run after
  // the other, when that is faster for its meshes (chosen by timing).
  bool seq = false;
  double seq_ms = 0, batch_ms = 0;
  // A batch of one order may also step its runs as one union operator
  // (use == 3): one tuned element kernel, one streaming gather and one source
  // launch per step over all its meshes, on copies of the runs' states taken
  // at the start of each advance and handed back at its end.
  std::unique_ptr<UnionGroup> uni;
  bool force_union = false;  // mj_mb_set_config(-2)
  ~mj_mb() {
    for (auto& g : graph)
      if (g) cudaGraphExecDestroy(g);
  }
};

namespace {

// The batch kernel of configuration T: the single-order instance when every
// mesh has one order, else the all-orders kernel.
template <int T>
const void* mb_kernel(const mj_mb* mb) {
  return mb->only ? mb_one_order_kernel(T, mb->only) : reinterpret_cast<const void*>(k_mesh_batch_step<T, 0>);
}

template <int T>
int mb_launch_t(mj_mb* mb, const MbLists& L, int k, cudaStream_t s) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(L.grid);
  cfg.blockDim = dim3(T);
  cfg.dynamicSmemBytes = MbPlan<T>::kSmem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  const Work* work = L.work.as<Work>();
  const Chunk* chunks = L.chunks.as<Chunk>();
  SyncState* sync = mb->sync.as<SyncState>();
  int* err = mb->err.as<int>();
  unsigned long long* stamps = mb->profile ? mb->stamps.as<unsigned long long>() : nullptr;
  int n_work = L.n_work, n_chunks = L.n_chunks;
  void* args[] = {&mb->table, &work, &n_work, &chunks, &n_chunks, &sync, &k, &err, &stamps};
  MJ_CUDA(cudaLaunchKernelExC(&cfg, mb_kernel<T>(mb), args));
  count_launch();
  return MJ_OK;
}

// Step k (relative to the uploaded table) of every run of the batch with the
// runs' own kernels, one run after the other.
int mb_launch_seq(mj_mb* mb, int k, cudaStream_t s) {
  for (size_t r = 0; r < mb->runs.size(); r++) {
    mj_lf* lf = mb->runs[r];
    const MeshDev& m = mb->h_mesh[r];
    float* cur = ((k + m.cur_par) & 1) == 0 ? m.ua : m.ub;  // U^n, overwritten by U^{n+2}
    const float* next = ((k + m.cur_par) & 1) == 0 ? m.ub : m.ua;
    const int rc = lf_step_on(lf, cur, next, (k + m.qc_par) & 1, s);
    if (rc) return rc;
  }
  return MJ_OK;
}

// Step k of a union batch, i steps after the runs' states were copied into
// the union: the union's two state buffers swap roles with the parity of i.
int mb_launch_union(mj_mb* mb, int k, int i, cudaStream_t s) {
  UnionGroup* u = mb->uni.get();
  mj_lf* lf = u->lf.get();
  float* cur = (i & 1) ? lf->ub.as<float>() : lf->ua.as<float>();
  const float* next = (i & 1) ? lf->ua.as<float>() : lf->ub.as<float>();
  if (int rc = lf_step_on(lf, cur, next, i & 1, s)) return rc;
  const int blocks = std::max(1, std::min((u->n_src + 255) / 256, 1024));
  k_union_sources<<<blocks, 256, 0, s>>>(u->table, k, u->sdof.as<int>(), u->srun.as<int>(), u->sval.as<float>(),
                                         u->n_src, lf->inv_mass64.as<double>(), cur);
  count_launch();
  MJ_CUDA(cudaGetLastError());
  return MJ_OK;
}

// Step k of the batch in form `which` (0/1: one kernel of 256/128 threads;
// 2: one launch per order group; 3: the union), i steps into the advance.
int mb_launch(mj_mb* mb, int which, int k, int i, cudaStream_t s) {
  if (which == 2) {  // one launch per order group (or its runs' own kernels, or its union)
    for (auto& g : mb->groups) {
      const int rc = g->seq ? mb_launch_seq(g.get(), k, s) : mb_launch(g.get(), g->use, k, i, s);
      if (rc) return rc;
    }
    return MJ_OK;
  }
  if (which == 3) return mb_launch_union(mb, k, i, s);
  return which == 0 ? mb_launch_t<256>(mb, mb->cfg[0], k, s) : mb_launch_t<128>(mb, mb->cfg[1], k, s);
}

// Kernel launches of one step in the batch's chosen form.
uint64_t mb_launches_per_step(const mj_mb* mb) {
  if (mb->use == 3) return 3;  // element kernel, streaming gather, sources
  if (mb->use != 2) return 1;
  uint64_t n = 0;
  for (auto& g : mb->groups) n += g->seq ? 2 * g->runs.size() : mb_launches_per_step(g.get());
  return n;
}

// The union copies of the runs' states: in, before the steps of an advance
// (U^n, U^{n+1} of every run at its offset); out, after `steps` steps and the
// runs' role update, back into each run's own buffers.
int union_copy(mj_mb* mb, bool in, int steps, cudaStream_t s) {
  UnionGroup* u = mb->uni.get();
  float* A = u->lf->ua.as<float>();
  float* B = u->lf->ub.as<float>();
  float* ucur = (steps & 1) ? B : A;
  float* unext = (steps & 1) ? A : B;
  for (size_t r = 0; r < mb->runs.size(); r++) {
    mj_lf* lf = mb->runs[r];
    const size_t bytes = sizeof(float) * lf->n_dof;
    float* c = ucur + u->dof_off[r];
    float* x = unext + u->dof_off[r];
    if (in) {
      MJ_CUDA(cudaMemcpyAsync(c, lf->cur(), bytes, cudaMemcpyDeviceToDevice, s));
      MJ_CUDA(cudaMemcpyAsync(x, lf->next(), bytes, cudaMemcpyDeviceToDevice, s));
    } else {
      MJ_CUDA(cudaMemcpyAsync(lf->cur(), c, bytes, cudaMemcpyDeviceToDevice, s));
      MJ_CUDA(cudaMemcpyAsync(lf->next(), x, bytes, cudaMemcpyDeviceToDevice, s));
    }
  }
  return MJ_OK;
}

// union_copy for every union the batch's chosen form steps.
int mb_union_copy(mj_mb* mb, bool in, int steps, cudaStream_t s) {
  if (mb->use == 3) return union_copy(mb, in, steps, s);
  if (mb->use == 2)
    for (auto& g : mb->groups)
      if (!g->seq && g->use == 3)
        if (int rc = union_copy(g.get(), in, steps, s)) return rc;
  return MJ_OK;
}

// Factors of a run's operator changed since they were copied into the union
// (mj_op_set_element_scale): copy them again.
int mb_union_refresh(mj_mb* mb, cudaStream_t s) {
  for (auto& g : mb->groups)
    if (int rc = mb_union_refresh(g.get(), s)) return rc;
  UnionGroup* u = mb->uni.get();
  if (!u) return MJ_OK;
  for (size_t r = 0; r < mb->runs.size(); r++) {
    const mj_op* op = mb->runs[r]->op;
    if (u->fac_version[r] == op->fac_version) continue;
    if (int rc = union_copy_factors(u->op.get(), op, u->elt_off[r], s)) return rc;
    u->fac_version[r] = op->fac_version;
  }
  return MJ_OK;
}

// The union of a batch of one order, with every run's sources at the run's
// offset; a batch too large for one union's int32 indexing gets none.
int mb_union_create(mj_mb* mb) {
  std::unique_ptr<UnionGroup> u(new UnionGroup());
  const int rc = lf_union_create(mb->runs, &u->op, &u->lf, &u->dof_off, &u->elt_off);
  if (rc == MJ_ERR_ARG) return MJ_OK;
  if (rc) return rc;
  std::vector<int> sdof, srun;
  std::vector<float> sval;
  for (size_t r = 0; r < mb->runs.size(); r++) {
    mj_lf* lf = mb->runs[r];
    u->fac_version.push_back(lf->op->fac_version);
    if (!lf->n_src) continue;
    std::vector<int> idx(lf->n_src);
    std::vector<float> val(lf->n_src);
    MJ_CUDA(cudaMemcpy(idx.data(), lf->src_idx.ptr, sizeof(int) * lf->n_src, cudaMemcpyDeviceToHost));
    MJ_CUDA(cudaMemcpy(val.data(), lf->src_val.ptr, sizeof(float) * lf->n_src, cudaMemcpyDeviceToHost));
    for (int t = 0; t < lf->n_src; t++) {
      sdof.push_back(u->dof_off[r] + idx[t]);
      srun.push_back((int)r);
      sval.push_back(val[t]);
    }
  }
  u->n_src = (int)sdof.size();
  MJ_CUDA(u->sdof.alloc(sizeof(int) * std::max<size_t>(1, sdof.size())));
  MJ_CUDA(u->srun.alloc(sizeof(int) * std::max<size_t>(1, srun.size())));
  MJ_CUDA(u->sval.alloc(sizeof(float) * std::max<size_t>(1, sval.size())));
  if (u->n_src) {
    MJ_CUDA(cudaMemcpy(u->sdof.ptr, sdof.data(), sizeof(int) * sdof.size(), cudaMemcpyHostToDevice));
    MJ_CUDA(cudaMemcpy(u->srun.ptr, srun.data(), sizeof(int) * srun.size(), cudaMemcpyHostToDevice));
    MJ_CUDA(cudaMemcpy(u->sval.ptr, sval.data(), sizeof(float) * sval.size(), cudaMemcpyHostToDevice));
  }
  mb->uni = std::move(u);
  return MJ_OK;
}

// Tile and chunk lists of configuration T: tiles sorted by decreasing cost
// (dealt round-robin to the CTAs), chunks of at most kChunkDofs dofs (one
// warp's) whose 16-byte rounded range of contributions fits kRCap.
template <int T>
int mb_build_lists(mj_mb* mb, const std::vector<std::vector<int>>& src_dofs, MbLists& L) {
  using P = MbPlan<T>;
  std::vector<Work> work;
  std::vector<Chunk> chunks;
  for (size_t r = 0; r < mb->runs.size(); r++) {
    const mj_op* op = mb->runs[r]->op;
    const int E = MbCfg<T>::tile(op->n);
    const int tiles = (op->n_elt + E - 1) / E;  // tiles past n_elt hold only padding
    for (int t = 0; t < tiles; t++) work.push_back({(int)r, t});
    std::vector<char> is_src(op->n_dof, 0);
    for (int d : src_dofs[r]) is_src[d] = 1;
    for (int d = 0; d < op->n_dof;) {
      int e = std::min(op->n_dof, d + P::kChunkDofs);
      auto range = [&](int e2) { return ((op->h_ptr[e2] + 3) & ~3) - (op->h_ptr[d] & ~3); };
      while (range(e) > P::kRCap) e = d + std::max(4, ((e - d) / 2) & ~3);
      Chunk ch = {(int)r, d, e, op->h_ptr[d] & ~3, (op->h_ptr[e] + 3) & ~3, 0, 0, 0};
      for (int x = d; x < e; x++) ch.has_src |= is_src[x];
      chunks.push_back(ch);
      d = e;
    }
  }
  auto cost = [&](const Work& w) {
    const long long n = mb->h_mesh[w.mesh].n;
    return (long long)MbCfg<T>::tile((int)n) * n * n * n * n;
  };
  std::stable_sort(work.begin(), work.end(), [&](const Work& a, const Work& b) { return cost(a) > cost(b); });
  L.threads = T;
  L.smem = P::kSmem;
  L.n_work = (int)work.size();
  L.n_chunks = (int)chunks.size();
  MJ_CUDA(L.work.alloc(sizeof(Work) * std::max<size_t>(1, work.size())));
  MJ_CUDA(L.chunks.alloc(sizeof(Chunk) * std::max<size_t>(1, chunks.size())));
  MJ_CUDA(cudaMemcpy(L.work.ptr, work.data(), sizeof(Work) * work.size(), cudaMemcpyHostToDevice));
  MJ_CUDA(cudaMemcpy(L.chunks.ptr, chunks.data(), sizeof(Chunk) * chunks.size(), cudaMemcpyHostToDevice));
  const void* fn = mb_kernel<T>(mb);
  MJ_CHECK_ARG(fn, "mj_mb_create: no batch kernel for this order");
  MJ_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, P::kSmem));
  MJ_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&L.ctas_per_sm, fn, T, P::kSmem));
  MJ_CHECK_ARG(L.ctas_per_sm >= 1, "mj_mb_create: the batch kernel cannot be resident");
  L.grid = L.ctas_per_sm * sm_count();
  return MJ_OK;
}

// Uploads the per-run table for the runs' current roles (state buffers and
// counters); drops the captured graphs, which bake in the old parities.
void mb_upload(mj_mb* mb) {
  const size_t n = mb->runs.size();
  mb->base_cur.resize(n);
  mb->base_qc.resize(n);
  for (size_t r = 0; r < n; r++) {
    mj_lf* lf = mb->runs[r];
    mb->h_mesh[r].cur_par = lf->cur_is_a ? 0 : 1;
    mb->h_mesh[r].qc_par = lf->step & 1;
    mb->base_cur[r] = lf->cur_is_a ? 1 : 0;
    mb->base_qc[r] = lf->step & 1;
    mb->table.m[r] = mb->h_mesh[r];
    if (mb->uni)
      mb->uni->table.r[r] = {lf->ctr.as<int>(), lf->pulse_d.as<double>(), lf->dt * lf->dt, lf->n_pulse,
                             mb->h_mesh[r].qc_par};
  }
  mb->table.n = (int)n;
  if (mb->uni) mb->uni->table.n = (int)n;
  for (auto& g : mb->graph)
    if (g) {
      cudaGraphExecDestroy(g);
      g = nullptr;
    }
  for (auto& g : mb->groups) mb_upload(g.get());
}

// Offset (0 or 1) of the runs' current roles from the uploaded table, or -1
// when the runs moved by different parities (a run advanced on its own).
int mb_offset(const mj_mb* mb) {
  int off = -1;
  for (size_t r = 0; r < mb->runs.size(); r++) {
    const mj_lf* lf = mb->runs[r];
    const int dc = (lf->cur_is_a ? 1 : 0) ^ mb->base_cur[r];
    const int dq = (lf->step & 1) ^ mb->base_qc[r];
    if (dc != dq) return -1;
    if (off < 0) off = dc;
    else if (off != dc) return -1;
  }
  return off < 0 ? 0 : off;
}

int mb_check_err(mj_mb* mb, cudaStream_t s) {
  int herr = 0;
  for (auto& g : mb->groups) {
    const int rc = mb_check_err(g.get(), s);
    if (rc == MJ_ERR_STATE) herr = 1;
    else if (rc) return rc;
    if (g->seq)  // runs stepped with their own kernels report through their operators
      for (mj_lf* lf : g->runs)
        if (take_kernel_error(lf->op->err.ptr, s, "mj_mb_advance")) herr = 1;
  }
  if (mb->uni && take_kernel_error(mb->uni->op->err.ptr, s, "mj_mb_advance")) herr = 1;
  int own = 0;
  MJ_CUDA(cudaMemcpyAsync(&own, mb->err.ptr, sizeof(int), cudaMemcpyDeviceToHost, s));
  MJ_CUDA(cudaStreamSynchronize(s));
  herr |= own;
  if (herr) {
    cudaMemset(mb->err.ptr, 0, sizeof(int));
    cudaMemset(mb->sync.ptr, 0, sizeof(SyncState));
    set_error("mj_mb_advance: a bounded wait timed out (batch state is invalid)");
    return MJ_ERR_STATE;
  }
  return MJ_OK;
}

// Times the batch's forms on the batch itself (3 steps each after one
// warm-up) and keeps the fastest: one kernel of 256 or 128 threads; for
// several orders, one launch per order group (each group batched, on its
// runs' own kernels or as its union, whichever its own timing favours); for
// one order, the union of its runs.  The runs' states and step counters are
// saved before and restored after, so tuning leaves no trace.
int mb_autotune(mj_mb* mb, int off, cudaStream_t s) {
  const size_t n = mb->runs.size();
  std::vector<std::unique_ptr<DevBuf>> save(n);
  std::vector<int> ctr(2 * n);
  for (size_t r = 0; r < n; r++) {
    mj_lf* lf = mb->runs[r];
    save[r] = std::make_unique<DevBuf>();
    const size_t bytes = lf->ua.bytes;
    MJ_CUDA(save[r]->alloc(2 * bytes));
    MJ_CUDA(cudaMemcpyAsync(save[r]->ptr, lf->ua.ptr, bytes, cudaMemcpyDeviceToDevice, s));
    MJ_CUDA(cudaMemcpyAsync(static_cast<char*>(save[r]->ptr) + bytes, lf->ub.ptr, bytes, cudaMemcpyDeviceToDevice,
                            s));
    MJ_CUDA(cudaMemcpyAsync(&ctr[2 * r], lf->ctr.ptr, 2 * sizeof(int), cudaMemcpyDeviceToHost, s));
  }
  cudaEvent_t e0, e1;
  MJ_CUDA(cudaEventCreate(&e0));
  MJ_CUDA(cudaEventCreate(&e1));
  const uint64_t before = launch_counter().load();
  int best = 0;
  std::vector<int> forms = {0, 1};
  if (!mb->groups.empty()) forms.push_back(2);
  if (mb->uni) forms.push_back(3);
  for (int c : forms) {
    int rc = MJ_OK;
    if (c == 3) rc = union_copy(mb, true, 0, s);  // the union steps from the runs' states
    if (c == 2)  // each order group picks its form, then batched or its runs' own kernels
      for (auto& g : mb->groups) {
        if (!rc && g->use < 0) rc = mb_autotune(g.get(), off, s);
        if (!rc && g->use == 3) rc = union_copy(g.get(), true, 0, s);
        for (int form = 0; !rc && form < 2; form++) {
          g->seq = form == 1;
          rc = mb_launch(mb, 2, off, 0, s) == MJ_OK ? MJ_OK : MJ_ERR_CUDA;  // warm-up of the whole grouped step
          if (!rc) rc = cudaEventRecord(e0, s) == cudaSuccess ? MJ_OK : MJ_ERR_CUDA;
          for (int i = 1; !rc && i <= 3; i++)
            rc = g->seq ? mb_launch_seq(g.get(), off + i, s) : mb_launch(g.get(), g->use, off + i, i, s);
          if (!rc) rc = cudaEventRecord(e1, s) == cudaSuccess ? MJ_OK : MJ_ERR_CUDA;
          if (!rc) rc = mb_check_err(mb, s);
          float ms = 0.f;
          if (!rc) rc = cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess ? MJ_OK : MJ_ERR_CUDA;
          (form ? g->seq_ms : g->batch_ms) = ms / 3.0;
        }
        if (rc) break;
        g->seq = g->seq_ms < g->batch_ms;
      }
    if (!rc) rc = mb_launch(mb, c, off, 0, s);
    if (!rc) rc = cudaEventRecord(e0, s) == cudaSuccess ? MJ_OK : MJ_ERR_CUDA;
    for (int i = 1; !rc && i <= 3; i++) rc = mb_launch(mb, c, off + i, i, s);
    if (!rc) rc = cudaEventRecord(e1, s) == cudaSuccess ? MJ_OK : MJ_ERR_CUDA;
    if (!rc) rc = mb_check_err(mb, s);
    float ms = 0.f;
    if (!rc) rc = cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess ? MJ_OK : MJ_ERR_CUDA;
    if (rc) {
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      return rc;
    }
    mb->tune_ms[c] = ms / 3.0;
    if (mb->tune_ms[c] < mb->tune_ms[best]) best = c;
  }
  launch_counter().store(before);  // tuning launches are not the caller's steps
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  for (size_t r = 0; r < n; r++) {
    mj_lf* lf = mb->runs[r];
    const size_t bytes = lf->ua.bytes;
    MJ_CUDA(cudaMemcpyAsync(lf->ua.ptr, save[r]->ptr, bytes, cudaMemcpyDeviceToDevice, s));
    MJ_CUDA(cudaMemcpyAsync(lf->ub.ptr, static_cast<char*>(save[r]->ptr) + bytes, bytes, cudaMemcpyDeviceToDevice,
                            s));
    MJ_CUDA(cudaMemcpyAsync(lf->ctr.ptr, &ctr[2 * r], 2 * sizeof(int), cudaMemcpyHostToDevice, s));
  }
  MJ_CUDA(cudaStreamSynchronize(s));
  mb->use = best;
  return MJ_OK;
}

// A batch of the given runs; with split, a batch of several orders also gets
// one sub-batch per order (the grouped alternative its autotuner times).
int mb_create(int n_runs, mj_lf* const* runs, bool split, std::unique_ptr<mj_mb>* result) {
  std::unique_ptr<mj_mb> mb(new mj_mb());
  mb->runs.assign(runs, runs + n_runs);
  std::vector<const mj_op*> ops;
  double gm[kMaxNK + 1][kMaxNK * kMaxNK];
  bool have_g[kMaxNK + 1] = {};
  for (int r = 0; r < n_runs; r++) {
    mj_lf* lf = runs[r];
    MJ_CHECK_ARG(lf, "mj_mb_create: null run");
    const mj_op* op = lf->op;
    MJ_CHECK_ARG(op->precision == MJ_FP32, "mj_mb_create: every run needs an MJ_FP32 operator");
    MJ_CHECK_ARG(lf->time_order == 2, "mj_mb_create: every run needs the order-2 leap-frog");
    MJ_CHECK_ARG(op->n >= 2 && op->n <= kMaxNK, "mj_mb_create: order out of range");
    MJ_CHECK_ARG(std::find(ops.begin(), ops.end(), op) == ops.end(), "mj_mb_create: runs share an operator");
    ops.push_back(op);
    if (!have_g[op->n]) {
      std::copy(op->gradphi, op->gradphi + op->n * op->n, gm[op->n]);
      have_g[op->n] = true;
    } else {
      for (int a = 0; a < op->n * op->n; a++)
        MJ_CHECK_ARG(gm[op->n][a] == op->gradphi[a],
                     "mj_mb_create: runs of one order use different derivative matrices");
    }
  }
  int n_orders = 0;
  for (int n = 2; n <= kMaxNK; n++)
    if (have_g[n]) {
      n_orders++;
      mb->only = n;
      float v[kMaxNK * kMaxNK];
      for (int a = 0; a < n * n; a++) v[a] = (float)gm[n][a];
      MJ_CUDA(cudaMemcpyToSymbol(c_gmat32, v, sizeof(float) * n * n, sizeof(float) * kMaxNK * kMaxNK * n));
      if (int rc = mb_one_order_set_gmat(n, v)) return rc;
    }
  if (n_orders != 1) mb->only = 0;  // several orders: the all-orders kernel

  // per-run table, source masks and sorted sources
  mb->h_mesh.resize(n_runs);
  std::vector<std::vector<int>> src_dofs(n_runs);
  for (int r = 0; r < n_runs; r++) {
    mj_lf* lf = runs[r];
    mj_op* op = lf->op;
    MeshDev& m = mb->h_mesh[r];
    m.nodle_e = op->nodle_e.as<int>();
    m.fac_e = op->fac_e.as<float>();
    m.slot_e = op->slot_e.as<int>();
    m.R = op->R.as<float>();
    m.ptr = op->ptr.as<int>();
    m.ua = lf->ua.as<float>();
    m.ub = lf->ub.as<float>();
    m.minv = lf->minv.as<float>();
    m.inv_mass = lf->inv_mass64.as<double>();
    m.pulse = lf->pulse_d.as<double>();
    m.ctr = lf->ctr.as<int>();
    m.dt2 = lf->dt * lf->dt;
    m.n = op->n;
    m.n_dof = op->n_dof;
    m.n_src = lf->n_src;
    m.n_pulse = lf->n_pulse;
    const int words = (op->n_dof + 31) / 32;
    auto mask = std::make_unique<DevBuf>();
    auto sidx = std::make_unique<DevBuf>();
    auto sval = std::make_unique<DevBuf>();
    MJ_CUDA(mask->alloc(sizeof(unsigned) * std::max(1, words)));
    MJ_CUDA(sidx->alloc(sizeof(int) * std::max(1, lf->n_src)));
    MJ_CUDA(sval->alloc(sizeof(float) * std::max(1, lf->n_src)));
    std::vector<unsigned> hm(std::max(1, words), 0u);
    if (lf->n_src) {
      std::vector<int> idx(lf->n_src);
      std::vector<float> val(lf->n_src);
      MJ_CUDA(cudaMemcpy(idx.data(), lf->src_idx.ptr, sizeof(int) * lf->n_src, cudaMemcpyDeviceToHost));
      MJ_CUDA(cudaMemcpy(val.data(), lf->src_val.ptr, sizeof(float) * lf->n_src, cudaMemcpyDeviceToHost));
      std::vector<int> order(lf->n_src);
      std::iota(order.begin(), order.end(), 0);
      std::sort(order.begin(), order.end(), [&](int a, int b) { return idx[a] < idx[b]; });
      std::vector<int> si(lf->n_src);
      std::vector<float> sv(lf->n_src);
      for (int t = 0; t < lf->n_src; t++) {
        si[t] = idx[order[t]];
        sv[t] = val[order[t]];
        hm[si[t] >> 5] |= 1u << (si[t] & 31);
      }
      src_dofs[r] = si;
      MJ_CUDA(cudaMemcpy(sidx->ptr, si.data(), sizeof(int) * lf->n_src, cudaMemcpyHostToDevice));
      MJ_CUDA(cudaMemcpy(sval->ptr, sv.data(), sizeof(float) * lf->n_src, cudaMemcpyHostToDevice));
    }
    MJ_CUDA(cudaMemcpy(mask->ptr, hm.data(), sizeof(unsigned) * hm.size(), cudaMemcpyHostToDevice));
    m.src_mask = mask->as<unsigned>();
    m.src_idx = sidx->as<int>();
    m.src_val = sval->as<float>();
    mb->keep.push_back(std::move(mask));
    mb->keep.push_back(std::move(sidx));
    mb->keep.push_back(std::move(sval));
  }
  int dev = 0, coop = 0;
  MJ_CUDA(cudaGetDevice(&dev));
  MJ_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
  MJ_CHECK_ARG(coop, "mj_mb_create: the device does not support cooperative launches");
  {
    int rc = mb_build_lists<256>(mb.get(), src_dofs, mb->cfg[0]);
    if (!rc) rc = mb_build_lists<128>(mb.get(), src_dofs, mb->cfg[1]);
    if (rc) return rc;
  }
  MJ_CUDA(mb->sync.alloc(sizeof(SyncState)));
  MJ_CUDA(cudaMemset(mb->sync.ptr, 0, sizeof(SyncState)));
  MJ_CUDA(mb->err.alloc(sizeof(int)));
  MJ_CUDA(cudaMemset(mb->err.ptr, 0, sizeof(int)));
  MJ_CUDA(mb->stamps.alloc(sizeof(unsigned long long) * kStamps *
                           std::max(mb->cfg[0].grid, mb->cfg[1].grid)));
  mb->stream = runs[0]->stream;
  if (mb->only)
    if (int rc = mb_union_create(mb.get())) return rc;
  if (split && !mb->only) {
    for (int n = 2; n <= kMaxNK; n++) {
      if (!have_g[n]) continue;
      std::vector<mj_lf*> sub;
      for (int r = 0; r < n_runs; r++)
        if (runs[r]->op->n == n) sub.push_back(runs[r]);
      std::unique_ptr<mj_mb> g;
      const int rc = mb_create((int)sub.size(), sub.data(), false, &g);
      if (rc) return rc;
      mb->groups.push_back(std::move(g));
    }
  }
  mb_upload(mb.get());
  *result = std::move(mb);
  return MJ_OK;
}

}  // namespace

extern "C" {

int mj_mb_create(int n_runs, mj_lf* const* runs, mj_mb** out) {
  MJ_CHECK_ARG(out && runs && n_runs > 0, "mj_mb_create: null argument or no runs");
  MJ_CHECK_ARG(n_runs <= kMaxRuns, "mj_mb_create: at most 48 runs per batch");
  *out = nullptr;
  for (int r = 0; r < n_runs; r++) MJ_CHECK_ARG(runs[r], "mj_mb_create: null run");
  std::unique_ptr<mj_mb> mb;
  const int rc = mb_create(n_runs, runs, true, &mb);
  if (rc) return rc;
  *out = mb.release();
  return MJ_OK;
}

int mj_mb_destroy(mj_mb* mb) {
  delete mb;
  return MJ_OK;
}

int mj_mb_advance(mj_mb* mb, int nsteps, int use_graph) {
  MJ_CHECK_ARG(mb && nsteps >= 0, "mj_mb_advance: bad argument");
  for (mj_lf* lf : mb->runs) {
    if (!lf->initialised) {
      set_error("mj_mb_advance: a run is not initialised (mj_lf_init)");
      return MJ_ERR_STATE;
    }
  }
  cudaStream_t s = mb->stream;
  // every run's own stream has finished its work before the batch runs
  for (mj_lf* lf : mb->runs)
    if (lf->stream != s) MJ_CUDA(cudaStreamSynchronize(lf->stream));
  int off = mb_offset(mb);
  if (off < 0) {
    mb_upload(mb);
    off = 0;
  }
  if (int rc = mb_union_refresh(mb, s)) return rc;
  if (mb->use < 0) {
    const int rc = mb_autotune(mb, off, s);
    if (rc) return rc;
  }
  if (mb->use == 2)  // grouped by order (forced): every group needs its configuration
    for (auto& g : mb->groups)
      if (g->use < 0) {
        const int rc = mb_autotune(g.get(), off, s);
        if (rc) return rc;
      }
  if (int rc = mb_union_copy(mb, true, 0, s)) return rc;
  mb->last_graph = false;
  int done = 0;
  if (use_graph && !mb->profile && nsteps >= kGraphStepsMb) {
    if (!mb->graph[off]) {
      cudaStream_t cs;
      MJ_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
      cudaGraph_t g;
      const uint64_t before = launch_counter().load();
      MJ_CUDA(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
      for (int k = 0; k < kGraphStepsMb; k++) {
        const int rc = mb_launch(mb, mb->use, off + k, k, cs);
        if (rc) {
          cudaStreamEndCapture(cs, &g);
          cudaStreamDestroy(cs);
          return rc;
        }
      }
      MJ_CUDA(cudaStreamEndCapture(cs, &g));
      launch_counter().store(before);  // captured, not launched
      MJ_CUDA(cudaGraphInstantiate(&mb->graph[off], g, 0));
      cudaGraphDestroy(g);
      cudaStreamDestroy(cs);
    }
    const uint64_t per_step = mb_launches_per_step(mb);
    while (nsteps - done >= kGraphStepsMb) {
      MJ_CUDA(cudaGraphLaunch(mb->graph[off], s));
      count_launch(kGraphStepsMb * per_step);
      done += kGraphStepsMb;
    }
    mb->last_graph = true;
  }
  for (; done < nsteps; done++) {
    const int rc = mb_launch(mb, mb->use, off + done, done, s);
    if (rc) return rc;
  }
  for (mj_lf* lf : mb->runs) {
    lf->step += nsteps;
    if (nsteps & 1) lf->cur_is_a = !lf->cur_is_a;
  }
  if (int rc = mb_union_copy(mb, false, nsteps, s)) return rc;
  return mb_check_err(mb, s);
}

int mj_mb_profile(mj_mb* mb, int enable) {
  MJ_CHECK_ARG(mb, "mj_mb_profile: null batch");
  mb->profile = enable != 0;
  for (auto& g : mb->groups) g->profile = mb->profile;
  return MJ_OK;
}

int mj_mb_phase_ms(const mj_mb* mb, double* out) {
  MJ_CHECK_ARG(mb && out, "mj_mb_phase_ms: null argument");
  MJ_CHECK_ARG(mb->use >= 0, "mj_mb_phase_ms: no step has run");
  if (mb->use == 3) {  // the union's kernels carry no phase stamps
    for (int i = 0; i < 6; i++) out[i] = 0.0;
    return MJ_OK;
  }
  if (mb->use == 2) {  // grouped by order: each phase summed over the groups' batch-kernel launches
    for (int i = 0; i < 6; i++) out[i] = 0.0;
    for (auto& g : mb->groups) {
      if (g->seq) continue;
      double o[6];
      const int rc = mj_mb_phase_ms(g.get(), o);
      if (rc) return rc;
      for (int i = 0; i < 6; i++) out[i] += o[i];
    }
    return MJ_OK;
  }
  const int grid = mb->cfg[mb->use].grid;
  std::vector<unsigned long long> st(kStamps * (size_t)grid);
  MJ_CUDA(cudaMemcpy(st.data(), mb->stamps.ptr, sizeof(unsigned long long) * st.size(), cudaMemcpyDeviceToHost));
  unsigned long long t0 = ~0ull, p1max = 0, p2 = 0, end = 0;
  double p1sum = 0;
  double w1 = 0, w2 = 0;
  for (int b = 0; b < grid; b++) t0 = std::min(t0, st[kStamps * b]);
  for (int b = 0; b < grid; b++) {
    const unsigned long long* c = &st[kStamps * b];
    p1max = std::max(p1max, c[1]);
    p1sum += double(c[1] - t0);
    p2 = std::max(p2, c[2]);
    end = std::max(end, c[3]);
    w1 += double(c[4]);
    w2 += double(c[5]);
  }
  out[0] = double(p1max - t0) * 1e-6;  // phase 1 (last CTA to finish)
  out[1] = p1sum / grid * 1e-6;        // phase 1 (mean CTA)
  out[2] = double(p2 - p1max) * 1e-6;  // barrier release after the last arrival
  out[3] = double(end - p2) * 1e-6;    // phase 2 (last CTA)
  out[4] = w1 / grid * 1e-6;           // stage waits of phase 1 (mean CTA)
  out[5] = w2 / grid * 1e-6;           // chunk waits of phase 2 (mean CTA)
  return MJ_OK;
}

int mj_mb_info(const mj_mb* mb, int* grid, int* ctas_per_sm, int* n_tiles, int* n_chunks, int* graph,
               int* single_order) {
  MJ_CHECK_ARG(mb, "mj_mb_info: null batch");
  // the launch shape of a form: a batch kernel's lists, or the union's element
  // kernel (its tiles) and streaming gather (its chunks)
  auto shape = [](const mj_mb* b, int* gr, int* cps, int* tiles, int* chunks) {
    if (b->use == 3) {
      const mj_op* op = b->uni->op.get();
      *gr = op->grid_k1;
      *cps = std::max(1, op->grid_k1 / sm_count());
      *tiles = op->n_tiles;
      *chunks = b->uni->lf->n_stream_chunks;
      return;
    }
    const MbLists& L = b->cfg[std::max(0, std::min(1, b->use))];
    *gr = L.grid;
    *cps = L.ctas_per_sm;
    *tiles = L.n_work;
    *chunks = L.n_chunks;
  };
  int gr = 0, cps = 0, tiles = 0, chunks = 0;
  if (mb->use == 2) {  // grouped by order: the groups' totals, the launch shape of the largest group
    int best_tiles = -1;
    for (const auto& g : mb->groups) {
      int g1, c1, t1, k1;
      shape(g.get(), &g1, &c1, &t1, &k1);
      tiles += t1;
      chunks += k1;
      if (t1 > best_tiles) {
        best_tiles = t1;
        gr = g1;
        cps = c1;
      }
    }
  } else {
    shape(mb, &gr, &cps, &tiles, &chunks);
  }
  if (grid) *grid = gr;
  if (ctas_per_sm) *ctas_per_sm = cps;
  if (n_tiles) *n_tiles = tiles;
  if (n_chunks) *n_chunks = chunks;
  if (graph) *graph = mb->last_graph ? 1 : 0;
  if (single_order) *single_order = mb->only;
  return MJ_OK;
}

int mj_mb_set_config(mj_mb* mb, int threads) {
  MJ_CHECK_ARG(mb, "mj_mb_set_config: null batch");
  MJ_CHECK_ARG(threads == 0 || threads == 128 || threads == 256 || threads == -1 || threads == -2,
               "mj_mb_set_config: threads must be 0, 128, 256, -1 or -2");
  MJ_CHECK_ARG(threads != -1 || !mb->groups.empty(), "mj_mb_set_config: the batch has one order (no groups)");
  if (threads == -2) {  // the union: of the whole batch (one order) or of every order group
    if (mb->groups.empty()) {
      MJ_CHECK_ARG(mb->uni, "mj_mb_set_config: the batch is too large for one union");
      mb->use = 3;
    } else {
      for (auto& g : mb->groups) MJ_CHECK_ARG(g->uni, "mj_mb_set_config: a group is too large for one union");
      mb->use = 2;
      for (auto& g : mb->groups) {
        g->use = 3;
        g->seq = false;
      }
    }
  } else {
    mb->use = threads == 0 ? -1 : threads == 256 ? 0 : threads == 128 ? 1 : 2;
    for (auto& g : mb->groups) g->use = -1;  // groups tune again at the next advance
  }
  for (auto& g : mb->graph)
    if (g) {
      cudaGraphExecDestroy(g);
      g = nullptr;
    }
  return MJ_OK;
}

int mj_mb_grouping(const mj_mb* mb, int* grouped, int* n_groups, double* grouped_ms) {
  MJ_CHECK_ARG(mb, "mj_mb_grouping: null batch");
  if (grouped) *grouped = mb->use == 2 ? 1 : 0;
  if (n_groups) *n_groups = (int)mb->groups.size();
  if (grouped_ms) *grouped_ms = mb->tune_ms[2];
  return MJ_OK;
}

int mj_mb_group_info(const mj_mb* mb, int group, int* order, int* n_runs, int* own_kernels, double* batch_ms,
                     double* own_ms) {
  MJ_CHECK_ARG(mb && group >= 0 && group < (int)mb->groups.size(), "mj_mb_group_info: no such group");
  const mj_mb* g = mb->groups[group].get();
  if (order) *order = g->runs[0]->op->order;
  if (n_runs) *n_runs = (int)g->runs.size();
  if (own_kernels) *own_kernels = g->seq ? 1 : 0;
  if (batch_ms) *batch_ms = g->batch_ms;
  if (own_ms) *own_ms = g->seq_ms;
  return MJ_OK;
}

int mj_mb_tuning(const mj_mb* mb, int* threads, double* candidate_ms) {
  MJ_CHECK_ARG(mb, "mj_mb_tuning: null batch");
  if (threads) {
    // the batch kernel's configuration: the one in use, else the faster of
    // the two timed (of the first group when grouped)
    const mj_mb* b = mb->use == 2 ? mb->groups[0].get() : mb;
    int c = b->use;
    if (c != 0 && c != 1) c = (b->tune_ms[1] > 0 && b->tune_ms[1] < b->tune_ms[0]) ? 1 : 0;
    *threads = mb->use < 0 ? 0 : b->cfg[c].threads;
  }
  if (candidate_ms) {
    candidate_ms[0] = mb->tune_ms[0];
    candidate_ms[1] = mb->tune_ms[1];
  }
  return MJ_OK;
}

int mj_mb_union_info(const mj_mb* mb, int group, int* in_use, double* union_ms, int* tile_elems, int* n_dof) {
  MJ_CHECK_ARG(mb, "mj_mb_union_info: null batch");
  MJ_CHECK_ARG(group >= -1 && group < (int)mb->groups.size(), "mj_mb_union_info: no such group");
  const mj_mb* b = group < 0 ? mb : mb->groups[group].get();
  if (in_use) *in_use = (group < 0 ? mb->use == 3 : (mb->use == 2 && !b->seq && b->use == 3)) ? 1 : 0;
  if (union_ms) *union_ms = b->tune_ms[3];
  if (tile_elems) *tile_elems = b->uni ? b->uni->op->E : 0;
  if (n_dof) *n_dof = b->uni ? b->uni->op->n_dof : 0;
  return MJ_OK;
}

}  // extern "C"
