// Many right-hand sides on one mesh (FP32): ONE cooperative persistent kernel
// per leap-frog step of all S runs.
//
//   phase 1  element tiles (E elements) of the mesh, persistent CTAs; the
//            factors and Nodle of a tile arrive by 1-D bulk copy (TMA) two
//            tiles ahead and stay in shared memory for all S/W passes.  A
//            thread owns a z-line of one element for V right-hand sides held
//            in registers (LB thread lanes x V = W right-hand sides per
//            pass), so every shared-memory line access moves V values at
//            once (8- or 16-byte loads) and the factors are read once per V.
//            The operation order per right-hand side is that of
//            k_local_stiffness_rhs; results go to the dof-ordered R.
//   barrier  grid-wide, bounded (cooperative launch; mj_sync.cuh);
//   phase 2  dof chunks: u^{n+1}, u^n rows, the chunk's contiguous block of
//            R rows, dt^2/D and the CSR offsets arrive by bulk copy (two
//            buffers per CTA); then the sums, the leap-frog update and the
//            sources (grouped by dof) of every (dof, right-hand side).
// The variant (n, E, LB, V) is chosen at creation by timing the candidates
// of the order on the integrator itself.  The reference runs the S
// problems one after the other (MONTJOIE/src/Instationary/ModifiedEquation.cxx:290-345).
#include <cuda_runtime.h>

#include <algorithm>
#include <memory>
#include <vector>

#include "mj_rhs_step.cuh"

namespace mj {
namespace {

constexpr int kGraphStepsRs = 20;

// Order in which the threads of an element take its n*n z-lines.  A warp
// holds Z = 32/LB consecutive slots; each of its shared-memory line reads
// touches one x-line per distinct row j and one y-line per distinct column i
// among its z-lines.  Candidates: row-major, 2-D blocks, and strips of 2, 3 or
// 4 rows walked column by column, alternate strips in reverse (snake); the one
// with the fewest distinct rows + columns per warp, summed over the E
// elements of a tile, is kept (row-major on ties).  Every point's arithmetic
// is the same whichever thread does it.
void rs_zline_order(int n, int E, int LB, unsigned char* out) {
  const int Z = std::max(1, 32 / LB), NN = n * n;
  auto cost = [&](const std::vector<int>& ord) {
    int tot = 0;
    for (int w0 = 0; w0 < E * NN; w0 += Z) {
      std::vector<int> rows, cols;
      for (int sl = w0; sl < std::min(w0 + Z, E * NN); sl++) {
        const int e = sl / NN, q = ord[sl % NN];
        rows.push_back(e * n + q / n);
        cols.push_back(e * n + q % n);
      }
      std::sort(rows.begin(), rows.end());
      std::sort(cols.begin(), cols.end());
      tot += (int)(std::unique(rows.begin(), rows.end()) - rows.begin()) +
             (int)(std::unique(cols.begin(), cols.end()) - cols.begin());
    }
    return tot;
  };
  std::vector<std::vector<int>> cands;
  std::vector<int> ord;
  for (int q = 0; q < NN; q++) ord.push_back(q);
  cands.push_back(ord);
  {
    const int bw = Z >= 8 ? 4 : Z >= 2 ? 2 : 1, bh = std::max(1, Z / bw);
    ord.clear();
    for (int by = 0; by < n; by += bh)
      for (int bx = 0; bx < n; bx += bw)
        for (int y = by; y < std::min(by + bh, n); y++)
          for (int x = bx; x < std::min(bx + bw, n); x++) ord.push_back(y * n + x);
    cands.push_back(ord);
  }
  for (int bh = 2; bh <= 4; bh++) {
    ord.clear();
    for (int by = 0, strip = 0; by < n; by += bh, strip++)
      for (int c = 0; c < n; c++) {
        const int x = strip % 2 == 0 ? c : n - 1 - c;
        for (int y = by; y < std::min(by + bh, n); y++) ord.push_back(y * n + x);
      }
    cands.push_back(ord);
  }
  size_t best = 0;
  for (size_t c = 1; c < cands.size(); c++)
    if (cost(cands[c]) < cost(cands[best])) best = c;
  for (int q = 0; q < NN; q++) out[q] = (unsigned char)cands[best][q];
}



struct RsVariant {
  int n, E, LB, V, threads, smem, half;
};

const std::vector<RsVariant>& rs_variants() {
  static const std::vector<RsVariant> v = {
#define MJ_X(N_, E_, LB_, V_)                                                                          \
  {N_, E_, LB_, V_, RsPlan<N_, E_, LB_, V_>::T, RsPlan<N_, E_, LB_, V_>::kSmem, RsPlan<N_, E_, LB_, V_>::kHalf},
      MJ_RS_VARIANTS(MJ_X)
#undef MJ_X
  };
  return v;
}

int rs_prepare(const RsVariant& v, int* ctas) {
#define MJ_X(N_, E_, LB_, V_)                                                                               \
  if (v.n == N_ && v.E == E_ && v.LB == LB_ && v.V == V_) {                                                 \
    MJ_CUDA(cudaFuncSetAttribute(k_rhs_step<N_, E_, LB_, V_>, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                                 v.smem));                                                                 \
    MJ_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(ctas, k_rhs_step<N_, E_, LB_, V_>, v.threads,    \
                                                          v.smem));                                        \
    return MJ_OK;                                                                                           \
  }
  MJ_RS_VARIANTS(MJ_X)
#undef MJ_X
  set_error("no many-source step variant");
  return MJ_ERR_ARG;
}

int rs_launch(const RsVariant& v, int grid, const RsParams& prm, const RsChunk* chunks, int n_chunks,
              SyncState* sync, int par, int* err, cudaStream_t s, unsigned long long* stamps = nullptr) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(v.threads);
  cfg.dynamicSmemBytes = v.smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
#define MJ_X(N_, E_, LB_, V_)                                                                                \
  if (v.n == N_ && v.E == E_ && v.LB == LB_ && v.V == V_) {                                                  \
    MJ_CUDA(cudaLaunchKernelEx(&cfg, k_rhs_step<N_, E_, LB_, V_>, prm, chunks, n_chunks, sync, par, err,  \
                               stamps));                                                                     \
    count_launch();                                                                                          \
    return MJ_OK;                                                                                            \
  }
  MJ_RS_VARIANTS(MJ_X)
#undef MJ_X
  set_error("no many-source step variant");
  return MJ_ERR_ARG;
}

RsParams rs_params(mj_lfb* b, const RsVariant& v) {
  mj_op* op = b->op;
  RsParams p;
  p.fac_e = op->fac_e.as<float>();
  p.nodle_e = op->nodle_e.as<int>();
  p.slot_e = op->slot_e.as<int>();
  p.R = b->R.as<float>();
  p.ptr = op->ptr.as<int>();
  p.ua = b->ua.as<float>();
  p.ub = b->ub.as<float>();
  p.m = b->m.as<float>();
  p.pulse = b->pulse.as<double>();
  p.ctr = b->ctr.as<int>();
  p.src_dof = b->rs_src_dof.as<int>();
  p.src_ptr = b->rs_src_ptr.as<int>();
  p.src_rhs = b->rs_src_rhs.as<int>();
  p.src_val = b->rs_src_val.as<float>();
  p.uout = nullptr;
  p.ucopy = nullptr;
  p.ue = nullptr;
  p.gacc = nullptr;
  p.gcoef = nullptr;
  p.n_src_dof = b->rs_n_src_dof;
  p.n_pulse = b->n_pulse;
  p.S = b->S;
  p.n_tiles = op->n_elt_pad / v.E;
  rs_zline_order(v.n, v.E, v.LB, p.zmap);
  return p;
}

// Dof chunks of a variant: as many dofs as fit one phase-2 buffer (<= 512).
std::vector<RsChunk> rs_chunks(const mj_lfb* b, int half, const std::vector<char>& is_src) {
  const mj_op* op = b->op;
  const std::vector<int>& ptr = op->h_ptr;
  std::vector<RsChunk> out;
  for (int d = 0; d < op->n_dof;) {
    if (rs_buf(d, d + 1, ptr[d], ptr[d + 1], b->S).end > half) return {};
    int e = d + 1;
    while (e < op->n_dof && e - d < 512 && rs_buf(d, e + 1, ptr[d], ptr[e + 1], b->S).end <= half) e++;
    RsChunk ch = {d, e, ptr[d], ptr[e], 0, 0, 0, 0};
    for (int x = d; x < e; x++) ch.has_src |= is_src[x];
    out.push_back(ch);
    d = e;
  }
  return out;
}

int rs_check_err(mj_lfb* b, cudaStream_t s) {
  int herr = 0;
  MJ_CUDA(cudaMemcpyAsync(&herr, b->rs_err.ptr, sizeof(int), cudaMemcpyDeviceToHost, s));
  MJ_CUDA(cudaStreamSynchronize(s));
  if (herr) {
    cudaMemset(b->rs_err.ptr, 0, sizeof(int));
    cudaMemset(b->rs_sync.ptr, 0, sizeof(SyncState));
    set_error("mj_lfb_advance: a bounded wait of the step kernel timed out (state is invalid)");
    return MJ_ERR_STATE;
  }
  return MJ_OK;
}

}  // namespace

// Sources grouped by dof, chunk lists per candidate, and the variant choice:
// each candidate of the order runs 3 steps (after one warm-up) on the
// integrator's state, which mj_lfb_init resets afterwards.  Leaves
// b->fused = false when no variant fits (S too large for a chunk buffer).
int lfb_fused_setup(mj_lfb* b) {
  mj_op* op = b->op;
  {
    // derivative matrix of this order into this unit's constant memory
    float v[kMaxNK * kMaxNK];
    for (int a = 0; a < op->n * op->n; a++) v[a] = (float)op->gradphi[a];
    MJ_CUDA(cudaMemcpyToSymbol(c_gmat32, v, sizeof(float) * op->n * op->n, sizeof(float) * kMaxNK * kMaxNK * op->n));
    if (int rc = rs_en_set_gmat(op->n, v)) return rc;
  }
  // sources grouped by dof: sorted (dof, rhs) pairs from the device copies
  std::vector<int> si(b->n_src), sr(b->n_src);
  std::vector<float> sv(b->n_src);
  if (b->n_src) {
    MJ_CUDA(cudaMemcpy(si.data(), b->src_idx.ptr, sizeof(int) * b->n_src, cudaMemcpyDeviceToHost));
    MJ_CUDA(cudaMemcpy(sr.data(), b->src_rhs.ptr, sizeof(int) * b->n_src, cudaMemcpyDeviceToHost));
    MJ_CUDA(cudaMemcpy(sv.data(), b->src_val.ptr, sizeof(float) * b->n_src, cudaMemcpyDeviceToHost));
  }
  std::vector<int> order(b->n_src);
  for (int t = 0; t < b->n_src; t++) order[t] = t;
  std::sort(order.begin(), order.end(), [&](int x, int y) { return si[x] != si[y] ? si[x] < si[y] : sr[x] < sr[y]; });
  std::vector<int> dofs, dptr, rhs;
  std::vector<float> val;
  std::vector<char> is_src(op->n_dof, 0);
  for (int t = 0; t < b->n_src; t++) {
    const int e = order[t];
    if (dofs.empty() || dofs.back() != si[e]) {
      dofs.push_back(si[e]);
      dptr.push_back((int)rhs.size());
    }
    rhs.push_back(sr[e]);
    val.push_back(sv[e]);
    is_src[si[e]] = 1;
  }
  dptr.push_back((int)rhs.size());
  b->rs_n_src_dof = (int)dofs.size();
  MJ_CUDA(b->rs_src_dof.alloc(sizeof(int) * std::max<size_t>(1, dofs.size())));
  MJ_CUDA(b->rs_src_ptr.alloc(sizeof(int) * dptr.size()));
  MJ_CUDA(b->rs_src_rhs.alloc(sizeof(int) * std::max<size_t>(1, rhs.size())));
  MJ_CUDA(b->rs_src_val.alloc(sizeof(float) * std::max<size_t>(1, val.size())));
  if (!dofs.empty()) {
    MJ_CUDA(cudaMemcpy(b->rs_src_dof.ptr, dofs.data(), sizeof(int) * dofs.size(), cudaMemcpyHostToDevice));
    MJ_CUDA(cudaMemcpy(b->rs_src_rhs.ptr, rhs.data(), sizeof(int) * rhs.size(), cudaMemcpyHostToDevice));
    MJ_CUDA(cudaMemcpy(b->rs_src_val.ptr, val.data(), sizeof(float) * val.size(), cudaMemcpyHostToDevice));
  }
  MJ_CUDA(cudaMemcpy(b->rs_src_ptr.ptr, dptr.data(), sizeof(int) * dptr.size(), cudaMemcpyHostToDevice));
  MJ_CUDA(b->rs_sync.alloc(sizeof(SyncState)));
  MJ_CUDA(cudaMemset(b->rs_sync.ptr, 0, sizeof(SyncState)));
  MJ_CUDA(b->rs_err.alloc(sizeof(int)));
  MJ_CUDA(cudaMemset(b->rs_err.ptr, 0, sizeof(int)));

  int dev = 0, coop = 0;
  MJ_CUDA(cudaGetDevice(&dev));
  MJ_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
  b->fused = false;
  if (!coop) return MJ_OK;
  const std::vector<RsVariant>& all = rs_variants();
  cudaEvent_t e0, e1;
  MJ_CUDA(cudaEventCreate(&e0));
  MJ_CUDA(cudaEventCreate(&e1));
  const uint64_t before = launch_counter().load();
  double best = 1e300;
  int bi = -1;
  std::vector<DevBuf> lists(all.size());
  std::vector<int> counts(all.size(), 0), grids(all.size(), 0);
  for (size_t c = 0; c < all.size(); c++) {
    const RsVariant& v = all[c];
    if (v.n != op->n || b->S % (v.LB * v.V) != 0) continue;
    if (rs_buf(3, 4, 0, 8, b->S).end > v.half) continue;  // one dof (up to 8 contributions) must fit
    int ctas = 0;
    if (rs_prepare(v, &ctas) != MJ_OK || ctas < 1) continue;
    const std::vector<RsChunk> ch = rs_chunks(b, v.half, is_src);
    if (ch.empty()) continue;  // a dof with too many contributions for one buffer
    MJ_CUDA(lists[c].alloc(sizeof(RsChunk) * ch.size()));
    MJ_CUDA(cudaMemcpy(lists[c].ptr, ch.data(), sizeof(RsChunk) * ch.size(), cudaMemcpyHostToDevice));
    counts[c] = (int)ch.size();
    grids[c] = ctas * sm_count();
    const RsParams prm = rs_params(b, v);
    int rc = rs_launch(v, grids[c], prm, lists[c].as<RsChunk>(), counts[c], b->rs_sync.as<SyncState>(), 0,
                       b->rs_err.as<int>(), b->stream);
    if (!rc) rc = cudaEventRecord(e0, b->stream) == cudaSuccess ? MJ_OK : MJ_ERR_CUDA;
    for (int k = 1; !rc && k <= 3; k++)
      rc = rs_launch(v, grids[c], prm, lists[c].as<RsChunk>(), counts[c], b->rs_sync.as<SyncState>(), k & 1,
                     b->rs_err.as<int>(), b->stream);
    if (!rc) rc = cudaEventRecord(e1, b->stream) == cudaSuccess ? MJ_OK : MJ_ERR_CUDA;
    if (!rc) rc = rs_check_err(b, b->stream);
    float ms = 0.f;
    if (!rc) rc = cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess ? MJ_OK : MJ_ERR_CUDA;
    if (rc) {
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      return rc;
    }
    b->rs_tune_ms.push_back(ms / 3.0);
    b->rs_tune_variant.push_back((int)c);
    if (ms < best) {
      best = ms;
      bi = (int)c;
    }
  }
  launch_counter().store(before);  // tuning launches are not steps of the caller
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (bi < 0) return MJ_OK;
  b->rs_variant = bi;
  b->rs_threads = all[bi].threads;
  b->rs_grid = grids[bi];
  b->rs_n_chunks = counts[bi];
  b->rs_chunks.release();
  std::swap(b->rs_chunks.ptr, lists[bi].ptr);
  std::swap(b->rs_chunks.bytes, lists[bi].bytes);
  b->fused = true;
  return MJ_OK;
}

// Forces the one-kernel step's variant (n of the operator, E, LB, V): its
// chunk list and persistent grid as the creation-time timing would set them;
// captured graphs of the previous variant are dropped.
int lfb_set_step_variant(mj_lfb* b, int E, int LB, int V) {
  mj_op* op = b->op;
  const std::vector<RsVariant>& all = rs_variants();
  int c = -1;
  for (size_t k = 0; k < all.size(); k++)
    if (all[k].n == op->n && all[k].E == E && all[k].LB == LB && all[k].V == V) c = (int)k;
  if (c < 0) {
    set_error("mj_lfb_set_step_variant: no one-kernel step variant with these parameters for this order");
    return MJ_ERR_ARG;
  }
  const RsVariant& v = all[c];
  if (b->S % (v.LB * v.V) != 0) {
    set_error("mj_lfb_set_step_variant: the number of right-hand sides is not a multiple of the variant's pass");
    return MJ_ERR_ARG;
  }
  int ctas = 0;
  if (int rc = rs_prepare(v, &ctas)) return rc;
  std::vector<char> is_src(op->n_dof, 0);
  if (b->n_src) {
    std::vector<int> si(b->n_src);
    MJ_CUDA(cudaMemcpy(si.data(), b->src_idx.ptr, sizeof(int) * b->n_src, cudaMemcpyDeviceToHost));
    for (int d : si) is_src[d] = 1;
  }
  const std::vector<RsChunk> ch = rs_chunks(b, v.half, is_src);
  if (ch.empty() || ctas < 1) {
    set_error("mj_lfb_set_step_variant: the variant does not fit this integrator");
    return MJ_ERR_ARG;
  }
  MJ_CUDA(b->rs_chunks.alloc(sizeof(RsChunk) * ch.size()));
  MJ_CUDA(cudaMemcpy(b->rs_chunks.ptr, ch.data(), sizeof(RsChunk) * ch.size(), cudaMemcpyHostToDevice));
  b->rs_variant = c;
  b->rs_threads = v.threads;
  b->rs_grid = ctas * sm_count();
  b->rs_n_chunks = (int)ch.size();
  for (auto& g : b->rs_graph)
    if (g) {
      cudaGraphExecDestroy(g);
      g = nullptr;
    }
  b->fused = true;
  return MJ_OK;
}

// mj_lfb_advance with one cooperative kernel per step.  Without traces,
// runs of 20 steps replay a CUDA graph captured for the current step parity.
int lfb_fused_advance(mj_lfb* b, int nsteps, double* traces, int trace_stride, bool use_graph) {
  const RsVariant& v = rs_variants()[b->rs_variant];
  const RsParams prm = rs_params(b, v);
  cudaStream_t s = b->stream;
  const bool diag = traces && b->n_rec;
  const bool prof = b->rs_profile;
  if (prof && b->rs_stamps.bytes < sizeof(unsigned long long) * 4 * b->rs_grid)
    MJ_CUDA(b->rs_stamps.alloc(sizeof(unsigned long long) * 4 * b->rs_grid));
  auto launch = [&](int par, cudaStream_t st) {
    return rs_launch(v, b->rs_grid, prm, b->rs_chunks.as<RsChunk>(), b->rs_n_chunks, b->rs_sync.as<SyncState>(),
                     par, b->rs_err.as<int>(), st,
                     prof ? b->rs_stamps.as<unsigned long long>() : (unsigned long long*)nullptr);
  };
  int done = 0;
  if (use_graph && !diag && !prof && nsteps >= kGraphStepsRs) {
    const int p0 = b->step & 1;
    if (!b->rs_graph[p0]) {
      cudaStream_t cs;
      MJ_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
      cudaGraph_t g;
      const uint64_t before = launch_counter().load();
      MJ_CUDA(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
      for (int k = 0; k < kGraphStepsRs; k++) {
        const int rc = launch((p0 + k) & 1, cs);
        if (rc) {
          cudaStreamEndCapture(cs, &g);
          cudaStreamDestroy(cs);
          return rc;
        }
      }
      MJ_CUDA(cudaStreamEndCapture(cs, &g));
      launch_counter().store(before);  // captured, not launched
      MJ_CUDA(cudaGraphInstantiate(&b->rs_graph[p0], g, 0));
      cudaGraphDestroy(g);
      cudaStreamDestroy(cs);
    }
    while (nsteps - done >= kGraphStepsRs) {
      MJ_CUDA(cudaGraphLaunch(b->rs_graph[p0], s));
      count_launch(kGraphStepsRs);
      done += kGraphStepsRs;
      b->step += kGraphStepsRs;
    }
  }
  for (; done < nsteps; done++) {
    if (diag) lfb_receivers(b, b->cur(), nsteps, done, s);
    const int rc = launch(b->step & 1, s);
    if (rc) return rc;
    b->cur_is_a = !b->cur_is_a;
    b->step++;
  }
  if (diag)
    for (int r = 0; r < b->n_rec * b->S; r++)
      MJ_CUDA(cudaMemcpyAsync(traces + (size_t)r * trace_stride, b->traces_d.as<double>() + (size_t)r * nsteps,
                              sizeof(double) * nsteps, cudaMemcpyDeviceToHost, s));
  return rs_check_err(b, s);
}

// One step of the one-kernel form on caller-given states: U^n = u0,
// U^{n+1} = u1, U^{n+2} written to out (out may be u0); the pulse index is
// ctr[0] (set by the caller), sources only when `sources`.  Used by the
// adjoint's checkpoint replays and its adjoint steps.
int lfb_fused_step_on(mj_lfb* b, float* u0, float* u1, float* out, bool sources, cudaStream_t s) {
  const RsVariant& v = rs_variants()[b->rs_variant];
  RsParams prm = rs_params(b, v);
  prm.ua = u0;
  prm.ub = u1;
  prm.uout = out;
  if (!sources) {
    prm.n_src_dof = 0;
    prm.n_pulse = 0;
  }
  return rs_launch(v, b->rs_grid, prm, b->rs_chunks.as<RsChunk>(), b->rs_n_chunks, b->rs_sync.as<SyncState>(), 0,
                   b->rs_err.as<int>(), s);
}

// lfb_fused_step_on without sources, in the EN form: also
// gacc[e] += gcoef[e] * sum_s sum_q ue[dof_q][s] (A_e u1)_q.  *done = false,
// with nothing launched, when the EN form of the step's variant does not fit
// (its shared memory grows with S); the caller then runs the plain step and
// the ENERGY kernel, which give the same bits.
int lfb_fused_step_en(mj_lfb* b, float* u0, float* u1, float* out, const float* ue, double* gacc,
                      const double* gcoef, cudaStream_t s, bool* done) {
  *done = false;
  const RsVariant& v = rs_variants()[b->rs_variant];
  if (b->rs_en_variant != b->rs_variant) {
    int ctas = 0;
    if (int rc = rs_en_prepare(v.n, v.E, v.LB, v.V, b->S, &ctas)) return rc;
    b->rs_en_variant = b->rs_variant;
    b->rs_en_grid = ctas * sm_count();
  }
  if (b->rs_en_grid < 1) return MJ_OK;
  RsParams prm = rs_params(b, v);
  prm.ua = u0;
  prm.ub = u1;
  prm.uout = out;
  prm.n_src_dof = 0;
  prm.n_pulse = 0;
  prm.ue = ue;
  prm.gacc = gacc;
  prm.gcoef = gcoef;
  const int rc = rs_en_launch(v.n, v.E, v.LB, v.V, b->S, b->rs_en_grid, prm, b->rs_chunks.as<RsChunk>(),
                              b->rs_n_chunks, b->rs_sync.as<SyncState>(), 0, b->rs_err.as<int>(), s);
  *done = rc == MJ_OK;
  return rc;
}

// Error flag of the one-kernel step (bounded waits), reset when set.
int lfb_fused_check(mj_lfb* b, cudaStream_t s) { return rs_check_err(b, s); }

// One ordinary step of the one-kernel form (the integrator's own states and
// step counter); copy: where a second copy of the new state goes, or nullptr.
int lfb_fused_step(mj_lfb* b, cudaStream_t s, float* copy) {
  const RsVariant& v = rs_variants()[b->rs_variant];
  RsParams prm = rs_params(b, v);
  prm.ucopy = copy;
  return rs_launch(v, b->rs_grid, prm, b->rs_chunks.as<RsChunk>(), b->rs_n_chunks, b->rs_sync.as<SyncState>(),
                   b->step & 1, b->rs_err.as<int>(), s);
}

// Phase times (ms) of the last profiled step: element phase (last CTA,
// mean CTA), barrier release, dof phase.
int lfb_phase_ms(const mj_lfb* b, double* out) {
  if (!b->rs_stamps.ptr) {
    set_error("mj_lfb_phase_ms: no profiled step has run (mj_lfb_profile)");
    return MJ_ERR_STATE;
  }
  const int grid = b->rs_grid;
  std::vector<unsigned long long> st(4 * (size_t)grid);
  MJ_CUDA(cudaMemcpy(st.data(), b->rs_stamps.ptr, sizeof(unsigned long long) * st.size(), cudaMemcpyDeviceToHost));
  unsigned long long t0 = ~0ull, p1max = 0, p2 = 0, end = 0;
  double p1sum = 0;
  for (int c = 0; c < grid; c++) t0 = std::min(t0, st[4 * c]);
  for (int c = 0; c < grid; c++) {
    p1max = std::max(p1max, st[4 * c + 1]);
    p1sum += double(st[4 * c + 1] - t0);
    p2 = std::max(p2, st[4 * c + 2]);
    end = std::max(end, st[4 * c + 3]);
  }
  out[0] = double(p1max - t0) * 1e-6;
  out[1] = p1sum / grid * 1e-6;
  out[2] = double(p2 - p1max) * 1e-6;
  out[3] = double(end - p2) * 1e-6;
  return MJ_OK;
}

}  // namespace mj
