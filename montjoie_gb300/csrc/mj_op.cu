// Operator (MltAdd) and leap-frog integrator behind the C ABI.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "mj_common.cuh"
#include "mj_internal.cuh"
#include "mj_kernels.cuh"

#include <mutex>

namespace mj {

namespace {
thread_local std::string g_last_error;
}

void set_error(const std::string& msg) { g_last_error = msg; }

std::atomic<uint64_t>& launch_counter() {
  static std::atomic<uint64_t> c{0};
  return c;
}

int sm_count() {
  int dev = 0, n = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 1;
  if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 1;
  return n > 0 ? n : 1;
}

// Sum of the per-block partial norms by one warp in a fixed order (lane l
// sums partials l, l+32, ..., then a fixed shuffle tree): deterministic.
template <typename Real>
__global__ void k_cast_from_f64(const double* __restrict__ a, Real* __restrict__ b, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) b[i] = Real(a[i]);
}
template <typename Real>
__global__ void k_cast_to_f64(const Real* __restrict__ a, double* __restrict__ b, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) b[i] = double(a[i]);
}

// Power-iteration helpers (mj_op_power_iteration): per-block sums of squares
// (the host adds the block sums in block order), y *= w, x = y / s.
__global__ void k_sumsq_blocks(const double* __restrict__ a, int n, double* __restrict__ partial) {
  __shared__ double sh[256];
  double acc = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) acc += a[i] * a[i];
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = sh[0];
}
__global__ void k_mul(double* __restrict__ y, const double* __restrict__ w, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) y[i] *= w[i];
}
__global__ void k_div(const double* __restrict__ y, double s, double* __restrict__ x, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) x[i] = y[i] / s;
}

}  // namespace mj

using namespace mj;


namespace {

// One launch of the element kernel with the operator's tuned variant (its
// instance compiled with a bulk-copy wait limit of 0 while the test hook
// mj_debug_set_wait_limits asks for it and one exists).
void launch_k1(mj_op* op, const void* x, cudaStream_t s) {
  if (k1_waits_run_out() && !op->packed) {
    const bool done =
        op->warp ? k1_launch_w_f32_waits_out(op->n, op->E, op->grid_k1, x, op->nodle_e.as<int>(), op->fac_e.ptr,
                                            op->R.ptr, op->slot_e.as<int>(), op->n_tiles, op->err.as<int>(), s)
        : op->precision == MJ_FP64 && !op->vec
            ? k1_launch_f64_waits_out(op->n, op->E, op->grid_k1, x, op->nodle_e.as<int>(), op->fac_e.ptr, op->R.ptr,
                                      op->slot_e.as<int>(), op->n_tiles, op->err.as<int>(), s)
            : false;
    if (done) {
      count_launch();
      return;
    }
  }
  if (op->warp) {
    k1_launch_w_f32(op->n, op->E, op->packed, op->grid_k1, x, (op->packed ? op->nodle_pk : op->nodle_e).as<int>(),
                    op->fac_e.ptr, op->R.ptr, (op->packed ? op->ptr : op->slot_e).as<int>(), op->n_tiles,
                    op->err.as<int>(), s);
    count_launch();
    return;
  }
  if (op->fs) {
    k1_launch_fs_f32(op->n, op->E, op->grid_k1, x, op->nodle_e.as<int>(), op->fac_e.ptr, op->R.ptr,
                     op->slot_e.as<int>(), op->n_tiles, op->err.as<int>(), s);
    count_launch();
    return;
  }
  if (op->precision == MJ_FP64)
    k1_launch_f64(op->n, op->E, op->vec, op->grid_k1, x, op->nodle_e.as<int>(), op->fac_e.ptr, op->R.ptr,
                  op->slot_e.as<int>(), op->n_tiles, op->err.as<int>(), s);
  else
    k1_launch_f32(op->n, op->E, op->vec, op->grid_k1, x, op->nodle_e.as<int>(), op->fac_e.ptr, op->R.ptr,
                  op->slot_e.as<int>(), op->n_tiles, op->err.as<int>(), s);
  count_launch();
}

template <typename Real>
void launch_k1(mj_op* op, const void* x, cudaStream_t s) {
  launch_k1(op, x, s);
}

// Autotuner: every instantiated tile size E of this order, on a persistent
// grid of (CTAs per SM x SMs) CTAs, is timed with CUDA events on the
// operator's own data (3 launches after 1 warm-up); the fastest is kept.
// Small meshes skip the timing and take the variant with the most resident
// threads.
int autotune_k1(mj_op* op) {
  const std::vector<int> cands = k1_tile_candidates(op->n);
  const int sms = sm_count();
  const size_t esz = op->precision == MJ_FP64 ? sizeof(double) : sizeof(float);
  DevBuf x;
  MJ_CUDA(x.alloc(esz * op->n_dof));
  MJ_CUDA(cudaMemset(x.ptr, 0, esz * op->n_dof));
  cudaEvent_t e0, e1;
  MJ_CUDA(cudaEventCreate(&e0));
  MJ_CUDA(cudaEventCreate(&e1));
  double best = 1e300;
  int bestE = -1, bestGrid = 1;
  bool bestVec = false, bestWarp = false, bestPacked = false, bestFs = false;
  const bool time_it = (long long)op->n_elt * op->Q >= 2000000;
  // layouts: 0 compact, 1 vector lines, 2 one element per warp, 3 the same
  // with packed connectivity, 4 compact with one factor stage (2-4: FP32)
  std::vector<int> layouts = {0};
  if (op->precision == MJ_FP32) {
    layouts = {0, 1, 2};
    if (op->nodle_pk.ptr) layouts.push_back(3);
    layouts.push_back(4);
  }
  for (int lay : layouts)
    for (int E : ((lay == 2 || lay == 3) ? k1_warp_tile_candidates(op->n) : cands)) {
      const bool vec = lay == 1, warp = lay == 2 || lay == 3, packed = lay == 3, fs = lay == 4;
      int ctas = 0;
      const int rc = warp ? k1_prepare_w_f32(op->n, E, packed, &ctas)
                     : fs ? k1_prepare_fs_f32(op->n, E, &ctas)
                          : op->precision == MJ_FP64 ? k1_prepare_f64(op->n, E, vec, &ctas)
                                                     : k1_prepare_f32(op->n, E, vec, &ctas);
      if (rc != MJ_OK) continue;
      const int tiles = op->n_elt_pad / E;
      const int grid = std::max(1, std::min(tiles, ctas * sms));
      double ms = 0.0;
      if (time_it) {
        op->E = E; op->vec = vec; op->warp = warp; op->packed = packed; op->fs = fs; op->grid_k1 = grid;
        op->n_tiles = tiles;
        launch_k1(op, x.ptr, op->stream);
        MJ_CUDA(cudaEventRecord(e0, op->stream));
        for (int rep = 0; rep < 3; rep++) launch_k1(op, x.ptr, op->stream);
        MJ_CUDA(cudaEventRecord(e1, op->stream));
        MJ_CUDA(cudaEventSynchronize(e1));
        float f = 0.f;
        MJ_CUDA(cudaEventElapsedTime(&f, e0, e1));
        ms = f / 3.0;
      } else {
        ms = -double(ctas) * E * op->n * op->n + (vec ? 0.5 : 0.0) + (warp ? 0.75 : 0.0) +
             (packed ? 0.1 : 0.0) + (fs ? 0.25 : 0.0);  // most resident threads first
      }
      op->tune_E.push_back(E);
      op->tune_vec.push_back(lay);
      op->tune_ms.push_back(ms);
      if (ms < best) {
        best = ms; bestE = E; bestGrid = grid; bestVec = vec; bestWarp = warp; bestPacked = packed; bestFs = fs;
      }
    }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (bestE < 0) {
    set_error("mj_op_create: no element kernel variant fits this device");
    return MJ_ERR_CUDA;
  }
  op->E = bestE;
  op->vec = bestVec;
  op->warp = bestWarp;
  op->packed = bestPacked;
  op->fs = bestFs;
  op->grid_k1 = bestGrid;
  // the chosen variant's shared-memory attribute must be the one set last
  {
    int ctas = 0;
    const int rc = bestWarp ? k1_prepare_w_f32(op->n, bestE, bestPacked, &ctas)
                   : bestFs ? k1_prepare_fs_f32(op->n, bestE, &ctas)
                            : op->precision == MJ_FP64 ? k1_prepare_f64(op->n, bestE, bestVec, &ctas)
                                                       : k1_prepare_f32(op->n, bestE, bestVec, &ctas);
    if (rc) return rc;
  }
  op->n_tiles = op->n_elt_pad / bestE;
  MJ_CUDA(cudaMemset(op->err.ptr, 0, sizeof(int)));
  MJ_CUDA(cudaGetLastError());
  return MJ_OK;
}

}  // namespace

int mj::take_kernel_error(void* dev_flag, cudaStream_t s, const char* what) {
  int herr = 0;
  MJ_CUDA(cudaMemcpyAsync(&herr, dev_flag, sizeof(int), cudaMemcpyDeviceToHost, s));
  MJ_CUDA(cudaStreamSynchronize(s));
  if (!herr) return MJ_OK;
  MJ_CUDA(cudaMemsetAsync(dev_flag, 0, sizeof(int), s));
  MJ_CUDA(cudaStreamSynchronize(s));
  set_error(std::string(what) + ": a bounded wait of a kernel on its bulk copies timed out (results invalid)");
  return MJ_ERR_CUDA;
}

namespace {
struct WaitLimitRegistry {
  std::mutex m;
  std::vector<mj::WaitLimitSetter> setters;
};
WaitLimitRegistry& wait_limit_registry() {
  static WaitLimitRegistry r;
  return r;
}
}  // namespace

bool& mj::k1_waits_run_out() {
  static bool on = false;
  return on;
}

void mj::register_wait_limit_setter(mj::WaitLimitSetter f) {
  WaitLimitRegistry& r = wait_limit_registry();
  std::lock_guard<std::mutex> lock(r.m);
  r.setters.push_back(f);
}

int mj::stream_grid(int n) {
  long g = (n + 255) / 256;
  return (int)std::max(1L, std::min<long>(g, (long)sm_count() * 16));
}

namespace {

template <typename Real>
int mltadd_impl(mj_op* op, double alpha, const void* x, double beta, void* y, cudaStream_t s) {
  launch_k1<Real>(op, x, s);
  k_gather_mltadd<Real><<<stream_grid(op->n_dof), 256, 0, s>>>(op->R.as<Real>(), op->ptr.as<int>(), Real(alpha),
                                                                Real(beta), static_cast<Real*>(y), op->n_dof);
  count_launch();
  MJ_CUDA(cudaGetLastError());
  return MJ_OK;
}


// Copies a host double vector into a device vector of the operator precision.
int upload_vec(mj_op* op, const double* h, void* d, DevBuf& stage, cudaStream_t s) {
  const int n = op->n_dof;
  if (op->precision == MJ_FP64) {
    MJ_CUDA(cudaMemcpyAsync(d, h, sizeof(double) * n, cudaMemcpyHostToDevice, s));
    return MJ_OK;
  }
  if (stage.bytes < sizeof(double) * n) MJ_CUDA(stage.alloc(sizeof(double) * n));
  MJ_CUDA(cudaMemcpyAsync(stage.ptr, h, sizeof(double) * n, cudaMemcpyHostToDevice, s));
  k_cast_from_f64<float><<<stream_grid(n), 256, 0, s>>>(stage.as<double>(), static_cast<float*>(d), n);
  count_launch();
  MJ_CUDA(cudaGetLastError());
  return MJ_OK;
}

int download_vec(mj_op* op, const void* d, double* h, DevBuf& stage, cudaStream_t s) {
  const int n = op->n_dof;
  if (op->precision == MJ_FP64) {
    MJ_CUDA(cudaMemcpyAsync(h, d, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
    return MJ_OK;
  }
  if (stage.bytes < sizeof(double) * n) MJ_CUDA(stage.alloc(sizeof(double) * n));
  k_cast_to_f64<float><<<stream_grid(n), 256, 0, s>>>(static_cast<const float*>(d), stage.as<double>(), n);
  count_launch();
  MJ_CUDA(cudaGetLastError());
  MJ_CUDA(cudaMemcpyAsync(h, stage.ptr, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
  return MJ_OK;
}

size_t elem_size(int precision) { return precision == MJ_FP64 ? sizeof(double) : sizeof(float); }

}  // namespace

extern "C" {

const char* mj_last_error(void) { return g_last_error.c_str(); }

const char* mj_version(void) { return "montjoie_gb300 0.1 (sm_103a)"; }

uint64_t mj_kernel_launches(void) { return launch_counter().load(); }

}  // extern "C"

namespace {

// Element-major connectivity, incidence slots and CSR of an operator from the
// reference-layout Nodle (host), uploaded; the factors are left to the caller
// (host factors: mj_op_create; device geometry: mj_op_create_geometry).
int op_layout(mj_op* op, const mj_mesh_desc* mesh, const double* gradphi, int precision, const char* who) {
  const int r = mesh->order;
  MJ_CHECK_ARG(r >= 1 && r <= kMaxOrder, std::string(who) + ": order must be in [1, 8]");
  MJ_CHECK_ARG(mesh->n_elt > 0 && mesh->n_dof > 0, std::string(who) + ": empty mesh");
  MJ_CHECK_ARG(mesh->nodle, std::string(who) + ": nodle is required");
  MJ_CHECK_ARG(precision == MJ_FP64 || precision == MJ_FP32, std::string(who) + ": precision must be MJ_FP64 or MJ_FP32");
  const int n = r + 1, Q = n * n * n, NN = n * n;
  const long long total_pts = (long long)mesh->n_elt * Q;
  MJ_CHECK_ARG(total_pts < (1LL << 31) - 1, std::string(who) + ": n_elt*(r+1)^3 exceeds int32 indexing");
  op->order = r; op->n = n; op->Q = Q; op->n_elt = mesh->n_elt; op->n_dof = mesh->n_dof;
  op->precision = precision;
  op->Qp = elem_slots(n);
  op->n_elt_pad = (mesh->n_elt + kElemPad - 1) / kElemPad * kElemPad;
  op->r_len = (size_t)op->n_elt_pad * op->Qp;
  MJ_CHECK_ARG(op->r_len < (size_t)INT32_MAX - 1, std::string(who) + ": mesh too large for int32 incidences");
  if (gradphi) {
    for (int a = 0; a < NN; a++) op->gradphi[a] = gradphi[a];
  } else {
    double pts[kMaxN], wts[kMaxN];
    gauss_lobatto(r, pts, wts);
    gl_derivative_matrix(r, pts, op->gradphi);
  }
  for (int a = 0; a < NN; a++)
    MJ_CHECK_ARG(std::isfinite(op->gradphi[a]), std::string(who) + ": non-finite derivative matrix");

  const std::vector<int> num = hex_local_numbering(r);
  const size_t Qp = (size_t)op->Qp;
  std::vector<int> nodle_e(op->r_len, 0);
  std::vector<int> count(op->n_dof + 1, 0);
  for (long long t = 0; t < total_pts; t++) {
    const int d = mesh->nodle[t];
    MJ_CHECK_ARG(d >= 0 && d < mesh->n_dof, std::string(who) + ": Nodle entry out of [0, n_dof)");
    count[d + 1]++;
  }
  for (int d = 0; d < op->n_dof; d++)
    MJ_CHECK_ARG(count[d + 1] > 0, std::string(who) + ": a dof belongs to no element");
  op->h_ptr.assign(op->n_dof + 1, 0);
  for (int d = 0; d < op->n_dof; d++) op->h_ptr[d + 1] = op->h_ptr[d] + count[d + 1];
  op->n_inc = (size_t)total_pts;
  // slot of every element point: its position in the dof-ordered incidence
  // list; padding points write to the spare entry R[n_inc]
  std::vector<int> slot_e(op->r_len, (int)op->n_inc);
  std::vector<int> fill(op->h_ptr.begin(), op->h_ptr.end() - 1);
  std::vector<int> ql_of(Q);  // element-major slot p -> local index
  for (int k = 0; k < n; k++)
    for (int j = 0; j < n; j++)
      for (int i = 0; i < n; i++) ql_of[(k * n + j) * n + i] = num[(i * n + j) * n + k];
  // Walk R slots in increasing order so each dof's incidences come out sorted.
  for (int e = 0; e < mesh->n_elt; e++) {
    const int32_t* row = mesh->nodle + (size_t)e * Q;
    int* ne = nodle_e.data() + (size_t)e * Qp;
    int* se = slot_e.data() + (size_t)e * Qp;
    for (int p = 0; p < Q; p++) {
      const int d = row[ql_of[p]];
      ne[p] = d;
      se[p] = fill[d]++;
    }
  }
  // packed connectivity for the FP32 warp-per-element kernel: dof | rank << kPkDofBits
  // (rank = the slot's place among the dof's incidences), padding -> the spare dof n_dof
  int max_deg = 0;
  for (int d = 0; d < op->n_dof; d++) max_deg = std::max(max_deg, count[d + 1]);
  if (precision == MJ_FP32 && !k1_warp_tile_candidates(n).empty() && op->n_dof < (1 << kPkDofBits) &&
      max_deg <= kPkMaxRank + 1) {
    std::vector<int> pk(op->r_len, op->n_dof);
    for (int e = 0; e < mesh->n_elt; e++)
      for (int p = 0; p < Q; p++) {
        const size_t rp = (size_t)e * Qp + p;
        const int d = nodle_e[rp];
        pk[rp] = (int)((unsigned)d | ((unsigned)(slot_e[rp] - op->h_ptr[d]) << kPkDofBits));
      }
    MJ_CUDA(op->nodle_pk.alloc(sizeof(int) * op->r_len));
    MJ_CUDA(cudaMemcpy(op->nodle_pk.ptr, pk.data(), sizeof(int) * op->r_len, cudaMemcpyHostToDevice));
  }
  const size_t esz = elem_size(precision);
  MJ_CUDA(op->nodle_e.alloc(sizeof(int) * op->r_len));
  MJ_CUDA(op->slot_e.alloc(sizeof(int) * op->r_len));
  MJ_CUDA(op->fac_e.alloc((size_t)op->n_elt_pad * 6 * Qp * esz));
  // 3 spare entries past the dummy slot: 16-byte rounded bulk copies of a
  // dof range of R stay inside the buffer
  MJ_CUDA(op->R.alloc(esz * (op->n_inc + 4)));
  MJ_CUDA(op->ptr.alloc(sizeof(int) * (op->n_dof + 8)));  // padded like R
  MJ_CUDA(cudaMemset(op->ptr.ptr, 0, sizeof(int) * (op->n_dof + 8)));
  MJ_CUDA(cudaMemcpy(op->nodle_e.ptr, nodle_e.data(), sizeof(int) * op->r_len, cudaMemcpyHostToDevice));
  MJ_CUDA(cudaMemcpy(op->slot_e.ptr, slot_e.data(), sizeof(int) * op->r_len, cudaMemcpyHostToDevice));
  MJ_CUDA(cudaMemcpy(op->ptr.ptr, op->h_ptr.data(), sizeof(int) * (op->n_dof + 1), cudaMemcpyHostToDevice));
  MJ_CUDA(cudaMemset(op->R.ptr, 0, esz * (op->n_inc + 4)));
  MJ_CUDA(op->err.alloc(sizeof(int)));
  MJ_CUDA(cudaMemset(op->err.ptr, 0, sizeof(int)));
  return MJ_OK;
}

// Derivative matrix into constant memory and the element-kernel autotuner.
int op_finish(mj_op* op) {
  int rc = op->precision == MJ_FP64 ? k1_set_gmat_f64(op->n, op->gradphi) : k1_set_gmat_f32(op->n, op->gradphi);
  if (rc) return rc;
  return autotune_k1(op);
}

}  // namespace

extern "C" {

int mj_op_create(const mj_mesh_desc* mesh, const mj_geom_desc* geom, int precision, mj_op** out) {
  MJ_CHECK_ARG(mesh && geom && out, "mj_op_create: null argument");
  *out = nullptr;
  MJ_CHECK_ARG(geom->factors, "mj_op_create: nodle and factors are required");
  if (mesh->order >= 1 && mesh->order <= kMaxOrder && mesh->n_elt > 0) {
    const size_t nf = (size_t)mesh->n_elt * (mesh->order + 1) * (mesh->order + 1) * (mesh->order + 1) * 6;
    for (size_t t = 0; t < nf; t++)
      if (!std::isfinite(geom->factors[t])) {
        set_error("mj_op_create: non-finite stiffness factor");
        return MJ_ERR_NONFINITE;
      }
  }
  std::unique_ptr<mj_op> op(new mj_op());
  int rc = op_layout(op.get(), mesh, geom->gradphi, precision, "mj_op_create");
  if (rc) return rc;
  const int n = op->n, Q = op->Q;
  const size_t Qp = (size_t)op->Qp;
  const std::vector<int> num = hex_local_numbering(op->order);
  std::vector<unsigned char> fac_bytes(op->fac_e.bytes, 0);
  double* fac64 = reinterpret_cast<double*>(fac_bytes.data());
  float* fac32 = reinterpret_cast<float*>(fac_bytes.data());
  for (int e = 0; e < op->n_elt; e++)
    for (int k = 0; k < n; k++)
      for (int j = 0; j < n; j++)
        for (int i = 0; i < n; i++) {
          const int p = (k * n + j) * n + i;
          const size_t src = (size_t)e * Q + num[(i * n + j) * n + k];
          for (int c = 0; c < 6; c++) {
            const double v = geom->factors[src * 6 + c];
            const size_t fp = ((size_t)e * 6 + c) * Qp + p;
            if (precision == MJ_FP64) fac64[fp] = v;
            else fac32[fp] = (float)v;
          }
        }
  MJ_CUDA(cudaMemcpy(op->fac_e.ptr, fac_bytes.data(), fac_bytes.size(), cudaMemcpyHostToDevice));
  rc = op_finish(op.get());
  if (rc) return rc;
  *out = op.release();
  return MJ_OK;
}

int mj_op_create_geometry(const mj_mesh_desc* mesh, const double* verts, const double* mu, int precision,
                          mj_op** out) {
  MJ_CHECK_ARG(mesh && verts && mu && out, "mj_op_create_geometry: null argument");
  *out = nullptr;
  for (int e = 0; e < mesh->n_elt; e++)
    MJ_CHECK_ARG(std::isfinite(mu[e]) && mu[e] >= 0, "mj_op_create_geometry: mu must be finite and >= 0");
  std::unique_ptr<mj_op> op(new mj_op());
  int rc = op_layout(op.get(), mesh, nullptr, precision, "mj_op_create_geometry");
  if (rc) return rc;
  cudaStream_t s = op->stream;
  MJ_CUDA(op->verts.alloc(sizeof(double) * 24 * op->n_elt));
  MJ_CUDA(cudaMemcpyAsync(op->verts.ptr, verts, sizeof(double) * 24 * op->n_elt, cudaMemcpyHostToDevice, s));
  DevBuf dmu, bad;
  MJ_CUDA(dmu.alloc(sizeof(double) * op->n_elt));
  MJ_CUDA(cudaMemcpyAsync(dmu.ptr, mu, sizeof(double) * op->n_elt, cudaMemcpyHostToDevice, s));
  MJ_CUDA(bad.alloc(sizeof(int)));
  MJ_CUDA(cudaMemsetAsync(bad.ptr, 0, sizeof(int), s));
  MJ_CUDA(cudaMemsetAsync(op->fac_e.ptr, 0, op->fac_e.bytes, s));  // padding elements and slots
  rc = geometry_elem_major(op->order, op->n_elt, op->Qp, op->verts.as<double>(), dmu.as<double>(),
                           precision == MJ_FP64 ? op->fac_e.as<double>() : nullptr,
                           precision == MJ_FP32 ? op->fac_e.as<float>() : nullptr, nullptr, nullptr, bad.as<int>(), s);
  if (rc) return rc;
  int hbad = 0;
  MJ_CUDA(cudaMemcpyAsync(&hbad, bad.ptr, sizeof(int), cudaMemcpyDeviceToHost, s));
  MJ_CUDA(cudaStreamSynchronize(s));
  if (hbad) {
    set_error("mj_op_create_geometry: " + std::to_string(hbad) + " quadrature points with non-positive Jacobian");
    return MJ_ERR_GEOMETRY;
  }
  rc = op_finish(op.get());
  if (rc) return rc;
  *out = op.release();
  return MJ_OK;
}

namespace {
// rho J w (center == NULL) or J w g(x) summed per dof on the device, into `d_out` (device, n_dof).
int op_assemble(mj_op* op, const double* rho, const double* center, double radius, double* d_out, const char* who) {
  if (!op->verts.ptr) {
    set_error(std::string(who) + ": the operator was not built from its geometry (mj_op_create_geometry)");
    return MJ_ERR_STATE;
  }
  cudaStream_t s = op->stream;
  const size_t pts = op->r_len;
  DevBuf jw, xq, tmp, drho, bad;
  MJ_CUDA(jw.alloc(sizeof(double) * pts));
  if (center) MJ_CUDA(xq.alloc(sizeof(double) * 3 * pts));
  MJ_CUDA(tmp.alloc(sizeof(double) * (op->n_inc + 1)));
  MJ_CUDA(bad.alloc(sizeof(int)));
  MJ_CUDA(cudaMemsetAsync(bad.ptr, 0, sizeof(int), s));
  if (rho) {
    MJ_CUDA(drho.alloc(sizeof(double) * op->n_elt));
    MJ_CUDA(cudaMemcpyAsync(drho.ptr, rho, sizeof(double) * op->n_elt, cudaMemcpyHostToDevice, s));
  }
  int rc = geometry_elem_major(op->order, op->n_elt, op->Qp, op->verts.as<double>(), nullptr, nullptr, nullptr,
                               jw.as<double>(), center ? xq.as<double>() : nullptr, bad.as<int>(), s);
  if (rc) return rc;
  return assemble_points(op->order, op->n_elt, op->Qp, jw.as<double>(), xq.as<double>(), drho.as<double>(),
                         op->slot_e.as<int>(), op->ptr.as<int>(), op->n_dof, center, radius, tmp.as<double>(), d_out,
                         s);
}
}  // namespace

int mj_op_lumped_mass(mj_op* op, const double* rho, double* mass_out) {
  MJ_CHECK_ARG(op && mass_out, "mj_op_lumped_mass: null argument");
  if (rho)
    for (int e = 0; e < op->n_elt; e++)
      MJ_CHECK_ARG(std::isfinite(rho[e]) && rho[e] > 0, "mj_op_lumped_mass: rho must be finite and > 0");
  DevBuf d;
  MJ_CUDA(d.alloc(sizeof(double) * op->n_dof));
  int rc = op_assemble(op, rho, nullptr, 0.0, d.as<double>(), "mj_op_lumped_mass");
  if (rc) return rc;
  MJ_CUDA(cudaMemcpyAsync(mass_out, d.ptr, sizeof(double) * op->n_dof, cudaMemcpyDeviceToHost, op->stream));
  MJ_CUDA(cudaStreamSynchronize(op->stream));
  return MJ_OK;
}

int mj_op_gaussian_source(mj_op* op, const double* center, double radius, int capacity, int32_t* idx_out,
                          double* val_out, int* n_out) {
  MJ_CHECK_ARG(op && center && n_out, "mj_op_gaussian_source: null argument");
  MJ_CHECK_ARG(radius > 0 && std::isfinite(radius), "mj_op_gaussian_source: radius must be positive");
  DevBuf d;
  MJ_CUDA(d.alloc(sizeof(double) * op->n_dof));
  int rc = op_assemble(op, nullptr, center, radius, d.as<double>(), "mj_op_gaussian_source");
  if (rc) return rc;
  std::vector<double> F(op->n_dof);
  MJ_CUDA(cudaMemcpyAsync(F.data(), d.ptr, sizeof(double) * op->n_dof, cudaMemcpyDeviceToHost, op->stream));
  MJ_CUDA(cudaStreamSynchronize(op->stream));
  int cnt = 0;
  for (int i = 0; i < op->n_dof; i++)
    if (F[i] != 0.0) {
      if (idx_out && val_out && cnt < capacity) {
        idx_out[cnt] = i;
        val_out[cnt] = F[i];
      }
      cnt++;
    }
  *n_out = cnt;
  if ((idx_out || val_out) && cnt > capacity) {
    set_error("mj_op_gaussian_source: " + std::to_string(cnt) + " source dofs exceed the capacity " +
              std::to_string(capacity));
    return MJ_ERR_ARG;
  }
  return MJ_OK;
}

int mj_op_power_iteration(mj_op* op, const double* inv_mass, const double* x0, int iters, double* lambda_max) {
  MJ_CHECK_ARG(op && inv_mass && x0 && lambda_max && iters > 0, "mj_op_power_iteration: bad argument");
  const int n = op->n_dof;
  cudaStream_t s = op->stream;
  const size_t esz = elem_size(op->precision);
  DevBuf x64, y64, w, xo, yo, part;
  constexpr int kBlocks = 1024;
  MJ_CUDA(x64.alloc(sizeof(double) * n));
  MJ_CUDA(y64.alloc(sizeof(double) * n));
  MJ_CUDA(w.alloc(sizeof(double) * n));
  MJ_CUDA(part.alloc(sizeof(double) * kBlocks));
  if (op->precision == MJ_FP32) {
    MJ_CUDA(xo.alloc(esz * n));
    MJ_CUDA(yo.alloc(esz * n));
  }
  MJ_CUDA(cudaMemcpyAsync(x64.ptr, x0, sizeof(double) * n, cudaMemcpyHostToDevice, s));
  MJ_CUDA(cudaMemcpyAsync(w.ptr, inv_mass, sizeof(double) * n, cudaMemcpyHostToDevice, s));
  std::vector<double> hp(kBlocks);
  auto norm = [&](const DevBuf& v, double* out) -> int {
    k_sumsq_blocks<<<kBlocks, 256, 0, s>>>(v.as<double>(), n, part.as<double>());
    count_launch();
    MJ_CUDA(cudaMemcpyAsync(hp.data(), part.ptr, sizeof(double) * kBlocks, cudaMemcpyDeviceToHost, s));
    MJ_CUDA(cudaStreamSynchronize(s));
    double t = 0.0;
    for (double v2 : hp) t += v2;
    *out = std::sqrt(t);
    return MJ_OK;
  };
  const int g = stream_grid(n);
  double lam = 0.0;
  for (int it = 0; it < iters; it++) {
    // y = A x in the operator's precision (the host MltVector's arithmetic), then D^-1 y in FP64
    if (op->precision == MJ_FP32) {
      k_cast_from_f64<float><<<g, 256, 0, s>>>(x64.as<double>(), xo.as<float>(), n);
      count_launch();
      int rc = mltadd_impl<float>(op, 1.0, xo.ptr, 0.0, yo.ptr, s);
      if (rc) return rc;
      k_cast_to_f64<float><<<g, 256, 0, s>>>(yo.as<float>(), y64.as<double>(), n);
      count_launch();
    } else {
      int rc = mltadd_impl<double>(op, 1.0, x64.ptr, 0.0, y64.ptr, s);
      if (rc) return rc;
    }
    k_mul<<<g, 256, 0, s>>>(y64.as<double>(), w.as<double>(), n);
    count_launch();
    double ny = 0.0, nx = 0.0;
    int rc = norm(y64, &ny);
    if (rc) return rc;
    rc = norm(x64, &nx);
    if (rc) return rc;
    if (!(ny > 0.0) || !(nx > 0.0)) {
      set_error("mj_op_power_iteration: the iterate vanished or is not finite");
      return MJ_ERR_NONFINITE;
    }
    lam = ny / nx;
    k_div<<<g, 256, 0, s>>>(y64.as<double>(), ny, x64.as<double>(), n);
    count_launch();
  }
  MJ_CUDA(cudaGetLastError());
  *lambda_max = lam;
  return take_kernel_error(op->err.ptr, s, "mj_op_power_iteration");
}

int mj_op_destroy(mj_op* op) {
  delete op;
  return MJ_OK;
}

int mj_op_info(const mj_op* op, int* order, int* n_elt, int* n_dof, int* precision, size_t* device_bytes) {
  MJ_CHECK_ARG(op, "mj_op_info: null operator");
  if (order) *order = op->order;
  if (n_elt) *n_elt = op->n_elt;
  if (n_dof) *n_dof = op->n_dof;
  if (precision) *precision = op->precision;
  if (device_bytes) *device_bytes = op->device_bytes();
  return MJ_OK;
}

int mj_op_tuning(const mj_op* op, int* tile_elems, int* vector_lines, int* grid, int* n_candidates,
                 double* candidate_ms) {
  MJ_CHECK_ARG(op, "mj_op_tuning: null operator");
  if (tile_elems) *tile_elems = op->E;
  if (vector_lines) *vector_lines = op->fs ? 4 : op->packed ? 3 : op->warp ? 2 : op->vec ? 1 : 0;
  if (grid) *grid = op->grid_k1;
  if (n_candidates) *n_candidates = (int)op->tune_ms.size();
  if (candidate_ms)
    for (size_t c = 0; c < op->tune_ms.size(); c++) candidate_ms[c] = op->tune_ms[c];
  return MJ_OK;
}

int mj_op_set_variant(mj_op* op, int tile_elems, int vector_lines) {
  MJ_CHECK_ARG(op, "mj_op_set_variant: null operator");
  MJ_CHECK_ARG(vector_lines >= 0 && vector_lines <= 4, "mj_op_set_variant: layout must be 0, 1, 2, 3 or 4");
  MJ_CHECK_ARG(vector_lines != 3 || op->nodle_pk.ptr, "mj_op_set_variant: no packed connectivity for this operator");
  const bool warp = vector_lines == 2 || vector_lines == 3, vec = vector_lines == 1, packed = vector_lines == 3;
  const bool fs = vector_lines == 4;
  const std::vector<int> cands = warp ? k1_warp_tile_candidates(op->n) : k1_tile_candidates(op->n);
  MJ_CHECK_ARG(std::find(cands.begin(), cands.end(), tile_elems) != cands.end(),
               "mj_op_set_variant: no element kernel with this tile size and layout for this order");
  MJ_CHECK_ARG(vector_lines == 0 || op->precision == MJ_FP32,
               "mj_op_set_variant: the vector-line, warp and one-factor-stage layouts are FP32 only");
  int ctas = 0;
  const int rc = warp ? k1_prepare_w_f32(op->n, tile_elems, packed, &ctas)
                 : fs ? k1_prepare_fs_f32(op->n, tile_elems, &ctas)
                      : op->precision == MJ_FP64 ? k1_prepare_f64(op->n, tile_elems, false, &ctas)
                                                 : k1_prepare_f32(op->n, tile_elems, vec, &ctas);
  if (rc) return rc;
  op->E = tile_elems;
  op->vec = vec;
  op->warp = warp;
  op->packed = packed;
  op->fs = fs;
  op->n_tiles = op->n_elt_pad / tile_elems;
  op->grid_k1 = std::max(1, std::min(op->n_tiles, ctas * sm_count()));
  return MJ_OK;
}

int mj_op_mltadd_device(mj_op* op, double alpha, const void* x, double beta, void* y, void* stream) {
  MJ_CHECK_ARG(op && x && y, "mj_op_mltadd_device: null argument");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  return op->precision == MJ_FP64 ? mltadd_impl<double>(op, alpha, x, beta, y, s)
                                  : mltadd_impl<float>(op, alpha, x, beta, y, s);
}

int mj_op_mltadd(mj_op* op, double alpha, const double* x, double beta, double* y) {
  MJ_CHECK_ARG(op && x && y, "mj_op_mltadd: null argument");
  const size_t esz = elem_size(op->precision);
  const int n = op->n_dof;
  if (op->xbuf.bytes < esz * n) MJ_CUDA(op->xbuf.alloc(esz * n));
  if (op->ybuf.bytes < esz * n) MJ_CUDA(op->ybuf.alloc(esz * n));
  DevBuf stage;
  cudaStream_t s = op->stream;
  int rc = upload_vec(op, x, op->xbuf.ptr, stage, s);
  if (rc) return rc;
  if (beta != 0.0) {
    rc = upload_vec(op, y, op->ybuf.ptr, stage, s);
    if (rc) return rc;
  }
  rc = mj_op_mltadd_device(op, alpha, op->xbuf.ptr, beta, op->ybuf.ptr, s);
  if (rc) return rc;
  rc = download_vec(op, op->ybuf.ptr, y, stage, s);
  if (rc) return rc;
  return take_kernel_error(op->err.ptr, s, "mj_op_mltadd");
}

int mj_debug_set_wait_limits(long long mbar_polls, long long barrier_polls, long long barrier_ns) {
  mj::k1_waits_run_out() = mbar_polls == 0;
  mj::WaitLimits w;
  w.barrier_polls =
      barrier_polls >= 0 ? (long)std::min<long long>(barrier_polls, mj::kBarrierPolls) : mj::kBarrierPolls;
  w.barrier_ns = barrier_ns >= 0 ? std::min<unsigned long long>(barrier_ns, mj::kBarrierNs) : mj::kBarrierNs;
  WaitLimitRegistry& r = wait_limit_registry();
  std::lock_guard<std::mutex> lock(r.m);
  for (mj::WaitLimitSetter f : r.setters)
    if (f(w)) {
      set_error("mj_debug_set_wait_limits: cudaMemcpyToSymbol failed");
      return MJ_ERR_CUDA;
    }
  return MJ_OK;
}

}  // extern "C"

namespace {

// Sources sorted by dof with a per-dof bit mask, looked up inside the
// order-4 and streaming gathers.
int lf_sorted_sources(mj_lf* lf) {
  const int n = lf->n_dof;
  const size_t esz = elem_size(lf->op->precision);
  // sources sorted by dof with a per-dof bit mask (looked up inside the gathers)
  const int ns = lf->n_src, words = (n + 31) / 32;
  std::vector<int> idx(std::max(1, ns));
  std::vector<unsigned char> val(esz * std::max(1, ns));
  if (ns) {
    MJ_CUDA(cudaMemcpy(idx.data(), lf->src_idx.ptr, sizeof(int) * ns, cudaMemcpyDeviceToHost));
    MJ_CUDA(cudaMemcpy(val.data(), lf->src_val.ptr, esz * ns, cudaMemcpyDeviceToHost));
  }
  std::vector<int> order_(ns);
  for (int t = 0; t < ns; t++) order_[t] = t;
  std::sort(order_.begin(), order_.end(), [&](int a, int b) { return idx[a] < idx[b]; });
  std::vector<int> si(std::max(1, ns), 0);
  std::vector<unsigned char> sv(esz * std::max(1, ns), 0);
  std::vector<unsigned> mask(std::max(1, words), 0u);
  for (int t = 0; t < ns; t++) {
    si[t] = idx[order_[t]];
    std::memcpy(&sv[esz * t], &val[esz * order_[t]], esz);
    mask[si[t] >> 5] |= 1u << (si[t] & 31);
  }
  MJ_CUDA(lf->src_sidx.alloc(sizeof(int) * si.size()));
  MJ_CUDA(lf->src_sval.alloc(sv.size()));
  MJ_CUDA(lf->src_mask.alloc(sizeof(unsigned) * mask.size()));
  MJ_CUDA(cudaMemcpy(lf->src_sidx.ptr, si.data(), sizeof(int) * si.size(), cudaMemcpyHostToDevice));
  MJ_CUDA(cudaMemcpy(lf->src_sval.ptr, sv.data(), sv.size(), cudaMemcpyHostToDevice));
  MJ_CUDA(cudaMemcpy(lf->src_mask.ptr, mask.data(), sizeof(unsigned) * mask.size(), cudaMemcpyHostToDevice));
  lf->n_src_sorted = ns;
  return MJ_OK;
}

// Dof chunks of the streaming gather: start on a multiple of 4, at most
// kStreamDofs dofs, the 16-byte rounded range of their contributions within
// kStreamRCap; then the launch shape.
int lf_stream_setup(mj_lf* lf) {
  const mj_op* op = lf->op;
  const std::vector<int>& ptr = op->h_ptr;
  std::vector<char> is_src(op->n_dof, 0);
  {
    std::vector<int> idx(std::max(1, lf->n_src));
    if (lf->n_src)
      MJ_CUDA(cudaMemcpy(idx.data(), lf->src_idx.ptr, sizeof(int) * lf->n_src, cudaMemcpyDeviceToHost));
    for (int t = 0; t < lf->n_src; t++) is_src[idx[t]] = 1;
  }
  std::vector<StreamChunk> chunks;
  for (int d = 0; d < op->n_dof;) {
    int e = std::min(op->n_dof, d + kStreamDofs);
    auto range = [&](int e2) { return ((ptr[e2] + 3) & ~3) - (ptr[d] & ~3); };
    while (range(e) > kStreamRCap) e = d + std::max(4, ((e - d) / 2) & ~3);
    if (range(e) > kStreamRCap) {
      set_error("streaming gather: a dof has too many contributions for one chunk buffer");
      return MJ_ERR_ARG;
    }
    StreamChunk ch = {d, e, ptr[d] & ~3, (ptr[e] + 3) & ~3, 0, 0, 0, 0};
    for (int x = d; x < e; x++) ch.has_src |= is_src[x];
    chunks.push_back(ch);
    d = e;
  }
  MJ_CUDA(lf->stream_chunks.alloc(sizeof(StreamChunk) * chunks.size()));
  MJ_CUDA(cudaMemcpy(lf->stream_chunks.ptr, chunks.data(), sizeof(StreamChunk) * chunks.size(),
                     cudaMemcpyHostToDevice));
  lf->n_stream_chunks = (int)chunks.size();
  MJ_CUDA(cudaFuncSetAttribute(k_gather_leapfrog_stream<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               kStreamSmem));
  MJ_CUDA(cudaFuncSetAttribute(k_gather_leapfrog_stream<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               kStreamSmem));
  int ctas = 0;
  MJ_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&ctas, k_gather_leapfrog_stream<false>, kStreamThreads,
                                                        kStreamSmem));
  MJ_CHECK_ARG(ctas >= 1, "streaming gather cannot be resident");
  lf->stream_grid_ = std::max(1, std::min(lf->n_stream_chunks, ctas * sm_count()));
  MJ_CUDA(lf->stream_partial.alloc(sizeof(double) * lf->stream_grid_));
  return MJ_OK;
}

}  // namespace

extern "C" {

// ------------------------------------------------------------------ leap-frog

int mj_lf_create(mj_op* op, const mj_lf_desc* desc, mj_lf** out) {
  MJ_CHECK_ARG(op && desc && out, "mj_lf_create: null argument");
  *out = nullptr;
  MJ_CHECK_ARG(desc->dt > 0 && std::isfinite(desc->dt), "mj_lf_create: dt must be positive");
  MJ_CHECK_ARG(desc->mass, "mj_lf_create: mass is required");
  MJ_CHECK_ARG(desc->n_src >= 0 && (desc->n_src == 0 || (desc->src_idx && desc->src_val)),
               "mj_lf_create: bad source arrays");
  MJ_CHECK_ARG(desc->n_pulse >= 0 && (desc->n_pulse == 0 || desc->pulse), "mj_lf_create: bad pulse array");
  MJ_CHECK_ARG(desc->n_rec >= 0 && (desc->n_rec == 0 || (desc->rec_idx && desc->rec_w && desc->n_rec_w > 0)),
               "mj_lf_create: bad receiver arrays");
  const int n = op->n_dof;
  std::unique_ptr<mj_lf> lf(new mj_lf());
  lf->op = op; lf->dt = desc->dt; lf->n_dof = n; lf->stream = op->stream;
  const size_t esz = elem_size(op->precision);

  std::vector<double> invD(n);
  for (int i = 0; i < n; i++) {
    MJ_CHECK_ARG(std::isfinite(desc->mass[i]) && desc->mass[i] > 0, "mj_lf_create: mass must be positive");
    invD[i] = desc->inv_mass ? desc->inv_mass[i] : 1.0 / desc->mass[i];
  }
  // sparse source (one entry per dof; applied by k_source after each update)
  std::vector<char> seen(n, 0);
  for (int s = 0; s < desc->n_src; s++) {
    const int d = desc->src_idx[s];
    MJ_CHECK_ARG(d >= 0 && d < n, "mj_lf_create: source index out of range");
    MJ_CHECK_ARG(!seen[d], "mj_lf_create: duplicate source index");
    seen[d] = 1;
  }
  MJ_CUDA(lf->src_idx.alloc(sizeof(int) * std::max(1, desc->n_src)));
  if (desc->n_src)
    MJ_CUDA(cudaMemcpy(lf->src_idx.ptr, desc->src_idx, sizeof(int) * desc->n_src, cudaMemcpyHostToDevice));
  lf->n_src = desc->n_src;
  MJ_CUDA(lf->src_val.alloc(esz * std::max(1, desc->n_src)));
  MJ_CUDA(lf->inv_mass64.alloc(sizeof(double) * n));
  MJ_CUDA(cudaMemcpy(lf->inv_mass64.ptr, invD.data(), sizeof(double) * n, cudaMemcpyHostToDevice));
  if (op->precision == MJ_FP64) {
    if (desc->n_src)
      MJ_CUDA(cudaMemcpy(lf->src_val.ptr, desc->src_val, sizeof(double) * desc->n_src, cudaMemcpyHostToDevice));
    MJ_CUDA(lf->mass.alloc(sizeof(double) * n));
    MJ_CUDA(lf->minv.alloc(sizeof(double) * n));
    MJ_CUDA(cudaMemcpy(lf->mass.ptr, desc->mass, sizeof(double) * n, cudaMemcpyHostToDevice));
    MJ_CUDA(cudaMemcpy(lf->minv.ptr, invD.data(), sizeof(double) * n, cudaMemcpyHostToDevice));
  } else {
    std::vector<float> sv(std::max(1, desc->n_src)), m(n);
    for (int s = 0; s < desc->n_src; s++) sv[s] = (float)desc->src_val[s];
    for (int i = 0; i < n; i++) m[i] = (float)(desc->dt * desc->dt * invD[i]);
    MJ_CUDA(cudaMemcpy(lf->src_val.ptr, sv.data(), sizeof(float) * sv.size(), cudaMemcpyHostToDevice));
    MJ_CUDA(lf->minv.alloc(sizeof(float) * (n + 4)));
    MJ_CUDA(cudaMemset(lf->minv.ptr, 0, sizeof(float) * (n + 4)));
    MJ_CUDA(cudaMemcpy(lf->minv.ptr, m.data(), sizeof(float) * n, cudaMemcpyHostToDevice));
  }
  lf->n_pulse = desc->n_pulse;
  MJ_CUDA(lf->pulse_d.alloc(sizeof(double) * std::max(1, desc->n_pulse)));
  if (desc->n_pulse)
    MJ_CUDA(cudaMemcpy(lf->pulse_d.ptr, desc->pulse, sizeof(double) * desc->n_pulse, cudaMemcpyHostToDevice));
  MJ_CUDA(lf->ctr.alloc(sizeof(int) * 2));
  MJ_CUDA(cudaMemset(lf->ctr.ptr, 0, sizeof(int) * 2));
  if (desc->norm_weight) {
    MJ_CUDA(lf->norm_w.alloc(sizeof(double) * n));
    MJ_CUDA(cudaMemcpy(lf->norm_w.ptr, desc->norm_weight, sizeof(double) * n, cudaMemcpyHostToDevice));
    if (op->precision == MJ_FP32) {  // the FP32 norm rounds the weights to FP32: read them so (8 B per dof less)
      std::vector<float> w32(desc->norm_weight, desc->norm_weight + n);
      MJ_CUDA(lf->norm_w32.alloc(sizeof(float) * n));
      MJ_CUDA(cudaMemcpy(lf->norm_w32.ptr, w32.data(), sizeof(float) * n, cudaMemcpyHostToDevice));
      lf->norm_is_mass = std::equal(desc->norm_weight, desc->norm_weight + n, desc->mass);
    }
  }
  lf->n_rec = desc->n_rec;
  lf->n_rec_w = desc->n_rec_w;
  if (desc->n_rec) {
    const size_t m = (size_t)desc->n_rec * desc->n_rec_w;
    for (size_t t = 0; t < m; t++)
      MJ_CHECK_ARG(desc->rec_idx[t] >= 0 && desc->rec_idx[t] < n, "mj_lf_create: receiver dof out of range");
    MJ_CUDA(lf->rec_idx.alloc(sizeof(int) * m));
    MJ_CUDA(lf->rec_w.alloc(sizeof(double) * m));
    MJ_CUDA(cudaMemcpy(lf->rec_idx.ptr, desc->rec_idx, sizeof(int) * m, cudaMemcpyHostToDevice));
    MJ_CUDA(cudaMemcpy(lf->rec_w.ptr, desc->rec_w, sizeof(double) * m, cudaMemcpyHostToDevice));
  }
  // state vectors padded by 4 entries (16-byte rounded bulk copies of dof ranges)
  MJ_CUDA(lf->ua.alloc(esz * (n + 4)));
  MJ_CUDA(lf->ub.alloc(esz * (n + 4)));
  MJ_CUDA(cudaMemset(lf->ua.ptr, 0, esz * (n + 4)));
  MJ_CUDA(cudaMemset(lf->ub.ptr, 0, esz * (n + 4)));
  lf->norm_blocks = std::min(stream_grid(n), 1024);
  MJ_CUDA(lf->partial.alloc(sizeof(double) * lf->norm_blocks));
  MJ_CUDA(lf->flag.alloc(sizeof(int)));
  MJ_CUDA(lf->diag_done.alloc(sizeof(unsigned)));
  MJ_CUDA(cudaMemset(lf->diag_done.ptr, 0, sizeof(unsigned)));
  MJ_CUDA(lf->diag_where.alloc(sizeof(DiagDev)));
  MJ_CUDA(cudaMemset(lf->flag.ptr, 0, sizeof(int)));
  if (op->precision == MJ_FP32) {
    int rc = lf_sorted_sources(lf.get());
    if (!rc) rc = lf_stream_setup(lf.get());
    if (rc) return rc;
    lf->stream_gather = true;
  }
  *out = lf.release();
  return MJ_OK;
}

int mj_lf_destroy(mj_lf* lf) {
  delete lf;
  return MJ_OK;
}

int mj_lf_set_stream(mj_lf* lf, void* stream) {
  MJ_CHECK_ARG(lf, "mj_lf_set_stream: null integrator");
  lf->stream = static_cast<cudaStream_t>(stream);
  return MJ_OK;
}

}  // extern "C"

namespace {

template <typename Real>
int lf_init_impl(mj_lf* lf, const double* u0, const double* du0) {
  mj_op* op = lf->op;
  cudaStream_t s = lf->stream;
  const int n = lf->n_dof;
  DevBuf stage;
  int rc = upload_vec(op, u0, lf->ua.ptr, stage, s);
  if (rc) return rc;
  const Real* du0_d = nullptr;
  if (du0) {
    if (lf->du0.bytes < sizeof(Real) * n) MJ_CUDA(lf->du0.alloc(sizeof(Real) * n));
    rc = upload_vec(op, du0, lf->du0.ptr, stage, s);
    if (rc) return rc;
    du0_d = lf->du0.as<Real>();
  }
  if (lf->time_order == 4) {
    // order-4 start (SetInitialConditionS, ModifiedEquation.cxx:125-175):
    // d2 = invD(-A u0), d3 = invD(-A du0), then U^1 by the Taylor step with
    // d4 = invD(-A d2)
    launch_k1<Real>(op, lf->ua.ptr, s);
    k_gather_scaled<Real><<<stream_grid(n), 256, 0, s>>>(op->R.as<Real>(), op->ptr.as<int>(),
                                                          lf->inv_mass64.as<double>(), lf->z4.as<Real>(), n);
    const Real* d3 = nullptr;
    if (du0_d) {
      launch_k1<Real>(op, du0_d, s);
      k_gather_scaled<Real><<<stream_grid(n), 256, 0, s>>>(op->R.as<Real>(), op->ptr.as<int>(),
                                                            lf->inv_mass64.as<double>(), lf->d3_4.as<Real>(), n);
      d3 = lf->d3_4.as<Real>();
      count_launch();
    }
    launch_k1<Real>(op, lf->z4.ptr, s);
    k_gather_o4_init<Real><<<stream_grid(n), 256, 0, s>>>(op->R.as<Real>(), op->ptr.as<int>(),
                                                           lf->inv_mass64.as<double>(), lf->ua.as<Real>(), du0_d,
                                                           lf->z4.as<Real>(), d3, lf->dt, lf->ub.as<Real>(), n);
    count_launch(2);
  } else {
    launch_k1<Real>(op, lf->ua.ptr, s);
    k_gather_init<Real><<<stream_grid(n), 256, 0, s>>>(op->R.as<Real>(), op->ptr.as<int>(),
                                                        lf->ua.as<Real>(), du0_d, lf->inv_mass64.as<double>(),
                                                        lf->dt, lf->ub.as<Real>(), n);
    count_launch();
  }
  MJ_CUDA(cudaGetLastError());
  lf->cur_is_a = true;
  lf->step = 0;
  lf->initialised = true;
  MJ_CUDA(cudaMemsetAsync(lf->flag.ptr, 0, sizeof(int), s));
  MJ_CUDA(cudaMemsetAsync(lf->ctr.ptr, 0, sizeof(int) * 2, s));
  MJ_CUDA(cudaStreamSynchronize(s));
  return MJ_OK;
}

// Norm and receiver traces of the current iterate in one launch: plain
// launches write column `col` of norms_d / traces_d (row stride `stride`);
// with `where` (graph capture) the kernel reads the arrays and the column
// base from device memory and adds `col`.
template <typename Real>
void lf_diag_launch(mj_lf* lf, const void* u, double* norms_d, double* traces_d, int stride, int col,
                    const DiagDev* where, cudaStream_t s) {
  const int nb = (norms_d || where) && lf->norm_w.ptr ? lf->norm_blocks : 0;
  const int rb = (traces_d || where) && lf->n_rec ? (lf->n_rec * 32 + 255) / 256 : 0;
  if (nb + rb == 0) return;
  const DiagDev direct = {norms_d, traces_d, stride, 0, INT_MAX};
  k_diag<Real><<<nb + rb, 256, 0, s>>>(static_cast<const Real*>(u), lf->norm_w.as<double>(), lf->norm_w32.as<float>(),
                                      lf->n_dof, nb, lf->partial.as<double>(), lf->diag_done.as<unsigned>(),
                                      lf->flag.as<int>(), lf->rec_idx.as<int>(), lf->rec_w.as<double>(),
                                      rb ? lf->n_rec : 0, lf->n_rec_w, where, direct, col);
  count_launch();
}

template <typename Real>
int lf_diag(mj_lf* lf, double* norms_d, double* traces_d, int stride, int col) {
  lf_diag_launch<Real>(lf, lf->cur(), norms_d, traces_d, stride, col, nullptr, lf->stream);
  MJ_CUDA(cudaGetLastError());
  return MJ_OK;
}

// Launches of one leap-frog step (capturable): element kernel on U^{n+1},
// then gather + source + update writing U^{n+2} over U^n.  qc = parity of
// the pulse counter holding this step's index.
// Steps per captured CUDA graph (even, so the state buffers and the pulse
// counters are back in their roles after each replay).
constexpr int kGraphSteps = 20;

// Kernels one step launches (launch accounting of graph replays).
int lf_kernels_per_step(const mj_lf* lf) {
  if (lf->time_order == 4) return 4;
  if (lf->stream_gather && lf->op->precision == MJ_FP32) return 2;
  return 2 + (lf->n_src > 0);
}

// One order-4 step: element product of U^{n+1}, first gather (P, Z),
// element product of Z, second gather + update over U^n.
template <typename Real>
void lf_step4_launch(mj_lf* lf, void* cur, const void* next, int qc, cudaStream_t s, bool prof) {
  mj_op* op = lf->op;
  const int n = lf->n_dof;
  const Real dt2 = Real(lf->dt * lf->dt);
  constexpr bool EXACT = sizeof(Real) == 8;
  if (prof) cudaEventRecord(lf->ev[lf->ev_used], s);
  launch_k1<Real>(op, next, s);
  if (prof) cudaEventRecord(lf->ev[lf->ev_used + 1], s);
  if (!EXACT && lf->stream_grid_ > 0) {  // FP32: the streaming forms
    const float* Rf = op->R.as<float>();
    k_gather_o4_stream<0><<<lf->stream_grid_, kStreamThreads, kStreamSmem, s>>>(
        Rf, op->ptr.as<int>(), lf->ctr.as<int>(), qc, lf->pulse_d.as<double>(), lf->n_pulse,
        lf->src_mask.as<unsigned>(), lf->src_sidx.as<int>(), lf->src_sval.as<float>(), lf->n_src_sorted, nullptr,
        nullptr, lf->minv.as<float>(), lf->w4.as<float>(), lf->z4.as<float>(), lf->stream_chunks.as<StreamChunk>(),
        lf->n_stream_chunks, float(dt2), op->err.as<int>());
    launch_k1<Real>(op, lf->z4.ptr, s);
    k_gather_o4_stream<1><<<lf->stream_grid_, kStreamThreads, kStreamSmem, s>>>(
        Rf, op->ptr.as<int>(), lf->ctr.as<int>(), qc, lf->pulse3_d.as<double>(), lf->n_pulse3,
        lf->src_mask.as<unsigned>(), lf->src_sidx.as<int>(), lf->src_sval.as<float>(), lf->n_src_sorted,
        static_cast<float*>(cur), static_cast<const float*>(next), lf->minv.as<float>(), lf->w4.as<float>(), nullptr,
        lf->stream_chunks.as<StreamChunk>(), lf->n_stream_chunks, float(dt2), op->err.as<int>());
  } else {
    k_gather_o4a<Real, EXACT><<<stream_grid(n), 256, 0, s>>>(
        op->R.as<Real>(), op->ptr.as<int>(), lf->ctr.as<int>(), qc, lf->pulse_d.as<double>(), lf->n_pulse,
        lf->src_mask.as<unsigned>(), lf->src_sidx.as<int>(), lf->src_sval.as<Real>(), lf->n_src_sorted,
        lf->minv.as<Real>(), dt2, lf->w4.as<Real>(), lf->z4.as<Real>(), n);
    launch_k1<Real>(op, lf->z4.ptr, s);
    k_gather_o4b<Real, EXACT><<<stream_grid(n), 256, 0, s>>>(
        op->R.as<Real>(), op->ptr.as<int>(), lf->ctr.as<int>(), qc, lf->pulse3_d.as<double>(), lf->n_pulse3,
        lf->src_mask.as<unsigned>(), lf->src_sidx.as<int>(), lf->src_sval.as<Real>(), lf->n_src_sorted,
        lf->w4.as<Real>(), static_cast<Real*>(cur), static_cast<const Real*>(next),
        EXACT ? lf->mass.as<Real>() : nullptr, lf->minv.as<Real>(), dt2, n);
  }
  count_launch(2);
  if (prof) {
    cudaEventRecord(lf->ev[lf->ev_used + 2], s);
    lf->ev_used += 3;
  }
}

// Diagnostics fused into the step: the FP32 order-2 step with the streaming
// gather computes the norm and the receivers of the iterate it produces.
bool lf_fused_diag(const mj_lf* lf) {
  return lf->stream_gather && lf->op->precision == MJ_FP32 && lf->time_order == 2;
}

// dg: the step's fused diagnostics (streaming gather only), or nullptr.
template <typename Real>
void lf_step_launch(mj_lf* lf, void* cur, const void* next, int qc, cudaStream_t s, bool prof,
                    const StreamDiag* dg = nullptr) {
  if (lf->time_order == 4) {
    lf_step4_launch<Real>(lf, cur, next, qc, s, prof);
    return;
  }
  mj_op* op = lf->op;
  const int n = lf->n_dof;
  if (prof) cudaEventRecord(lf->ev[lf->ev_used], s);
  launch_k1<Real>(op, next, s);
  if (prof) cudaEventRecord(lf->ev[lf->ev_used + 1], s);
  const double dt2 = lf->dt * lf->dt;
  if (lf->stream_gather && op->precision == MJ_FP32) {
    auto k2 = dg ? k_gather_leapfrog_stream<true> : k_gather_leapfrog_stream<false>;
    k2<<<lf->stream_grid_, kStreamThreads, kStreamSmem, s>>>(
        op->R.as<float>(), op->ptr.as<int>(), lf->ctr.as<int>(), qc, static_cast<float*>(cur),
        static_cast<const float*>(next), lf->minv.as<float>(), lf->stream_chunks.as<StreamChunk>(),
        lf->n_stream_chunks, lf->src_mask.as<unsigned>(), lf->src_sidx.as<int>(), lf->src_sval.as<float>(),
        lf->n_src_sorted, lf->pulse_d.as<double>(), lf->n_pulse, lf->inv_mass64.as<double>(), dt2,
        op->err.as<int>(), dg ? *dg : StreamDiag{});
    count_launch();
    if (prof) {
      cudaEventRecord(lf->ev[lf->ev_used + 2], s);
      lf->ev_used += 3;
    }
    return;
  }
  if (op->precision == MJ_FP64) {
    k_gather_leapfrog<Real, true><<<stream_grid(n), 256, 0, s>>>(
        op->R.as<Real>(), op->ptr.as<int>(), lf->ctr.as<int>(), qc, static_cast<Real*>(cur),
        static_cast<const Real*>(next), lf->mass.as<Real>(), lf->minv.as<Real>(), Real(dt2), n);
  } else {
    k_gather_leapfrog<Real, false><<<stream_grid(n), 256, 0, s>>>(
        op->R.as<Real>(), op->ptr.as<int>(), lf->ctr.as<int>(), qc, static_cast<Real*>(cur),
        static_cast<const Real*>(next), nullptr, lf->minv.as<Real>(), Real(dt2), n);
  }
  if (lf->n_src) {
    k_source<Real><<<(lf->n_src + 255) / 256, 256, 0, s>>>(lf->src_idx.as<int>(), lf->src_val.as<Real>(), lf->n_src,
                                                           lf->pulse_d.as<double>(), lf->n_pulse, lf->ctr.as<int>(),
                                                           qc, lf->inv_mass64.as<double>(), dt2,
                                                           static_cast<Real*>(cur));
    count_launch();
  }
  count_launch();
  if (prof) {
    cudaEventRecord(lf->ev[lf->ev_used + 2], s);
    lf->ev_used += 3;
  }
}

// The StreamDiag of a step whose new iterate goes to column where.col + col.
StreamDiag lf_stream_diag(mj_lf* lf, const DiagDev* dd, DiagDev direct, int col) {
  StreamDiag g = {};
  // norm weights equal to the mass (no density): dt^2 / (dt^2/D) from the staged dt^2/D, no weight stream
  const bool from_m = lf->norm_is_mass && lf->norm_w32.ptr;
  g.w32 = from_m ? nullptr : lf->norm_w32.as<float>();
  g.m = lf->minv.as<float>();
  g.wdt2 = from_m ? (float)(lf->dt * lf->dt) : 0.f;
  g.partial = lf->stream_partial.as<double>();
  g.done = lf->diag_done.as<unsigned>();
  g.flag = lf->flag.as<int>();
  g.rec_idx = lf->rec_idx.as<int>();
  g.rec_w = lf->rec_w.as<double>();
  g.n_rec = lf->n_rec;
  g.n_w = lf->n_rec_w;
  g.dd = dd;
  g.direct = direct;
  g.col = col;
  return g;
}

template <typename Real>
int lf_step(mj_lf* lf, const StreamDiag* dg = nullptr) {
  const bool prof = lf->profile && lf->ev_used + 3 <= (int)lf->ev.size() - 3 * kGraphSteps;
  lf_step_launch<Real>(lf, lf->cur(), lf->next(), lf->step & 1, lf->stream, prof, dg);
  MJ_CUDA(cudaGetLastError());
  lf->cur_is_a = !lf->cur_is_a;  // new cur = old next; new next = overwritten old cur
  lf->step++;
  return MJ_OK;
}

// Captures kGraphSteps steps; with prof, event records around each kernel
// (events 0..3*kGraphSteps-1 of the pool) are part of the graph, so the last
// replay's per-kernel times can be read back.
// diag: each step starts with the fused norm/receiver launch of its iterate
// (arrays and column base read from lf->diag_where, the column advanced by
// kGraphSteps at the end of the graph).
template <typename Real>
int lf_capture(mj_lf* lf, bool prof, cudaGraphExec_t* out, bool diag = false) {
  cudaStream_t cs;
  MJ_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
  cudaGraph_t g;
  const uint64_t before = launch_counter().load();
  MJ_CUDA(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
  bool a = true;
  const int ev_saved = lf->ev_used;
  const int ev_base = (int)lf->ev.size() - 3 * kGraphSteps;  // the graph's own events, apart from plain steps'
  lf->ev_used = ev_base;
  for (int k = 0; k < kGraphSteps; k++) {
    void* cur = a ? lf->ua.ptr : lf->ub.ptr;
    void* nxt = a ? lf->ub.ptr : lf->ua.ptr;
    if (diag && lf_fused_diag(lf)) {  // the step writes its new iterate's column (k + 2)
      const StreamDiag dg = lf_stream_diag(lf, lf->diag_where.as<DiagDev>(), DiagDev{}, k + 2);
      lf_step_launch<Real>(lf, cur, nxt, k & 1, cs, prof, &dg);
    } else {
      if (diag) lf_diag_launch<Real>(lf, cur, nullptr, nullptr, 0, k, lf->diag_where.as<DiagDev>(), cs);
      lf_step_launch<Real>(lf, cur, nxt, k & 1, cs, prof);
    }
    a = !a;
  }
  if (diag) {
    k_diag_advance<<<1, 1, 0, cs>>>(lf->diag_where.as<DiagDev>(), kGraphSteps);
    count_launch();
  }
  lf->ev_used = ev_saved;
  MJ_CUDA(cudaStreamEndCapture(cs, &g));
  launch_counter().store(before);  // captured, not launched
  MJ_CUDA(cudaGraphInstantiate(out, g, 0));
  cudaGraphDestroy(g);
  cudaStreamDestroy(cs);
  return MJ_OK;
}

template <typename Real>
int lf_advance_impl(mj_lf* lf, int nsteps, double* norms, double* traces, int stride, bool final_diag) {
  const int cols = nsteps + (final_diag ? 1 : 0);
  double* nd = nullptr;
  double* td = nullptr;
  if (norms && lf->norm_w.ptr) {
    if (lf->norms_d.bytes < sizeof(double) * cols) MJ_CUDA(lf->norms_d.alloc(sizeof(double) * cols));
    nd = lf->norms_d.as<double>();
  }
  if (traces && lf->n_rec) {
    MJ_CHECK_ARG(stride >= cols, "mj_lf_advance: trace_stride smaller than the number of recorded iterates");
    const size_t b = sizeof(double) * (size_t)lf->n_rec * cols;
    if (lf->traces_d.bytes < b) MJ_CUDA(lf->traces_d.alloc(b));
    td = lf->traces_d.as<double>();
  }
  int s0 = 0;
  bool replayed_prof = false;
  if (!nd && !td && !lf->profile && lf->use_graph && nsteps >= kGraphSteps + 1) {
    if (lf->step & 1) {  // realign: replays start on an even step with ua holding U^n
      lf_step_launch<Real>(lf, lf->cur(), lf->next(), lf->step & 1, lf->stream, false);
      MJ_CUDA(cudaGetLastError());
      lf->cur_is_a = !lf->cur_is_a;
      lf->step++;
      s0 = 1;
    }
    if (!lf->graph) {
      int rc = lf_capture<Real>(lf, false, &lf->graph);
      if (rc) return rc;
    }
    while (nsteps - s0 >= kGraphSteps) {
      MJ_CUDA(cudaGraphLaunch(lf->graph, lf->stream));
      count_launch((uint64_t)kGraphSteps * lf_kernels_per_step(lf));
      s0 += kGraphSteps;
      lf->step += kGraphSteps;
    }
    MJ_CUDA(cudaGetLastError());
  }
  // Diagnostics: the norm and the traces of iterate s go to column s.  The
  // state holds iterates s (handed out) and s+1, and step s produces s+2.
  // With the fused form step s writes column s+2 (nothing past the call's
  // columns), and iterates 0 and 1 have launches of their own.
  const bool fused = (nd || td) && lf_fused_diag(lf);
  const DiagDev direct = {nd, td, cols, 0, cols};
  auto plain_step = [&](int s) -> int {
    if (fused) {
      const StreamDiag dg = lf_stream_diag(lf, nullptr, direct, s + 2);
      return lf_step<Real>(lf, &dg);
    }
    if (nd || td) {
      const int rc = lf_diag<Real>(lf, nd, td, cols, s);
      if (rc) return rc;
    }
    return lf_step<Real>(lf);
  };
  if (fused)  // iterates 0 and 1 with the same arithmetic as the fused steps
    for (int c = 0; c < std::min(cols, 2); c++) {
      const StreamDiag dg = lf_stream_diag(lf, nullptr, direct, c);
      k_stream_diag<<<lf->stream_grid_, kStreamThreads, 0, lf->stream>>>(
          static_cast<const float*>(c == 0 ? lf->cur() : lf->next()), lf->stream_chunks.as<StreamChunk>(),
          lf->n_stream_chunks, dg);
      count_launch();
    }
  if ((nd || td) && !lf->profile && lf->use_graph && nsteps >= kGraphSteps + 1) {
    // diagnosed steps: graph replays whose kernels read the arrays and the
    // column from diag_where
    if (lf->step & 1) {  // realign on an even step
      const int rc = plain_step(0);
      if (rc) return rc;
      s0 = 1;
    }
    if (!lf->graph_diag) {
      const int rc = lf_capture<Real>(lf, false, &lf->graph_diag, true);
      if (rc) return rc;
    }
    const DiagDev where = {nd, td, cols, s0, cols};
    k_diag_set<<<1, 1, 0, lf->stream>>>(lf->diag_where.as<DiagDev>(), where);
    count_launch();
    while (nsteps - s0 >= kGraphSteps) {
      MJ_CUDA(cudaGraphLaunch(lf->graph_diag, lf->stream));
      count_launch((uint64_t)kGraphSteps * (lf_kernels_per_step(lf) + (fused ? 0 : 1)) + 1);
      s0 += kGraphSteps;
      lf->step += kGraphSteps;
    }
    MJ_CUDA(cudaGetLastError());
  }
  for (int s = s0; s < nsteps; s++) {
    const int rc = plain_step(s);
    if (rc) return rc;
  }
  if (final_diag && !fused) {
    const int rc = lf_diag<Real>(lf, nd, td, cols, nsteps);
    if (rc) return rc;
  }
  cudaStream_t s = lf->stream;
  if (nd) MJ_CUDA(cudaMemcpyAsync(norms, nd, sizeof(double) * cols, cudaMemcpyDeviceToHost, s));
  if (td)
    for (int k = 0; k < lf->n_rec; k++)
      MJ_CUDA(cudaMemcpyAsync(traces + (size_t)k * stride, td + (size_t)k * cols, sizeof(double) * cols,
                              cudaMemcpyDeviceToHost, s));
  int flag = 0;
  MJ_CUDA(cudaMemcpyAsync(&flag, lf->flag.ptr, sizeof(int), cudaMemcpyDeviceToHost, s));
  {
    const int rc = take_kernel_error(lf->op->err.ptr, s, "mj_lf_advance");
    if (rc) return rc;
  }
  if (replayed_prof) {  // per-kernel times of the last replay
    const int base = (int)lf->ev.size() - 3 * kGraphSteps;
    for (int k = 0; k < kGraphSteps; k++) {
      float a = 0.f, b = 0.f;
      MJ_CUDA(cudaEventElapsedTime(&a, lf->ev[base + 3 * k], lf->ev[base + 3 * k + 1]));
      MJ_CUDA(cudaEventElapsedTime(&b, lf->ev[base + 3 * k + 1], lf->ev[base + 3 * k + 2]));
      lf->prof_elem_ms += a;
      lf->prof_update_ms += b;
      lf->prof_steps++;
    }
  }
  for (int e = 0; e + 3 <= lf->ev_used; e += 3) {
    float a = 0.f, b = 0.f;
    MJ_CUDA(cudaEventElapsedTime(&a, lf->ev[e], lf->ev[e + 1]));
    MJ_CUDA(cudaEventElapsedTime(&b, lf->ev[e + 1], lf->ev[e + 2]));
    lf->prof_elem_ms += a;
    lf->prof_update_ms += b;
    lf->prof_steps++;
  }
  lf->ev_used = 0;
  if (norms)  // the first recorded norm that is not finite or above the limit
    for (int c = 0; c < cols; c++) {
      if (!std::isfinite(norms[c])) {
        set_error("mj_lf_advance: non-finite norm at column " + std::to_string(c) + " (unstable run?)");
        return MJ_ERR_NONFINITE;
      }
      if (std::fabs(norms[c]) > lf->norm_max) {
        // GetNormeSolution's guard (VarInstationary.cxx:2741-2745), which aborts there
        set_error("mj_lf_advance: norm of the solution " + std::to_string(norms[c]) + " at column " +
                  std::to_string(c) + " above the limit " + std::to_string(lf->norm_max) + " (unstable run?)");
        return MJ_ERR_NONFINITE;
      }
    }
  if (flag) {
    set_error("mj_lf_advance: non-finite norm (unstable run?)");
    return MJ_ERR_NONFINITE;
  }
  return MJ_OK;
}

}  // namespace

extern "C" {

int mj_lf_init(mj_lf* lf, const double* u0, const double* du0) {
  MJ_CHECK_ARG(lf && u0, "mj_lf_init: null argument");
  return lf->op->precision == MJ_FP64 ? lf_init_impl<double>(lf, u0, du0) : lf_init_impl<float>(lf, u0, du0);
}

int mj_lf_advance(mj_lf* lf, int nsteps, double* norms, double* traces, int trace_stride) {
  MJ_CHECK_ARG(lf, "mj_lf_advance: null integrator");
  MJ_CHECK_ARG(nsteps >= 0, "mj_lf_advance: negative step count");
  if (!lf->initialised) {
    set_error("mj_lf_advance: mj_lf_init must be called first");
    return MJ_ERR_STATE;
  }
  return lf->op->precision == MJ_FP64 ? lf_advance_impl<double>(lf, nsteps, norms, traces, trace_stride, false)
                                      : lf_advance_impl<float>(lf, nsteps, norms, traces, trace_stride, false);
}

int mj_lf_get_state(mj_lf* lf, double* u_n, double* u_np1) {
  MJ_CHECK_ARG(lf, "mj_lf_get_state: null integrator");
  if (!lf->initialised) {
    set_error("mj_lf_get_state: mj_lf_init must be called first");
    return MJ_ERR_STATE;
  }
  DevBuf stage;
  int rc;
  if (u_n && (rc = download_vec(lf->op, lf->cur(), u_n, stage, lf->stream))) return rc;
  if (u_np1 && (rc = download_vec(lf->op, lf->next(), u_np1, stage, lf->stream))) return rc;
  MJ_CUDA(cudaStreamSynchronize(lf->stream));
  return MJ_OK;
}

int mj_lf_run(mj_lf* lf, const double* u0, const double* du0, int nsteps, double* u_final, double* norms,
              double* traces, int trace_stride) {
  MJ_CHECK_ARG(lf && u0, "mj_lf_run: null argument");
  MJ_CHECK_ARG(nsteps >= 0, "mj_lf_run: negative step count");
  int rc = mj_lf_init(lf, u0, du0);
  if (rc) return rc;
  rc = lf->op->precision == MJ_FP64 ? lf_advance_impl<double>(lf, nsteps, norms, traces, trace_stride, true)
                                    : lf_advance_impl<float>(lf, nsteps, norms, traces, trace_stride, true);
  if (rc) return rc;
  if (u_final) return mj_lf_get_state(lf, u_final, nullptr);
  return MJ_OK;
}

int mj_lf_set_scheme(mj_lf* lf, int order, int n_pulse_d2, const double* pulse_d2) {
  MJ_CHECK_ARG(lf, "mj_lf_set_scheme: null integrator");
  MJ_CHECK_ARG(order == 2 || order == 4, "mj_lf_set_scheme: order must be 2 or 4");
  MJ_CHECK_ARG(order == 2 || n_pulse_d2 == 0 || pulse_d2, "mj_lf_set_scheme: null pulse_d2");
  MJ_CHECK_ARG(n_pulse_d2 >= 0, "mj_lf_set_scheme: negative n_pulse_d2");
  for (cudaGraphExec_t* g : {&lf->graph, &lf->graph_prof, &lf->graph_diag})
    if (*g) {
      cudaGraphExecDestroy(*g);
      *g = nullptr;
    }
  lf->initialised = false;
  lf->time_order = order;
  if (order == 2) return MJ_OK;
  const int n = lf->n_dof;
  const size_t esz = elem_size(lf->op->precision);
  MJ_CUDA(lf->w4.alloc(esz * n));
  MJ_CUDA(lf->z4.alloc(esz * n));
  MJ_CUDA(lf->d3_4.alloc(esz * n));
  lf->n_pulse3 = n_pulse_d2;
  MJ_CUDA(lf->pulse3_d.alloc(sizeof(double) * std::max(1, n_pulse_d2)));
  if (n_pulse_d2)
    MJ_CUDA(cudaMemcpy(lf->pulse3_d.ptr, pulse_d2, sizeof(double) * n_pulse_d2, cudaMemcpyHostToDevice));
  {
    const int rc = lf_sorted_sources(lf);
    if (rc) return rc;
  }
  return MJ_OK;
}

int mj_lf_set_norm_max(mj_lf* lf, double norm_max) {
  MJ_CHECK_ARG(lf, "mj_lf_set_norm_max: null integrator");
  MJ_CHECK_ARG(norm_max > 0.0, "mj_lf_set_norm_max: the limit must be positive");
  lf->norm_max = norm_max;
  return MJ_OK;
}

int mj_lf_set_stream_gather(mj_lf* lf, int enable) {
  MJ_CHECK_ARG(lf, "mj_lf_set_stream_gather: null integrator");
  MJ_CHECK_ARG(!enable || lf->op->precision == MJ_FP32, "mj_lf_set_stream_gather: FP32 integrators only");
  for (cudaGraphExec_t* g : {&lf->graph, &lf->graph_prof, &lf->graph_diag})
    if (*g) {
      cudaGraphExecDestroy(*g);
      *g = nullptr;
    }
  lf->stream_gather = enable != 0;
  return MJ_OK;
}

int mj_lf_set_graph(mj_lf* lf, int enable) {
  MJ_CHECK_ARG(lf, "mj_lf_set_graph: null integrator");
  lf->use_graph = enable != 0;
  return MJ_OK;
}

int mj_lf_profile(mj_lf* lf, int enable, double* elem_ms, double* update_ms, int* steps) {
  MJ_CHECK_ARG(lf, "mj_lf_profile: null integrator");
  if (elem_ms) *elem_ms = lf->prof_elem_ms;
  if (update_ms) *update_ms = lf->prof_update_ms;
  if (steps) *steps = lf->prof_steps;
  if (enable && !lf->profile) {
    const int n_ev = 3 * 1024;
    while ((int)lf->ev.size() < n_ev) {
      cudaEvent_t e;
      MJ_CUDA(cudaEventCreate(&e));
      lf->ev.push_back(e);
    }
    lf->prof_elem_ms = lf->prof_update_ms = 0.0;
    lf->prof_steps = 0;
    lf->ev_used = 0;
  }
  lf->profile = enable != 0;
  return MJ_OK;
}

int mj_lf_device_state(mj_lf* lf, void** u_n, void** u_np1, int* step) {
  MJ_CHECK_ARG(lf, "mj_lf_device_state: null integrator");
  if (u_n) *u_n = lf->cur();
  if (u_np1) *u_np1 = lf->next();
  if (step) *step = lf->step;
  return MJ_OK;
}

}  // extern "C"

int mj::lf_step_on(mj_lf* lf, void* cur, const void* next, int qc, cudaStream_t s) {
  if (lf->op->precision == MJ_FP64) lf_step_launch<double>(lf, cur, next, qc, s, false);
  else lf_step_launch<float>(lf, cur, next, qc, s, false);
  MJ_CUDA(cudaGetLastError());
  return MJ_OK;
}

// ---- union of several runs of one order (mesh batch) ------------------------

namespace mj {

// Element-major connectivity and slots of one run, shifted into the union:
// points of the element get the run's dof and incidence offsets, padding
// points the union's spare dof 0 and spare slot.
static __global__ void k_union_remap(const int* __restrict__ nodle, const int* __restrict__ slot, long long n, int Qp,
                              int Q, int dof_off, int inc_off, int pad_slot, int* __restrict__ onodle,
                              int* __restrict__ oslot) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    if ((int)(t % Qp) < Q) {
      onodle[t] = nodle[t] + dof_off;
      oslot[t] = slot[t] + inc_off;
    } else {
      onodle[t] = 0;
      oslot[t] = pad_slot;
    }
  }
}

static __global__ void k_fill_int(int* __restrict__ a, long long n, int v) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x)
    a[t] = v;
}

static int grid_for_len(long long n) { return (int)std::max(1LL, std::min<long long>((n + 255) / 256, 4096)); }

}  // namespace mj

int mj::union_copy_factors(mj_op* uop, const mj_op* op, int elt_off, cudaStream_t s) {
  const size_t per = (size_t)6 * op->Qp * sizeof(float);
  MJ_CUDA(cudaMemcpyAsync(uop->fac_e.as<char>() + (size_t)elt_off * per, op->fac_e.ptr, (size_t)op->n_elt * per,
                          cudaMemcpyDeviceToDevice, s));
  return MJ_OK;
}

int mj::lf_union_create(const std::vector<mj_lf*>& runs, std::unique_ptr<mj_op>* uop_out,
                        std::unique_ptr<mj_lf>* ulf_out, std::vector<int>* dof_off, std::vector<int>* elt_off) {
  MJ_CHECK_ARG(!runs.empty(), "union: no runs");
  const mj_op* op0 = runs[0]->op;
  long long n_elt = 0, n_dof = 0, n_inc = 0;
  dof_off->clear();
  elt_off->clear();
  for (mj_lf* lf : runs) {
    const mj_op* op = lf->op;
    MJ_CHECK_ARG(op->precision == MJ_FP32 && op->n == op0->n && lf->time_order == 2,
                 "union: the runs need FP32 operators of one order and the order-2 scheme");
    for (int a = 0; a < op->n * op->n; a++)
      MJ_CHECK_ARG(op->gradphi[a] == op0->gradphi[a], "union: the runs use different derivative matrices");
    dof_off->push_back((int)n_dof);
    elt_off->push_back((int)n_elt);
    n_elt += op->n_elt;
    n_dof += op->n_dof;
    n_inc += (long long)op->n_inc;
  }
  const int Qp = op0->Qp, Q = op0->Q;
  const long long n_elt_pad = (n_elt + kElemPad - 1) / kElemPad * kElemPad;
  MJ_CHECK_ARG(n_dof < INT32_MAX - 8 && n_inc < INT32_MAX - 8 && n_elt_pad * Qp < INT32_MAX - 1 &&
                   n_elt * Q < (1LL << 31) - 1,
               "union: the runs together exceed int32 indexing");
  std::unique_ptr<mj_op> u(new mj_op());
  u->order = op0->order; u->n = op0->n; u->Q = Q; u->Qp = Qp;
  u->n_elt = (int)n_elt; u->n_elt_pad = (int)n_elt_pad; u->n_dof = (int)n_dof; u->precision = MJ_FP32;
  u->r_len = (size_t)n_elt_pad * Qp;
  u->n_inc = (size_t)n_inc;
  std::copy(op0->gradphi, op0->gradphi + op0->n * op0->n, u->gradphi);
  u->h_ptr.assign((size_t)n_dof + 1, 0);
  for (size_t r = 0; r < runs.size(); r++) {
    const mj_op* op = runs[r]->op;
    const int base = op->h_ptr[0];  // 0
    const int inc0 = u->h_ptr[(*dof_off)[r]];
    for (int d = 0; d < op->n_dof; d++) u->h_ptr[(size_t)(*dof_off)[r] + d + 1] = inc0 + op->h_ptr[d + 1] - base;
  }
  cudaStream_t s = u->stream;
  MJ_CUDA(u->nodle_e.alloc(sizeof(int) * u->r_len));
  MJ_CUDA(u->slot_e.alloc(sizeof(int) * u->r_len));
  MJ_CUDA(u->fac_e.alloc((size_t)n_elt_pad * 6 * Qp * sizeof(float)));
  MJ_CUDA(u->R.alloc(sizeof(float) * (u->n_inc + 4)));
  MJ_CUDA(u->ptr.alloc(sizeof(int) * ((size_t)n_dof + 8)));
  MJ_CUDA(u->err.alloc(sizeof(int)));
  MJ_CUDA(cudaMemsetAsync(u->err.ptr, 0, sizeof(int), s));
  MJ_CUDA(cudaMemsetAsync(u->ptr.ptr, 0, sizeof(int) * ((size_t)n_dof + 8), s));
  MJ_CUDA(cudaMemsetAsync(u->R.ptr, 0, sizeof(float) * (u->n_inc + 4), s));
  MJ_CUDA(cudaMemsetAsync(u->fac_e.ptr, 0, u->fac_e.bytes, s));
  MJ_CUDA(cudaMemsetAsync(u->nodle_e.ptr, 0, u->nodle_e.bytes, s));
  k_fill_int<<<grid_for_len((long long)u->r_len), 256, 0, s>>>(u->slot_e.as<int>(), (long long)u->r_len,
                                                                (int)u->n_inc);
  count_launch();
  for (size_t r = 0; r < runs.size(); r++) {
    const mj_op* op = runs[r]->op;
    const long long len = (long long)op->n_elt * Qp;
    const size_t at = (size_t)(*elt_off)[r] * Qp;
    k_union_remap<<<grid_for_len(len), 256, 0, s>>>(op->nodle_e.as<int>(), op->slot_e.as<int>(), len, Qp, Q,
                                                    (*dof_off)[r], u->h_ptr[(*dof_off)[r]], (int)u->n_inc,
                                                    u->nodle_e.as<int>() + at, u->slot_e.as<int>() + at);
    count_launch();
    if (int rc = union_copy_factors(u.get(), op, (*elt_off)[r], s)) return rc;
  }
  MJ_CUDA(cudaMemcpyAsync(u->ptr.ptr, u->h_ptr.data(), sizeof(int) * ((size_t)n_dof + 1), cudaMemcpyHostToDevice, s));
  MJ_CUDA(cudaStreamSynchronize(s));
  MJ_CUDA(cudaGetLastError());
  if (int rc = op_finish(u.get())) return rc;

  // the union's integrator state: dt^2/D and 1/D of every run at its offset,
  // no sources (applied per run by the batch), its own step counters
  std::unique_ptr<mj_lf> lf(new mj_lf());
  lf->op = u.get(); lf->dt = 1.0; lf->n_dof = (int)n_dof; lf->stream = s;
  MJ_CUDA(lf->minv.alloc(sizeof(float) * ((size_t)n_dof + 4)));
  MJ_CUDA(cudaMemsetAsync(lf->minv.ptr, 0, lf->minv.bytes, s));
  MJ_CUDA(lf->inv_mass64.alloc(sizeof(double) * (size_t)n_dof));
  MJ_CUDA(lf->ua.alloc(sizeof(float) * ((size_t)n_dof + 4)));
  MJ_CUDA(lf->ub.alloc(sizeof(float) * ((size_t)n_dof + 4)));
  MJ_CUDA(cudaMemsetAsync(lf->ua.ptr, 0, lf->ua.bytes, s));
  MJ_CUDA(cudaMemsetAsync(lf->ub.ptr, 0, lf->ub.bytes, s));
  for (size_t r = 0; r < runs.size(); r++) {
    const mj_lf* src = runs[r];
    const size_t off = (size_t)(*dof_off)[r];
    MJ_CUDA(cudaMemcpyAsync(lf->minv.as<float>() + off, src->minv.ptr, sizeof(float) * src->n_dof,
                            cudaMemcpyDeviceToDevice, s));
    MJ_CUDA(cudaMemcpyAsync(lf->inv_mass64.as<double>() + off, src->inv_mass64.ptr, sizeof(double) * src->n_dof,
                            cudaMemcpyDeviceToDevice, s));
  }
  MJ_CUDA(lf->ctr.alloc(sizeof(int) * 2));
  MJ_CUDA(cudaMemsetAsync(lf->ctr.ptr, 0, sizeof(int) * 2, s));
  MJ_CUDA(lf->pulse_d.alloc(sizeof(double)));
  MJ_CUDA(cudaMemsetAsync(lf->pulse_d.ptr, 0, sizeof(double), s));
  lf->n_pulse = 0;
  lf->n_src = 0;
  lf->stream_gather = true;
  lf->initialised = true;
  MJ_CUDA(cudaStreamSynchronize(s));
  if (int rc = lf_stream_setup(lf.get())) return rc;
  *uop_out = std::move(u);
  *ulf_out = std::move(lf);
  return MJ_OK;
}
