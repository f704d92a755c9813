// Many right-hand sides on one mesh: S independent leap-frog runs (one per
// source) advanced together, FP32, state stored [dof][S] so every dof row of
// S values moves as one contiguous block.  The factors and connectivity are
// streamed once per step for all S runs.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <memory>
#include <vector>

#include "mj_internal.cuh"
#include "mj_k1.cuh"

namespace mj {
namespace {

// ---- element kernel variants for many right-hand sides (FP32) -----------

template <int N, int E, int L>
int rhs_prepare_one(int* ctas) {
  using P = K1Plan<float, N, E, L>;
  int dev = 0, optin = 0;
  MJ_CUDA(cudaGetDevice(&dev));
  MJ_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  if ((int)P::total > optin || P::threads > 1024) {
    set_error("many-RHS element kernel variant does not fit");
    return MJ_ERR_ARG;
  }
  MJ_CUDA(cudaFuncSetAttribute(k_local_stiffness_rhs<N, E, L>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)P::total));
  MJ_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(ctas, k_local_stiffness_rhs<N, E, L>, P::threads, P::total));
  if (*ctas < 1) {
    set_error("many-RHS element kernel variant cannot be resident");
    return MJ_ERR_ARG;
  }
  return MJ_OK;
}

template <int N, int E, int L>
void rhs_launch_one(int grid, const float* x, const int* nodle_e, const float* fac_e, float* R, const int* slot_e,
                    int n_tiles, int S, int* err, cudaStream_t s) {
  using P = K1Plan<float, N, E, L>;
  k_local_stiffness_rhs<N, E, L><<<grid, P::threads, P::total, s>>>(x, nodle_e, fac_e, R, slot_e, n_tiles, S, err);
}

#define MJ_RHS_VARIANTS(X)                                                                                     \
  X(2, 4, 32) X(2, 8, 16) X(2, 8, 8) X(3, 2, 32) X(3, 4, 16) X(3, 4, 8) X(4, 1, 32) X(4, 2, 16) X(4, 2, 8)    \
  X(5, 1, 32) X(5, 1, 16) X(5, 2, 8)                                                                           \
  X(6, 1, 16) X(6, 1, 8) X(7, 1, 16) X(7, 1, 8) X(8, 1, 8) X(9, 1, 8)

int rhs_prepare(int n, int E, int L, int* ctas) {
#define MJ_X(NV, EV, LV) \
  if (n == NV && E == EV && L == LV) return rhs_prepare_one<NV, EV, LV>(ctas);
  MJ_RHS_VARIANTS(MJ_X)
#undef MJ_X
  set_error("no many-RHS element kernel variant for this order");
  return MJ_ERR_ARG;
}

// Dynamic shared memory of the ENERGY variant: the plan's bytes, then the
// per-(element, source, z-line) sums of the element product.
template <int N, int E, int L>
size_t energy_smem(int S) {
  using P = K1Plan<float, N, E, L>;
  return P::total + sizeof(float) * (size_t)E * S * N * N;
}

template <int N, int E, int L>
int energy_prepare_one(int S, int* ctas) {
  using P = K1Plan<float, N, E, L>;
  int dev = 0, optin = 0;
  MJ_CUDA(cudaGetDevice(&dev));
  MJ_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  const size_t bytes = energy_smem<N, E, L>(S);
  if (bytes > (size_t)optin) {
    set_error("adjoint gradient kernel: too many sources for its shared memory");
    return MJ_ERR_ARG;
  }
  MJ_CUDA(cudaFuncSetAttribute(k_local_stiffness_rhs<N, E, L, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)bytes));
  MJ_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(ctas, k_local_stiffness_rhs<N, E, L, true>, P::threads,
                                                        bytes));
  if (*ctas < 1) {
    set_error("adjoint gradient kernel cannot be resident");
    return MJ_ERR_ARG;
  }
  return MJ_OK;
}

template <int N, int E, int L>
void energy_launch_one(int grid, const float* x, const int* nodle_e, const float* fac_e, int n_tiles, int S, int* err,
                       const float* lam, double* gacc, const double* coef, cudaStream_t s) {
  using P = K1Plan<float, N, E, L>;
  k_local_stiffness_rhs<N, E, L, true><<<grid, P::threads, energy_smem<N, E, L>(S), s>>>(
      x, nodle_e, fac_e, nullptr, nullptr, n_tiles, S, err, lam, gacc, coef);
}

// Sets up the ENERGY variant of (n, E, L) for S sources; *ctas: its CTAs per
// SM (its shared memory is larger than the plain variant's, so its persistent
// grid is sized on its own).
int energy_prepare(int n, int E, int L, int S, int* ctas) {
#define MJ_X(NV, EV, LV) \
  if (n == NV && E == EV && L == LV) return energy_prepare_one<NV, EV, LV>(S, ctas);
  MJ_RHS_VARIANTS(MJ_X)
#undef MJ_X
  set_error("no energy kernel variant for this order");
  return MJ_ERR_ARG;
}

void energy_launch(int n, int E, int L, int grid, const float* x, const int* nodle_e, const float* fac_e, int n_tiles,
                   int S, int* err, const float* lam, double* gacc, const double* coef, cudaStream_t s) {
#define MJ_X(NV, EV, LV)                                                                              \
  if (n == NV && E == EV && L == LV) {                                                                \
    energy_launch_one<NV, EV, LV>(grid, x, nodle_e, fac_e, n_tiles, S, err, lam, gacc, coef, s);      \
    return;                                                                                           \
  }
  MJ_RHS_VARIANTS(MJ_X)
#undef MJ_X
}

void rhs_launch(int n, int E, int L, int grid, const float* x, const int* nodle_e, const float* fac_e, float* R,
                const int* slot_e, int n_tiles, int S, int* err, cudaStream_t s) {
#define MJ_X(NV, EV, LV)                                                                     \
  if (n == NV && E == EV && L == LV) {                                                       \
    rhs_launch_one<NV, EV, LV>(grid, x, nodle_e, fac_e, R, slot_e, n_tiles, S, err, s);      \
    return;                                                                                  \
  }
  MJ_RHS_VARIANTS(MJ_X)
#undef MJ_X
}

// ---- per-(dof, rhs) kernels ------------------------------------------------

// Gather + leap-frog, thread per (dof d, right-hand side s):
//   U[d][s] <- 2 U1 - U0 + (dt^2/D_d) (-(A U1)[d][s])
// The contributions to dof d sit in R[ptr[d] .. ptr[d+1]) (rows of S), so a
// warp streams contiguous memory.  Block 0 advances the step counter
// ctr[1-q] = ctr[q] + 1 (sources: k_source_rhs).  uout may alias u0
// (each thread reads its entry first).
__global__ void k_gather_leapfrog_rhs(const float* __restrict__ R, const int* __restrict__ ptr,
                                      int* __restrict__ ctr, int q, const float* u0, const float* __restrict__ u1,
                                      float* uout, const float* __restrict__ m, int n_dof, int S) {
  if (ctr && blockIdx.x == 0 && threadIdx.x == 0) ctr[1 - q] = ctr[q] + 1;
  const long long total = (long long)n_dof * S;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const int d = (int)(t / S);
    const int s = (int)(t - (long long)d * S);
    float y = 0.f;
    const int q1 = __ldg(ptr + d + 1);
    for (int e = __ldg(ptr + d); e < q1; e++) y += __ldg(R + (size_t)e * S + s);
    uout[t] = 2.f * __ldg(u1 + t) - u0[t] + __ldg(m + d) * (-y);
  }
}

// Sources of the step just taken: u[idx[t]][rhs[t]] += (dt^2/D) p val[t],
// p = pulse[ctr[q]] (no pulse past n_pulse).  (dof, rhs) pairs are unique.
__global__ void k_source_rhs(const int* __restrict__ idx, const int* __restrict__ rhs, const float* __restrict__ val,
                             int n_src, const double* __restrict__ pulse, int n_pulse, const int* __restrict__ ctr,
                             int q, const float* __restrict__ m, float* __restrict__ u, int S) {
  const int step = ctr[q];
  if (step >= n_pulse) return;
  const float p = (float)pulse[step];
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n_src; t += gridDim.x * blockDim.x) {
    const int d = idx[t];
    u[(size_t)d * S + rhs[t]] += m[d] * p * val[t];
  }
}

// Adjoint source: lam[d][s] += invD[d] * sum_{(k,w) at d} w * res[k][s][col]
// over the dofs touched by receivers (rdof, CSR rptr/rk/rw).
__global__ void k_inject_rhs(const int* __restrict__ rdof, const int* __restrict__ rptr, const int* __restrict__ rk,
                             const double* __restrict__ rw, int n_rd, const double* __restrict__ res, int res_stride,
                             int col, const double* __restrict__ inv_mass, float* __restrict__ lam, int S) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n_rd * S) return;
  const int i = t / S, s = t - i * S;
  double acc = 0.0;
  for (int e = rptr[i]; e < rptr[i + 1]; e++) acc += rw[e] * res[((size_t)rk[e] * S + s) * res_stride + col];
  const int d = rdof[i];
  lam[(size_t)d * S + s] += (float)(inv_mass[d] * acc);
}

// fac = scale[e] * orig for every element (media update of an operator).
template <typename Real>
__global__ void k_scale_factors(const Real* __restrict__ orig, const double* __restrict__ scale, Real* __restrict__ fac,
                                int n_elt, int per_elt) {
  const long long total = (long long)n_elt * per_elt;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x)
    fac[t] = Real(double(orig[t]) * scale[t / per_elt]);
}

// First step U1 = U0 + dt (dU0 + dt/2 D^-1 (-A U0)) for every right-hand side.
// du0 and u1 may be the same array (each thread reads its entry before writing it).
__global__ void k_gather_init_rhs(const float* __restrict__ R, const int* __restrict__ ptr,
                                  const float* __restrict__ u0, const float* du0,
                                  const double* __restrict__ inv_mass, double dt, float* u1, int n_dof, int S) {
  const long long total = (long long)n_dof * S;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const int d = (int)(t / S);
    const int s = (int)(t - (long long)d * S);
    float y = 0.f;
    for (int e = ptr[d]; e < ptr[d + 1]; e++) y += R[(size_t)e * S + s];
    double v = double(-y) * inv_mass[d];
    v *= 0.5 * dt;
    v += du0 ? double(du0[t]) : 0.0;
    v *= dt;
    u1[t] = float(v + double(u0[t]));
  }
}

// Receiver k, right-hand side s: sum_t W[k][t] U[idx[k][t]][s], FP64 sum;
// written to out[(k*S + s)*stride + col].
__global__ void k_receivers_rhs(const float* __restrict__ u, const int* __restrict__ idx,
                                const double* __restrict__ w, int n_rec, int n_w, int S,
                                double* __restrict__ out, int stride, int col) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n_rec * S) return;
  const int k = t / S, s = t - k * S;
  double acc = 0.0;
  for (int a = 0; a < n_w; a++) acc += w[(size_t)k * n_w + a] * double(u[(size_t)idx[(size_t)k * n_w + a] * S + s]);
  out[(size_t)t * stride + col] = acc;
}

__global__ void k_cast_f64_to_f32(const double* __restrict__ a, float* __restrict__ b, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    b[i] = (float)a[i];
}
__global__ void k_cast_f32_to_f64(const float* __restrict__ a, double* __restrict__ b, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    b[i] = (double)a[i];
}

int grid_for(long long n) {
  return (int)std::max<long long>(1, std::min<long long>((n + 255) / 256, (long long)sm_count() * 16));
}

}  // namespace

// Receiver values of every run before a step: out column `col` of
// b->traces_d (stride = steps of the call).
void lfb_receivers(mj_lfb* b, const float* u, int stride, int col, cudaStream_t s) {
  const int threads = 128, blocks = (b->n_rec * b->S + threads - 1) / threads;
  k_receivers_rhs<<<blocks, threads, 0, s>>>(u, b->rec_idx.as<int>(), b->rec_w.as<double>(), b->n_rec, b->n_rec_w,
                                             b->S, b->traces_d.as<double>(), stride, col);
  count_launch();
}

// Derivative matrix of order n into this unit's constant memory.
int k1_set_gmat_rhs(int n, const double* g) {
  float v[kMaxNK * kMaxNK];
  for (int a = 0; a < n * n; a++) v[a] = (float)g[a];
  MJ_CUDA(cudaMemcpyToSymbol(c_gmat32, v, sizeof(float) * n * n, sizeof(float) * kMaxNK * kMaxNK * n));
  return MJ_OK;
}

std::vector<RhsVariant> k1_rhs_candidates(int n) {
  switch (n) {
    case 2: return {{4, 32}, {8, 16}, {8, 8}};
    case 3: return {{2, 32}, {4, 16}, {4, 8}};
    case 4: return {{1, 32}, {2, 16}, {2, 8}};
    case 5: return {{1, 32}, {1, 16}, {2, 8}};
    case 6: return {{1, 16}, {1, 8}};
    case 7: return {{1, 16}, {1, 8}};
    case 8: return {{1, 8}};
    case 9: return {{1, 8}};
  }
  return {};
}

}  // namespace mj

using namespace mj;


namespace {

void lfb_k1(mj_lfb* b, const float* x, cudaStream_t s) {
  mj_op* op = b->op;
  rhs_launch(op->n, b->E, b->L, b->grid, x, op->nodle_e.as<int>(), op->fac_e.as<float>(), b->R.as<float>(),
             op->slot_e.as<int>(), b->n_tiles, b->S, op->err.as<int>(), s);
  count_launch();
}

// One leap-frog step of all right-hand sides; q = parity of the pulse counter.
void lfb_step_launch(mj_lfb* b, float* cur, const float* next, int q, cudaStream_t s) {
  lfb_k1(b, next, s);
  const long long total = (long long)b->n_dof * b->S;
  k_gather_leapfrog_rhs<<<grid_for(total), 256, 0, s>>>(b->R.as<float>(), b->op->ptr.as<int>(), b->ctr.as<int>(), q,
                                                        cur, next, cur, b->m.as<float>(), b->n_dof, b->S);
  count_launch();
  if (b->n_src) {
    k_source_rhs<<<(b->n_src + 255) / 256, 256, 0, s>>>(b->src_idx.as<int>(), b->src_rhs.as<int>(),
                                                        b->src_val.as<float>(), b->n_src, b->pulse.as<double>(),
                                                        b->n_pulse, b->ctr.as<int>(), q, b->m.as<float>(), cur, b->S);
    count_launch();
  }
}

int lfb_autotune(mj_lfb* b) {
  mj_op* op = b->op;
  const int sms = sm_count();
  cudaEvent_t e0, e1;
  MJ_CUDA(cudaEventCreate(&e0));
  MJ_CUDA(cudaEventCreate(&e1));
  double best = 1e300;
  int bi = -1;
  const std::vector<RhsVariant> cands = k1_rhs_candidates(op->n);
  for (int c = 0; c < (int)cands.size(); c++) {
    const RhsVariant v = cands[c];
    if (b->S % v.L) continue;
    int ctas = 0;
    if (rhs_prepare(op->n, v.E, v.L, &ctas) != MJ_OK) continue;
    b->E = v.E; b->L = v.L; b->n_tiles = op->n_elt_pad / v.E;
    b->grid = std::max(1, std::min(b->n_tiles, ctas * sms));
    lfb_k1(b, b->ua.as<float>(), b->stream);
    MJ_CUDA(cudaEventRecord(e0, b->stream));
    for (int rep = 0; rep < 2; rep++) lfb_k1(b, b->ua.as<float>(), b->stream);
    MJ_CUDA(cudaEventRecord(e1, b->stream));
    MJ_CUDA(cudaEventSynchronize(e1));
    float f = 0.f;
    MJ_CUDA(cudaEventElapsedTime(&f, e0, e1));
    b->tune_ms.push_back(f / 2.0);
    if (f < best) { best = f; bi = c; }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (bi < 0) {
    set_error("mj_lfb_create: no many-RHS element kernel variant fits (n_rhs must be a multiple of 8)");
    return MJ_ERR_ARG;
  }
  const RhsVariant v = cands[bi];
  int ctas = 0;
  int rc = rhs_prepare(op->n, v.E, v.L, &ctas);
  if (rc) return rc;
  b->E = v.E; b->L = v.L; b->n_tiles = op->n_elt_pad / v.E;
  b->grid = std::max(1, std::min(b->n_tiles, ctas * sms));
  MJ_CUDA(cudaMemset(op->err.ptr, 0, sizeof(int)));
  return MJ_OK;
}

}  // namespace

extern "C" {

int mj_lfb_create(mj_op* op, const mj_lfb_desc* d, mj_lfb** out) {
  MJ_CHECK_ARG(op && d && out, "mj_lfb_create: null argument");
  *out = nullptr;
  MJ_CHECK_ARG(op->precision == MJ_FP32, "mj_lfb_create: the many-RHS integrator needs an MJ_FP32 operator");
  MJ_CHECK_ARG(d->n_rhs >= 8 && d->n_rhs % 8 == 0 && d->n_rhs <= 4096, "mj_lfb_create: n_rhs must be a multiple of 8 in [8, 4096]");
  MJ_CHECK_ARG(d->dt > 0 && std::isfinite(d->dt), "mj_lfb_create: dt must be positive");
  MJ_CHECK_ARG(d->mass, "mj_lfb_create: mass is required");
  MJ_CHECK_ARG(d->n_src >= 0 && (d->n_src == 0 || (d->src_idx && d->src_rhs && d->src_val)),
               "mj_lfb_create: bad source arrays");
  MJ_CHECK_ARG(d->n_pulse >= 0 && (d->n_pulse == 0 || d->pulse), "mj_lfb_create: bad pulse array");
  MJ_CHECK_ARG(d->n_rec >= 0 && (d->n_rec == 0 || (d->rec_idx && d->rec_w && d->n_rec_w > 0)),
               "mj_lfb_create: bad receiver arrays");
  const int n = op->n_dof, S = d->n_rhs;
  std::unique_ptr<mj_lfb> b(new mj_lfb());
  b->op = op; b->S = S; b->n_dof = n; b->dt = d->dt; b->stream = op->stream;
  std::vector<double> invD(n);
  std::vector<float> m(n);
  for (int i = 0; i < n; i++) {
    MJ_CHECK_ARG(std::isfinite(d->mass[i]) && d->mass[i] > 0, "mj_lfb_create: mass must be positive");
    invD[i] = d->inv_mass ? d->inv_mass[i] : 1.0 / d->mass[i];
    m[i] = (float)(d->dt * d->dt * invD[i]);
  }
  // sparse sources, one entry per (dof, rhs) pair
  std::vector<std::pair<int, int>> pairs;
  for (int t = 0; t < d->n_src; t++) {
    MJ_CHECK_ARG(d->src_idx[t] >= 0 && d->src_idx[t] < n, "mj_lfb_create: source index out of range");
    MJ_CHECK_ARG(d->src_rhs[t] >= 0 && d->src_rhs[t] < S, "mj_lfb_create: source right-hand side out of range");
    pairs.push_back({d->src_idx[t], d->src_rhs[t]});
  }
  std::sort(pairs.begin(), pairs.end());
  for (size_t t = 1; t < pairs.size(); t++)
    MJ_CHECK_ARG(pairs[t] != pairs[t - 1], "mj_lfb_create: duplicate (source dof, right-hand side) pair");
  std::vector<float> sv(std::max(1, d->n_src));
  std::vector<int> sr(std::max(1, d->n_src), 0), si(std::max(1, d->n_src), 0);
  for (int t = 0; t < d->n_src; t++) { sv[t] = (float)d->src_val[t]; sr[t] = d->src_rhs[t]; si[t] = d->src_idx[t]; }
  b->n_src = d->n_src;
  const size_t rows = (size_t)n * S;
  MJ_CUDA(b->R.alloc(sizeof(float) * (op->n_inc + 1) * S));
  MJ_CUDA(b->src_idx.alloc(sizeof(int) * si.size()));
  MJ_CUDA(b->src_val.alloc(sizeof(float) * sv.size()));
  MJ_CUDA(b->src_rhs.alloc(sizeof(int) * sr.size()));
  MJ_CUDA(b->m.alloc(sizeof(float) * (n + 8)));  // padded: 16-byte rounded bulk copies of dof ranges
  MJ_CUDA(cudaMemset(b->m.ptr, 0, sizeof(float) * (n + 8)));
  MJ_CUDA(b->inv_mass64.alloc(sizeof(double) * n));
  MJ_CUDA(b->pulse.alloc(sizeof(double) * std::max(1, d->n_pulse)));
  MJ_CUDA(b->ctr.alloc(sizeof(int) * 2));
  MJ_CUDA(b->ua.alloc(sizeof(float) * rows));
  MJ_CUDA(b->ub.alloc(sizeof(float) * rows));
  MJ_CUDA(cudaMemcpy(b->src_idx.ptr, si.data(), sizeof(int) * si.size(), cudaMemcpyHostToDevice));
  MJ_CUDA(cudaMemcpy(b->src_val.ptr, sv.data(), sizeof(float) * sv.size(), cudaMemcpyHostToDevice));
  MJ_CUDA(cudaMemcpy(b->src_rhs.ptr, sr.data(), sizeof(int) * sr.size(), cudaMemcpyHostToDevice));
  MJ_CUDA(cudaMemcpy(b->m.ptr, m.data(), sizeof(float) * n, cudaMemcpyHostToDevice));
  MJ_CUDA(cudaMemcpy(b->inv_mass64.ptr, invD.data(), sizeof(double) * n, cudaMemcpyHostToDevice));
  if (d->n_pulse) MJ_CUDA(cudaMemcpy(b->pulse.ptr, d->pulse, sizeof(double) * d->n_pulse, cudaMemcpyHostToDevice));
  b->n_pulse = d->n_pulse;
  MJ_CUDA(cudaMemset(b->ctr.ptr, 0, sizeof(int) * 2));
  MJ_CUDA(cudaMemset(b->ua.ptr, 0, sizeof(float) * rows));
  MJ_CUDA(cudaMemset(b->ub.ptr, 0, sizeof(float) * rows));
  b->n_rec = d->n_rec;
  b->n_rec_w = d->n_rec_w;
  if (d->n_rec) {
    const size_t mrec = (size_t)d->n_rec * d->n_rec_w;
    for (size_t t = 0; t < mrec; t++)
      MJ_CHECK_ARG(d->rec_idx[t] >= 0 && d->rec_idx[t] < n, "mj_lfb_create: receiver dof out of range");
    MJ_CUDA(b->rec_idx.alloc(sizeof(int) * mrec));
    MJ_CUDA(b->rec_w.alloc(sizeof(double) * mrec));
    MJ_CUDA(cudaMemcpy(b->rec_idx.ptr, d->rec_idx, sizeof(int) * mrec, cudaMemcpyHostToDevice));
    MJ_CUDA(cudaMemcpy(b->rec_w.ptr, d->rec_w, sizeof(double) * mrec, cudaMemcpyHostToDevice));
  }
  int rc = k1_set_gmat_rhs(op->n, op->gradphi);
  if (rc) return rc;
  rc = lfb_autotune(b.get());
  if (rc) return rc;
  rc = lfb_fused_setup(b.get());
  if (rc) return rc;
  *out = b.release();
  return MJ_OK;
}

int mj_lfb_destroy(mj_lfb* b) {
  delete b;
  return MJ_OK;
}

int mj_lfb_init(mj_lfb* b, const double* u0, const double* du0) {
  MJ_CHECK_ARG(b, "mj_lfb_init: null integrator");
  cudaStream_t s = b->stream;
  const long long rows = (long long)b->n_dof * b->S;
  if (b->stage.bytes < sizeof(double) * rows) MJ_CUDA(b->stage.alloc(sizeof(double) * rows));
  // U^0
  if (u0) {
    MJ_CUDA(cudaMemcpyAsync(b->stage.ptr, u0, sizeof(double) * rows, cudaMemcpyHostToDevice, s));
    k_cast_f64_to_f32<<<grid_for(rows), 256, 0, s>>>(b->stage.as<double>(), b->ua.as<float>(), rows);
    count_launch();
  } else {
    MJ_CUDA(cudaMemsetAsync(b->ua.ptr, 0, sizeof(float) * rows, s));
  }
  // dU^0 staged in ub, overwritten by U^1 below (each thread reads its own entry first)
  const float* du = nullptr;
  if (du0) {
    MJ_CUDA(cudaMemcpyAsync(b->stage.ptr, du0, sizeof(double) * rows, cudaMemcpyHostToDevice, s));
    k_cast_f64_to_f32<<<grid_for(rows), 256, 0, s>>>(b->stage.as<double>(), b->ub.as<float>(), rows);
    count_launch();
    du = b->ub.as<float>();
  }
  lfb_k1(b, b->ua.as<float>(), s);
  k_gather_init_rhs<<<grid_for(rows), 256, 0, s>>>(b->R.as<float>(), b->op->ptr.as<int>(),
                                                   b->ua.as<float>(), du, b->inv_mass64.as<double>(), b->dt,
                                                   b->ub.as<float>(), b->n_dof, b->S);
  count_launch();
  MJ_CUDA(cudaMemsetAsync(b->ctr.ptr, 0, sizeof(int) * 2, s));
  MJ_CUDA(cudaGetLastError());
  MJ_CUDA(cudaStreamSynchronize(s));
  b->cur_is_a = true;
  b->step = 0;
  b->initialised = true;
  return MJ_OK;
}

// Advances nsteps steps of every right-hand side.  With use_graph, chunks of
// 2*k steps replay one captured CUDA graph (instantiated on first use);
// traces (if not NULL and receivers were given) are sampled before every
// step into traces[(k*S + s)*trace_stride + step_in_call] (no graph then).
int mj_lfb_advance(mj_lfb* b, int nsteps, double* traces, int trace_stride, int use_graph) {
  MJ_CHECK_ARG(b, "mj_lfb_advance: null integrator");
  MJ_CHECK_ARG(nsteps >= 0, "mj_lfb_advance: negative step count");
  if (!b->initialised) {
    set_error("mj_lfb_advance: mj_lfb_init must be called first");
    return MJ_ERR_STATE;
  }
  cudaStream_t s = b->stream;
  const bool diag = traces && b->n_rec;
  if (diag) {
    MJ_CHECK_ARG(trace_stride >= nsteps, "mj_lfb_advance: trace_stride smaller than nsteps");
    const size_t bytes = sizeof(double) * (size_t)b->n_rec * b->S * nsteps;
    if (b->traces_d.bytes < bytes) MJ_CUDA(b->traces_d.alloc(bytes));
  }
  if (b->fused) return lfb_fused_advance(b, nsteps, traces, trace_stride, use_graph != 0);
  int done = 0;
  const int G = 20;  // steps per captured graph (even: buffers and counters return to their roles)
  if (use_graph && !diag && nsteps >= G + 1) {
    if (b->step & 1) {  // realign: graphs start on an even step with ua holding U^n
      lfb_step_launch(b, b->cur(), b->next(), b->step & 1, s);
      b->cur_is_a = !b->cur_is_a;
      b->step++;
      done++;
    }
    if (!b->graph) {
      cudaStream_t cs;
      MJ_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
      cudaGraph_t g;
      const uint64_t launches_before = launch_counter().load();
      MJ_CUDA(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
      bool a = true;
      for (int k = 0; k < G; k++) {
        float* cur = (a ? b->ua : b->ub).as<float>();
        float* nxt = (a ? b->ub : b->ua).as<float>();
        lfb_step_launch(b, cur, nxt, k & 1, cs);
        a = !a;
      }
      MJ_CUDA(cudaStreamEndCapture(cs, &g));
      launch_counter().store(launches_before);  // captured, not launched
      MJ_CUDA(cudaGraphInstantiate(&b->graph, g, 0));
      cudaGraphDestroy(g);
      cudaStreamDestroy(cs);
      b->graph_steps = G;
    }
    while (nsteps - done >= G) {
      MJ_CUDA(cudaGraphLaunch(b->graph, s));
      count_launch((uint64_t)G * (2 + (b->n_src > 0)));
      done += G;
      b->step += G;
    }
  }
  for (; done < nsteps; done++) {
    if (diag) {
      const int threads = 128, blocks = (b->n_rec * b->S + threads - 1) / threads;
      k_receivers_rhs<<<blocks, threads, 0, s>>>(b->cur(), b->rec_idx.as<int>(), b->rec_w.as<double>(), b->n_rec,
                                                 b->n_rec_w, b->S, b->traces_d.as<double>(), nsteps, done);
      count_launch();
    }
    lfb_step_launch(b, b->cur(), b->next(), b->step & 1, s);
    b->cur_is_a = !b->cur_is_a;
    b->step++;
  }
  MJ_CUDA(cudaGetLastError());
  if (diag)
    for (int r = 0; r < b->n_rec * b->S; r++)
      MJ_CUDA(cudaMemcpyAsync(traces + (size_t)r * trace_stride, b->traces_d.as<double>() + (size_t)r * nsteps,
                              sizeof(double) * nsteps, cudaMemcpyDeviceToHost, s));
  return take_kernel_error(b->op->err.ptr, s, "mj_lfb_advance");
}

int mj_lfb_get_state(mj_lfb* b, double* u_n, double* u_np1) {
  MJ_CHECK_ARG(b, "mj_lfb_get_state: null integrator");
  cudaStream_t s = b->stream;
  const long long rows = (long long)b->n_dof * b->S;
  if (b->stage.bytes < sizeof(double) * rows) MJ_CUDA(b->stage.alloc(sizeof(double) * rows));
  const float* src[2] = {b->cur(), b->next()};
  double* dst[2] = {u_n, u_np1};
  for (int k = 0; k < 2; k++) {
    if (!dst[k]) continue;
    k_cast_f32_to_f64<<<grid_for(rows), 256, 0, s>>>(src[k], b->stage.as<double>(), rows);
    count_launch();
    MJ_CUDA(cudaMemcpyAsync(dst[k], b->stage.ptr, sizeof(double) * rows, cudaMemcpyDeviceToHost, s));
    MJ_CUDA(cudaStreamSynchronize(s));
  }
  return MJ_OK;
}

int mj_lfb_set_fused(mj_lfb* b, int enable) {
  MJ_CHECK_ARG(b, "mj_lfb_set_fused: null integrator");
  if (enable && b->rs_variant < 0) {
    set_error("mj_lfb_set_fused: no one-kernel step variant fits this integrator");
    return MJ_ERR_STATE;
  }
  b->fused = enable != 0;
  return MJ_OK;
}

int mj_lfb_set_step_variant(mj_lfb* b, int tile_elems, int lanes, int sources_per_thread) {
  MJ_CHECK_ARG(b, "mj_lfb_set_step_variant: null integrator");
  return lfb_set_step_variant(b, tile_elems, lanes, sources_per_thread);
}

int mj_lfb_profile(mj_lfb* b, int enable) {
  MJ_CHECK_ARG(b, "mj_lfb_profile: null integrator");
  b->rs_profile = enable != 0;
  return MJ_OK;
}

int mj_lfb_phase_ms(const mj_lfb* b, double* out) {
  MJ_CHECK_ARG(b && out, "mj_lfb_phase_ms: null argument");
  return lfb_phase_ms(b, out);
}

int mj_lfb_step_info(const mj_lfb* b, int* fused, int* threads, int* grid, int* n_candidates, double* candidate_ms) {
  MJ_CHECK_ARG(b, "mj_lfb_step_info: null integrator");
  if (fused) *fused = b->fused ? 1 : 0;
  if (threads) *threads = b->rs_threads;
  if (grid) *grid = b->rs_grid;
  if (n_candidates) *n_candidates = (int)b->rs_tune_ms.size();
  if (candidate_ms)
    for (size_t c = 0; c < b->rs_tune_ms.size(); c++) candidate_ms[c] = b->rs_tune_ms[c];
  return MJ_OK;
}

int mj_lfb_info(const mj_lfb* b, int* n_rhs, int* tile_elems, int* lanes, int* grid, int* step) {
  MJ_CHECK_ARG(b, "mj_lfb_info: null integrator");
  if (n_rhs) *n_rhs = b->S;
  if (tile_elems) *tile_elems = b->E;
  if (lanes) *lanes = b->L;
  if (grid) *grid = b->grid;
  if (step) *step = b->step;
  return MJ_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Discrete adjoint of the many-source leap-frog (no reference counterpart).
// ---------------------------------------------------------------------------

// One action of a binomial (revolve) checkpoint schedule over the chain of
// forward states P_k = (U^k, U^{k+1}), k = 1..N-1, whose adjoint visits
// P_{N-1}, ..., P_1 in that order (adjoint step m = k+1 needs U^k).
struct RevAction {
  enum Kind { RESTORE, ADVANCE, STORE, VISIT } kind;
  int step;  // RESTORE/STORE: the state's k; ADVANCE: target k; VISIT: k
  int slot;  // RESTORE/STORE: snapshot slot
};

struct mj_adj {
  mj_lfb* b = nullptr;
  int N = 0, K = 0, J = 0;           // steps, checkpoint interval, checkpoints
  size_t rows = 0;                   // n_dof * S
  DevBuf ckpt;                       // J x 2 states (U^{jK}, U^{jK+1})
  DevBuf seg;                        // K states of the segment being replayed
  DevBuf la, lb;                     // adjoint states
  DevBuf traces, res;                // n_rec x S x (N+1), FP64
  DevBuf grad, coef;                 // per element (padded), FP64
  DevBuf rdof, rptr, rk, rw;         // receiver injection CSR
  int n_rd = 0;
  bool have_forward = false;
  // binomial (revolve) schedule: snaps snapshot slots of one state pair each
  bool revolve = false;
  int snaps = 0;
  std::vector<RevAction> plan;       // whole schedule; plan[first_visit] is the first VISIT
  size_t first_visit = 0;
  std::vector<std::pair<int, int>> sweep_stores;  // (k, slot) stored by the forward sweep
  DevBuf slots;                      // snaps x 2 states
  DevBuf work;                       // 3 states: the current pair and the next state
  long long backward_steps = 0;      // forward steps recomputed by the backward sweep
  bool store_all = false;            // uniform with K = N: seg keeps U^0 .. U^{N-1} from the forward sweep
  int energy_grid = 1;               // persistent grid of the gradient kernel
};

namespace {

void adj_receivers(mj_adj* a, const float* u, int col, cudaStream_t s) {
  mj_lfb* b = a->b;
  const int threads = 128, blocks = (b->n_rec * b->S + threads - 1) / threads;
  k_receivers_rhs<<<blocks, threads, 0, s>>>(u, b->rec_idx.as<int>(), b->rec_w.as<double>(), b->n_rec, b->n_rec_w,
                                             b->S, a->traces.as<double>(), a->N + 1, col);
  count_launch();
}

// out = 2*u1 - u0 + dt^2 D^-1 (-A u1 + pulse[step] F): the forward update with
// an explicit step index (pulse counter set on the host first).
int adj_forward_step(mj_adj* a, const float* u0, const float* u1, float* out, int step, cudaStream_t s) {
  mj_lfb* b = a->b;
  MJ_CUDA(cudaMemcpyAsync(b->ctr.as<int>(), &step, sizeof(int), cudaMemcpyHostToDevice, s));
  if (b->fused)  // the one-kernel step (bitwise the same arithmetic)
    return lfb_fused_step_on(b, const_cast<float*>(u0), const_cast<float*>(u1), out, true, s);
  lfb_k1(b, u1, s);
  const long long total = (long long)b->n_dof * b->S;
  k_gather_leapfrog_rhs<<<grid_for(total), 256, 0, s>>>(b->R.as<float>(), b->op->ptr.as<int>(), b->ctr.as<int>(), 0,
                                                        u0, u1, out, b->m.as<float>(), b->n_dof, b->S);
  count_launch();
  if (b->n_src) {
    k_source_rhs<<<(b->n_src + 255) / 256, 256, 0, s>>>(b->src_idx.as<int>(), b->src_rhs.as<int>(),
                                                        b->src_val.as<float>(), b->n_src, b->pulse.as<double>(),
                                                        b->n_pulse, b->ctr.as<int>(), 0, b->m.as<float>(), out, b->S);
    count_launch();
  }
  MJ_CUDA(cudaGetLastError());
  return MJ_OK;
}

// Binomial checkpointing (Griewank and Walther's revolve): the fewest
// forward steps that visit the chain states x_{b-1}, ..., x_a in reverse
// order, x_a being held in a snapshot and s more snapshots free, by dynamic
// programming: cost(l, 0) = l(l-1)/2 (every state recomputed from x_a) and
// cost(l, s) = min_c [c + cost(l-c, s-1) + cost(c, s)] (advance c steps,
// store, reverse the right part with one snapshot fewer, then the left part).
struct RevolvePlanner {
  int L, S;
  std::vector<long long> cost;
  std::vector<int> arg;
  std::vector<RevAction>* out;
  std::vector<int> free_slots;
  RevolvePlanner(int L_, int S_) : L(L_), S(S_), cost((size_t)(L_ + 1) * (S_ + 1)), arg((size_t)(L_ + 1) * (S_ + 1)) {
    for (int l = 0; l <= L; l++) C(l, 0) = (long long)l * (l - 1) / 2;
    for (int s = 1; s <= S; s++) {
      C(0, s) = C(1, s) = 0;
      for (int l = 2; l <= L; l++) {
        long long best = -1;
        int bc = 1;
        for (int c = 1; c < l; c++) {
          const long long v = c + C(l - c, s - 1) + C(c, s);
          if (best < 0 || v < best) { best = v; bc = c; }
        }
        C(l, s) = best;
        A(l, s) = bc;
      }
    }
  }
  long long& C(int l, int s) { return cost[(size_t)l * (S + 1) + s]; }
  int& A(int l, int s) { return arg[(size_t)l * (S + 1) + s]; }
  void reverse(int a, int b, int s, int slot_a) {
    const int l = b - a;
    if (l <= 0) return;
    if (l == 1) {
      out->push_back({RevAction::RESTORE, a, slot_a});
      out->push_back({RevAction::VISIT, a, -1});
      return;
    }
    if (s == 0) {
      for (int k = b - 1; k >= a; k--) {
        out->push_back({RevAction::RESTORE, a, slot_a});
        if (k > a) out->push_back({RevAction::ADVANCE, k, -1});
        out->push_back({RevAction::VISIT, k, -1});
      }
      return;
    }
    const int c = A(l, s);
    const int t = free_slots.back();
    free_slots.pop_back();
    out->push_back({RevAction::RESTORE, a, slot_a});
    out->push_back({RevAction::ADVANCE, a + c, -1});
    out->push_back({RevAction::STORE, a + c, t});
    reverse(a + c, b, s - 1, t);
    free_slots.push_back(t);
    reverse(a, a + c, s, slot_a);
  }
};

// The gradient of the misfit in the element coefficients is the sum over
// n = 2 .. N of coef_e (A_e lambda^n)^T U^{n-1} (lambda^{N+1} = 0 and
// U^0 = 0 add nothing).  Term n is taken where A_e lambda^n is computed
// anyway: in adjoint step n - 1, from U^{n-1} (adj_visit with um), except the
// last term of a run of steps, which adj_term adds.  Every schedule adds the
// terms in the order n = N, N-1, ..., 2, each with the same FP32 sums, so all
// give the same bits.

// ENERGY kernel: gacc[e] += coef[e] * (A_e x)^T u.
void adj_term(mj_adj* a, const float* x, const float* u, cudaStream_t s) {
  mj_lfb* b = a->b;
  mj_op* op = b->op;
  energy_launch(op->n, b->E, b->L, a->energy_grid, x, op->nodle_e.as<int>(), op->fac_e.as<float>(), b->n_tiles, b->S,
                op->err.as<int>(), u, a->grad.as<double>(), a->coef.as<double>(), s);
  count_launch();
}

// Adjoint step m: lambda^m from lambda^{m+1}, lambda^{m+2} and the residual
// of column m.  With um = U^m (m < N), also the gradient term n = m + 1,
// coef_e (A_e lambda^{m+1})^T U^m: inside the one-kernel step (its EN form)
// or by the ENERGY kernel.
int adj_visit(mj_adj* a, const float* um, int m, float*& lam1, float*& lam2, cudaStream_t s) {
  mj_lfb* b = a->b;
  mj_op* op = b->op;
  const int S = b->S, N = a->N;
  if (b->fused) {  // lambda^m = 2 lambda^{m+1} - lambda^{m+2} + m (-A lambda^{m+1}), one kernel
    bool done = false;
    if (um) {
      const int rc = lfb_fused_step_en(b, lam2, lam1, lam2, um, a->grad.as<double>(), a->coef.as<double>(), s, &done);
      if (rc) return rc;
    }
    if (!done) {
      if (um) adj_term(a, lam1, um, s);
      const int rc = lfb_fused_step_on(b, lam2, lam1, lam2, false, s);
      if (rc) return rc;
    }
  } else {
    lfb_k1(b, lam1, s);
    if (um) adj_term(a, lam1, um, s);
    const long long total = (long long)a->rows;
    k_gather_leapfrog_rhs<<<grid_for(total), 256, 0, s>>>(b->R.as<float>(), op->ptr.as<int>(), nullptr, 0, lam2,
                                                          lam1, lam2, b->m.as<float>(), b->n_dof, S);
    count_launch();
  }
  const int inj_blocks = (a->n_rd * S + 127) / 128;
  k_inject_rhs<<<inj_blocks, 128, 0, s>>>(a->rdof.as<int>(), a->rptr.as<int>(), a->rk.as<int>(), a->rw.as<double>(),
                                          a->n_rd, a->res.as<double>(), N + 1, m, b->inv_mass64.as<double>(), lam2,
                                          S);
  count_launch();
  std::swap(lam1, lam2);  // lam1 = lambda^m, lam2 = lambda^{m+1}
  MJ_CUDA(cudaGetLastError());
  return MJ_OK;
}

}  // namespace

extern "C" {

int mj_op_set_element_scale(mj_op* op, const double* scale) {
  MJ_CHECK_ARG(op && scale, "mj_op_set_element_scale: null argument");
  for (int e = 0; e < op->n_elt; e++)
    MJ_CHECK_ARG(std::isfinite(scale[e]) && scale[e] >= 0, "mj_op_set_element_scale: scale must be finite and >= 0");
  const size_t esz = op->precision == MJ_FP64 ? sizeof(double) : sizeof(float);
  const int per_elt = 6 * op->Qp;
  if (!op->fac_orig.ptr) {
    MJ_CUDA(op->fac_orig.alloc(op->fac_e.bytes));
    MJ_CUDA(cudaMemcpy(op->fac_orig.ptr, op->fac_e.ptr, op->fac_e.bytes, cudaMemcpyDeviceToDevice));
  }
  std::vector<double> sc(op->n_elt_pad, 0.0);
  for (int e = 0; e < op->n_elt; e++) sc[e] = scale[e];
  DevBuf d;
  MJ_CUDA(d.alloc(sizeof(double) * sc.size()));
  MJ_CUDA(cudaMemcpy(d.ptr, sc.data(), sizeof(double) * sc.size(), cudaMemcpyHostToDevice));
  const long long total = (long long)op->n_elt_pad * per_elt;
  if (esz == sizeof(double))
    k_scale_factors<double><<<grid_for(total), 256, 0, op->stream>>>(op->fac_orig.as<double>(), d.as<double>(),
                                                                     op->fac_e.as<double>(), op->n_elt_pad, per_elt);
  else
    k_scale_factors<float><<<grid_for(total), 256, 0, op->stream>>>(op->fac_orig.as<float>(), d.as<double>(),
                                                                    op->fac_e.as<float>(), op->n_elt_pad, per_elt);
  count_launch();
  MJ_CUDA(cudaGetLastError());
  MJ_CUDA(cudaStreamSynchronize(op->stream));
  op->fac_version++;
  return MJ_OK;
}

}  // extern "C"

namespace {

// Buffers and receiver tables shared by both checkpoint schedules.
int adj_common_init(mj_adj* a) {
  mj_lfb* b = a->b;
  const int nsteps = a->N;
  MJ_CUDA(a->la.alloc(sizeof(float) * a->rows));
  MJ_CUDA(a->lb.alloc(sizeof(float) * a->rows));
  const size_t tr = (size_t)b->n_rec * b->S * (nsteps + 1);
  MJ_CUDA(a->traces.alloc(sizeof(double) * tr));
  MJ_CUDA(a->res.alloc(sizeof(double) * tr));
  mj_op* op = b->op;
  MJ_CUDA(a->grad.alloc(sizeof(double) * op->n_elt_pad));
  MJ_CUDA(a->coef.alloc(sizeof(double) * op->n_elt_pad));
  // receiver injection CSR (dofs touched by receivers -> (receiver, weight))
  std::vector<int> ridx((size_t)b->n_rec * b->n_rec_w);
  std::vector<double> rwt(ridx.size());
  MJ_CUDA(cudaMemcpy(ridx.data(), b->rec_idx.ptr, sizeof(int) * ridx.size(), cudaMemcpyDeviceToHost));
  MJ_CUDA(cudaMemcpy(rwt.data(), b->rec_w.ptr, sizeof(double) * rwt.size(), cudaMemcpyDeviceToHost));
  std::vector<std::pair<int, int>> ent;  // (dof, t)
  for (size_t t = 0; t < ridx.size(); t++) ent.push_back({ridx[t], (int)t});
  std::sort(ent.begin(), ent.end());
  std::vector<int> rdof, rptr{0}, rk;
  std::vector<double> rw;
  for (size_t i = 0; i < ent.size(); i++) {
    if (i == 0 || ent[i].first != ent[i - 1].first) {
      if (i) rptr.push_back((int)rk.size());
      rdof.push_back(ent[i].first);
    }
    rk.push_back(ent[i].second / b->n_rec_w);
    rw.push_back(rwt[ent[i].second]);
  }
  rptr.push_back((int)rk.size());
  a->n_rd = (int)rdof.size();
  MJ_CUDA(a->rdof.alloc(sizeof(int) * rdof.size()));
  MJ_CUDA(a->rptr.alloc(sizeof(int) * rptr.size()));
  MJ_CUDA(a->rk.alloc(sizeof(int) * rk.size()));
  MJ_CUDA(a->rw.alloc(sizeof(double) * rw.size()));
  MJ_CUDA(cudaMemcpy(a->rdof.ptr, rdof.data(), sizeof(int) * rdof.size(), cudaMemcpyHostToDevice));
  MJ_CUDA(cudaMemcpy(a->rptr.ptr, rptr.data(), sizeof(int) * rptr.size(), cudaMemcpyHostToDevice));
  MJ_CUDA(cudaMemcpy(a->rk.ptr, rk.data(), sizeof(int) * rk.size(), cudaMemcpyHostToDevice));
  MJ_CUDA(cudaMemcpy(a->rw.ptr, rw.data(), sizeof(double) * rw.size(), cudaMemcpyHostToDevice));
  int ctas = 0;
  if (int rc = energy_prepare(op->n, b->E, b->L, b->S, &ctas)) return rc;
  a->energy_grid = std::max(1, std::min(b->n_tiles, ctas * sm_count()));
  return MJ_OK;
}

}  // namespace

extern "C" {

int mj_adj_create(mj_lfb* b, int nsteps, int checkpoint_every, mj_adj** out) {
  MJ_CHECK_ARG(b && out, "mj_adj_create: null argument");
  *out = nullptr;
  MJ_CHECK_ARG(nsteps >= 2, "mj_adj_create: at least 2 steps");
  MJ_CHECK_ARG(b->n_rec > 0, "mj_adj_create: the integrator needs receivers");
  std::unique_ptr<mj_adj> a(new mj_adj());
  a->b = b;
  a->N = nsteps;
  a->K = checkpoint_every > 0 ? checkpoint_every : std::max(2, (int)std::ceil(std::sqrt((double)nsteps)));
  MJ_CHECK_ARG(a->K >= 2, "mj_adj_create: checkpoint interval must be >= 2");
  // an interval of nsteps or more keeps every forward state: one segment the
  // forward sweep fills itself, nothing recomputed
  a->store_all = a->K >= nsteps;
  if (a->store_all) a->K = nsteps;
  a->J = (nsteps + a->K - 1) / a->K;
  a->rows = (size_t)b->n_dof * b->S;
  if (a->store_all) {
    size_t free_b = 0, total_b = 0;
    MJ_CUDA(cudaMemGetInfo(&free_b, &total_b));
    const double need = double(sizeof(float)) * a->rows * (a->K + 2);
    MJ_CHECK_ARG(need < 0.9 * double(free_b),
                 "mj_adj_create: keeping every state needs " + std::to_string(need / 1e9) + " GB, " +
                     std::to_string(free_b / 1e9) + " GB free (use a shorter checkpoint interval)");
  }
  MJ_CUDA(a->ckpt.alloc(sizeof(float) * a->rows * 2 * a->J));
  MJ_CUDA(a->seg.alloc(sizeof(float) * a->rows * a->K));
  for (int j = 0; j < a->J && !a->store_all; j++) {  // replays: U^{n0+2} .. U^{n1-1} of every segment
    const int n0 = j * a->K, n1 = std::min(n0 + a->K, nsteps);
    a->backward_steps += std::max(0, n1 - n0 - 2);
  }
  const int rc = adj_common_init(a.get());
  if (rc) return rc;
  *out = a.release();
  return MJ_OK;
}

int mj_adj_create_revolve(mj_lfb* b, int nsteps, int snapshots, mj_adj** out) {
  MJ_CHECK_ARG(b && out, "mj_adj_create_revolve: null argument");
  *out = nullptr;
  MJ_CHECK_ARG(nsteps >= 2, "mj_adj_create_revolve: at least 2 steps");
  MJ_CHECK_ARG(snapshots >= 1, "mj_adj_create_revolve: at least one snapshot");
  MJ_CHECK_ARG(b->n_rec > 0, "mj_adj_create_revolve: the integrator needs receivers");
  const int L = nsteps - 1;  // chain x_1 .. x_{N-1}
  const int S = std::min(snapshots, std::max(1, L)) - 1;  // free slots besides the one holding x_1
  MJ_CHECK_ARG((double)L * L * (S + 1) <= 4e8,
               "mj_adj_create_revolve: schedule too large to plan (steps^2 x snapshots above 4e8)");
  std::unique_ptr<mj_adj> a(new mj_adj());
  a->b = b;
  a->N = nsteps;
  a->revolve = true;
  a->snaps = S + 1;
  a->rows = (size_t)b->n_dof * b->S;
  RevolvePlanner pl(L, S);
  pl.out = &a->plan;
  for (int t = S; t >= 1; t--) pl.free_slots.push_back(t);
  pl.reverse(1, nsteps, S, 0);
  // The forward sweep does the plan's leading restores, advances and stores
  // itself (it passes every state in order) and ends on x_{N-1}, the first
  // state visited: the backward sweep starts at the first VISIT.
  a->sweep_stores.push_back({1, 0});
  while (a->first_visit < a->plan.size() && a->plan[a->first_visit].kind != RevAction::VISIT) {
    const RevAction& x = a->plan[a->first_visit++];
    if (x.kind == RevAction::STORE) a->sweep_stores.push_back({x.step, x.slot});
  }
  int cur = -1;
  for (size_t i = a->first_visit; i < a->plan.size(); i++) {
    const RevAction& x = a->plan[i];
    if (x.kind == RevAction::RESTORE) cur = x.step;
    if (x.kind == RevAction::ADVANCE) { a->backward_steps += x.step - cur; cur = x.step; }
  }
  MJ_CUDA(a->slots.alloc(sizeof(float) * a->rows * 2 * a->snaps));
  MJ_CUDA(a->work.alloc(sizeof(float) * a->rows * 3));
  const int rc = adj_common_init(a.get());
  if (rc) return rc;
  *out = a.release();
  return MJ_OK;
}

int mj_revolve_schedule(int nsteps, int snapshots, int capacity, int* actions, int* n_actions,
                        long long* backward_steps) {
  MJ_CHECK_ARG(nsteps >= 2 && snapshots >= 1, "mj_revolve_schedule: nsteps >= 2 and snapshots >= 1");
  const int L = nsteps - 1;
  const int S = std::min(snapshots, std::max(1, L)) - 1;
  MJ_CHECK_ARG((double)L * L * (S + 1) <= 4e8, "mj_revolve_schedule: schedule too large to plan");
  std::vector<RevAction> plan;
  RevolvePlanner pl(L, S);
  pl.out = &plan;
  for (int t = S; t >= 1; t--) pl.free_slots.push_back(t);
  pl.reverse(1, nsteps, S, 0);
  if (n_actions) *n_actions = (int)plan.size();
  if (actions) {
    MJ_CHECK_ARG(capacity >= (int)plan.size(), "mj_revolve_schedule: action buffer too small");
    for (size_t i = 0; i < plan.size(); i++) {
      actions[3 * i] = (int)plan[i].kind;
      actions[3 * i + 1] = plan[i].step;
      actions[3 * i + 2] = plan[i].slot;
    }
  }
  if (backward_steps) *backward_steps = pl.C(L, S);
  return MJ_OK;
}

int mj_adj_info(const mj_adj* a, int* revolve, int* snapshots, long long* forward_steps, size_t* device_bytes) {
  MJ_CHECK_ARG(a, "mj_adj_info: null argument");
  if (revolve) *revolve = a->revolve ? 1 : 0;
  if (snapshots) *snapshots = a->revolve ? a->snaps : a->store_all ? a->N : a->J;
  if (forward_steps) *forward_steps = (long long)a->N + a->backward_steps;
  if (device_bytes) *device_bytes = a->ckpt.bytes + a->seg.bytes + a->slots.bytes + a->work.bytes;
  return MJ_OK;
}

int mj_adj_destroy(mj_adj* a) {
  delete a;
  return MJ_OK;
}

int mj_adj_forward(mj_adj* a, double* traces) {
  MJ_CHECK_ARG(a, "mj_adj_forward: null argument");
  mj_lfb* b = a->b;
  cudaStream_t s = b->stream;
  int rc = mj_lfb_init(b, nullptr, nullptr);  // zero initial conditions
  if (rc) return rc;
  const size_t bytes = sizeof(float) * a->rows;
  float* ck = a->revolve ? a->slots.as<float>() : a->ckpt.as<float>();
  size_t next_store = 0;  // revolve: the next (k, slot) of sweep_stores (increasing k)
  for (int n = 0; n <= a->N; n++) {
    adj_receivers(a, b->cur(), n, s);
    if (n == a->N) break;
    int slot = -1;
    if (!a->revolve && n % a->K == 0) slot = n / a->K;
    if (a->revolve && next_store < a->sweep_stores.size() && a->sweep_stores[next_store].first == n)
      slot = a->sweep_stores[next_store++].second;
    if (slot >= 0) {
      float* dst = ck + (size_t)slot * 2 * a->rows;
      MJ_CUDA(cudaMemcpyAsync(dst, b->cur(), bytes, cudaMemcpyDeviceToDevice, s));
      MJ_CUDA(cudaMemcpyAsync(dst + a->rows, b->next(), bytes, cudaMemcpyDeviceToDevice, s));
    }
    // every state kept: U^0 and U^1 copied here, U^{n+2} (n + 2 < N) written by the one-kernel step itself
    if (a->store_all && (n < 2 || !b->fused))
      MJ_CUDA(cudaMemcpyAsync(a->seg.as<float>() + (size_t)n * a->rows, b->cur(), bytes, cudaMemcpyDeviceToDevice,
                              s));
    if (a->revolve && n == a->N - 1) {  // x_{N-1}, the first state the backward sweep visits
      float* w = a->work.as<float>();
      MJ_CUDA(cudaMemcpyAsync(w, b->cur(), bytes, cudaMemcpyDeviceToDevice, s));
      MJ_CUDA(cudaMemcpyAsync(w + a->rows, b->next(), bytes, cudaMemcpyDeviceToDevice, s));
    }
    if (b->fused) {
      float* copy = a->store_all && n + 2 < a->N ? a->seg.as<float>() + (size_t)(n + 2) * a->rows : nullptr;
      const int rc = lfb_fused_step(b, s, copy);
      if (rc) return rc;
    } else {
      lfb_step_launch(b, b->cur(), b->next(), b->step & 1, s);
    }
    b->cur_is_a = !b->cur_is_a;
    b->step++;
  }
  MJ_CUDA(cudaGetLastError());
  if (b->fused) {
    const int rc = lfb_fused_check(b, s);
    if (rc) return rc;
  }
  if (traces)
    MJ_CUDA(cudaMemcpyAsync(traces, a->traces.ptr, sizeof(double) * b->n_rec * b->S * (a->N + 1),
                            cudaMemcpyDeviceToHost, s));
  MJ_CUDA(cudaStreamSynchronize(s));
  a->have_forward = true;
  return MJ_OK;
}

int mj_adj_backward(mj_adj* a, const double* residual, const double* coef, double* grad) {
  MJ_CHECK_ARG(a && residual && coef && grad, "mj_adj_backward: null argument");
  if (!a->have_forward) {
    set_error("mj_adj_backward: mj_adj_forward must run first");
    return MJ_ERR_STATE;
  }
  mj_lfb* b = a->b;
  mj_op* op = b->op;
  cudaStream_t s = b->stream;
  const int N = a->N, K = a->K, S = b->S;
  const size_t rows = a->rows, bytes = sizeof(float) * rows;
  MJ_CUDA(cudaMemcpyAsync(a->res.ptr, residual, sizeof(double) * b->n_rec * S * (N + 1), cudaMemcpyHostToDevice, s));
  std::vector<double> cf(op->n_elt_pad, 0.0);
  for (int e = 0; e < op->n_elt; e++) cf[e] = coef[e];
  MJ_CUDA(cudaMemcpyAsync(a->coef.ptr, cf.data(), sizeof(double) * cf.size(), cudaMemcpyHostToDevice, s));
  MJ_CUDA(cudaMemsetAsync(a->grad.ptr, 0, sizeof(double) * op->n_elt_pad, s));
  MJ_CUDA(cudaMemsetAsync(a->la.ptr, 0, bytes, s));
  MJ_CUDA(cudaMemsetAsync(a->lb.ptr, 0, bytes, s));
  float* lam1 = a->la.as<float>();  // lambda^{m+1}
  float* lam2 = a->lb.as<float>();  // lambda^{m+2}
  if (a->revolve) {
    // current pair (U^k, U^{k+1}) in w[0], w[1]; w[2] receives U^{k+2}
    float* w[3] = {a->work.as<float>(), a->work.as<float>() + rows, a->work.as<float>() + 2 * rows};
    float* sl = a->slots.as<float>();
    int cur = a->N - 1;  // the forward sweep left x_{N-1} in w[0], w[1]
    for (size_t i = a->first_visit; i < a->plan.size(); i++) {
      const RevAction& x = a->plan[i];
      if (x.kind == RevAction::RESTORE) {
        if (cur == x.step) continue;  // already the current pair
        MJ_CUDA(cudaMemcpyAsync(w[0], sl + (size_t)x.slot * 2 * rows, bytes, cudaMemcpyDeviceToDevice, s));
        MJ_CUDA(cudaMemcpyAsync(w[1], sl + (size_t)x.slot * 2 * rows + rows, bytes, cudaMemcpyDeviceToDevice, s));
        cur = x.step;
      } else if (x.kind == RevAction::ADVANCE) {
        for (; cur < x.step; cur++) {
          const int rc = adj_forward_step(a, w[0], w[1], w[2], cur, s);
          if (rc) return rc;
          float* t = w[0];
          w[0] = w[1]; w[1] = w[2]; w[2] = t;
        }
      } else if (x.kind == RevAction::STORE) {
        MJ_CUDA(cudaMemcpyAsync(sl + (size_t)x.slot * 2 * rows, w[0], bytes, cudaMemcpyDeviceToDevice, s));
        MJ_CUDA(cudaMemcpyAsync(sl + (size_t)x.slot * 2 * rows + rows, w[1], bytes, cudaMemcpyDeviceToDevice, s));
      } else {  // VISIT x_k: adjoint step m = k + 1, U^m in w[1]
        const int m = x.step + 1;
        const int rc = adj_visit(a, m < N ? w[1] : nullptr, m, lam1, lam2, s);
        if (rc) return rc;
      }
    }
    adj_term(a, lam1, w[0], s);  // n = 2: lambda^2 and U^1 (the last visit is x_1)
  }
  float* seg = a->seg.as<float>();
  const float* ck = a->ckpt.as<float>();
  for (int j = a->revolve ? -1 : a->J - 1; j >= 0; j--) {
    const int n0 = j * K, n1 = std::min(n0 + K, N);
    // replay U^{n0} .. U^{n1-1} of the segment from its checkpoint (kept by
    // the forward sweep when every state is stored)
    if (!a->store_all) {
      MJ_CUDA(cudaMemcpyAsync(seg, ck + (size_t)j * 2 * rows, bytes, cudaMemcpyDeviceToDevice, s));
      if (n1 - n0 >= 2)
        MJ_CUDA(cudaMemcpyAsync(seg + rows, ck + (size_t)j * 2 * rows + rows, bytes, cudaMemcpyDeviceToDevice, s));
    }
    for (int n = n0; !a->store_all && n + 2 <= n1 - 1; n++) {
      int rc = adj_forward_step(a, seg + (size_t)(n - n0) * rows, seg + (size_t)(n + 1 - n0) * rows,
                                seg + (size_t)(n + 2 - n0) * rows, n, s);
      if (rc) return rc;
    }
    // adjoint steps m = n1 .. lo with the gradient terms n = n1 .. lo + 1
    // (U^{n1} was the next segment's first state: its term n1 + 1 is done),
    // then the term n = lo with lambda^lo and U^{lo-1}
    const int lo = std::max(n0 + 1, 2);
    for (int m = n1; m >= lo; m--) {
      const int rc = adj_visit(a, m < n1 ? seg + (size_t)(m - n0) * rows : nullptr, m, lam1, lam2, s);
      if (rc) return rc;
    }
    adj_term(a, lam1, seg + (size_t)(lo - 1 - n0) * rows, s);
  }
  if (b->fused) {
    const int rc = lfb_fused_check(b, s);
    if (rc) return rc;
  }
  std::vector<double> g(op->n_elt_pad);
  MJ_CUDA(cudaMemcpyAsync(g.data(), a->grad.ptr, sizeof(double) * g.size(), cudaMemcpyDeviceToHost, s));
  {
    const int rc = take_kernel_error(op->err.ptr, s, "mj_adj_backward");
    if (rc) return rc;
  }
  for (int e = 0; e < op->n_elt; e++) grad[e] = g[e];
  return MJ_OK;
}

}  // extern "C"
