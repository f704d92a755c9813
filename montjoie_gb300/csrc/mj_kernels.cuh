// Device kernels of the matrix-free Q_r hexahedral stiffness operator and the
// leap-frog update (sm_103a).
//
// Data layout in HBM ("tile layout").  Elements are grouped in tiles of E
// consecutive elements; one CTA processes one tile at a time with E*n*n
// threads, thread (el, j, i) owning the line of n points (i, j, k=0..n-1) of
// element el.  A tile holds TQ = E*n^3 points, stored with a stride TS =
// TQ rounded up to 4 so each tile block is 16-byte aligned; inside a tile,
// point (el, i, j, k) sits at p = (k*E + el)*n*n + j*n + i:
//   nodle_t[tile*TS + p]                (int32 global dof)
//   fac_t  [(tile*6 + c)*TS + p]        (c = xx,xy,xz,yy,yz,zz)
//   R      [tile*TS + p]                (element-local A*u)
// The global result is gathered per dof from R through a CSR incidence list
// (owner computes: deterministic, no atomics).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace mj {

constexpr int kMaxNK = 9;  // largest n = r + 1 of the kernels

using ::uint32_t;
using ::uint64_t;

// Derivative matrices g[a*N + b] = phi_a'(x_b) of every order, in constant
// memory (one slot per n = r+1 and precision, written when an operator of
// that order is created): entries picked by unrolled loop indices become
// constant-bank operands, rows picked by thread index use the constant cache.
__constant__ double c_gmat64[kMaxNK + 1][kMaxNK * kMaxNK];
__constant__ float c_gmat32[kMaxNK + 1][kMaxNK * kMaxNK];

template <typename Real>
struct GConst;
template <>
struct GConst<double> {
  __device__ static const double* get(int n) { return c_gmat64[n]; }
};
template <>
struct GConst<float> {
  __device__ static const float* get(int n) { return c_gmat32[n]; }
};

// ---------------------------------------------------------------------------
// Bulk-copy (TMA) and mbarrier helpers.  Every wait is bounded: after
// kSpinLimit unsuccessful polls the waiter gives up and the kernel reports
// the timeout through an error flag instead of hanging.
// ---------------------------------------------------------------------------
constexpr long kSpinLimit = 1L << 22;

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
}

// 1-D bulk copy global -> shared, completion counted on `bar` (16-byte aligned
// addresses, size a multiple of 16).
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity) {
  for (long it = 0; it < kSpinLimit; ++it)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

// Padded tile stride: points per tile rounded up to 4 elements, so every
// per-tile block of int32 / float / double starts on a 16-byte boundary.
__host__ __device__ constexpr int tile_stride(int tq) { return (tq + 3) / 4 * 4; }

// ---------------------------------------------------------------------------
// K1: element-local stiffness product, sum-factorised.
//
// Per element (MltAdd_ElementH1_Scalar, ProdMatVectScalarH1.cxx:256-668):
//   u(i,j,k)  = x[Nodle(e, num(i,j,k))]                        gather
//   gx(l,m,p) = sum_a G[a][l] u(a,m,p)   (gy, gz likewise)      Rh^T
//   v = B(l,m,p) (gx,gy,gz)                                    geometry
//   Y(i,j,k)  = sum_a G[i][a] vx(a,j,k) + G[j][a] vy(i,a,k) + G[k][a] vz(i,j,a)   Rh
//   R = Y                                                      (scatter: K2)
// The z contractions run in registers (each thread owns a z-line); the x and
// y contractions read the element's values from shared memory.
//
// Staging: a persistent CTA walks its tiles; the factors and connectivity of
// each tile are one contiguous block each, brought into shared memory by
// 1-D bulk copies (cp.async.bulk, the TMA engine) two tiles ahead of use
// (double buffer, one mbarrier per stage).  The gather of the next tile's
// u values is issued before the divergence of the current tile.
// Shared memory (dynamic): 2 x [6*TS Real factors | TS int nodle] + 3 x TQ Real
// work arrays + 2 mbarriers.
// ---------------------------------------------------------------------------
template <typename Real, int N, int E>
struct K1Smem {
  static constexpr int NN = N * N;
  static constexpr int TQ = E * N * NN;
  static constexpr int TS = tile_stride(TQ);
  static constexpr size_t fac_bytes = sizeof(Real) * 6 * TS;
  static constexpr size_t nod_bytes = sizeof(int) * TS;
  static constexpr size_t stage_bytes = fac_bytes + nod_bytes;
  static constexpr size_t work_bytes = ((sizeof(Real) * 3 * TQ + 15) / 16) * 16;
  static constexpr size_t total = 2 * stage_bytes + work_bytes + 2 * sizeof(uint64_t);
};

template <typename Real, int N, int E>
__global__ void __launch_bounds__(E* N* N)
    k_local_stiffness(const Real* __restrict__ x, const int* __restrict__ nodle_t,
                      const Real* __restrict__ fac_t, Real* __restrict__ R, int n_tiles,
                      int* __restrict__ err) {
  using L = K1Smem<Real, N, E>;
  const Real* __restrict__ Gm = GConst<Real>::get(N);
  constexpr int NN = L::NN, TQ = L::TQ, TS = L::TS;
  extern __shared__ __align__(128) unsigned char smem[];
  // stage st: factors at smem + st*stage_bytes, connectivity right after them
  auto s_fac = [&](int st) { return reinterpret_cast<Real*>(smem + st * L::stage_bytes); };
  auto s_nod = [&](int st) { return reinterpret_cast<int*>(smem + st * L::stage_bytes + L::fac_bytes); };
  Real* s_u = reinterpret_cast<Real*>(smem + 2 * L::stage_bytes);
  Real* s_vx = s_u + TQ;
  Real* s_vy = s_vx + TQ;
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem + 2 * L::stage_bytes + L::work_bytes);

  const int t = threadIdx.x;
  const int el = t / NN;
  const int ij = t - el * NN;
  const int j = ij / N;
  const int i = ij - j * N;
  Real gci[N], gcj[N], gri[N], grj[N];
#pragma unroll
  for (int a = 0; a < N; a++) {
    gci[a] = Gm[a * N + i];
    gcj[a] = Gm[a * N + j];
    gri[a] = Gm[i * N + a];
    grj[a] = Gm[j * N + a];
  }
  const int s_line_x = (el * N * N + j) * N;  // + k*NN + a   : row (j,k) along x
  const int s_line_y = el * N * NN + i;       // + k*NN + a*N : row (i,k) along y

  if (t == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    fence_mbar_init();
  }
  __syncthreads();
  auto issue = [&](int stage, int tile) {
    if (t == 0 && tile < n_tiles) {
      mbar_expect_tx(&bar[stage], (uint32_t)L::stage_bytes);
      bulk_g2s(s_fac(stage), fac_t + (size_t)tile * 6 * TS, (uint32_t)L::fac_bytes, &bar[stage]);
      bulk_g2s(s_nod(stage), nodle_t + (size_t)tile * TS, (uint32_t)L::nod_bytes, &bar[stage]);
    }
  };
  const int g = gridDim.x;
  int tile = blockIdx.x;
  issue(0, tile);
  issue(1, tile + g);
  uint32_t ph = 0u;  // bit st: parity of the next completion of stage st
  Real u[N];
  if (tile < n_tiles) {
    const bool ok = mbar_wait_bounded(&bar[0], ph & 1u);
    if (__syncthreads_or(!ok)) {
      if (t == 0) atomicExch(err, 1);
      return;
    }
    ph ^= 1u;
    const int* nd = s_nod(0);
#pragma unroll
    for (int k = 0; k < N; k++) u[k] = __ldg(x + nd[k * E * NN + t]);
  }
  for (int it = 0; tile < n_tiles; tile += g, ++it) {
    const int s = it & 1;
#pragma unroll
    for (int k = 0; k < N; k++) s_u[(el * N + k) * NN + ij] = u[k];
    __syncthreads();

    const Real* f = s_fac(s) + t;
    Real vz[N];
#pragma unroll
    for (int k = 0; k < N; k++) {
      Real gx = 0, gy = 0, gz = 0;
#pragma unroll
      for (int a = 0; a < N; a++) {
        gz += Gm[a * N + k] * u[a];
        gx += gci[a] * s_u[s_line_x + k * NN + a];
        gy += gcj[a] * s_u[s_line_y + k * NN + a * N];
      }
      const Real* fk = f + k * E * NN;
      const Real bxx = fk[0], bxy = fk[TS], bxz = fk[2 * TS];
      const Real byy = fk[3 * TS], byz = fk[4 * TS], bzz = fk[5 * TS];
      s_vx[(el * N + k) * NN + ij] = bxx * gx + bxy * gy + bxz * gz;
      s_vy[(el * N + k) * NN + ij] = bxy * gx + byy * gy + byz * gz;
      vz[k] = bxz * gx + byz * gy + bzz * gz;
    }
    __syncthreads();

    // gather of the next tile's u, in flight during the divergence below
    const int nt = tile + g;
    if (nt < n_tiles) {
      const int so = s ^ 1;
      const bool ok = mbar_wait_bounded(&bar[so], (ph >> so) & 1u);
      if (__syncthreads_or(!ok)) {
        if (t == 0) atomicExch(err, 1);
        return;
      }
      ph ^= 1u << so;
      const int* nd = s_nod(so);
#pragma unroll
      for (int k = 0; k < N; k++) u[k] = __ldg(x + nd[k * E * NN + t]);
    }

    Real* Rt = R + (size_t)tile * TS + t;
#pragma unroll
    for (int k = 0; k < N; k++) {
      Real y = 0;
#pragma unroll
      for (int a = 0; a < N; a++) {
        y += gri[a] * s_vx[s_line_x + k * NN + a];
        y += grj[a] * s_vy[s_line_y + k * NN + a * N];
        y += Gm[k * N + a] * vz[a];
      }
      Rt[k * E * NN] = y;
    }
    __syncthreads();  // stage s and the work arrays are free again
    if (t == 0) fence_proxy_async();
    issue(s, tile + 2 * g);
  }
}

// ---------------------------------------------------------------------------
// K2a: y <- beta*y + alpha * sum over the incidences of dof i of R  (MltAdd).
// ---------------------------------------------------------------------------
template <typename Real>
__global__ void k_gather_mltadd(const Real* __restrict__ R, const int* __restrict__ ptr,
                                const int* __restrict__ pos, Real alpha, Real beta,
                                Real* __restrict__ y, int n_dof) {
  for (int d = blockIdx.x * blockDim.x + threadIdx.x; d < n_dof; d += gridDim.x * blockDim.x) {
    Real s = 0;
    const int q1 = __ldg(ptr + d + 1);
    for (int q = __ldg(ptr + d); q < q1; q++) s += __ldg(R + __ldg(pos + q));
    y[d] = (beta == Real(0)) ? alpha * s : beta * y[d] + alpha * s;
  }
}

// ---------------------------------------------------------------------------
// K2b: gather + source + leap-frog update, one dof per thread.
//   Ah = -(A U1)_i + p F_i        (ApplyOperatorKh + AddScalarTimeSource)
//   FP64 (EXACT): a = dt2*Ah - D u0;  a += 2 D u1;  u_new = invD a
//                 (ModifiedEquation.cxx:311-333, operation order kept)
//   FP32:         u_new = 2 u1 - u0 + m Ah,  m = dt^2 / D
// Source entries are CSR entries with pos < 0 (slot -pos-1 of src_val), placed
// after the element entries of the dof.  u_new overwrites u0 in place.
// ---------------------------------------------------------------------------
template <typename Real, bool EXACT>
__global__ void k_gather_leapfrog(const Real* __restrict__ R, const int* __restrict__ ptr,
                                  const int* __restrict__ pos, const Real* __restrict__ src_val,
                                  Real pulse, Real* __restrict__ u0, const Real* __restrict__ u1,
                                  const Real* __restrict__ mass, const Real* __restrict__ minv,
                                  Real dt2, int n_dof) {
  for (int d = blockIdx.x * blockDim.x + threadIdx.x; d < n_dof; d += gridDim.x * blockDim.x) {
    Real s = 0;
    const int q1 = __ldg(ptr + d + 1);
    for (int q = __ldg(ptr + d); q < q1; q++) {
      const int p = __ldg(pos + q);
      s += (p >= 0) ? __ldg(R + p) : -pulse * __ldg(src_val + (-p - 1));
    }
    const Real ah = -s;
    if (EXACT) {
      const Real Dd = __ldg(mass + d);
      Real a = dt2 * ah - Dd * u0[d];
      a += Real(2) * Dd * __ldg(u1 + d);
      u0[d] = a * __ldg(minv + d);
    } else {
      u0[d] = Real(2) * __ldg(u1 + d) - u0[d] + __ldg(minv + d) * ah;
    }
  }
}

// First step U1 = U0 + dt*(du0 + dt/2 * invD*(-A U0))   (SetInitialConditionS)
template <typename Real>
__global__ void k_gather_init(const Real* __restrict__ R, const int* __restrict__ ptr,
                              const int* __restrict__ pos, const Real* __restrict__ u0,
                              const Real* __restrict__ du0, const double* __restrict__ inv_mass,
                              double dt, Real* __restrict__ u1, int n_dof) {
  for (int d = blockIdx.x * blockDim.x + threadIdx.x; d < n_dof; d += gridDim.x * blockDim.x) {
    Real s = 0;
    const int q1 = __ldg(ptr + d + 1);
    for (int q = __ldg(ptr + d); q < q1; q++) {
      const int p = __ldg(pos + q);
      if (p >= 0) s += __ldg(R + p);
    }
    double v = double(-s) * inv_mass[d];
    v *= 0.5 * dt;
    v += du0 ? double(du0[d]) : 0.0;
    v *= dt;
    u1[d] = Real(v + double(u0[d]));
  }
}

// ---------------------------------------------------------------------------
// K3: weighted norm sum_i M_i u_i^2 in FP64 (GetNormeSolution,
// VarInstationary.cxx:2696-2745, with M_i the J*w summed over the points on
// dof i).  Two passes, fixed summation order (deterministic).
// ---------------------------------------------------------------------------
template <typename Real>
__global__ void k_norm_partial(const Real* __restrict__ u, const double* __restrict__ w, int n,
                               double* __restrict__ partial) {
  __shared__ double sh[32];
  double acc = 0.0;
  for (int d = blockIdx.x * blockDim.x + threadIdx.x; d < n; d += gridDim.x * blockDim.x) {
    const double v = double(u[d]);
    acc += w[d] * v * v;
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x < 32) {
    acc = (threadIdx.x < (blockDim.x >> 5)) ? sh[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if (threadIdx.x == 0) partial[blockIdx.x] = acc;
  }
}

__global__ void k_norm_final(const double* __restrict__ partial, int nparts, double* __restrict__ out,
                             int* __restrict__ nonfinite_flag);

// ---------------------------------------------------------------------------
// K6: receiver traces r_k = sum_t W[k][t] u[idx[k][t]], one warp per receiver.
// ---------------------------------------------------------------------------
template <typename Real>
__global__ void k_receivers(const Real* __restrict__ u, const int* __restrict__ idx,
                            const double* __restrict__ w, int n_rec, int n_w,
                            double* __restrict__ out, int stride, int col) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= n_rec) return;
  double acc = 0.0;
  for (int t = lane; t < n_w; t += 32) acc += w[(size_t)warp * n_w + t] * double(u[idx[(size_t)warp * n_w + t]]);
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if (lane == 0) out[(size_t)warp * stride + col] = acc;
}

}  // namespace mj
