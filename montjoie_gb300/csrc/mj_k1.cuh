// Element kernels (K1) of the matrix-free Q_r hexahedral stiffness operator
// (sm_103a): single right-hand side and many right-hand sides.
//
// Data layout in HBM ("element-major").  Every element owns Qp = n^3 rounded
// up to 4 consecutive slots; point (i,j,k) of element e (i along x) is slot
// p = (k*n + j)*n + i:
//   nodle_e[e*Qp + p]            int32 global dof
//   fac_e  [(e*6 + c)*Qp + p]    the six factors (c = xx,xy,xz,yy,yz,zz)
//   slot_e [e*Qp + p]            where the element kernel writes that point's
//                                result: its position q in the dof-ordered
//                                incidence list (CSR), so R[ptr[d] .. ptr[d+1])
//                                holds the contributions to dof d
//   R      [q]                   element-local A*u (single RHS)
//   R      [q*S + s]             element-local A*u (S right-hand sides)
// The element count is padded to a multiple of 240 with empty elements
// (Nodle 0, factors 0), so every tile size E that divides 240 covers the mesh
// with whole tiles and E can be chosen at run time (the autotuner does).
// A tile of E consecutive elements is one contiguous block per array, so it
// is brought into shared memory by one 1-D bulk copy per array.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "mj_wait.cuh"

namespace mj {

using ::uint32_t;
using ::uint64_t;

constexpr int kMaxNK = 9;  // largest n = r + 1 of the kernels

// Derivative matrices g[a*n + b] = phi_a'(x_b) of every order in constant
// memory (one slot per n and precision; each translation unit that launches
// element kernels keeps its own copy, written at operator creation).
static __constant__ double c_gmat64[kMaxNK + 1][kMaxNK * kMaxNK];
static __constant__ float c_gmat32[kMaxNK + 1][kMaxNK * kMaxNK];

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
// Bulk-copy (TMA) and mbarrier helpers.  Every wait is bounded: after LIMIT
// unsuccessful polls (kSpinLimit; 0 in the test instances) the waiter gives
// up and the kernel reports the timeout through an error flag instead of
// hanging.  Before returning, the CTA drains the copies it still has in
// flight (mbar_wait_drain, always with the full kSpinLimit) so that no copy
// lands in shared memory after the CTA has exited.
// ---------------------------------------------------------------------------

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// Orders this thread's generic-proxy global accesses with async-proxy (bulk
// copy) accesses: global data written by plain stores and read back by bulk
// copies in the same kernel (after a grid barrier) needs it on both sides.
__device__ __forceinline__ void fence_proxy_async_global() {
  asm volatile("fence.proxy.async.global;" ::: "memory");
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

// L2 eviction priority for data a launch reads exactly once (factors,
// connectivity, incidence slots, the streamed vectors of the gathers): evict
// first, so that the state vector gathered by the element kernel, and written
// by the previous step's gather, stays in L2.
__device__ __forceinline__ uint64_t l2_evict_first_policy() {
  uint64_t pol;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
  return pol;
}

// bulk_g2s with an L2 cache policy (l2_evict_first_policy).
__device__ __forceinline__ void bulk_g2s_hint(void* dst, const void* src, uint32_t bytes, uint64_t* bar,
                                              uint64_t pol) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], %2, [%3], %4;" ::
          "r"(smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar)), "l"(pol)
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

template <long LIMIT = kSpinLimit>
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity) {
  for (long it = 0; it < LIMIT; ++it)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

// Wait of a CTA that is giving up after a timed-out wait: lets a copy still in
// flight into this stage complete (bounded by the full kSpinLimit).  Out of
// line, so that the rarely taken failure path leaves the kernels' register
// allocation as it is.
static __device__ __noinline__ void mbar_wait_drain(uint64_t* bar, uint32_t parity) {
  for (long it = 0; it < kSpinLimit; ++it)
    if (mbar_try_wait(bar, parity)) return;
}

// Sums of the staged contributions of V dofs of one thread (dof-ordered
// CSR: dof dl[v] owns sR[sp[dl] - q0 .. sp[dl + 1] - q0)).  Each sum is
// 0 + R[qa] + R[qa + 1] + ... in CSR order, the order of the plain gather;
// the first terms of all V dofs are loaded together before the rest, so
// their latencies overlap.
template <int V>
__device__ __forceinline__ void contrib_sums(const int* sp, const float* sR, int q0, const int (&dl)[V],
                                             const bool (&on)[V], float (&s)[V]) {
  int qa[V], qb[V];
  float first[V];
#pragma unroll
  for (int v = 0; v < V; v++) {
    qa[v] = on[v] ? sp[dl[v]] - q0 : 0;
    qb[v] = on[v] ? sp[dl[v] + 1] - q0 : 0;
  }
#pragma unroll
  for (int v = 0; v < V; v++) first[v] = qa[v] < qb[v] ? sR[qa[v]] : 0.f;
#pragma unroll
  for (int v = 0; v < V; v++) {
    s[v] = 0.f;
    if (qa[v] < qb[v]) s[v] += first[v];
    for (int q = qa[v] + 1; q < qb[v]; q++) s[v] += sR[q];
  }
}

// Loads the first RW values of a 16-byte aligned shared-memory line with
// 16-byte loads.
template <int RW>
__device__ __forceinline__ void load_line(const float* p, float (&r)[RW]) {
#pragma unroll
  for (int v = 0; v < RW / 4; v++) {
    const float4 q = reinterpret_cast<const float4*>(p)[v];
    r[4 * v] = q.x; r[4 * v + 1] = q.y; r[4 * v + 2] = q.z; r[4 * v + 3] = q.w;
  }
}
template <int RW>
__device__ __forceinline__ void load_line(const double* p, double (&r)[RW]) {
#pragma unroll
  for (int v = 0; v < RW / 2; v++) {
    const double2 q = reinterpret_cast<const double2*>(p)[v];
    r[2 * v] = q.x; r[2 * v + 1] = q.y;
  }
}

// One row of the factor tensor applied to the gradient, (a, b, c) . (x, y, z),
// in the one order every element kernel uses: fma(c, z, fma(b, y, a * x)).
template <typename Real>
__device__ __forceinline__ Real fac_dot(Real a, Real x, Real b, Real y, Real c, Real z) {
  return fma(c, z, fma(b, y, a * x));
}

// Shared-memory plan of one element kernel: two stages of [factors | Nodle]
// for a tile of E elements, work arrays, two mbarriers.  L = right-hand
// sides handled per pass (1 for the single-RHS kernel).
template <typename Real, int N, int E, int L, bool VEC = false>
struct K1Plan {
  static constexpr int NN = N * N;
  static constexpr int Q = N * NN;
  static constexpr int Qp = elem_slots(N);
  // single RHS: lines of n values padded to RW so a line is a few 16-byte loads
  static constexpr int RW = ((N * (int)sizeof(Real) + 15) / 16) * 16 / (int)sizeof(Real);
  static constexpr size_t fac_bytes = sizeof(Real) * 6 * E * Qp;
  static constexpr size_t nod_bytes = sizeof(int) * E * Qp;
  static constexpr size_t stage_bytes = fac_bytes + nod_bytes;
  static constexpr size_t work_bytes = VEC ? sizeof(Real) * 4 * E * NN * RW
                                          : ((sizeof(Real) * 3 * E * Q * L + 15) / 16) * 16;
  static constexpr size_t total = 2 * stage_bytes + work_bytes + 2 * sizeof(uint64_t);
  static constexpr int threads = E * NN * L;
};

// ---------------------------------------------------------------------------
// K1, single right-hand side: element-local stiffness product, sum-factorised.
//
// Per element (MltAdd_ElementH1_Scalar, ProdMatVectScalarH1.cxx:256-668):
//   u(i,j,k)  = x[Nodle(e, num(i,j,k))]                        gather
//   gx(l,m,p) = sum_a G[a][l] u(a,m,p)   (gy, gz likewise)      Rh^T
//   v = B(l,m,p) (gx,gy,gz)                                    geometry
//   Y(i,j,k)  = sum_a G[i][a] vx(a,j,k) + G[j][a] vy(i,a,k) + G[k][a] vz(i,j,a)   Rh
//   R = Y                                                      (scatter: K2)
// E*n*n threads, thread (el, j, i) owning the z-line (i, j, k = 0..n-1) of
// element el of the tile: z contractions in registers, x and y through shared
// memory.  A persistent CTA walks tiles blockIdx.x, +gridDim.x, ...; the
// factors and Nodle of a tile arrive by bulk copy two tiles ahead (double
// buffer, one mbarrier per stage) and the gather of the next tile's u is in
// flight during the current tile's divergence.
// ---------------------------------------------------------------------------
//
// Two work-array layouts, both timed by the autotuner: VEC = false keeps one
// compact copy of u, vx, vy ([el][k][j][i]; y lines read with stride n);
// VEC = true keeps x-lines and y-lines as separate padded copies so every
// line is read with 16-byte loads (more shared memory, fewer instructions).
template <typename Real, int N, int E, bool VEC = false, long SPIN = kSpinLimit>
__global__ void __launch_bounds__(E* N* N)
    k_local_stiffness(const Real* __restrict__ x, const int* __restrict__ nodle_e,
                      const Real* __restrict__ fac_e, Real* __restrict__ R, const int* __restrict__ slot_e,
                      int n_tiles, int* __restrict__ err) {
  using P = K1Plan<Real, N, E, 1, VEC>;
  constexpr int NN = P::NN, Qp = P::Qp;
  const Real* __restrict__ Gm = GConst<Real>::get(N);
  extern __shared__ __align__(128) unsigned char smem[];
  auto s_fac = [&](int st) { return reinterpret_cast<Real*>(smem + st * P::stage_bytes); };
  auto s_nod = [&](int st) { return reinterpret_cast<int*>(smem + st * P::stage_bytes + P::fac_bytes); };
  // VEC: x-lines (el, k, j) hold i = 0..n-1, y-lines (el, k, i) hold j, each
  // padded to RW; compact: one array per quantity, index (el*n + k)*n*n + j*n + i
  constexpr int RW = VEC ? P::RW : N;
  constexpr int YS = VEC ? 1 : N;   // stride along a y-line
  Real* s_ux = reinterpret_cast<Real*>(smem + 2 * P::stage_bytes);
  Real* s_uy = VEC ? s_ux + E * NN * RW : s_ux;
  Real* s_vx = s_uy + E * NN * RW;
  Real* s_vy = s_vx + E * NN * RW;
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem + 2 * P::stage_bytes + P::work_bytes);

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
  const int lx = (el * N * N + j) * RW;                        // + k*N*RW: x-line (el,k,j); entry i
  const int ly = VEC ? (el * N * N + i) * RW : el * N * NN + i;  // + k*N*RW: y-line (el,k,i); entry j*YS
  const int pe = el * Qp + ij;            // slot (k = 0) of this thread in the tile block

  if (t == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    fence_mbar_init();
  }
  __syncthreads();
  auto issue = [&](int stage, int tile) {
    if (t == 0 && tile < n_tiles) {
      mbar_expect_tx(&bar[stage], (uint32_t)P::stage_bytes);
      const uint64_t pol = l2_evict_first_policy();
      bulk_g2s_hint(s_fac(stage), fac_e + (size_t)tile * E * 6 * Qp, (uint32_t)P::fac_bytes, &bar[stage], pol);
      bulk_g2s_hint(s_nod(stage), nodle_e + (size_t)tile * E * Qp, (uint32_t)P::nod_bytes, &bar[stage], pol);
    }
  };
  const int g = gridDim.x;
  int tile = blockIdx.x;
  issue(0, tile);
  issue(1, tile + g);
  uint32_t ph = 0u;  // bit st: parity of the next completion of stage st
  Real u[N];
  if (tile < n_tiles) {
    const bool ok = mbar_wait_bounded<SPIN>(&bar[0], ph & 1u);
    if (__syncthreads_or(!ok)) {
      if (t == 0) {  // report; both stages may still have a copy in flight
        atomicExch(err, 1);
        mbar_wait_drain(&bar[0], 0u);
        if (tile + g < n_tiles) mbar_wait_drain(&bar[1], 0u);
      }
      return;
    }
    ph ^= 1u;
    const int* nd = s_nod(0) + pe;
#pragma unroll
    for (int k = 0; k < N; k++) u[k] = __ldg(x + nd[k * NN]);
  }
  for (int it = 0; tile < n_tiles; tile += g, ++it) {
    const int s = it & 1;
#pragma unroll
    for (int k = 0; k < N; k++) {
      s_ux[lx + k * N * RW + i] = u[k];
      if (VEC) s_uy[ly + k * N * RW + j] = u[k];
    }
    __syncthreads();

    const Real* f = s_fac(s) + el * 6 * Qp + ij;
    Real vz[N];
#pragma unroll
    for (int k = 0; k < N; k++) {
      Real rx[RW], ry[RW];
      if constexpr (VEC) {
        load_line<RW>(s_ux + lx + k * N * RW, rx);
        load_line<RW>(s_uy + ly + k * N * RW, ry);
      } else {
#pragma unroll
        for (int a = 0; a < N; a++) {
          rx[a] = s_ux[lx + k * N * RW + a];
          ry[a] = s_uy[ly + k * N * RW + a * YS];
        }
      }
      Real gx = 0, gy = 0, gz = 0;
#pragma unroll
      for (int a = 0; a < N; a++) {
        gz += Gm[a * N + k] * u[a];
        gx += gci[a] * rx[a];
        gy += gcj[a] * ry[a];
      }
      const Real* fk = f + k * NN;
      const Real bxx = fk[0], bxy = fk[Qp], bxz = fk[2 * Qp];
      const Real byy = fk[3 * Qp], byz = fk[4 * Qp], bzz = fk[5 * Qp];
      s_vx[lx + k * N * RW + i] = fac_dot(bxx, gx, bxy, gy, bxz, gz);
      s_vy[ly + k * N * RW + j * YS] = fac_dot(bxy, gx, byy, gy, byz, gz);
      vz[k] = fac_dot(bxz, gx, byz, gy, bzz, gz);
    }
    __syncthreads();

    // gather of the next tile's u, in flight during the divergence below
    const int nt = tile + g;
    if (nt < n_tiles) {
      const int so = s ^ 1;
      const bool ok = mbar_wait_bounded<SPIN>(&bar[so], (ph >> so) & 1u);
      if (__syncthreads_or(!ok)) {
        if (t == 0) {  // report; stage so's copy may be in flight (stage s is not reissued yet)
          atomicExch(err, 1);
          mbar_wait_drain(&bar[so], (ph >> so) & 1u);
        }
        return;
      }
      ph ^= 1u << so;
      const int* nd = s_nod(so) + pe;
#pragma unroll
      for (int k = 0; k < N; k++) u[k] = __ldg(x + nd[k * NN]);
    }

    const int* st = slot_e + ((size_t)tile * E + el) * Qp + ij;
#pragma unroll
    for (int k = 0; k < N; k++) {
      Real rx[RW], ry[RW];
      if constexpr (VEC) {
        load_line<RW>(s_vx + lx + k * N * RW, rx);
        load_line<RW>(s_vy + ly + k * N * RW, ry);
      } else {
#pragma unroll
        for (int a = 0; a < N; a++) {
          rx[a] = s_vx[lx + k * N * RW + a];
          ry[a] = s_vy[ly + k * N * RW + a * YS];
        }
      }
      Real y = 0;
#pragma unroll
      for (int a = 0; a < N; a++) {
        y += gri[a] * rx[a];
        y += grj[a] * ry[a];
        y += Gm[k * N + a] * vz[a];
      }
      R[__ldg(st + k * NN)] = y;
    }
    __syncthreads();  // stage s and the work arrays are free again
    if (t == 0) fence_proxy_async();
    issue(s, tile + 2 * g);
  }
}

// ---------------------------------------------------------------------------
// K1, compact layout with ONE factor stage (FS).  The factors of a tile are
// read only by the gradient half of the product, so the next tile's factors
// are copied into the same stage while the current tile's divergence runs;
// Nodle keeps two stages, since the next tile's u is gathered during that
// divergence.  At high order the factors are 6/7 of a stage, so a CTA needs
// little more than half the shared memory of k_local_stiffness and more CTAs
// fit on an SM.  The arithmetic is that of k_local_stiffness (compact), term
// for term, so both give the same bits.
// ---------------------------------------------------------------------------
template <typename Real, int N, int E>
struct K1PlanFS {
  static constexpr int NN = N * N;
  static constexpr int Q = N * NN;
  static constexpr int Qp = elem_slots(N);
  static constexpr size_t fac_bytes = sizeof(Real) * 6 * E * Qp;
  static constexpr size_t nod_bytes = sizeof(int) * E * Qp;
  static constexpr size_t work_bytes = ((sizeof(Real) * 3 * E * Q + 15) / 16) * 16;
  static constexpr size_t total = fac_bytes + 2 * nod_bytes + work_bytes + 3 * sizeof(uint64_t);
  static constexpr int threads = E * NN;
};

template <typename Real, int N, int E, long SPIN = kSpinLimit>
__global__ void __launch_bounds__(E* N* N)
    k_local_stiffness_fs(const Real* __restrict__ x, const int* __restrict__ nodle_e,
                         const Real* __restrict__ fac_e, Real* __restrict__ R, const int* __restrict__ slot_e,
                         int n_tiles, int* __restrict__ err) {
  using P = K1PlanFS<Real, N, E>;
  constexpr int NN = P::NN, Q = P::Q, Qp = P::Qp;
  const Real* __restrict__ Gm = GConst<Real>::get(N);
  extern __shared__ __align__(128) unsigned char smem[];
  Real* s_fac = reinterpret_cast<Real*>(smem);
  auto s_nod = [&](int st) { return reinterpret_cast<int*>(smem + P::fac_bytes + st * P::nod_bytes); };
  // work arrays [el][k][j][i]
  Real* s_u = reinterpret_cast<Real*>(smem + P::fac_bytes + 2 * P::nod_bytes);
  Real* s_vx = s_u + E * Q;
  Real* s_vy = s_vx + E * Q;
  // bar[0], bar[1]: the Nodle stages; bar[2]: the factor stage
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem + P::fac_bytes + 2 * P::nod_bytes + P::work_bytes);

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
  const int lx = el * Q + j * N;  // + k*NN + a: x-line (el, k, j)
  const int ly = el * Q + i;      // + k*NN + a*N: y-line (el, k, i)
  const int pe = el * Qp + ij;

  if (t == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    mbar_init(&bar[2], 1);
    fence_mbar_init();
  }
  __syncthreads();
  auto issue_nod = [&](int st, int tile) {
    if (t == 0 && tile < n_tiles) {
      mbar_expect_tx(&bar[st], (uint32_t)P::nod_bytes);
      bulk_g2s_hint(s_nod(st), nodle_e + (size_t)tile * E * Qp, (uint32_t)P::nod_bytes, &bar[st],
                    l2_evict_first_policy());
    }
  };
  auto issue_fac = [&](int tile) {
    if (t == 0 && tile < n_tiles) {
      mbar_expect_tx(&bar[2], (uint32_t)P::fac_bytes);
      bulk_g2s_hint(s_fac, fac_e + (size_t)tile * E * 6 * Qp, (uint32_t)P::fac_bytes, &bar[2],
                    l2_evict_first_policy());
    }
  };
  const int g = gridDim.x;
  int tile = blockIdx.x;
  issue_nod(0, tile);
  issue_fac(tile);
  issue_nod(1, tile + g);
  uint32_t ph = 0u;  // bits 0, 1: parity of the next completion of Nodle stage 0, 1; bit 2: of the factor stage
  Real u[N];
  if (tile < n_tiles) {
    const bool ok = mbar_wait_bounded<SPIN>(&bar[0], 0u);
    if (__syncthreads_or(!ok)) {
      if (t == 0) {  // report; every copy issued above may still be in flight
        atomicExch(err, 1);
        mbar_wait_drain(&bar[0], 0u);
        mbar_wait_drain(&bar[2], 0u);
        if (tile + g < n_tiles) mbar_wait_drain(&bar[1], 0u);
      }
      return;
    }
    ph ^= 1u;
    const int* nd = s_nod(0) + pe;
#pragma unroll
    for (int k = 0; k < N; k++) u[k] = __ldg(x + nd[k * NN]);
  }
  for (int it = 0; tile < n_tiles; tile += g, ++it) {
    const int s = it & 1;
#pragma unroll
    for (int k = 0; k < N; k++) s_u[lx + k * NN + i] = u[k];
    // this tile's factors (the vote is also the barrier after staging u)
    {
      const bool ok = mbar_wait_bounded<SPIN>(&bar[2], (ph >> 2) & 1u);
      if (__syncthreads_or(!ok)) {
        if (t == 0) {  // report; this tile's factors and the next tile's Nodle may be in flight
          atomicExch(err, 1);
          mbar_wait_drain(&bar[2], (ph >> 2) & 1u);
          if (tile + g < n_tiles) mbar_wait_drain(&bar[s ^ 1], (ph >> (s ^ 1)) & 1u);
        }
        return;
      }
      ph ^= 4u;
    }
    const Real* f = s_fac + el * 6 * Qp + ij;
    Real vz[N];
#pragma unroll
    for (int k = 0; k < N; k++) {
      Real rx[N], ry[N];
#pragma unroll
      for (int a = 0; a < N; a++) {
        rx[a] = s_u[lx + k * NN + a];
        ry[a] = s_u[ly + k * NN + a * N];
      }
      Real gx = 0, gy = 0, gz = 0;
#pragma unroll
      for (int a = 0; a < N; a++) {
        gz += Gm[a * N + k] * u[a];
        gx += gci[a] * rx[a];
        gy += gcj[a] * ry[a];
      }
      const Real* fk = f + k * NN;
      const Real bxx = fk[0], bxy = fk[Qp], bxz = fk[2 * Qp];
      const Real byy = fk[3 * Qp], byz = fk[4 * Qp], bzz = fk[5 * Qp];
      s_vx[lx + k * NN + i] = fac_dot(bxx, gx, bxy, gy, bxz, gz);
      s_vy[ly + k * NN + j * N] = fac_dot(bxy, gx, byy, gy, byz, gz);
      vz[k] = fac_dot(bxz, gx, byz, gy, bzz, gz);
    }
    __syncthreads();  // the factor stage and s_u are free
    if (t == 0) fence_proxy_async();
    issue_fac(tile + g);  // the next tile's factors, during this divergence

    // gather of the next tile's u, in flight during the divergence below
    const int nt = tile + g;
    if (nt < n_tiles) {
      const int so = s ^ 1;
      const bool ok = mbar_wait_bounded<SPIN>(&bar[so], (ph >> so) & 1u);
      if (__syncthreads_or(!ok)) {
        if (t == 0) {  // report; Nodle stage so and the factors just issued may be in flight
          atomicExch(err, 1);
          mbar_wait_drain(&bar[so], (ph >> so) & 1u);
          mbar_wait_drain(&bar[2], (ph >> 2) & 1u);
        }
        return;
      }
      ph ^= 1u << so;
      const int* nd = s_nod(so) + pe;
#pragma unroll
      for (int k = 0; k < N; k++) u[k] = __ldg(x + nd[k * NN]);
    }

    const int* st = slot_e + ((size_t)tile * E + el) * Qp + ij;
#pragma unroll
    for (int k = 0; k < N; k++) {
      Real rx[N], ry[N];
#pragma unroll
      for (int a = 0; a < N; a++) {
        rx[a] = s_vx[lx + k * NN + a];
        ry[a] = s_vy[ly + k * NN + a * N];
      }
      Real y = 0;
#pragma unroll
      for (int a = 0; a < N; a++) {
        y += gri[a] * rx[a];
        y += grj[a] * ry[a];
        y += Gm[k * N + a] * vz[a];
      }
      R[__ldg(st + k * NN)] = y;
    }
    __syncthreads();  // Nodle stage s and the work arrays are free again
    if (t == 0) fence_proxy_async();
    issue_nod(s, tile + 2 * g);
  }
}

// ---------------------------------------------------------------------------
// K1, warp-per-element layout (n*n <= 32, i.e. orders up to 4): element el
// of the tile belongs to warp el, lane (j, i) owning the z-line (i, j, .);
// lanes >= n*n idle.  The compact work arrays of an element are touched by
// its own warp only, so the exchanges of u and of the fluxes need warp
// barriers, not block barriers: one block barrier per tile remains (stage
// release, which also carries the timeout vote of the warps' bounded stage
// waits).  Same operation order as k_local_stiffness.
// ---------------------------------------------------------------------------
// Packed connectivity (PK): an entry of nodle_pk holds the dof in its low
// kPkDofBits bits and, above them, the element's rank among the dof's
// elements, so the result slot is ptr[dof] + rank: the slot array stream is
// replaced by a gather of ptr at the dofs already gathered for u.  Padding
// entries name the spare dof n_dof (slot ptr[n_dof] = the dummy slot).
constexpr int kPkDofBits = 27;
constexpr int kPkMaxRank = (1 << (32 - kPkDofBits)) - 1;  // 31

template <typename Real, int N, int E, long SPIN = kSpinLimit, bool PK = false>
__global__ void __launch_bounds__(E * 32)
    k_local_stiffness_w(const Real* __restrict__ x, const int* __restrict__ nodle_e,
                        const Real* __restrict__ fac_e, Real* __restrict__ R, const int* __restrict__ slot_e,
                        int n_tiles, int* __restrict__ err) {
  // PK: nodle_e is the packed connectivity and slot_e the CSR offsets ptr
  static_assert(N * N <= 32, "one element per warp");
  using P = K1Plan<Real, N, E, 1, false>;
  constexpr int NN = P::NN, Q = P::Q, Qp = P::Qp;
  const Real* __restrict__ Gm = GConst<Real>::get(N);
  extern __shared__ __align__(128) unsigned char smem[];
  auto s_fac = [&](int st) { return reinterpret_cast<Real*>(smem + st * P::stage_bytes); };
  auto s_nod = [&](int st) { return reinterpret_cast<int*>(smem + st * P::stage_bytes + P::fac_bytes); };
  Real* s_u = reinterpret_cast<Real*>(smem + 2 * P::stage_bytes);
  Real* s_vx = s_u + E * Q;
  Real* s_vy = s_vx + E * Q;
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem + 2 * P::stage_bytes + P::work_bytes);

  const int t = threadIdx.x;
  const int el = t >> 5;
  const int lane = t & 31;
  const bool act = lane < NN;
  const int ij = act ? lane : 0;
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
  const int lx = el * Q + j * N;  // + k*NN + a: x-line (el, k, j)
  const int ly = el * Q + i;      // + k*NN + a*N: y-line (el, k, i)
  const int pe = el * Qp + ij;

  if (t == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    fence_mbar_init();
  }
  __syncthreads();
  auto issue = [&](int stage, int tile) {
    if (t == 0 && tile < n_tiles) {
      mbar_expect_tx(&bar[stage], (uint32_t)P::stage_bytes);
      const uint64_t pol = l2_evict_first_policy();
      bulk_g2s_hint(s_fac(stage), fac_e + (size_t)tile * E * 6 * Qp, (uint32_t)P::fac_bytes, &bar[stage], pol);
      bulk_g2s_hint(s_nod(stage), nodle_e + (size_t)tile * E * Qp, (uint32_t)P::nod_bytes, &bar[stage], pol);
    }
  };
  const int g = gridDim.x;
  int tile = blockIdx.x;
  issue(0, tile);
  issue(1, tile + g);
  uint32_t ph = 0u;
  Real u[N];
  int slot[N];  // PK: result slots of the gathered tile's points
  if (tile < n_tiles) {
    const bool ok = mbar_wait_bounded<SPIN>(&bar[0], ph & 1u);
    if (__syncthreads_or(!ok)) {
      if (t == 0) {  // report; both stages may still have a copy in flight
        atomicExch(err, 1);
        mbar_wait_drain(&bar[0], 0u);
        if (tile + g < n_tiles) mbar_wait_drain(&bar[1], 0u);
      }
      return;
    }
    ph ^= 1u;
    const int* nd = s_nod(0) + pe;
    if (act) {
#pragma unroll
      for (int k = 0; k < N; k++) {
        const int w = nd[k * NN];
        const int d = PK ? (w & ((1 << kPkDofBits) - 1)) : w;
        u[k] = __ldg(x + d);
        if constexpr (PK) slot[k] = __ldg(slot_e + d) + (int)((unsigned)w >> kPkDofBits);
      }
    }
  }
  for (int it = 0; tile < n_tiles; tile += g, ++it) {
    const int s = it & 1;
    if (act) {
#pragma unroll
      for (int k = 0; k < N; k++) s_u[lx + k * NN + i] = u[k];
    }
    __syncwarp();
    const Real* f = s_fac(s) + el * 6 * Qp + ij;
    Real vz[N];
    if (act) {
#pragma unroll
      for (int k = 0; k < N; k++) {
        Real rx[N], ry[N];
#pragma unroll
        for (int a = 0; a < N; a++) {
          rx[a] = s_u[lx + k * NN + a];
          ry[a] = s_u[ly + k * NN + a * N];
        }
        Real gx = 0, gy = 0, gz = 0;
#pragma unroll
        for (int a = 0; a < N; a++) {
          gz += Gm[a * N + k] * u[a];
          gx += gci[a] * rx[a];
          gy += gcj[a] * ry[a];
        }
        const Real* fk = f + k * NN;
        const Real bxx = fk[0], bxy = fk[Qp], bxz = fk[2 * Qp];
        const Real byy = fk[3 * Qp], byz = fk[4 * Qp], bzz = fk[5 * Qp];
        s_vx[lx + k * NN + i] = fac_dot(bxx, gx, bxy, gy, bxz, gz);
        s_vy[ly + k * NN + j * N] = fac_dot(bxy, gx, byy, gy, byz, gz);
        vz[k] = fac_dot(bxz, gx, byz, gy, bzz, gz);
      }
    }
    __syncwarp();
    // next tile's stage (every warp waits for it itself) and u gather, in
    // flight during the divergence
    const int nt = tile + g;
    bool bad = false;
    int nslot[N];  // PK: the next tile's result slots
    if (nt < n_tiles) {
      const int so = s ^ 1;
      const bool ok = mbar_wait_bounded<SPIN>(&bar[so], (ph >> so) & 1u);
      bad = __any_sync(0xffffffffu, !ok);
      ph ^= 1u << so;
      if (!bad && act) {
        const int* nd = s_nod(so) + pe;
#pragma unroll
        for (int k = 0; k < N; k++) {
          const int w = nd[k * NN];
          const int d = PK ? (w & ((1 << kPkDofBits) - 1)) : w;
          u[k] = __ldg(x + d);
          if constexpr (PK) nslot[k] = __ldg(slot_e + d) + (int)((unsigned)w >> kPkDofBits);
        }
      }
    }
    if (act) {
      const int* st = slot_e + ((size_t)tile * E + el) * Qp + ij;
#pragma unroll
      for (int k = 0; k < N; k++) {
        Real y = 0;
#pragma unroll
        for (int a = 0; a < N; a++) {
          y += gri[a] * s_vx[lx + k * NN + a];
          y += grj[a] * s_vy[ly + k * NN + a * N];
          y += Gm[k * N + a] * vz[a];
        }
        if constexpr (PK) R[slot[k]] = y;
        else R[__ldg(st + k * NN)] = y;
      }
    }
    if constexpr (PK) {
#pragma unroll
      for (int k = 0; k < N; k++) slot[k] = nslot[k];
    }
    if (__syncthreads_or(bad)) {  // stage s and the work arrays are free; any wait timed out?
      if (t == 0) {  // report; stage s^1's copy may be in flight (parity before the flip above)
        atomicExch(err, 1);
        mbar_wait_drain(&bar[s ^ 1], ((ph >> (s ^ 1)) & 1u) ^ 1u);
      }
      return;
    }
    if (t == 0) fence_proxy_async();
    issue(s, tile + 2 * g);
  }
}

// ---------------------------------------------------------------------------
// K1, many right-hand sides (FP32 state [dof][S], S a multiple of L):
// the same element product for S independent right-hand sides sharing the
// mesh.  L lanes (consecutive threads) carry L right-hand sides of one
// z-line, so every gather of a dof row and every write of R moves L
// contiguous values; the factors and Nodle of a tile are staged once and
// reused for all S/L passes.  E*n*n*L threads.
// ENERGY variant (adjoint gradient): instead of writing R, each element
// accumulates gacc[e] += coef[e] * sum_s sum_q lam[dof_q][s] (A_e x_s)_q,
// i.e. lam^T A_e x summed over the right-hand sides, in FP64 (one CTA owns
// an element per launch, so the update needs no atomics in global memory).
// The sum has one order whatever E and L, so every tuned variant gives the
// same bits: each (source s, z-line q) sums its points in k order (FP32
// FMAs) into shared memory (E*S*NN floats past the plan's bytes, see
// k1_rhs_energy_smem); after the passes, lane l of warp el adds each source
// s = l, l+32, ...: its z-lines q = 0..NN-1 in order in FP32 (FP64 adds on
// the GB300's narrow FP64 pipe cost more than the element's other work),
// then that sum into an FP64 accumulator; a fixed shuffle tree adds the lanes.
// ---------------------------------------------------------------------------
template <int N, int E, int L, bool ENERGY = false>
__global__ void __launch_bounds__(E* N* N* L)
    k_local_stiffness_rhs(const float* __restrict__ x, const int* __restrict__ nodle_e,
                          const float* __restrict__ fac_e, float* __restrict__ R, const int* __restrict__ slot_e,
                          int n_tiles, int S, int* __restrict__ err, const float* __restrict__ lam = nullptr,
                          double* __restrict__ gacc = nullptr, const double* __restrict__ coef = nullptr) {
  using P = K1Plan<float, N, E, L>;
  constexpr int NN = P::NN, Qp = P::Qp;
  const float* __restrict__ Gm = GConst<float>::get(N);
  extern __shared__ __align__(128) unsigned char smem[];
  auto s_fac = [&](int st) { return reinterpret_cast<float*>(smem + st * P::stage_bytes); };
  auto s_nod = [&](int st) { return reinterpret_cast<int*>(smem + st * P::stage_bytes + P::fac_bytes); };
  float* s_u = reinterpret_cast<float*>(smem + 2 * P::stage_bytes);
  float* s_vx = s_u + E * N * NN * L;
  float* s_vy = s_vx + E * N * NN * L;
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem + 2 * P::stage_bytes + P::work_bytes);

  const int lane = threadIdx.x % L;
  const int w = threadIdx.x / L;
  const int el = w / NN;
  const int ij = w - el * NN;
  const int j = ij / N;
  const int i = ij - j * N;
  float gci[N], gcj[N], gri[N], grj[N];
#pragma unroll
  for (int a = 0; a < N; a++) {
    gci[a] = Gm[a * N + i];
    gcj[a] = Gm[a * N + j];
    gri[a] = Gm[i * N + a];
    grj[a] = Gm[j * N + a];
  }
  // work arrays: value (el, k, j, i) of lane l at ((el*N + k)*NN + j*N + i)*L + l
  const int s_base = el * N * NN;
  const int s_line_x = s_base + j * N;
  const int s_line_y = s_base + i;
  const int pe = el * Qp + ij;

  if (threadIdx.x == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    fence_mbar_init();
  }
  __syncthreads();
  auto issue = [&](int stage, int tile) {
    if (threadIdx.x == 0 && tile < n_tiles) {
      mbar_expect_tx(&bar[stage], (uint32_t)P::stage_bytes);
      const uint64_t pol = l2_evict_first_policy();
      bulk_g2s_hint(s_fac(stage), fac_e + (size_t)tile * E * 6 * Qp, (uint32_t)P::fac_bytes, &bar[stage], pol);
      bulk_g2s_hint(s_nod(stage), nodle_e + (size_t)tile * E * Qp, (uint32_t)P::nod_bytes, &bar[stage], pol);
    }
  };
  const int g = gridDim.x;
  int tile = blockIdx.x;
  issue(0, tile);
  issue(1, tile + g);
  uint32_t ph = 0u;
  const int passes = S / L;
  float* s_ez = reinterpret_cast<float*>(smem + P::total);  // ENERGY: [el][source][z-line]
  for (int it = 0; tile < n_tiles; tile += g, ++it) {
    const int s = it & 1;
    const bool ok = mbar_wait_bounded(&bar[s], (ph >> s) & 1u);
    if (__syncthreads_or(!ok)) {
      if (threadIdx.x == 0) {  // report; stage s and, if issued, stage s^1 may have copies in flight
        atomicExch(err, 1);
        mbar_wait_drain(&bar[s], (ph >> s) & 1u);
        if (tile + g < n_tiles) mbar_wait_drain(&bar[s ^ 1], (ph >> (s ^ 1)) & 1u);
      }
      return;
    }
    ph ^= 1u << s;
    const int* nd = s_nod(s) + pe;
    const float* f = s_fac(s) + el * 6 * Qp + ij;
    int dofs[N];
#pragma unroll
    for (int k = 0; k < N; k++) dofs[k] = nd[k * NN];
    for (int pass = 0; pass < passes; ++pass) {
      const int col = pass * L + lane;
      float u[N];
#pragma unroll
      for (int k = 0; k < N; k++) {
        u[k] = __ldg(x + (size_t)dofs[k] * S + col);
        s_u[(s_base + k * NN + ij) * L + lane] = u[k];
      }
      __syncthreads();
      float vz[N];
#pragma unroll
      for (int k = 0; k < N; k++) {
        // explicit FMAs in the order of k_rhs_step, so both forms round alike
        float gx = 0, gy = 0, gz = 0;
#pragma unroll
        for (int a = 0; a < N; a++) {
          gz = fmaf(Gm[a * N + k], u[a], gz);
          gx = fmaf(gci[a], s_u[(s_line_x + k * NN + a) * L + lane], gx);
          gy = fmaf(gcj[a], s_u[(s_line_y + k * NN + a * N) * L + lane], gy);
        }
        const float* fk = f + k * NN;
        const float bxx = fk[0], bxy = fk[Qp], bxz = fk[2 * Qp];
        const float byy = fk[3 * Qp], byz = fk[4 * Qp], bzz = fk[5 * Qp];
        s_vx[(s_base + k * NN + ij) * L + lane] = fmaf(bxz, gz, fmaf(bxy, gy, bxx * gx));
        s_vy[(s_base + k * NN + ij) * L + lane] = fmaf(byz, gz, fmaf(byy, gy, bxy * gx));
        vz[k] = fmaf(bzz, gz, fmaf(byz, gy, bxz * gx));
      }
      __syncthreads();
      const int* st = slot_e + ((size_t)tile * E + el) * Qp + ij;
      float ez = 0.f;  // ENERGY: this z-line's sum for source col
#pragma unroll
      for (int k = 0; k < N; k++) {
        float y = 0;
#pragma unroll
        for (int a = 0; a < N; a++) {
          y = fmaf(gri[a], s_vx[(s_line_x + k * NN + a) * L + lane], y);
          y = fmaf(grj[a], s_vy[(s_line_y + k * NN + a * N) * L + lane], y);
          y = fmaf(Gm[k * N + a], vz[a], y);
        }
        if (ENERGY) ez = fmaf(y, __ldg(lam + (size_t)dofs[k] * S + col), ez);
        else R[(size_t)__ldg(st + k * NN) * S + col] = y;
      }
      if constexpr (ENERGY) s_ez[((size_t)el * S + col) * NN + ij] = ez;
      __syncthreads();
    }
    if constexpr (ENERGY) {  // E*NN*L >= 32*E threads: warp el sums element el
      const int w = threadIdx.x >> 5, l32 = threadIdx.x & 31;
      if (w < E) {
        double acc = 0.0;
        for (int src = l32; src < S; src += 32) {
          const float* row = s_ez + ((size_t)w * S + src) * NN;
          float zs = 0.f;  // the element's z-lines of this source, in order, in FP32
          for (int q = 0; q < NN; q++) zs += row[q];
          acc += (double)zs;
        }
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
        if (l32 == 0) {
          const size_t e = (size_t)tile * E + w;
          gacc[e] += coef[e] * acc;
        }
      }
    }
    if (threadIdx.x == 0) fence_proxy_async();
    issue(s, tile + 2 * g);
  }
}

}  // namespace mj
