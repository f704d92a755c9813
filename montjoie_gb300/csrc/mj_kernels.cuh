// Per-dof kernels of the operator and the leap-frog (sm_103a): the sum of
// the element-local results R, which the element kernels (mj_k1.cuh) wrote
// in dof order (owner computes: deterministic, no atomics), fused with the
// leap-frog update; the source term; the norm and receiver diagnostics.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "mj_k1.cuh"

namespace mj {

// Sums of the contributions of V dofs d[v] of one thread straight from
// global memory (dof-ordered CSR), each 0 + R[q0] + R[q0 + 1] + ... in CSR
// order; the offsets and the first terms of all V dofs are loaded together
// so their latencies overlap.
template <typename Real, int V>
__device__ __forceinline__ void contrib_sums_global(const Real* __restrict__ R, const int* __restrict__ ptr,
                                                    const int (&d)[V], const bool (&on)[V], Real (&s)[V]) {
  int qa[V], qb[V];
  Real first[V];
#pragma unroll
  for (int v = 0; v < V; v++) {
    qa[v] = on[v] ? __ldg(ptr + d[v]) : 0;
    qb[v] = on[v] ? __ldg(ptr + d[v] + 1) : 0;
  }
#pragma unroll
  for (int v = 0; v < V; v++) first[v] = qa[v] < qb[v] ? __ldg(R + qa[v]) : Real(0);
#pragma unroll
  for (int v = 0; v < V; v++) {
    s[v] = Real(0);
    if (qa[v] < qb[v]) s[v] += first[v];
    for (int q = qa[v] + 1; q < qb[v]; q++) s[v] += __ldg(R + q);
  }
}

// Dofs per thread and pass of the grid-stride gathers below.
constexpr int kGatherV = 4;

// ---------------------------------------------------------------------------
// K2a: y <- beta*y + alpha * sum R[ptr[d] .. ptr[d+1])  (MltAdd).  The element
// kernel wrote every contribution to dof d into that contiguous range, so
// each warp streams one contiguous block of R.
// ---------------------------------------------------------------------------
template <typename Real>
__global__ void k_gather_mltadd(const Real* __restrict__ R, const int* __restrict__ ptr, Real alpha, Real beta,
                                Real* __restrict__ y, int n_dof) {
  constexpr int V = kGatherV;
  for (int base = blockIdx.x * blockDim.x * V; base < n_dof; base += gridDim.x * blockDim.x * V) {
    int dv[V];
    bool on[V];
    Real sv[V];
#pragma unroll
    for (int v = 0; v < V; v++) {
      dv[v] = base + v * blockDim.x + threadIdx.x;
      on[v] = dv[v] < n_dof;
    }
    contrib_sums_global<Real, V>(R, ptr, dv, on, sv);
#pragma unroll
    for (int v = 0; v < V; v++)
      if (on[v]) y[dv[v]] = (beta == Real(0)) ? alpha * sv[v] : beta * y[dv[v]] + alpha * sv[v];
  }
}

// ---------------------------------------------------------------------------
// K2b: gather + leap-frog update, one dof per thread (sources: K2c).
//   Ah = -(A U1)_i                (ApplyOperatorKh)
//   FP64 (EXACT): a = dt2*Ah - D u0;  a += 2 D u1;  u_new = invD a
//                 (ModifiedEquation.cxx:311-333, operation order kept)
//   FP32:         u_new = 2 u1 - u0 + m Ah,  m = dt^2 / D
// u_new overwrites u0 in place.  Block 0 advances the step counter:
// ctr[1-qc] = ctr[qc] + 1 (two counters, so a captured sequence of steps
// needs no host update of the pulse index).
// ---------------------------------------------------------------------------
template <typename Real, bool EXACT>
__global__ void k_gather_leapfrog(const Real* __restrict__ R, const int* __restrict__ ptr, int* __restrict__ ctr,
                                  int qc, Real* __restrict__ u0, const Real* __restrict__ u1,
                                  const Real* __restrict__ mass, const Real* __restrict__ minv, Real dt2, int n_dof) {
  if (blockIdx.x == 0 && threadIdx.x == 0) ctr[1 - qc] = ctr[qc] + 1;
  constexpr int V = kGatherV;
  for (int base = blockIdx.x * blockDim.x * V; base < n_dof; base += gridDim.x * blockDim.x * V) {
    int dv[V];
    bool on[V];
    Real sv[V];
#pragma unroll
    for (int v = 0; v < V; v++) {
      dv[v] = base + v * blockDim.x + threadIdx.x;
      on[v] = dv[v] < n_dof;
    }
    contrib_sums_global<Real, V>(R, ptr, dv, on, sv);
#pragma unroll
    for (int v = 0; v < V; v++) {
      if (!on[v]) continue;
      const int d = dv[v];
      const Real ah = -sv[v];
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
}

// ---------------------------------------------------------------------------
// K2c: source term of the step just taken, added to the new state at the
// source dofs: u[d] += coef_d * p * F_d with coef = dt^2/D (the source enters
// Ah as +p F, AddScalarTimeSource, VarInstationary.cxx:2392-2407).  p is
// pulse[ctr[qc]] (the counter K2b read), no pulse past n_pulse.
// ---------------------------------------------------------------------------
template <typename Real>
__global__ void k_source(const int* __restrict__ idx, const Real* __restrict__ val, int n_src,
                         const double* __restrict__ pulses, int n_pulse, const int* __restrict__ ctr, int qc,
                         const double* __restrict__ inv_mass, double dt2, Real* __restrict__ u) {
  const int step = ctr[qc];
  if (step >= n_pulse) return;
  const double p = pulses[step];
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n_src; t += gridDim.x * blockDim.x) {
    const int d = idx[t];
    u[d] = Real(double(u[d]) + dt2 * inv_mass[d] * p * double(val[t]));
  }
}

// First step U1 = U0 + dt*(du0 + dt/2 * invD*(-A U0))   (SetInitialConditionS)
template <typename Real>
__global__ void k_gather_init(const Real* __restrict__ R, const int* __restrict__ ptr,
                              const Real* __restrict__ u0, const Real* __restrict__ du0,
                              const double* __restrict__ inv_mass, double dt, Real* __restrict__ u1, int n_dof) {
  for (int d = blockIdx.x * blockDim.x + threadIdx.x; d < n_dof; d += gridDim.x * blockDim.x) {
    Real s = 0;
    const int q1 = __ldg(ptr + d + 1);
    for (int q = __ldg(ptr + d); q < q1; q++) s += __ldg(R + q);
    double v = double(-s) * inv_mass[d];
    v *= 0.5 * dt;
    v += du0 ? double(du0[d]) : 0.0;
    v *= dt;
    u1[d] = Real(v + double(u0[d]));
  }
}

// ---------------------------------------------------------------------------
// Order-4 modified-equation leap-frog (ModifiedEquationIterator with order 4,
// MONTJOIE/src/Instationary/ModifiedEquation.cxx:346-408), without damping:
// two element products per step, on U^{n+1} and on Z.  Sources are looked up
// per dof (bit mask + sorted list) inside the gathers.
// ---------------------------------------------------------------------------
__device__ __forceinline__ int sorted_position(const int* __restrict__ idx, int n, int d) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (__ldg(idx + mid) < d) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

template <typename Real>
__device__ __forceinline__ double source_at(const unsigned* __restrict__ mask, const int* __restrict__ sidx,
                                            const Real* __restrict__ sval, int nsrc, int d) {
  if (nsrc == 0 || !((__ldg(mask + (d >> 5)) >> (d & 31)) & 1u)) return 0.0;
  return double(sval[sorted_position(sidx, nsrc, d)]);
}

// First gather of a step, pulse p = pulse[ctr[qc]]:
//   EXACT (FP64): P = (-(A U^{n+1}) + p F) dt^2,  Z = invD P     (w <- P, z <- Z)
//   FP32:         w = -(A U^{n+1}) + p F,         z = (dt^2/D) w

template <typename Real, bool EXACT>
__global__ void k_gather_o4a(const Real* __restrict__ R, const int* __restrict__ ptr, const int* __restrict__ ctr,
                             int qc, const double* __restrict__ pulse, int n_pulse,
                             const unsigned* __restrict__ mask, const int* __restrict__ sidx,
                             const Real* __restrict__ sval, int nsrc, const Real* __restrict__ minv, Real dt2,
                             Real* __restrict__ w, Real* __restrict__ z, int n_dof) {
  const int step = ctr[qc];
  const double p = step < n_pulse ? pulse[step] : 0.0;
  constexpr int V = kGatherV;
  for (int base = blockIdx.x * blockDim.x * V; base < n_dof; base += gridDim.x * blockDim.x * V) {
    int dv[V];
    bool on[V];
    Real sv[V];
#pragma unroll
    for (int v = 0; v < V; v++) {
      dv[v] = base + v * blockDim.x + threadIdx.x;
      on[v] = dv[v] < n_dof;
    }
    contrib_sums_global<Real, V>(R, ptr, dv, on, sv);
#pragma unroll
    for (int v = 0; v < V; v++) {
      if (!on[v]) continue;
      const int d = dv[v];
      Real a = -sv[v];
      if (p != 0.0) {
        const double f = source_at(mask, sidx, sval, nsrc, d);
        if (f != 0.0) a = EXACT ? a + Real(p) * Real(f) : Real(double(a) + p * f);
      }
      if (EXACT) {
        a *= dt2;
        w[d] = a;
        z[d] = a * __ldg(minv + d);
      } else {
        w[d] = a;
        z[d] = __ldg(minv + d) * a;
      }
    }
  }
}

// Second gather and the update written over u0 = U^n, pulse'' p3 = pulse3[ctr[qc]]:
//   Y = -(A Z) + dt^2 p3 F
//   EXACT: a = P + (dt^2/12) Y + 2 D U^{n+1} - D U^n,  U^{n+2} = invD a
//   FP32:  U^{n+2} = 2 U^{n+1} - U^n + (dt^2/D)(w + Y/12)
// Block 0 advances the step counter: ctr[1-qc] = ctr[qc] + 1.
template <typename Real, bool EXACT>
__global__ void k_gather_o4b(const Real* __restrict__ R, const int* __restrict__ ptr, int* __restrict__ ctr, int qc,
                             const double* __restrict__ pulse3, int n_pulse3, const unsigned* __restrict__ mask,
                             const int* __restrict__ sidx, const Real* __restrict__ sval, int nsrc,
                             const Real* __restrict__ w, Real* __restrict__ u0, const Real* __restrict__ u1,
                             const Real* __restrict__ mass, const Real* __restrict__ minv, Real dt2, int n_dof) {
  if (blockIdx.x == 0 && threadIdx.x == 0) ctr[1 - qc] = ctr[qc] + 1;
  const int step = ctr[qc];
  const double p3 = step < n_pulse3 ? pulse3[step] : 0.0;
  constexpr int V = kGatherV;
  for (int base = blockIdx.x * blockDim.x * V; base < n_dof; base += gridDim.x * blockDim.x * V) {
    int dv[V];
    bool on[V];
    Real sv[V];
#pragma unroll
    for (int v = 0; v < V; v++) {
      dv[v] = base + v * blockDim.x + threadIdx.x;
      on[v] = dv[v] < n_dof;
    }
    contrib_sums_global<Real, V>(R, ptr, dv, on, sv);
#pragma unroll
    for (int v = 0; v < V; v++) {
      if (!on[v]) continue;
      const int d = dv[v];
      Real y = -sv[v];
      if (p3 != 0.0) {
        const double f = source_at(mask, sidx, sval, nsrc, d);
        if (f != 0.0) y = EXACT ? y + Real(double(dt2) * p3) * Real(f) : Real(double(y) + double(dt2) * p3 * f);
      }
      if (EXACT) {
        const Real Dd = __ldg(mass + d);
        Real a = __ldg(w + d);
        a += (dt2 / Real(12)) * y;
        a += Real(2) * Dd * __ldg(u1 + d);
        a += -Dd * u0[d];
        u0[d] = a * __ldg(minv + d);
      } else {
        u0[d] = Real(2) * __ldg(u1 + d) - u0[d] + __ldg(minv + d) * (__ldg(w + d) + y * Real(1.0 / 12));
      }
    }
  }
}

// out = invD * (-(A x)): the second and third time derivatives of the
// order-4 start (SetInitialConditionS, ModifiedEquation.cxx:142-157).
template <typename Real>
__global__ void k_gather_scaled(const Real* __restrict__ R, const int* __restrict__ ptr,
                                const double* __restrict__ inv_mass, Real* __restrict__ out, int n_dof) {
  for (int d = blockIdx.x * blockDim.x + threadIdx.x; d < n_dof; d += gridDim.x * blockDim.x) {
    Real s = 0;
    const int q1 = __ldg(ptr + d + 1);
    for (int q = __ldg(ptr + d); q < q1; q++) s += __ldg(R + q);
    out[d] = Real(double(-s) * inv_mass[d]);
  }
}

// U^1 of the order-4 start in the reference's Horner form
// (ModifiedEquation.cxx:159-163): d4 = invD(-(A d2)),
// U^1 = U^0 + dt(du0 + dt(d2/2 + dt(d3/6 + dt d4/24))).
template <typename Real>
__global__ void k_gather_o4_init(const Real* __restrict__ R, const int* __restrict__ ptr,
                                 const double* __restrict__ inv_mass, const Real* __restrict__ u0,
                                 const Real* __restrict__ du0, const Real* __restrict__ d2,
                                 const Real* __restrict__ d3, double dt, Real* __restrict__ u1, int n_dof) {
  for (int d = blockIdx.x * blockDim.x + threadIdx.x; d < n_dof; d += gridDim.x * blockDim.x) {
    Real s = 0;
    const int q1 = __ldg(ptr + d + 1);
    for (int q = __ldg(ptr + d); q < q1; q++) s += __ldg(R + q);
    const double d4 = double(-s) * inv_mass[d];
    double v = d4 * (1.0 / 24);
    v *= dt;
    v += (d3 ? double(d3[d]) : 0.0) * (1.0 / 6);
    v *= dt;
    v += double(d2[d]) * (1.0 / 2);
    v *= dt;
    v += du0 ? double(du0[d]) : 0.0;
    v *= dt;
    v += double(u0[d]);
    u1[d] = Real(v);
  }
}

// ---------------------------------------------------------------------------
// K2s: the FP32 gather + leap-frog update + source as a streaming kernel.
// Persistent CTAs walk chunks of at most kStreamDofs dofs (starting on a
// multiple of 4).  A chunk's u^{n+1}, u^n, dt^2/D, CSR offsets and its
// contiguous range of contributions R[ptr[d0] .. ptr[d1]) arrive by 1-D bulk
// copies (16-byte rounded; every buffer carries spare entries past its end)
// into a ring of kStreamNB shared-memory buffers: the next kStreamNB - 1
// chunks' copies are in flight while one chunk is summed.  Same arithmetic as k_gather_leapfrog<float, false> followed by
// k_source (the source in FP64 after the update), so the states agree bit
// for bit.  Every mbarrier wait is bounded (error flag on timeout).
// ---------------------------------------------------------------------------
// Shape measured at 64^3 Q4 (K2 alone, CUDA events): 256 threads, 2 buffers
// of 12 KB and chunks of up to 512 dofs (8 CTAs per SM) take 0.077 ms against
// 0.094 ms for 2 x 32 KB / 1024 dofs (3 CTAs per SM); deeper rings at fewer
// CTAs per SM were slower still: the summing, not the copies, sets the pace.
constexpr int kStreamThreads = 256;
constexpr int kStreamNB = 2;                              // buffers per CTA
constexpr int kStreamDofs = 512;
constexpr int kStreamBuf = 12288;                         // bytes per chunk buffer
constexpr int kStreamM = 2 * kStreamDofs * 4;             // offsets inside a buffer
constexpr int kStreamP = kStreamM + (kStreamDofs + 4) * 4;
constexpr int kStreamR = kStreamP + (kStreamDofs + 8) * 4;
constexpr int kStreamRCap = (kStreamBuf - kStreamR) / 4;  // R entries one chunk may stage
constexpr int kStreamSmem = kStreamNB * kStreamBuf + 8 * kStreamNB;
static_assert(kStreamM % 16 == 0 && kStreamP % 16 == 0 && kStreamR % 16 == 0 && kStreamBuf % 16 == 0,
              "aligned buffer segments");
static_assert(kStreamDofs % kStreamThreads == 0 && kStreamNB >= 2 && kStreamNB <= 8, "chunk shape");

// Where a diagnostic launch writes: the column of the iterate in the norm
// array and in each receiver's row of the trace array (row stride `stride`);
// nothing is written at columns >= ncols.  Graph replays read it from device
// memory (the column advances by one graph's steps per replay); plain
// launches pass it by value.
struct DiagDev {
  double* norms;
  double* traces;
  int stride, col, ncols;
};

// Norm and receivers of the new iterate, fused into the streaming gather
// (FP32): weights rounded to FP32, one partial per CTA, the finished-CTA
// counter (zero between launches), the non-finite flag, the receivers, and
// where to write: (dd ? *dd : direct), column where.col + col.
struct StreamDiag {
  const float* w32;    // the FP32 norm weights, or NULL: weights = wdt2 / m (norm weights equal to the mass)
  const float* m;      // dt^2/D (k_stream_diag, with w32 == NULL)
  float wdt2;          // dt^2 in FP32 (w32 == NULL), else 0; 0 with w32 == NULL: no norm
  double* partial;
  unsigned* done;
  int* flag;
  const int* rec_idx;
  const double* rec_w;
  int n_rec, n_w;
  const DiagDev* dd;
  DiagDev direct;
  int col;
};

struct StreamChunk {
  int d0, d1, q0, q1;  // dofs [d0, d1); R range [q0, q1) rounded to multiples of 4
  int has_src, pad0, pad1, pad2;
};

// One dof's term of the fused norm, rounded the same way wherever it is
// computed: FP32 w*u, then one FP32 fused multiply-add.
__device__ __forceinline__ float stream_norm_term(float w, float u, float acc) {
  return __fmaf_rn(__fmul_rn(w, u), u, acc);
}

// End of a fused-diagnostics launch over the streaming chunks (grid G):
// block tree of the threads' sums, one partial per CTA; the last CTA to
// finish adds the partials in a fixed order and samples the receivers from
// the finished state u.
__device__ __forceinline__ void stream_diag_finish(double nacc, const StreamDiag& dg, const float* u, int G) {
  __shared__ double sh[kStreamThreads / 32];
  __shared__ bool last;
  const int t = threadIdx.x;
  for (int o = 16; o > 0; o >>= 1) nacc += __shfl_down_sync(0xffffffffu, nacc, o);
  if ((t & 31) == 0) sh[t >> 5] = nacc;
  __syncthreads();  // also: every thread's state writes are done
  if (t < 32) {
    double a = t < kStreamThreads / 32 ? sh[t] : 0.0;
    for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
    if (t == 0) {
      dg.partial[blockIdx.x] = a;
      __threadfence();
      last = atomicAdd(dg.done, 1u) == (unsigned)G - 1u;
    }
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  const DiagDev where = dg.dd ? *dg.dd : dg.direct;
  const int col = where.col + dg.col;
  const int warp = t >> 5, lane = t & 31;
  if (col < where.ncols) {
    if (warp == 0) {
      // lane l adds partials l, l+32, ... in that order; the loads of four
      // of them are issued together so their latencies overlap
      double s = 0.0;
      int q = lane;
      for (; q + 3 * 32 < G; q += 4 * 32) {
        double p[4];
#pragma unroll
        for (int b = 0; b < 4; b++) p[b] = __ldcg(dg.partial + q + b * 32);
#pragma unroll
        for (int b = 0; b < 4; b++) s += p[b];
      }
      for (; q < G; q += 32) s += __ldcg(dg.partial + q);
      for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
      if (lane == 0) {
        if (where.norms) where.norms[col] = s;
        if (!isfinite(s)) *dg.flag = 1;
      }
    }
    if (where.traces)
      for (int r = warp; r < dg.n_rec; r += kStreamThreads / 32) {
        // the same order of terms; indices, then states, loaded two terms at a time
        const int* idx = dg.rec_idx + (size_t)r * dg.n_w;
        const double* wr = dg.rec_w + (size_t)r * dg.n_w;
        double acc = 0.0;
        int q = lane;
        for (; q + 32 < dg.n_w; q += 2 * 32) {
          const int i0 = idx[q], i1 = idx[q + 32];
          const float u0v = __ldcg(u + i0), u1v = __ldcg(u + i1);
          acc += wr[q] * double(u0v);
          acc += wr[q + 32] * double(u1v);
        }
        for (; q < dg.n_w; q += 32) acc += wr[q] * double(__ldcg(u + idx[q]));
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
        if (lane == 0) where.traces[(size_t)r * where.stride + col] = acc;
      }
  }
  if (t == 0) *dg.done = 0u;
}

// DIAG: the norm and the receiver traces of U^{n+2} as well (StreamDiag):
// each thread sums w*u^2 of its dofs in FP32 per chunk and accumulates in
// FP64, then a block tree gives one partial per CTA; the last CTA to finish
// adds the partials in a fixed order (deterministic for a given grid) and
// samples the receivers from the finished state.
template <bool DIAG>
__global__ void __launch_bounds__(kStreamThreads, 8)  // 8 CTAs per SM: 32 registers at most
    k_gather_leapfrog_stream(const float* __restrict__ R, const int* __restrict__ ptr, int* __restrict__ ctr, int qc,
                             float* __restrict__ u0, const float* __restrict__ u1, const float* __restrict__ m,
                             const StreamChunk* __restrict__ chunks, int n_chunks,
                             const unsigned* __restrict__ mask, const int* __restrict__ sidx,
                             const float* __restrict__ sval, int nsrc, const double* __restrict__ pulse, int n_pulse,
                             const double* __restrict__ inv_mass, double dt2, int* __restrict__ err, StreamDiag dg) {
  extern __shared__ __align__(128) unsigned char smem[];
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem + kStreamNB * kStreamBuf);
  const int t = threadIdx.x, G = gridDim.x;
  if (blockIdx.x == 0 && t == 0) ctr[1 - qc] = ctr[qc] + 1;
  const int step = ctr[qc];
  const bool src_on = nsrc > 0 && step < n_pulse;
  const double p = src_on ? pulse[step] : 0.0;
  auto issue = [&](int c, int b) {
    if (c >= n_chunks) return;
    const StreamChunk ch = chunks[c];
    unsigned char* dst = smem + b * kStreamBuf;
    const uint32_t sb = (uint32_t)(((ch.d1 - ch.d0 + 3) & ~3) * 4);
    const uint32_t pb = (uint32_t)(((ch.d1 - ch.d0 + 1 + 3) & ~3) * 4);
    const uint32_t rb = (uint32_t)((ch.q1 - ch.q0) * 4);
    mbar_expect_tx(&bar[b], 3u * sb + pb + rb);
    const uint64_t pol = l2_evict_first_policy();  // all read once; the new state, stored, stays in L2
    bulk_g2s_hint(dst, u1 + ch.d0, sb, &bar[b], pol);
    bulk_g2s_hint(dst + kStreamDofs * 4, u0 + ch.d0, sb, &bar[b], pol);
    bulk_g2s_hint(dst + kStreamM, m + ch.d0, sb, &bar[b], pol);
    bulk_g2s_hint(dst + kStreamP, ptr + ch.d0, pb, &bar[b], pol);
    bulk_g2s_hint(dst + kStreamR, R + ch.q0, rb, &bar[b], pol);
  };
  if (t == 0) {
    for (int b = 0; b < kStreamNB; b++) mbar_init(&bar[b], 1);
    fence_mbar_init();
    for (int b = 0; b < kStreamNB; b++) issue(blockIdx.x + b * G, b);
  }
  __syncthreads();
  uint32_t ph = 0u;  // bit b: parity of buffer b's next completion
  int b = 0;
  double nacc = 0.0;  // DIAG: this thread's sum of w u^2
  constexpr int V = kStreamDofs / kStreamThreads;
  for (int c = blockIdx.x; c < n_chunks; c += G, b = (b + 1 == kStreamNB ? 0 : b + 1)) {
    const StreamChunk ch = chunks[c];
    const bool ok = mbar_wait_bounded(&bar[b], (ph >> b) & 1u);
    if (__syncthreads_or(!ok)) {
      // report, wait (bounded) for this CTA's copies still in flight, and
      // still take part in the diagnostics' finished-CTA count
      if (t == 0) atomicExch(err, 1);
      for (int i = 0, cb = b; i < kStreamNB; i++, cb = (cb + 1 == kStreamNB ? 0 : cb + 1))
        if (c + i * G < n_chunks) mbar_wait_drain(&bar[cb], (ph >> cb) & 1u);
      break;
    }
    ph ^= 1u << b;
    const unsigned char* buf = smem + b * kStreamBuf;
    const float* su1 = reinterpret_cast<const float*>(buf);
    const float* su0 = su1 + kStreamDofs;
    const float* sm = reinterpret_cast<const float*>(buf + kStreamM);
    const int* sp = reinterpret_cast<const int*>(buf + kStreamP);
    const float* sR = reinterpret_cast<const float*>(buf + kStreamR);
    int dls[V];
    bool on[V];
    float sums[V];
#pragma unroll
    for (int v = 0; v < V; v++) {
      dls[v] = v * kStreamThreads + t;
      on[v] = ch.d0 + dls[v] < ch.d1;
    }
    contrib_sums<V>(sp, sR, ch.q0, dls, on, sums);
    float wsum = 0.f;
#pragma unroll
    for (int v = 0; v < V; v++) {
      const int dl = dls[v];
      const int d = ch.d0 + dl;
      if (on[v]) {
        const float ah = -sums[v];
        float un = 2.f * su1[dl] - su0[dl] + sm[dl] * ah;
        if (src_on && ch.has_src) {
          const double f = source_at(mask, sidx, sval, nsrc, d);
          if (f != 0.0) un = float(double(un) + dt2 * inv_mass[d] * p * f);
        }
        u0[d] = un;
        if (DIAG && dg.w32) wsum = stream_norm_term(__ldg(dg.w32 + d), un, wsum);
        else if (DIAG && dg.wdt2 != 0.f) wsum = stream_norm_term(__fdiv_rn(dg.wdt2, sm[dl]), un, wsum);
      }
    }
    if (DIAG) nacc += double(wsum);
    __syncthreads();  // buffer b is free
    if (t == 0) {
      fence_proxy_async();
      issue(c + kStreamNB * G, b);
    }
  }
  if constexpr (DIAG) stream_diag_finish(nacc, dg, u0, G);
}

// The order-4 gathers of the FP32 form as streaming kernels, on the chunks,
// buffers and grid of k_gather_leapfrog_stream:
//   MODE 0 (first gather):  w = -(A U^{n+1}) + p F,  z = (dt^2/D) w;
//   MODE 1 (second gather and update, advancing the step counter):
//     U^{n+2} = 2 U^{n+1} - U^n + (dt^2/D)(w + Y/12),  Y = -(A Z) + dt^2 p'' F.
// The same arithmetic as k_gather_o4a / k_gather_o4b<float, false>.
template <int MODE>
__global__ void __launch_bounds__(kStreamThreads, 8)
    k_gather_o4_stream(const float* __restrict__ R, const int* __restrict__ ptr, int* __restrict__ ctr, int qc,
                       const double* __restrict__ pulse, int n_pulse, const unsigned* __restrict__ mask,
                       const int* __restrict__ sidx, const float* __restrict__ sval, int nsrc,
                       float* __restrict__ u0, const float* __restrict__ u1, const float* __restrict__ m,
                       float* __restrict__ w, float* __restrict__ z, const StreamChunk* __restrict__ chunks,
                       int n_chunks, float dt2, int* __restrict__ err) {
  extern __shared__ __align__(128) unsigned char smem[];
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem + kStreamNB * kStreamBuf);
  const int t = threadIdx.x, G = gridDim.x;
  if (MODE == 1 && blockIdx.x == 0 && t == 0) ctr[1 - qc] = ctr[qc] + 1;
  const int step = ctr[qc];
  const double p = step < n_pulse ? pulse[step] : 0.0;
  auto issue = [&](int c, int b) {
    if (c >= n_chunks) return;
    const StreamChunk ch = chunks[c];
    unsigned char* dst = smem + b * kStreamBuf;
    const uint32_t sb = (uint32_t)(((ch.d1 - ch.d0 + 3) & ~3) * 4);
    const uint32_t pb = (uint32_t)(((ch.d1 - ch.d0 + 1 + 3) & ~3) * 4);
    const uint32_t rb = (uint32_t)((ch.q1 - ch.q0) * 4);
    mbar_expect_tx(&bar[b], (MODE == 1 ? 3u : 1u) * sb + pb + rb);
    if (MODE == 1) {
      bulk_g2s(dst, u1 + ch.d0, sb, &bar[b]);
      bulk_g2s(dst + kStreamDofs * 4, u0 + ch.d0, sb, &bar[b]);
    }
    bulk_g2s(dst + kStreamM, m + ch.d0, sb, &bar[b]);
    bulk_g2s(dst + kStreamP, ptr + ch.d0, pb, &bar[b]);
    bulk_g2s(dst + kStreamR, R + ch.q0, rb, &bar[b]);
  };
  if (t == 0) {
    for (int b = 0; b < kStreamNB; b++) mbar_init(&bar[b], 1);
    fence_mbar_init();
    for (int b = 0; b < kStreamNB; b++) issue(blockIdx.x + b * G, b);
  }
  __syncthreads();
  uint32_t ph = 0u;
  int b = 0;
  for (int c = blockIdx.x; c < n_chunks; c += G, b = (b + 1 == kStreamNB ? 0 : b + 1)) {
    const StreamChunk ch = chunks[c];
    const bool ok = mbar_wait_bounded(&bar[b], (ph >> b) & 1u);
    if (__syncthreads_or(!ok)) {
      if (t == 0) atomicExch(err, 1);
      for (int i = 0, cb = b; i < kStreamNB; i++, cb = (cb + 1 == kStreamNB ? 0 : cb + 1))
        if (c + i * G < n_chunks) mbar_wait_drain(&bar[cb], (ph >> cb) & 1u);
      return;
    }
    ph ^= 1u << b;
    const unsigned char* buf = smem + b * kStreamBuf;
    const float* su1 = reinterpret_cast<const float*>(buf);
    const float* su0 = su1 + kStreamDofs;
    const float* sm = reinterpret_cast<const float*>(buf + kStreamM);
    const int* sp = reinterpret_cast<const int*>(buf + kStreamP);
    const float* sR = reinterpret_cast<const float*>(buf + kStreamR);
    constexpr int V = kStreamDofs / kStreamThreads;
    int dls[V];
    bool on[V];
    float sums[V];
#pragma unroll
    for (int v = 0; v < V; v++) {
      dls[v] = v * kStreamThreads + t;
      on[v] = ch.d0 + dls[v] < ch.d1;
    }
    contrib_sums<V>(sp, sR, ch.q0, dls, on, sums);
#pragma unroll
    for (int v = 0; v < V; v++) {
      if (!on[v]) continue;
      const int dl = dls[v];
      const int d = ch.d0 + dl;
      float a = -sums[v];
      if (p != 0.0 && ch.has_src) {
        const double f = source_at(mask, sidx, sval, nsrc, d);
        if (f != 0.0) a = MODE == 0 ? float(double(a) + p * f) : float(double(a) + double(dt2) * p * f);
      }
      if (MODE == 0) {
        w[d] = a;
        z[d] = sm[dl] * a;
      } else {
        u0[d] = 2.f * su1[dl] - su0[dl] + sm[dl] * (__ldg(w + d) + a * float(1.0 / 12));
      }
    }
    __syncthreads();  // buffer b is free
    if (t == 0) {
      fence_proxy_async();
      issue(c + kStreamNB * G, b);
    }
  }
}

// The fused diagnostics of a state u on their own (the iterates a call
// starts from): the same chunks, grid, grouping and reduction as the
// streaming gather's DIAG form, so every column has the same arithmetic.
__global__ void __launch_bounds__(kStreamThreads)
    k_stream_diag(const float* __restrict__ u, const StreamChunk* __restrict__ chunks, int n_chunks, StreamDiag dg) {
  const int t = threadIdx.x, G = gridDim.x;
  constexpr int V = kStreamDofs / kStreamThreads;
  double nacc = 0.0;
  if (dg.w32 || dg.wdt2 != 0.f)
    for (int c = blockIdx.x; c < n_chunks; c += G) {
      const StreamChunk ch = chunks[c];
      float wsum = 0.f;
#pragma unroll
      for (int v = 0; v < V; v++) {
        const int d = ch.d0 + v * kStreamThreads + t;
        if (d < ch.d1) {
          const float w = dg.w32 ? __ldg(dg.w32 + d) : __fdiv_rn(dg.wdt2, __ldg(dg.m + d));
          wsum = stream_norm_term(w, __ldg(u + d), wsum);
        }
      }
      nacc += double(wsum);
    }
  stream_diag_finish(nacc, dg, u, G);
}

// ---------------------------------------------------------------------------
// K3: weighted norm sum_i M_i u_i^2 accumulated in FP64 (GetNormeSolution,
// VarInstationary.cxx:2696-2745, with M_i the J*w summed over the points on
// dof i).  Two passes, fixed summation order (deterministic).
// ---------------------------------------------------------------------------
// Four terms w_i u_i^2 of one thread, summed for the FP64 accumulator:
// FP64 state: every term in FP64 (the plain form's norm history is pinned to
// the reference at 1e-10); FP32 state: the four products and their sum in
// FP32 (relative error ~1e-7, the state's own precision), one FP64 add.
template <typename Real>
__device__ __forceinline__ double norm_group(const double (&w)[4], const Real (&u)[4]);
template <>
__device__ __forceinline__ double norm_group<double>(const double (&w)[4], const double (&u)[4]) {
  return (w[0] * u[0] * u[0] + w[1] * u[1] * u[1]) + (w[2] * u[2] * u[2] + w[3] * u[3] * u[3]);
}
template <>
__device__ __forceinline__ double norm_group<float>(const double (&w)[4], const float (&u)[4]) {
  return double((float(w[0]) * u[0] * u[0] + float(w[1]) * u[1] * u[1]) +
                (float(w[2]) * u[2] * u[2] + float(w[3]) * u[3] * u[3]));
}

// Block `blk` of `nb` (blockDim.x threads) of the norm's first pass: each
// thread groups four strided terms into one FP64 accumulator, then a fixed
// warp and block tree; returns the block's sum in thread 0.  Deterministic
// for a given nb.  w32: for FP32 state, the weights rounded to FP32 once
// (norm_group<float> rounds them so), read in the grouped loop instead of
// the FP64 ones.
template <typename Real>
__device__ __forceinline__ double norm_block_sum(const Real* __restrict__ u, const double* __restrict__ w,
                                                 const float* __restrict__ w32, int n, int blk, int nb) {
  __shared__ double sh[32];
  double acc = 0.0;
  const int stride = nb * blockDim.x;
  int d = blk * blockDim.x + threadIdx.x;
  for (; d + 3 * stride < n; d += 4 * stride) {
    double wv[4];
    Real uv[4];
#pragma unroll
    for (int v = 0; v < 4; v++) {
      wv[v] = w32 ? double(__ldg(w32 + d + v * stride)) : __ldg(w + d + v * stride);
      uv[v] = __ldg(u + d + v * stride);
    }
    acc += norm_group<Real>(wv, uv);
  }
  for (; d < n; d += stride) {
    const double x = double(__ldg(u + d));
    acc += __ldg(w + d) * x * x;
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x < 32) {
    acc = (threadIdx.x < (blockDim.x >> 5)) ? sh[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  }
  return acc;
}

// K3 + K6 in one launch (GetNormeSolution, VarInstationary.cxx:2696-2745,
// and the receiver traces): blocks [0, nb) sum M_i u_i^2, and the last of
// them to finish adds the nb block sums in a fixed order (one warp, lane l
// takes blocks l, l+32, ..., then a shuffle tree), so the value does not
// depend on which block finishes last; blocks [nb, ...) take one receiver
// per warp, r_k = sum_t W[k][t] u[idx[k][t]].  `done` is zero between
// launches.  A non-finite norm sets *flag.
template <typename Real>
__global__ void __launch_bounds__(256)
    k_diag(const Real* __restrict__ u, const double* __restrict__ w, const float* __restrict__ w32, int n, int nb,
           double* __restrict__ partial, unsigned* __restrict__ done, int* __restrict__ flag,
           const int* __restrict__ rec_idx, const double* __restrict__ rec_w, int n_rec, int n_w,
           const DiagDev* __restrict__ dd, DiagDev direct, int k) {
  const DiagDev where = dd ? *dd : direct;
  const int col = where.col + k;
  const bool put = col < where.ncols;
  if ((int)blockIdx.x >= nb) {
    const int warp = (((int)blockIdx.x - nb) * (int)blockDim.x + (int)threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= n_rec) return;
    double acc = 0.0;
    for (int t = lane; t < n_w; t += 32)
      acc += rec_w[(size_t)warp * n_w + t] * double(u[rec_idx[(size_t)warp * n_w + t]]);
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if (lane == 0 && where.traces && put) where.traces[(size_t)warp * where.stride + col] = acc;
    return;
  }
  __shared__ bool last;
  const double b = norm_block_sum<Real>(u, w, w32, n, blockIdx.x, nb);
  if (threadIdx.x == 0) {
    partial[blockIdx.x] = b;
    __threadfence();
    last = atomicAdd(done, 1u) == (unsigned)nb - 1u;
  }
  __syncthreads();
  if (last && threadIdx.x < 32) {
    __threadfence();
    double s = 0.0;
    for (int q = threadIdx.x; q < nb; q += 32) s += __ldcg(partial + q);
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (threadIdx.x == 0) {
      if (where.norms && put) where.norms[col] = s;
      if (!isfinite(s)) *flag = 1;
      *done = 0u;
    }
  }
}

// A graph replay of diagnosed steps ends by moving the column on.
__global__ void k_diag_advance(DiagDev* dd, int steps) { dd->col += steps; }
__global__ void k_diag_set(DiagDev* dd, DiagDev v) { *dd = v; }

}  // namespace mj
