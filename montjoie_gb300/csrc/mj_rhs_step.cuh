// The one-kernel leap-frog step of S right-hand sides on one mesh (FP32):
// parameter blocks, phase-2 buffer layout and the cooperative kernel
// k_rhs_step, shared by the translation unit of the plain step
// (mj_rhs_step.cu) and that of the step which also accumulates the
// adjoint's gradient term (mj_rhs_step_en.cu).  Each unit has its own
// constant-memory copy of the derivative matrix (c_gmat32) and sets it.
#pragma once
#include <cuda_runtime.h>

#include "mj_internal.cuh"
#include "mj_k1.cuh"
#include "mj_sync.cuh"

namespace mj {

struct RsParams {
  const float* fac_e;
  const int* nodle_e;
  const int* slot_e;
  float* R;           // [slot][S]
  const int* ptr;     // CSR offsets (padded)
  float* ua;
  float* ub;
  const float* m;     // dt^2 / D (padded)
  const double* pulse;
  int* ctr;
  const int* src_dof;  // dofs carrying sources, sorted
  const int* src_ptr;  // their entries [src_ptr[i], src_ptr[i+1]) in
  const int* src_rhs;  //   (right-hand side, value) pairs
  const float* src_val;
  float* uout;         // where U^{n+2} goes (nullptr: over U^n)
  float* ucopy;        // a second copy of U^{n+2} (a kept forward state of the adjoint), or nullptr
  // step with the gradient term (EN form): ue = U^m, one state of the
  // forward run; gacc[e] += gcoef[e] * sum_s sum_q ue[dof_q][s] (A_e U^{n+1})_q
  const float* ue;
  double* gacc;
  const double* gcoef;
  int n_src_dof, n_pulse, S, n_tiles;
  unsigned char zmap[kMaxNK * kMaxNK];  // z-line (j*n + i) of each thread slot of an element (rs_zline_order)
};

// Phase-2 work: dofs [d0, d1), contributions R rows [q0, q1).
struct RsChunk {
  int d0, d1, q0, q1, has_src, pad0, pad1, pad2;
};

// Byte layout of a phase-2 buffer for a chunk (all offsets 16-byte aligned):
// u^{n+1} rows | u^n rows | R rows | dt^2/D from d0&~3 | offsets from d0&~3.
struct RsBuf {
  int u1, u0, r, m, p, end;
};
__host__ __device__ __forceinline__ RsBuf rs_buf(int d0, int d1, int q0, int q1, int S) {
  RsBuf b;
  const int D = d1 - d0, da = d0 & ~3;
  b.u1 = 0;
  b.u0 = D * S * 4;
  b.r = 2 * D * S * 4;
  b.m = b.r + (q1 - q0) * S * 4;
  b.p = b.m + (((d1 + 3) & ~3) - da) * 4;
  b.end = b.p + (((d1 + 1 + 3) & ~3) - da) * 4;
  return b;
}

// CTAs per SM the register allocation aims at (smaller CTAs: more of them)
__host__ __device__ constexpr int rs_min_ctas(int T) { return T <= 128 ? 4 : T <= 216 ? 3 : 1; }

// ---- variants: (n, E, LB, V) per order -------------------------------------
#define MJ_RS_VARIANTS(X)                                                                        \
  X(2, 8, 4, 4) X(2, 4, 8, 4) X(2, 16, 2, 4)                                                     \
  X(3, 4, 4, 4) X(3, 2, 8, 4) X(3, 8, 2, 4)                                                      \
  X(4, 2, 4, 4) X(4, 1, 8, 4) X(4, 4, 2, 4)                                                      \
  X(5, 1, 4, 4) X(5, 1, 8, 4) X(5, 2, 4, 4) X(5, 1, 8, 2) X(5, 2, 2, 4)                          \
  X(6, 1, 4, 4) X(6, 1, 4, 2) X(6, 1, 8, 2)                                                      \
  X(7, 1, 2, 4) X(7, 1, 4, 2) X(7, 1, 2, 2)                                                      \
  X(8, 1, 2, 2) X(8, 1, 2, 4) X(8, 1, 4, 2)                                                      \
  X(9, 1, 2, 2) X(9, 1, 1, 4) X(9, 1, 4, 2)

// The EN form of variant (n, E, LB, V) for S right-hand sides
// (mj_rhs_step_en.cu): sets its shared-memory size, *ctas = its CTAs per SM
// (0: it does not fit); launch like the plain form; its own copy of the
// derivative matrix of order n.
int rs_en_prepare(int n, int E, int LB, int V, int S, int* ctas);
int rs_en_launch(int n, int E, int LB, int V, int S, int grid, const RsParams& prm, const RsChunk* chunks,
                 int n_chunks, SyncState* sync, int par, int* err, cudaStream_t s);
int rs_en_set_gmat(int n, const float* g);

namespace {

template <int V>
__device__ __forceinline__ void vload(const float* p, float (&r)[V]) {
  if constexpr (V == 4) {
    const float4 q = *reinterpret_cast<const float4*>(p);
    r[0] = q.x; r[1] = q.y; r[2] = q.z; r[3] = q.w;
  } else if constexpr (V == 2) {
    const float2 q = *reinterpret_cast<const float2*>(p);
    r[0] = q.x; r[1] = q.y;
  } else {
    r[0] = *p;
  }
}

template <int V>
__device__ __forceinline__ void vload_g(const float* p, float (&r)[V]) {
  if constexpr (V == 4) {
    const float4 q = __ldg(reinterpret_cast<const float4*>(p));
    r[0] = q.x; r[1] = q.y; r[2] = q.z; r[3] = q.w;
  } else if constexpr (V == 2) {
    const float2 q = __ldg(reinterpret_cast<const float2*>(p));
    r[0] = q.x; r[1] = q.y;
  } else {
    r[0] = __ldg(p);
  }
}

template <int V>
__device__ __forceinline__ void vstore(float* p, const float (&r)[V]) {
  if constexpr (V == 4) {
    *reinterpret_cast<float4*>(p) = make_float4(r[0], r[1], r[2], r[3]);
  } else if constexpr (V == 2) {
    *reinterpret_cast<float2*>(p) = make_float2(r[0], r[1]);
  } else {
    *p = r[0];
  }
}

// acc[v] = fma(c, x[v], acc[v]) for the V right-hand sides of a thread, two
// at a time by the paired FP32 FMA of sm_100+ (__ffma2_rn: each lane rounds
// as fmaf, so the results are those of V scalar FMAs with half the issued
// instructions); mul: acc[v] = c * x[v].
template <int V>
__device__ __forceinline__ void fma_v(float (&acc)[V], float c, const float (&x)[V]) {
  if constexpr (V % 2 == 0) {
    const float2 c2 = make_float2(c, c);
#pragma unroll
    for (int v = 0; v < V; v += 2) {
      const float2 r = __ffma2_rn(c2, make_float2(x[v], x[v + 1]), make_float2(acc[v], acc[v + 1]));
      acc[v] = r.x;
      acc[v + 1] = r.y;
    }
  } else {
#pragma unroll
    for (int v = 0; v < V; v++) acc[v] = fmaf(c, x[v], acc[v]);
  }
}
template <int V>
__device__ __forceinline__ void mul_v(float (&acc)[V], float c, const float (&x)[V]) {
  if constexpr (V % 2 == 0) {
    const float2 c2 = make_float2(c, c);
#pragma unroll
    for (int v = 0; v < V; v += 2) {
      const float2 r = __fmul2_rn(c2, make_float2(x[v], x[v + 1]));
      acc[v] = r.x;
      acc[v + 1] = r.y;
    }
  } else {
#pragma unroll
    for (int v = 0; v < V; v++) acc[v] = c * x[v];
  }
}


template <int N, int E, int LB, int V>
struct RsPlan {
  static constexpr int NN = N * N, Q = N * NN, Qp = elem_slots(N);
  static constexpr int T = E * NN * LB;  // threads
  static constexpr int W = LB * V;       // right-hand sides per pass
  static constexpr int kStage = (E * Qp * 28 + 127) / 128 * 128;  // factors + Nodle of a tile
  static constexpr int kWork = (E * Q * W + 3) / 4 * 4;            // floats per work array
  static constexpr int kArea = 2 * kStage + 3 * kWork * 4;
  static constexpr int kSmem = kArea + 32;                         // + 4 mbarriers
  static constexpr int kHalf = kArea / 2 / 16 * 16;                // one phase-2 chunk buffer
  static_assert(kArea % 16 == 0, "mbarriers and buffers are aligned");
};

// EN form (adjoint gradient): besides the step, each element accumulates
// gacc[e] += gcoef[e] * sum_s sum_q ue[dof_q][s] (A_e U^{n+1})_q in the order
// of the ENERGY variant of k_local_stiffness_rhs run with x = U^{n+1} and
// lam = ue, so both give the same bits: each (source s, z-line q) sums its
// points in k order (FP32 FMAs) into shared memory (E*S*NN floats past the
// plan's bytes); after a tile's passes, lane l of a warp adds each source
// s = l, l+32, ...: its z-lines q = 0..NN-1 in order in FP32, then that sum
// into an FP64 accumulator; a fixed shuffle tree adds the lanes.  One CTA owns
// an element per launch.
template <int N, int E, int LB, int V, bool EN = false>
__global__ void __launch_bounds__(RsPlan<N, E, LB, V>::T, rs_min_ctas(RsPlan<N, E, LB, V>::T))
    k_rhs_step(const RsParams p, const RsChunk* __restrict__ chunks, int n_chunks, SyncState* sync, int par,
               int* err, unsigned long long* __restrict__ stamps) {
  using P = RsPlan<N, E, LB, V>;
  constexpr int NN = P::NN, Q = P::Q, Qp = P::Qp, W = P::W;
  static_assert(!EN || P::T >= 32, "the EN form sums an element per full warp");
  extern __shared__ __align__(128) unsigned char smem[];
  float* s_u = reinterpret_cast<float*>(smem + 2 * P::kStage);
  float* s_vx = s_u + P::kWork;
  float* s_vy = s_vx + P::kWork;
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem + P::kArea);
  float* s_ez = reinterpret_cast<float*>(smem + P::kSmem);  // EN: [el][source][z-line]
  const int t = threadIdx.x, G = gridDim.x, S = p.S;
  const int lb = t % LB;
  const int w = t / LB;
  const int el = w / NN;
  const int ij = p.zmap[w - el * NN];  // this thread's z-line (i, j)
  const int j = ij / N;
  const int i = ij - j * N;
  float* __restrict__ cur = par == 0 ? p.ua : p.ub;        // U^n, overwritten by U^{n+2}
  const float* __restrict__ nxt = par == 0 ? p.ub : p.ua;  // U^{n+1}
  // step counters: ctr[1-par] = ctr[par] + 1 (phase 2 reads ctr[par] only)
  if (blockIdx.x == 0 && t == 0) p.ctr[1 - par] = p.ctr[par] + 1;
  // optional phase time stamps of this CTA: start, phase 1 done, barrier passed, end
  if (stamps && t == 0) stamps[4 * blockIdx.x] = global_ns();

  const float* __restrict__ Gm = c_gmat32[N];
  float gci[N], gcj[N], gri[N], grj[N];
#pragma unroll
  for (int a = 0; a < N; a++) {
    gci[a] = Gm[a * N + i];
    gcj[a] = Gm[a * N + j];
    gri[a] = Gm[i * N + a];
    grj[a] = Gm[j * N + a];
  }
  // work-array offset of point q of this thread's element and lane block
  auto wix = [&](int q) { return ((el * Q + q) * LB + lb) * V; };

  // ---- phase 1
  auto issue = [&](int st, int tile) {
    if (tile < p.n_tiles) {
      unsigned char* dst = smem + st * P::kStage;
      mbar_expect_tx(&bar[st], (uint32_t)(E * Qp * 28));
      bulk_g2s(dst, p.fac_e + (size_t)tile * E * 6 * Qp, (uint32_t)(E * 6 * Qp * 4), &bar[st]);
      bulk_g2s(dst + E * 6 * Qp * 4, p.nodle_e + (size_t)tile * E * Qp, (uint32_t)(E * Qp * 4), &bar[st]);
    }
  };
  if (t == 0) {
    for (int b = 0; b < 4; b++) mbar_init(&bar[b], 1);  // 0,1: tile stages; 2,3: chunk buffers
    fence_mbar_init();
    issue(0, blockIdx.x);
    issue(1, blockIdx.x + G);
  }
  __syncthreads();
  uint32_t ph = 0u;
  for (int tile = blockIdx.x, it = 0; tile < p.n_tiles; tile += G, ++it) {
    const int s = it & 1;
    const bool ok = mbar_wait_bounded(&bar[s], (ph >> s) & 1u);
    if (__syncthreads_or(!ok)) {
      if (t == 0) {  // report; stage s and, if issued, stage s^1 may have copies in flight
        atomicExch(err, 1);
        mbar_wait_drain(&bar[s], (ph >> s) & 1u);
        if (tile + G < p.n_tiles) mbar_wait_drain(&bar[s ^ 1], (ph >> (s ^ 1)) & 1u);
      }
      return;
    }
    ph ^= 1u << s;
    const float* f = reinterpret_cast<const float*>(smem + s * P::kStage) + el * 6 * Qp + ij;
    const int* nd = reinterpret_cast<const int*>(smem + s * P::kStage + E * 6 * Qp * 4) + el * Qp + ij;
    int dofs[N];
#pragma unroll
    for (int k = 0; k < N; k++) dofs[k] = nd[k * NN];
    const int* __restrict__ st = p.slot_e + ((size_t)tile * E + el) * Qp + ij;
    for (int pass = 0; pass < S / W; pass++) {
      const int col = pass * W + lb * V;
      float u[N][V];
#pragma unroll
      for (int k = 0; k < N; k++) {
        vload_g<V>(nxt + (size_t)dofs[k] * S + col, u[k]);
        vstore<V>(s_u + wix(k * NN + ij), u[k]);
      }
      __syncthreads();
      // the operation order of k_local_stiffness_rhs, written out as explicit
      // FMAs so both forms round alike
      float vz[N][V];
#pragma unroll
      for (int k = 0; k < N; k++) {
        float gx[V], gy[V], gz[V];
#pragma unroll
        for (int v = 0; v < V; v++) gx[v] = gy[v] = gz[v] = 0.f;
#pragma unroll
        for (int a = 0; a < N; a++) {
          float rx[V], ry[V];
          vload<V>(s_u + wix(k * NN + j * N + a), rx);
          vload<V>(s_u + wix(k * NN + a * N + i), ry);
          fma_v<V>(gz, Gm[a * N + k], u[a]);
          fma_v<V>(gx, gci[a], rx);
          fma_v<V>(gy, gcj[a], ry);
        }
        const float* fk = f + k * NN;
        const float bxx = fk[0], bxy = fk[Qp], bxz = fk[2 * Qp];
        const float byy = fk[3 * Qp], byz = fk[4 * Qp], bzz = fk[5 * Qp];
        float ox[V], oy[V];
        mul_v<V>(ox, bxx, gx);
        fma_v<V>(ox, bxy, gy);
        fma_v<V>(ox, bxz, gz);
        mul_v<V>(oy, bxy, gx);
        fma_v<V>(oy, byy, gy);
        fma_v<V>(oy, byz, gz);
        mul_v<V>(vz[k], bxz, gx);
        fma_v<V>(vz[k], byz, gy);
        fma_v<V>(vz[k], bzz, gz);
        vstore<V>(s_vx + wix(k * NN + ij), ox);
        vstore<V>(s_vy + wix(k * NN + ij), oy);
      }
      __syncthreads();
      float ez[V];  // EN: this z-line's sums for sources col .. col+V-1
#pragma unroll
      for (int v = 0; v < V; v++) ez[v] = 0.f;
      // EN: this z-line's U^m values, loaded together before the loop (its R
      // stores could alias them for the compiler, which would then issue each
      // load only after the previous point's store)
      float uev[EN ? N : 1][V];
      if constexpr (EN) {
#pragma unroll
        for (int k = 0; k < N; k++) vload_g<V>(p.ue + (size_t)dofs[k] * S + col, uev[k]);
      }
#pragma unroll
      for (int k = 0; k < N; k++) {
        float y[V];
#pragma unroll
        for (int v = 0; v < V; v++) y[v] = 0.f;
#pragma unroll
        for (int a = 0; a < N; a++) {
          float rx[V], ry[V];
          vload<V>(s_vx + wix(k * NN + j * N + a), rx);
          vload<V>(s_vy + wix(k * NN + a * N + i), ry);
          fma_v<V>(y, gri[a], rx);
          fma_v<V>(y, grj[a], ry);
          fma_v<V>(y, Gm[k * N + a], vz[a]);
        }
        vstore<V>(p.R + (size_t)__ldg(st + k * NN) * S + col, y);
        if constexpr (EN) {
#pragma unroll
          for (int v = 0; v < V; v++) ez[v] = fmaf(y[v], uev[k][v], ez[v]);
        }
      }
      if constexpr (EN) {
#pragma unroll
        for (int v = 0; v < V; v++) s_ez[((size_t)el * S + col + v) * NN + ij] = ez[v];
      }
      __syncthreads();
    }
    if (t == 0) {
      fence_proxy_async();
      issue(s, tile + 2 * G);
    }
    if constexpr (EN) {  // full warps; warp w sums elements w, w + T/32, ...
      const int wq = t >> 5, l32 = t & 31;
      if (wq < P::T / 32)
        for (int e = wq; e < E; e += P::T / 32) {
          double acc = 0.0;
          for (int src = l32; src < S; src += 32) {
            const float* row = s_ez + ((size_t)e * S + src) * NN;
            float zs = 0.f;  // the element's z-lines of this source, in order, in FP32
            for (int q = 0; q < NN; q++) zs += row[q];
            acc += (double)zs;
          }
          for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
          if (l32 == 0) {
            const size_t ge = (size_t)tile * E + e;
            p.gacc[ge] += p.gcoef[ge] * acc;
          }
        }
    }
  }

  fence_proxy_async_global();  // this thread's R stores before the bulk copies of phase 2
  if (stamps && t == 0) stamps[4 * blockIdx.x + 1] = global_ns();
  if (!grid_barrier(sync, err)) return;
  if (stamps && t == 0) stamps[4 * blockIdx.x + 2] = global_ns();

  // ---- phase 2
  float* __restrict__ dst = p.uout ? p.uout : cur;
  const int step = p.ctr[par];
  const bool pulse_on = step < p.n_pulse;
  const float pf = pulse_on ? (float)p.pulse[step] : 0.f;
  const int S4 = S >> 2;
  auto issue_chunk = [&](int c, int b) {
    if (c >= n_chunks) return;
    const RsChunk ch = chunks[c];
    const RsBuf L = rs_buf(ch.d0, ch.d1, ch.q0, ch.q1, S);
    unsigned char* dst = smem + b * P::kHalf;
    const int da = ch.d0 & ~3;
    mbar_expect_tx(&bar[2 + b], (uint32_t)L.end);
    bulk_g2s(dst + L.u1, nxt + (size_t)ch.d0 * S, (uint32_t)(L.u0 - L.u1), &bar[2 + b]);
    bulk_g2s(dst + L.u0, cur + (size_t)ch.d0 * S, (uint32_t)(L.r - L.u0), &bar[2 + b]);
    bulk_g2s(dst + L.r, p.R + (size_t)ch.q0 * S, (uint32_t)(L.m - L.r), &bar[2 + b]);
    bulk_g2s(dst + L.m, p.m + da, (uint32_t)(L.p - L.m), &bar[2 + b]);
    bulk_g2s(dst + L.p, p.ptr + da, (uint32_t)(L.end - L.p), &bar[2 + b]);
  };
  if (t == 0) {
    fence_proxy_async();         // phase-1 use of this shared memory is over
    fence_proxy_async_global();  // every CTA's R stores (ordered by the barrier) before the copies
    issue_chunk(blockIdx.x, 0);
    issue_chunk(blockIdx.x + G, 1);
  }
  uint32_t ph2 = 0u;
  for (int c = blockIdx.x, it = 0; c < n_chunks; c += G, ++it) {
    const int b = it & 1;
    const RsChunk ch = chunks[c];
    const bool ok = mbar_wait_bounded(&bar[2 + b], (ph2 >> b) & 1u);
    if (__syncthreads_or(!ok)) {
      if (t == 0) {  // report; buffer b and, if issued, buffer b^1 may have copies in flight
        atomicExch(err, 1);
        mbar_wait_drain(&bar[2 + b], (ph2 >> b) & 1u);
        if (c + G < n_chunks) mbar_wait_drain(&bar[2 + (b ^ 1)], (ph2 >> (b ^ 1)) & 1u);
      }
      return;
    }
    ph2 ^= 1u << b;
    const unsigned char* buf = smem + b * P::kHalf;
    const RsBuf L = rs_buf(ch.d0, ch.d1, ch.q0, ch.q1, S);
    const float4* su1 = reinterpret_cast<const float4*>(buf + L.u1);
    const float4* su0 = reinterpret_cast<const float4*>(buf + L.u0);
    const float4* sR = reinterpret_cast<const float4*>(buf + L.r);
    const float* sm = reinterpret_cast<const float*>(buf + L.m);
    const int* sp = reinterpret_cast<const int*>(buf + L.p);
    const int da = ch.d0 & ~3;
    const int items = (ch.d1 - ch.d0) * S4;
    for (int item = t; item < items; item += P::T) {
      const int dl = item / S4;
      const int c4 = item - dl * S4;
      const int d = ch.d0 + dl;
      float4 y = make_float4(0.f, 0.f, 0.f, 0.f);
      const int qb = sp[d + 1 - da] - ch.q0;
      for (int q = sp[d - da] - ch.q0; q < qb; q++) {
        const float4 r = sR[q * S4 + c4];
        y.x += r.x; y.y += r.y; y.z += r.z; y.w += r.w;
      }
      const float4 a1 = su1[dl * S4 + c4], a0 = su0[dl * S4 + c4];
      const float md = sm[d - da];
      float un[4];
      un[0] = 2.f * a1.x - a0.x + md * (-y.x);
      un[1] = 2.f * a1.y - a0.y + md * (-y.y);
      un[2] = 2.f * a1.z - a0.z + md * (-y.z);
      un[3] = 2.f * a1.w - a0.w + md * (-y.w);
      if (ch.has_src && pulse_on) {
        int lo = 0, hi = p.n_src_dof - 1;
        while (lo < hi) {
          const int mid = (lo + hi) >> 1;
          if (__ldg(p.src_dof + mid) < d) lo = mid + 1;
          else hi = mid;
        }
        if (__ldg(p.src_dof + lo) == d)
          for (int e = __ldg(p.src_ptr + lo); e < __ldg(p.src_ptr + lo + 1); e++) {
            const int r = __ldg(p.src_rhs + e);
            if ((r >> 2) == c4) un[r & 3] += md * pf * __ldg(p.src_val + e);
          }
      }
      const float4 o = make_float4(un[0], un[1], un[2], un[3]);
      *reinterpret_cast<float4*>(dst + (size_t)d * S + 4 * c4) = o;
      if (p.ucopy) *reinterpret_cast<float4*>(p.ucopy + (size_t)d * S + 4 * c4) = o;
    }
    __syncthreads();  // buffer b is free
    if (t == 0) {
      fence_proxy_async();
      issue_chunk(c + 2 * G, b);
    }
  }
  if (stamps) {
    __syncthreads();
    if (t == 0) stamps[4 * blockIdx.x + 3] = global_ns();
  }
}

}  // namespace
}  // namespace mj
