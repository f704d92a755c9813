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

#include "mj_internal.cuh"
#include "mj_k1.cuh"
#include "mj_sync.cuh"

namespace mj {
namespace {

constexpr int kGraphStepsRs = 20;

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
  int n_src_dof, n_pulse, S, n_tiles;
  unsigned char zmap[kMaxNK * kMaxNK];  // z-line (j*n + i) of each thread slot of an element (rs_zline_order)
};

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

template <int N, int E, int LB, int V>
__global__ void __launch_bounds__(RsPlan<N, E, LB, V>::T, rs_min_ctas(RsPlan<N, E, LB, V>::T))
    k_rhs_step(const RsParams p, const RsChunk* __restrict__ chunks, int n_chunks, SyncState* sync, int par,
               int* err, unsigned long long* __restrict__ stamps) {
  using P = RsPlan<N, E, LB, V>;
  constexpr int NN = P::NN, Q = P::Q, Qp = P::Qp, W = P::W;
  extern __shared__ __align__(128) unsigned char smem[];
  float* s_u = reinterpret_cast<float*>(smem + 2 * P::kStage);
  float* s_vx = s_u + P::kWork;
  float* s_vy = s_vx + P::kWork;
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem + P::kArea);
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
      }
      __syncthreads();
    }
    if (t == 0) {
      fence_proxy_async();
      issue(s, tile + 2 * G);
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
      *reinterpret_cast<float4*>(dst + (size_t)d * S + 4 * c4) = make_float4(un[0], un[1], un[2], un[3]);
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

// Error flag of the one-kernel step (bounded waits), reset when set.
int lfb_fused_check(mj_lfb* b, cudaStream_t s) { return rs_check_err(b, s); }

// One ordinary step of the one-kernel form (the integrator's own states and
// step counter).
int lfb_fused_step(mj_lfb* b, cudaStream_t s) {
  const RsVariant& v = rs_variants()[b->rs_variant];
  const RsParams prm = rs_params(b, v);
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
