// Device side of the many-mesh batch step (k_mesh_batch_step and its
// helpers), shared by the all-orders kernels (mj_multi.cu) and the
// single-order kernels (mj_multi_one.cu).  Everything here sits in an
// anonymous namespace: each translation unit holds its own copy of the
// kernels and of the derivative-matrix constant bank, and the host passes
// the same plain structures to either.
#pragma once

#include <cuda_runtime.h>

#include <type_traits>

#include "mj_internal.cuh"
#include "mj_k1.cuh"
#include "mj_sync.cuh"

namespace mj {
namespace {

constexpr int kGraphStepsMb = 20;
constexpr int cmax(int a, int b) { return a > b ? a : b; }

// Launch configuration T (threads per CTA): elements per tile E(n) for
// n = r + 1 points per axis (E divides the element padding 240, E*n*n <= T),
// and the shared-memory plan derived from it.
template <int T>
struct MbCfg;
template <>
struct MbCfg<256> {
  static constexpr int threads = 256, min_ctas = 2;
  __host__ __device__ static constexpr int tile(int n) {
    return n == 2 ? 60 : n == 3 ? 24 : n == 4 ? 16 : n == 5 ? 10 : n == 6 ? 6 : n == 7 ? 4 : n == 8 ? 3 : 2;
  }
};
template <>
struct MbCfg<128> {
  static constexpr int threads = 128, min_ctas = 4;
  __host__ __device__ static constexpr int tile(int n) {
    return n == 2 ? 30 : n == 3 ? 12 : n == 4 ? 8 : n == 5 ? 5 : n == 6 ? 3 : n == 7 ? 2 : 1;
  }
};

template <int T>
struct MbPlan {
  using C = MbCfg<T>;
  static_assert(C::threads == T, "configuration keyed by its thread count");
  static constexpr int stage_of(int n) { return C::tile(n) * elem_slots(n) * 28; }  // factors + Nodle
  static constexpr int work_of(int n) { return C::tile(n) * n * n * n; }
  static constexpr int stage_max =
      cmax(cmax(cmax(stage_of(2), stage_of(3)), cmax(stage_of(4), stage_of(5))),
           cmax(cmax(stage_of(6), stage_of(7)), cmax(stage_of(8), stage_of(9))));
  static constexpr int kStage = (stage_max + 127) / 128 * 128;
  // floats of one work array, a multiple of 4 so every array and the
  // mbarriers after them start on 16-byte boundaries
  static constexpr int kWork = (cmax(cmax(cmax(work_of(2), work_of(3)), cmax(work_of(4), work_of(5))),
                                     cmax(cmax(work_of(6), work_of(7)), cmax(work_of(8), work_of(9)))) +
                                3) / 4 * 4;
  static constexpr int kArea = 2 * kStage + 3 * kWork * 4;  // stages + work arrays (u, vx, vy)
  static constexpr int kMaxG = (kWork + T - 1) / T;         // gathered values per thread
  // phase 2: every warp streams its own dof chunks through two buffers
  // [u^{n+1} | u^n | dt^2/D | offsets | R range] carved from the same area
  static constexpr int kWarps = T / 32;
  static constexpr int kDofsPerLane = 8;
  static constexpr int kChunkDofs = 32 * kDofsPerLane;
  static constexpr int kP2Buf = kArea / (2 * kWarps) / 16 * 16;
  static constexpr int kP2Ptr = 3 * kChunkDofs * 4;
  static constexpr int kP2R = kP2Ptr + (kChunkDofs + 4) * 4;
  static constexpr int kRCap = (kP2Buf - kP2R) / 4;
  // mbarriers after the area: 2 tile stages, then 2 chunk buffers per warp
  static constexpr int kBars = 2 + 2 * kWarps;
  static constexpr int kSmem = kArea + 8 * kBars;
  static_assert(kStage % 128 == 0 && kArea % 16 == 0, "stages, work arrays and mbarriers are aligned");
  static_assert(2 * kWarps * kP2Buf <= kArea, "chunk buffers end before the mbarriers");
  static_assert(kP2R % 16 == 0 && kP2Buf % 16 == 0, "bulk-copy destinations are 16-byte aligned");
  // the chunk builder halves a chunk whose contributions do not fit, down to 4 dofs
  static_assert(kRCap >= 8 * 4 + 3, "4 dofs of Q1 (8 contributions each) must fit");
  static_assert(C::min_ctas * (kSmem + 1024) <= 228 * 1024, "CTAs per SM");
};

struct MeshDev {
  const int* nodle_e;
  const float* fac_e;
  const int* slot_e;
  float* R;
  const int* ptr;
  float* ua;
  float* ub;
  const float* minv;         // dt^2 / D
  const double* inv_mass;    // 1/D (FP64, source term)
  const unsigned* src_mask;  // bit d set: dof d carries a source entry
  const int* src_idx;        // source dofs, sorted
  const float* src_val;      // their values
  const double* pulse;
  int* ctr;                  // the run's two step counters
  double dt2;
  int n, n_dof, n_src, n_pulse;
  int cur_par;  // at step k of a launch sequence, cur = ua when (k + cur_par) is even
  int qc_par;   // ctr[(k + qc_par) & 1] holds the step index at step k
};

// Profile record per CTA: 4 time stamps and 2 wait totals (ns).
constexpr int kStamps = 6;

// Runs of one batch (the table is a kernel parameter: constant-bank reads).
constexpr int kMaxRuns = 48;
struct MeshTable {
  MeshDev m[kMaxRuns];
  int n;
};

struct Work {
  int mesh, tile;  // mesh < 0: none
};

// Phase-2 work: dofs [d0, d1) of one mesh (d0 a multiple of 4), the 16-byte
// rounded range [q0, q1) of their contributions in R, and whether any of the
// dofs carries a source entry.
struct Chunk {
  int mesh, d0, d1, q0, q1, has_src, pad0, pad1;
};

__device__ __forceinline__ const float* next_state(const MeshDev& m, int k) {
  return ((k + m.cur_par) & 1) == 0 ? m.ub : m.ua;  // U^{n+1}
}

// Bulk copies of a tile's factors and Nodle (contiguous in the element-major
// layout; 16-byte aligned offsets and sizes) into a stage.
template <int T>
__device__ __forceinline__ void issue_tile(const MeshDev& m, int tile, unsigned char* stage, uint64_t* bar) {
  const int E = MbCfg<T>::tile(m.n), Qp = elem_slots(m.n);
  const uint32_t fb = (uint32_t)(E * 6 * Qp * 4), nb = (uint32_t)(E * Qp * 4);
  mbar_expect_tx(bar, fb + nb);
  bulk_g2s(stage, m.fac_e + (size_t)tile * E * 6 * Qp, fb, bar);
  bulk_g2s(stage + fb, m.nodle_e + (size_t)tile * E * Qp, nb, bar);
}

template <int T>
__device__ __forceinline__ const int* stage_nodle(const unsigned char* stage, int n) {
  return reinterpret_cast<const int*>(stage + MbCfg<T>::tile(n) * 6 * elem_slots(n) * 4);
}

// Gather of a tile's u into registers: value idx = el*Q + r of the work
// array comes from x[Nodle(el, r)], Nodle staged at el*Qp + r.  NC > 0: the
// order is NC, known at compile time; NC = 0: the order is n_rt.
template <int T, int NC>
__device__ __forceinline__ void gather_tile(int n_rt, const float* __restrict__ x, const int* nod,
                                            float (&g)[MbPlan<T>::kMaxG]) {
  const int n = NC > 0 ? NC : n_rt;
  const int Q = n * n * n, Qp = elem_slots(n), EQ = MbCfg<T>::tile(n) * Q;
#pragma unroll
  for (int v = 0; v < MbPlan<T>::kMaxG; v++) {
    const int idx = threadIdx.x + v * T;
    if (idx < EQ) {
      const int el = idx / Q;
      g[v] = __ldg(x + nod[el * Qp + (idx - el * Q)]);
    }
  }
}

template <int T, int NC>
__device__ __forceinline__ void store_tile(int n_rt, float* s_u, const float (&g)[MbPlan<T>::kMaxG]) {
  const int n = NC > 0 ? NC : n_rt;
  const int EQ = MbCfg<T>::tile(n) * n * n * n;
#pragma unroll
  for (int v = 0; v < MbPlan<T>::kMaxG; v++) {
    const int idx = threadIdx.x + v * T;
    if (idx < EQ) s_u[idx] = g[v];
  }
}

// Element product of one tile (E elements of one mesh), the compact
// single-RHS scheme of k_local_stiffness in the same operation order:
// u from the work array (gathered during the previous tile), factors from
// the stage.  Between the gradient and the divergence it waits for the next
// tile's stage (nn > 0) and gathers that tile's u, which lands in the work
// array once the divergence is done.  Threads >= E*n*n only take part in the
// block barriers.  Returns false when the stage wait timed out.
// SAME: every tile of the batch has order N (the next tile's gather is
// specialised to it).
template <int T, int N, bool SAME>
__device__ __forceinline__ bool tile_run(float* R, const int* slot_e, int tile, const float* __restrict__ fac,
                                         float* s_u, float* s_vx, float* s_vy, int nn, const float* xn,
                                         const int* nodn, uint64_t* barn, uint32_t parn, bool prof,
                                         unsigned long long& wns) {
  constexpr int E = MbCfg<T>::tile(N), NN = N * N, Q = N * NN, Qp = elem_slots(N);
  const float* __restrict__ Gm = c_gmat32[N];
  const int t = threadIdx.x;
  const bool act = t < E * NN;
  const int el = act ? t / NN : 0;
  const int ij = t - el * NN;
  const int j = ij / N;
  const int i = ij - j * N;
  const int lx = el * Q + j * N;  // + k*NN + a: x-line (el, k, j)
  const int ly = el * Q + i;      // + k*NN + a*N: y-line (el, k, i)
  float vz[N];
  if (act) {
    float u[N], gci[N], gcj[N];
#pragma unroll
    for (int a = 0; a < N; a++) {
      u[a] = s_u[el * Q + a * NN + ij];
      gci[a] = Gm[a * N + i];
      gcj[a] = Gm[a * N + j];
    }
    const float* f = fac + el * 6 * Qp + ij;
#pragma unroll
    for (int k = 0; k < N; k++) {
      float rx[N], ry[N];
#pragma unroll
      for (int a = 0; a < N; a++) {
        rx[a] = s_u[lx + k * NN + a];
        ry[a] = s_u[ly + k * NN + a * N];
      }
      float gx = 0, gy = 0, gz = 0;
#pragma unroll
      for (int a = 0; a < N; a++) {
        gz += Gm[a * N + k] * u[a];
        gx += gci[a] * rx[a];
        gy += gcj[a] * ry[a];
      }
      const float* fk = f + k * NN;
      const float bxx = fk[0], bxy = fk[Qp], bxz = fk[2 * Qp];
      const float byy = fk[3 * Qp], byz = fk[4 * Qp], bzz = fk[5 * Qp];
      s_vx[lx + k * NN + i] = fac_dot(bxx, gx, bxy, gy, bxz, gz);
      s_vy[ly + k * NN + j * N] = fac_dot(bxy, gx, byy, gy, byz, gz);
      vz[k] = fac_dot(bxz, gx, byz, gy, bzz, gz);
    }
  }
  __syncthreads();  // s_u is free: the next tile's u may land there
  bool ok = true;
  if (nn) {
    const unsigned long long w0 = prof ? global_ns() : 0ull;
    ok = mbar_wait_bounded(barn, parn);
    if (prof) wns += global_ns() - w0;
  }
  if (__syncthreads_or(!ok)) return false;
  float g[MbPlan<T>::kMaxG];
  if (nn) gather_tile<T, SAME ? N : 0>(nn, xn, nodn, g);
  if (act) {
    float gri[N], grj[N];
#pragma unroll
    for (int a = 0; a < N; a++) {
      gri[a] = Gm[i * N + a];
      grj[a] = Gm[j * N + a];
    }
    const int* __restrict__ st = slot_e + ((size_t)tile * E + el) * Qp + ij;
#pragma unroll
    for (int k = 0; k < N; k++) {
      float rx[N], ry[N];
#pragma unroll
      for (int a = 0; a < N; a++) {
        rx[a] = s_vx[lx + k * NN + a];
        ry[a] = s_vy[ly + k * NN + a * N];
      }
      float y = 0;
#pragma unroll
      for (int a = 0; a < N; a++) {
        y += gri[a] * rx[a];
        y += grj[a] * ry[a];
        y += Gm[k * N + a] * vz[a];
      }
      R[__ldg(st + k * NN)] = y;
    }
  }
  if (nn) store_tile<T, SAME ? N : 0>(nn, s_u, g);
  return true;
}

// The tile product of order N as a function of its own, for the all-orders
// kernel's orders up to n = 6 (Q5): out of line they no longer weigh on the
// code of the costly high orders, which stay inline (measured on 24 meshes of
// orders 2,3,4,6,8: 1.99 -> 1.88 ms per step; with only n = 9 inline, 1.94).
// Shared memory is reached through the dynamic shared-memory symbol and
// offsets.  Returns the stage-wait time, or ~0 on a timeout.
template <int T, int N>
__device__ __noinline__ unsigned long long tile_run_out(float* R, const int* slot_e, int tile, int stage, int nn,
                                                        const float* xn, uint32_t parn, bool prof) {
  using P = MbPlan<T>;
  extern __shared__ __align__(128) unsigned char smem[];
  float* s_u = reinterpret_cast<float*>(smem + 2 * P::kStage);
  float* s_vx = s_u + P::kWork;
  float* s_vy = s_vx + P::kWork;
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem + P::kArea);
  const float* fac = reinterpret_cast<const float*>(smem + stage * P::kStage);
  const int* nodn = nn ? stage_nodle<T>(smem + (stage ^ 1) * P::kStage, nn) : nullptr;
  unsigned long long wns = 0;
  const bool ok = tile_run<T, N, false>(R, slot_e, tile, fac, s_u, s_vx, s_vy, nn, xn, nodn, &bar[stage ^ 1], parn,
                                        prof, wns);
  return ok ? wns : ~0ull;
}

// Position of d in the sorted source list (d is known to be present).
__device__ __forceinline__ int find_source(const int* __restrict__ idx, int n, int d) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (__ldg(idx + mid) < d) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// Bulk copies of a chunk into a phase-2 buffer.  The state, mass, offset and
// R buffers carry spare entries past their ends, so the 16-byte rounded
// sizes stay inside them.
template <int T>
__device__ __forceinline__ void issue_chunk(const MeshDev& m, const Chunk& ch, int k, unsigned char* buf,
                                            uint64_t* bar) {
  using P = MbPlan<T>;
  const int d0 = ch.d0, nd4 = (ch.d1 - ch.d0 + 3) & ~3;
  const bool a_cur = ((k + m.cur_par) & 1) == 0;
  const uint32_t sb = (uint32_t)nd4 * 4u, pb = (uint32_t)((ch.d1 - ch.d0 + 1 + 3) & ~3) * 4u;
  const uint32_t rb = (uint32_t)(ch.q1 - ch.q0) * 4u;
  mbar_expect_tx(bar, 3u * sb + pb + rb);
  bulk_g2s(buf, (a_cur ? m.ub : m.ua) + d0, sb, bar);
  bulk_g2s(buf + P::kChunkDofs * 4, (a_cur ? m.ua : m.ub) + d0, sb, bar);
  bulk_g2s(buf + 2 * P::kChunkDofs * 4, m.minv + d0, sb, bar);
  bulk_g2s(buf + P::kP2Ptr, m.ptr + d0, pb, bar);
  bulk_g2s(buf + P::kP2R, m.R + ch.q0, rb, bar);
}

__device__ __forceinline__ Chunk load_chunk(const Chunk* chunks, int n_chunks, int c) {
  Chunk ch;
  if (c < n_chunks) {
    const int4 a = __ldg(reinterpret_cast<const int4*>(chunks + c));
    const int4 b = __ldg(reinterpret_cast<const int4*>(chunks + c) + 1);
    ch.mesh = a.x; ch.d0 = a.y; ch.d1 = a.z; ch.q0 = a.w; ch.q1 = b.x; ch.has_src = b.y;
  } else {
    ch.mesh = -1; ch.d0 = ch.d1 = ch.q0 = ch.q1 = ch.has_src = 0;
  }
  ch.pad0 = ch.pad1 = 0;
  return ch;
}

__device__ __forceinline__ Work load_work(const Work* work, int n_work, int w) {
  if (w < n_work) {
    const int2 v = __ldg(reinterpret_cast<const int2*>(work + w));
    return {v.x, v.y};
  }
  return {-1, 0};
}

// ONLY = 0: meshes of any order (a switch on the tile's order); ONLY = n:
// every mesh of the batch has order n, and the kernel holds that order's
// code alone (measured faster than the same order's path in the all-orders
// kernel).
template <int T, int ONLY>
__global__ void __launch_bounds__(T, MbCfg<T>::min_ctas)
    k_mesh_batch_step(const __grid_constant__ MeshTable tab, const Work* __restrict__ work, int n_work,
                      const Chunk* __restrict__ chunks, int n_chunks, SyncState* sync, int k, int* err,
                      unsigned long long* __restrict__ stamps) {
  using P = MbPlan<T>;
  extern __shared__ __align__(128) unsigned char smem[];
  float* s_u = reinterpret_cast<float*>(smem + 2 * P::kStage);
  float* s_vx = s_u + P::kWork;
  float* s_vy = s_vx + P::kWork;
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem + P::kArea);
  const int t = threadIdx.x;
  const int G = gridDim.x;
  // optional profile of this CTA (thread 0): time stamps at the start, phase 1
  // done, barrier passed and the end, then the time spent in the stage waits
  // of phase 1 and in the chunk waits of phase 2
  const bool prof = stamps != nullptr;
  unsigned long long wns1 = 0, wns2 = 0;
  if (prof && t == 0) stamps[kStamps * blockIdx.x] = global_ns();

  // step counters: ctr[1-qc] = ctr[qc] + 1 (phase 2 reads ctr[qc] only)
  if (blockIdx.x == 0)
    for (int r = t; r < tab.n; r += blockDim.x) {
      const int qc = (k + tab.m[r].qc_par) & 1;
      tab.m[r].ctr[1 - qc] = tab.m[r].ctr[qc] + 1;
    }

  // ---- phase 1: element tiles b, b+G, b+2G, ... of the cost-sorted list,
  // the stage of the next tile in flight during the current one
  int w = blockIdx.x;
  Work cur = load_work(work, n_work, w);
  Work nxt = load_work(work, n_work, w + G);
  if (t == 0) {
    for (int b = 0; b < P::kBars; b++) mbar_init(&bar[b], 1);  // 0,1: tile stages; then 2 per warp
    fence_mbar_init();
    if (cur.mesh >= 0) issue_tile<T>(tab.m[cur.mesh], cur.tile, smem, &bar[0]);
    if (nxt.mesh >= 0) issue_tile<T>(tab.m[nxt.mesh], nxt.tile, smem + P::kStage, &bar[1]);
  }
  __syncthreads();
  uint32_t ph = 0u;  // bit s: parity of the next completion of stage s
  int s = 0;
  if (cur.mesh >= 0) {
    const unsigned long long w0 = prof ? global_ns() : 0ull;
    const bool ok = mbar_wait_bounded(&bar[0], 0u);
    if (prof) wns1 += global_ns() - w0;
    if (__syncthreads_or(!ok)) {
      if (t == 0) {  // report; both stages may still have a copy in flight
        atomicExch(err, 1);
        mbar_wait_drain(&bar[0], 0u);
        if (nxt.mesh >= 0) mbar_wait_drain(&bar[1], 0u);
      }
      return;
    }
    ph ^= 1u;
    const MeshDev& m = tab.m[cur.mesh];
    float g[P::kMaxG];
    gather_tile<T, ONLY>(m.n, next_state(m, k), stage_nodle<T>(smem, m.n), g);
    store_tile<T, ONLY>(m.n, s_u, g);
  }
  while (cur.mesh >= 0) {
    __syncthreads();  // the tile's u is in s_u
    const Work nn2 = load_work(work, n_work, w + 2 * G);  // issued into this stage at the end
    const MeshDev& m = tab.m[cur.mesh];
    const float* fac = reinterpret_cast<const float*>(smem + s * P::kStage);
    int nn = 0;
    const float* xn = nullptr;
    const int* nodn = nullptr;
    if (nxt.mesh >= 0) {
      const MeshDev& mn = tab.m[nxt.mesh];
      nn = mn.n;
      xn = next_state(mn, k);
      nodn = stage_nodle<T>(smem + (s ^ 1) * P::kStage, nn);
    }
    const uint32_t parn = (ph >> (s ^ 1)) & 1u;
    // the tile's order as a compile-time constant; SAME when the batch has one order
    auto run = [&](auto order) {
      constexpr int N = decltype(order)::value;
      if constexpr (ONLY == 0 && N <= 6) {  // low orders out of line
        const unsigned long long r = tile_run_out<T, N>(m.R, m.slot_e, cur.tile, s, nn, xn, parn, prof);
        if (r == ~0ull) return false;
        wns1 += r;
        return true;
      } else {
        return tile_run<T, N, (ONLY > 0)>(m.R, m.slot_e, cur.tile, fac, s_u, s_vx, s_vy, nn, xn, nodn, &bar[s ^ 1],
                                          parn, prof, wns1);
      }
    };
    bool ok;
    if constexpr (ONLY > 0) {
      ok = run(std::integral_constant<int, ONLY>{});
    } else {
      switch (m.n) {
        case 2: ok = run(std::integral_constant<int, 2>{}); break;
        case 3: ok = run(std::integral_constant<int, 3>{}); break;
        case 4: ok = run(std::integral_constant<int, 4>{}); break;
        case 5: ok = run(std::integral_constant<int, 5>{}); break;
        case 6: ok = run(std::integral_constant<int, 6>{}); break;
        case 7: ok = run(std::integral_constant<int, 7>{}); break;
        case 8: ok = run(std::integral_constant<int, 8>{}); break;
        default: ok = run(std::integral_constant<int, 9>{}); break;
      }
    }
    if (!ok) {
      if (t == 0) {  // report; the next tile's stage may be in flight (stage s is not reissued yet)
        atomicExch(err, 1);
        if (nxt.mesh >= 0) mbar_wait_drain(&bar[s ^ 1], parn);
      }
      return;
    }
    if (nxt.mesh >= 0) ph ^= 1u << (s ^ 1);
    __syncthreads();  // stage s and the work arrays are free
    if (t == 0 && nn2.mesh >= 0) {
      fence_proxy_async();
      issue_tile<T>(tab.m[nn2.mesh], nn2.tile, smem + s * P::kStage, &bar[s]);
    }
    s ^= 1;
    w += G;
    cur = nxt;
    nxt = nn2;
  }

  if (prof && t == 0) {
    stamps[kStamps * blockIdx.x + 1] = global_ns();
    stamps[kStamps * blockIdx.x + 4] = wns1;
  }
  fence_proxy_async_global();  // this thread's R stores before the bulk copies of phase 2
  if (!grid_barrier(sync, err)) return;
  if (prof && t == 0) stamps[kStamps * blockIdx.x + 2] = global_ns();

  // ---- phase 2: each warp walks its own dof chunks (global warp index,
  // stride the grid's warp count) through two buffers of its own.  A
  // chunk's u^{n+1}, u^n, dt^2/D, CSR offsets and contributions R[ptr[d0] ..
  // ptr[d1]) (contiguous: R is in dof order) arrive by bulk copy, the next
  // chunk's while this one is summed, updated and written back; warps sync
  // among their own lanes only.
  {
    const int lane = t & 31, wid = t >> 5;
    const int GW = G * P::kWarps;
    uint64_t* wbar = bar + 2 + 2 * wid;
    unsigned char* wbuf = smem + 2 * wid * P::kP2Buf;
    int c = blockIdx.x * P::kWarps + wid;
    Chunk ccur = load_chunk(chunks, n_chunks, c);
    Chunk cnxt = load_chunk(chunks, n_chunks, c + GW);
    if (lane == 0) {
      fence_proxy_async();         // phase-1 use of this shared memory is over
      fence_proxy_async_global();  // every CTA's R stores (ordered by the barrier) before the copies
      if (ccur.mesh >= 0) issue_chunk<T>(tab.m[ccur.mesh], ccur, k, wbuf, &wbar[0]);
      if (cnxt.mesh >= 0) issue_chunk<T>(tab.m[cnxt.mesh], cnxt, k, wbuf + P::kP2Buf, &wbar[1]);
    }
    uint32_t ph2 = 0u;
    for (int it = 0; ccur.mesh >= 0; ++it) {
      const Chunk cn2 = load_chunk(chunks, n_chunks, c + 2 * GW);
      const int b = it & 1;
      unsigned char* buf = wbuf + b * P::kP2Buf;
      const MeshDev& m = tab.m[ccur.mesh];
      const unsigned long long w0 = prof ? global_ns() : 0ull;
      const bool ok = mbar_wait_bounded(&wbar[b], (ph2 >> b) & 1u);
      if (prof) wns2 += global_ns() - w0;
      if (__any_sync(0xffffffffu, !ok)) {
        // report, then wait (bounded) for this warp's copies still in flight
        if (lane == 0) atomicExch(err, 1);
        mbar_wait_drain(&wbar[b], (ph2 >> b) & 1u);
        if (cnxt.mesh >= 0) mbar_wait_drain(&wbar[b ^ 1], (ph2 >> (b ^ 1)) & 1u);
        break;
      }
      ph2 ^= 1u << b;
      const float* su1 = reinterpret_cast<const float*>(buf);
      const float* su0 = su1 + P::kChunkDofs;
      const float* smv = su0 + P::kChunkDofs;
      const int* sptr = reinterpret_cast<const int*>(buf + P::kP2Ptr);
      const float* sR = reinterpret_cast<const float*>(buf + P::kP2R);
      float* __restrict__ u0 = ((k + m.cur_par) & 1) == 0 ? m.ua : m.ub;  // U^n, overwritten by U^{n+2}
      const int step = ccur.has_src ? m.ctr[(k + m.qc_par) & 1] : 0;
      constexpr int V = P::kDofsPerLane;
      int dls[V];
      bool on[V];
      float sums[V];
#pragma unroll
      for (int v = 0; v < V; v++) {
        dls[v] = v * 32 + lane;
        on[v] = ccur.d0 + dls[v] < ccur.d1;
      }
      contrib_sums<V>(sptr, sR, ccur.q0, dls, on, sums);
#pragma unroll
      for (int v = 0; v < V; v++) {
        const int dl = dls[v];
        const int d = ccur.d0 + dl;
        if (on[v]) {
          const float ah = -sums[v];
          float un = float(2) * su1[dl] - su0[dl] + smv[dl] * ah;
          if (ccur.has_src && ((__ldg(m.src_mask + (d >> 5)) >> (d & 31)) & 1u) && step < m.n_pulse) {
            const int ts = find_source(m.src_idx, m.n_src, d);
            un = float(double(un) + m.dt2 * __ldg(m.inv_mass + d) * __ldg(m.pulse + step) *
                                        double(__ldg(m.src_val + ts)));
          }
          u0[d] = un;
        }
      }
      __syncwarp();  // buffer b is free
      if (lane == 0 && cn2.mesh >= 0) {
        fence_proxy_async();
        issue_chunk<T>(tab.m[cn2.mesh], cn2, k, buf, &wbar[b]);
      }
      c += GW;
      ccur = cnxt;
      cnxt = cn2;
    }
  }
  if (prof) {
    __syncthreads();
    if (t == 0) {
      stamps[kStamps * blockIdx.x + 3] = global_ns();
      stamps[kStamps * blockIdx.x + 5] = wns2;
    }
  }

}

// Work lists of one launch configuration.
struct MbLists {
  int threads = 0, smem = 0, ctas_per_sm = 0, grid = 0;
  DevBuf work, chunks;
  int n_work = 0, n_chunks = 0;
};

}  // namespace
}  // namespace mj
