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
//   phase 2  dof chunks of all meshes, two buffers per CTA: the chunk's
//            u^{n+1}, u^n, dt^2/D, CSR offsets and its contiguous range of R
//            arrive by bulk copy (the next chunk's during this one), then
//            each dof's sum, leap-frog update and source term (a per-dof bit
//            mask marks source dofs).
// Two launch configurations are compiled (256 threads with large tiles, 128
// threads with small tiles and more CTAs per SM); the first advance times
// both on the batch itself and keeps the faster.
// The reference runs one ModifiedEquationIterator per problem, one after the
// other (MONTJOIE/src/Instationary/ModifiedEquation.cxx:290-345).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <memory>
#include <numeric>
#include <vector>

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
  static constexpr int kSmem = kArea + 32;                  // + 4 mbarriers
  static constexpr int kMaxG = (kWork + T - 1) / T;         // gathered values per thread
  // phase 2: two chunk buffers [u^{n+1} | u^n | dt^2/D | offsets | R range]
  static constexpr int kDofsPerThread = 4;
  static constexpr int kChunkDofs = T * kDofsPerThread;
  static constexpr int kP2Buf = kArea / 2 / 16 * 16;
  static constexpr int kP2Ptr = 3 * kChunkDofs * 4;
  static constexpr int kP2R = kP2Ptr + (kChunkDofs + 4) * 4;
  static constexpr int kRCap = (kP2Buf - kP2R) / 4;
  static_assert(kStage % 128 == 0 && kArea % 16 == 0, "stages, work arrays and mbarriers are aligned");
  static_assert(2 * kP2Buf <= kArea, "chunk buffers end before the mbarriers");
  static_assert(kP2R % 16 == 0, "bulk-copy destinations are 16-byte aligned");
  static_assert(kRCap >= 8 * kChunkDofs + 3, "a chunk of Q1 dofs (8 contributions each) must fit");
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

// Gather of a tile's u (any order) into registers: value idx = el*Q + r of
// the work array comes from x[Nodle(el, r)], Nodle staged at el*Qp + r.
template <int T>
__device__ __forceinline__ void gather_tile(int n, const float* __restrict__ x, const int* nod,
                                            float (&g)[MbPlan<T>::kMaxG]) {
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

template <int T>
__device__ __forceinline__ void store_tile(int n, float* s_u, const float (&g)[MbPlan<T>::kMaxG]) {
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
template <int T, int N>
__device__ __forceinline__ bool tile_run(const MeshDev& m, int tile, const float* __restrict__ fac, float* s_u,
                                         float* s_vx, float* s_vy, int nn, const float* xn, const int* nodn,
                                         uint64_t* barn, uint32_t parn) {
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
      s_vx[lx + k * NN + i] = bxx * gx + bxy * gy + bxz * gz;
      s_vy[ly + k * NN + j * N] = bxy * gx + byy * gy + byz * gz;
      vz[k] = bxz * gx + byz * gy + bzz * gz;
    }
  }
  __syncthreads();  // s_u is free: the next tile's u may land there
  bool ok = true;
  if (nn) ok = mbar_wait_bounded(barn, parn);
  if (__syncthreads_or(!ok)) return false;
  float g[MbPlan<T>::kMaxG];
  if (nn) gather_tile<T>(nn, xn, nodn, g);
  if (act) {
    float gri[N], grj[N];
#pragma unroll
    for (int a = 0; a < N; a++) {
      gri[a] = Gm[i * N + a];
      grj[a] = Gm[j * N + a];
    }
    const int* __restrict__ st = m.slot_e + ((size_t)tile * E + el) * Qp + ij;
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
      m.R[__ldg(st + k * NN)] = y;
    }
  }
  if (nn) store_tile<T>(nn, s_u, g);
  return true;
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

template <int T>
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
  // optional phase time stamps of this CTA: start, phase 1 done, barrier passed, end
  if (stamps && t == 0) stamps[4 * blockIdx.x] = global_ns();

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
    for (int b = 0; b < 4; b++) mbar_init(&bar[b], 1);  // 0,1: tile stages; 2,3: chunk buffers
    fence_mbar_init();
    if (cur.mesh >= 0) issue_tile<T>(tab.m[cur.mesh], cur.tile, smem, &bar[0]);
    if (nxt.mesh >= 0) issue_tile<T>(tab.m[nxt.mesh], nxt.tile, smem + P::kStage, &bar[1]);
  }
  __syncthreads();
  uint32_t ph = 0u;  // bit s: parity of the next completion of stage s
  int s = 0;
  if (cur.mesh >= 0) {
    const bool ok = mbar_wait_bounded(&bar[0], 0u);
    if (__syncthreads_or(!ok)) {
      if (t == 0) atomicExch(err, 1);
      return;
    }
    ph ^= 1u;
    const MeshDev& m = tab.m[cur.mesh];
    float g[P::kMaxG];
    gather_tile<T>(m.n, next_state(m, k), stage_nodle<T>(smem, m.n), g);
    store_tile<T>(m.n, s_u, g);
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
    bool ok;
    switch (m.n) {
      case 2: ok = tile_run<T, 2>(m, cur.tile, fac, s_u, s_vx, s_vy, nn, xn, nodn, &bar[s ^ 1], parn); break;
      case 3: ok = tile_run<T, 3>(m, cur.tile, fac, s_u, s_vx, s_vy, nn, xn, nodn, &bar[s ^ 1], parn); break;
      case 4: ok = tile_run<T, 4>(m, cur.tile, fac, s_u, s_vx, s_vy, nn, xn, nodn, &bar[s ^ 1], parn); break;
      case 5: ok = tile_run<T, 5>(m, cur.tile, fac, s_u, s_vx, s_vy, nn, xn, nodn, &bar[s ^ 1], parn); break;
      case 6: ok = tile_run<T, 6>(m, cur.tile, fac, s_u, s_vx, s_vy, nn, xn, nodn, &bar[s ^ 1], parn); break;
      case 7: ok = tile_run<T, 7>(m, cur.tile, fac, s_u, s_vx, s_vy, nn, xn, nodn, &bar[s ^ 1], parn); break;
      case 8: ok = tile_run<T, 8>(m, cur.tile, fac, s_u, s_vx, s_vy, nn, xn, nodn, &bar[s ^ 1], parn); break;
      default: ok = tile_run<T, 9>(m, cur.tile, fac, s_u, s_vx, s_vy, nn, xn, nodn, &bar[s ^ 1], parn); break;
    }
    if (!ok) {
      if (t == 0) atomicExch(err, 1);
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

  if (stamps && t == 0) stamps[4 * blockIdx.x + 1] = global_ns();
  fence_proxy_async_global();  // this thread's R stores before the bulk copies of phase 2
  if (!grid_barrier(sync, err)) return;
  if (stamps && t == 0) stamps[4 * blockIdx.x + 2] = global_ns();

  // ---- phase 2: dof chunks b, b+G, ..., two buffers per CTA.  A chunk's
  // u^{n+1}, u^n, dt^2/D, CSR offsets and contributions R[ptr[d0] ..
  // ptr[d1]) (contiguous: R is in dof order) arrive by bulk copy, the next
  // chunk's while this one is summed, updated and written back.
  int c = blockIdx.x;
  Chunk ccur = load_chunk(chunks, n_chunks, c);
  Chunk cnxt = load_chunk(chunks, n_chunks, c + G);
  if (t == 0) {
    fence_proxy_async();         // phase-1 use of this shared memory is over
    fence_proxy_async_global();  // every CTA's R stores (ordered by the barrier) before the copies
    if (ccur.mesh >= 0) issue_chunk<T>(tab.m[ccur.mesh], ccur, k, smem, &bar[2]);
    if (cnxt.mesh >= 0) issue_chunk<T>(tab.m[cnxt.mesh], cnxt, k, smem + P::kP2Buf, &bar[3]);
  }
  uint32_t ph2 = 0u;
  for (int it = 0; ccur.mesh >= 0; ++it) {
    const Chunk cn2 = load_chunk(chunks, n_chunks, c + 2 * G);
    const int b = it & 1;
    unsigned char* buf = smem + b * P::kP2Buf;
    const MeshDev& m = tab.m[ccur.mesh];
    const bool ok = mbar_wait_bounded(&bar[2 + b], (ph2 >> b) & 1u);
    if (__syncthreads_or(!ok)) {
      if (t == 0) atomicExch(err, 1);
      return;
    }
    ph2 ^= 1u << b;
    const float* su1 = reinterpret_cast<const float*>(buf);
    const float* su0 = su1 + P::kChunkDofs;
    const float* smv = su0 + P::kChunkDofs;
    const int* sptr = reinterpret_cast<const int*>(buf + P::kP2Ptr);
    const float* sR = reinterpret_cast<const float*>(buf + P::kP2R);
    float* __restrict__ u0 = ((k + m.cur_par) & 1) == 0 ? m.ua : m.ub;  // U^n, overwritten by U^{n+2}
    const int step = ccur.has_src ? m.ctr[(k + m.qc_par) & 1] : 0;
#pragma unroll
    for (int v = 0; v < P::kDofsPerThread; v++) {
      const int dl = v * T + t;
      const int d = ccur.d0 + dl;
      if (d < ccur.d1) {
        float sum = 0;
        const int qb = sptr[dl + 1] - ccur.q0;
        for (int q = sptr[dl] - ccur.q0; q < qb; q++) sum += sR[q];
        const float ah = -sum;
        float un = float(2) * su1[dl] - su0[dl] + smv[dl] * ah;
        if (ccur.has_src && ((__ldg(m.src_mask + (d >> 5)) >> (d & 31)) & 1u) && step < m.n_pulse) {
          const int ts = find_source(m.src_idx, m.n_src, d);
          un = float(double(un) + m.dt2 * __ldg(m.inv_mass + d) * __ldg(m.pulse + step) *
                                      double(__ldg(m.src_val + ts)));
        }
        u0[d] = un;
      }
    }
    __syncthreads();  // buffer b is free
    if (t == 0 && cn2.mesh >= 0) {
      fence_proxy_async();
      issue_chunk<T>(tab.m[cn2.mesh], cn2, k, buf, &bar[2 + b]);
    }
    c += G;
    ccur = cnxt;
    cnxt = cn2;
  }
  if (stamps) {
    __syncthreads();
    if (t == 0) stamps[4 * blockIdx.x + 3] = global_ns();
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

using namespace mj;

struct mj_mb {
  std::vector<mj_lf*> runs;
  DevBuf sync, err;
  MeshTable table;  // kernel parameter
  std::vector<std::unique_ptr<DevBuf>> keep;  // per-run source masks and sorted sources
  std::vector<MeshDev> h_mesh;
  MbLists cfg[2];   // 0: 256 threads, 1: 128 threads
  int use = -1;     // configuration in use (-1: not tuned yet)
  double tune_ms[2] = {0, 0};
  // launch parity of the uploaded table: per run (cur_is_a, step & 1) at upload
  std::vector<int> base_cur, base_qc;
  cudaGraphExec_t graph[2] = {nullptr, nullptr};  // 20 steps starting at k = 0 or k = 1
  bool last_graph = false;
  DevBuf stamps;        // per-CTA phase time stamps when profiling (plain launches only)
  bool profile = false;
  cudaStream_t stream = nullptr;
  ~mj_mb() {
    for (auto& g : graph)
      if (g) cudaGraphExecDestroy(g);
  }
};

namespace {

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
  MJ_CUDA(cudaLaunchKernelEx(&cfg, k_mesh_batch_step<T>, mb->table, (const Work*)L.work.as<Work>(), L.n_work,
                             (const Chunk*)L.chunks.as<Chunk>(), L.n_chunks, mb->sync.as<SyncState>(), k,
                             mb->err.as<int>(),
                             mb->profile ? mb->stamps.as<unsigned long long>() : (unsigned long long*)nullptr));
  count_launch();
  return MJ_OK;
}

int mb_launch(mj_mb* mb, int which, int k, cudaStream_t s) {
  return which == 0 ? mb_launch_t<256>(mb, mb->cfg[0], k, s) : mb_launch_t<128>(mb, mb->cfg[1], k, s);
}

// Tile and chunk lists of configuration T: tiles sorted by decreasing cost
// (dealt round-robin to the CTAs), chunks of at most kChunkDofs dofs whose
// 16-byte rounded range of contributions fits kRCap.
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
  MJ_CUDA(cudaFuncSetAttribute(k_mesh_batch_step<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, P::kSmem));
  MJ_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&L.ctas_per_sm, k_mesh_batch_step<T>, T, P::kSmem));
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
  }
  mb->table.n = (int)n;
  for (auto& g : mb->graph)
    if (g) {
      cudaGraphExecDestroy(g);
      g = nullptr;
    }
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
  MJ_CUDA(cudaMemcpyAsync(&herr, mb->err.ptr, sizeof(int), cudaMemcpyDeviceToHost, s));
  MJ_CUDA(cudaStreamSynchronize(s));
  if (herr) {
    cudaMemset(mb->err.ptr, 0, sizeof(int));
    cudaMemset(mb->sync.ptr, 0, sizeof(SyncState));
    set_error("mj_mb_advance: a bounded wait timed out (batch state is invalid)");
    return MJ_ERR_STATE;
  }
  return MJ_OK;
}

// Times both launch configurations on the batch itself (3 steps each after
// one warm-up) and keeps the faster.  The runs' states and step counters are
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
  for (int c = 0; c < 2; c++) {
    int rc = mb_launch(mb, c, off, s);
    if (!rc) rc = cudaEventRecord(e0, s) == cudaSuccess ? MJ_OK : MJ_ERR_CUDA;
    for (int i = 1; !rc && i <= 3; i++) rc = mb_launch(mb, c, off + i, s);
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

}  // namespace

extern "C" {

int mj_mb_create(int n_runs, mj_lf* const* runs, mj_mb** out) {
  MJ_CHECK_ARG(out && runs && n_runs > 0, "mj_mb_create: null argument or no runs");
  MJ_CHECK_ARG(n_runs <= kMaxRuns, "mj_mb_create: at most 48 runs per batch");
  *out = nullptr;
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
  for (int n = 2; n <= kMaxNK; n++)
    if (have_g[n]) {
      float v[kMaxNK * kMaxNK];
      for (int a = 0; a < n * n; a++) v[a] = (float)gm[n][a];
      MJ_CUDA(cudaMemcpyToSymbol(c_gmat32, v, sizeof(float) * n * n, sizeof(float) * kMaxNK * kMaxNK * n));
    }

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
  MJ_CUDA(mb->stamps.alloc(sizeof(unsigned long long) * 4 *
                           std::max(mb->cfg[0].grid, mb->cfg[1].grid)));
  mb->stream = runs[0]->stream;
  mb_upload(mb.get());
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
  if (mb->use < 0) {
    const int rc = mb_autotune(mb, off, s);
    if (rc) return rc;
  }
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
        const int rc = mb_launch(mb, mb->use, off + k, cs);
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
    while (nsteps - done >= kGraphStepsMb) {
      MJ_CUDA(cudaGraphLaunch(mb->graph[off], s));
      count_launch(kGraphStepsMb);
      done += kGraphStepsMb;
    }
    mb->last_graph = true;
  }
  for (; done < nsteps; done++) {
    const int rc = mb_launch(mb, mb->use, off + done, s);
    if (rc) return rc;
  }
  for (mj_lf* lf : mb->runs) {
    lf->step += nsteps;
    if (nsteps & 1) lf->cur_is_a = !lf->cur_is_a;
  }
  return mb_check_err(mb, s);
}

int mj_mb_profile(mj_mb* mb, int enable) {
  MJ_CHECK_ARG(mb, "mj_mb_profile: null batch");
  mb->profile = enable != 0;
  return MJ_OK;
}

int mj_mb_phase_ms(const mj_mb* mb, double* out) {
  MJ_CHECK_ARG(mb && out, "mj_mb_phase_ms: null argument");
  MJ_CHECK_ARG(mb->use >= 0, "mj_mb_phase_ms: no step has run");
  const int grid = mb->cfg[mb->use].grid;
  std::vector<unsigned long long> st(4 * (size_t)grid);
  MJ_CUDA(cudaMemcpy(st.data(), mb->stamps.ptr, sizeof(unsigned long long) * st.size(), cudaMemcpyDeviceToHost));
  unsigned long long t0 = ~0ull, p1max = 0, p2 = 0, end = 0;
  double p1sum = 0;
  for (int b = 0; b < grid; b++) t0 = std::min(t0, st[4 * b]);
  for (int b = 0; b < grid; b++) {
    p1max = std::max(p1max, st[4 * b + 1]);
    p1sum += double(st[4 * b + 1] - t0);
    p2 = std::max(p2, st[4 * b + 2]);
    end = std::max(end, st[4 * b + 3]);
  }
  out[0] = double(p1max - t0) * 1e-6;  // phase 1 (last CTA to finish)
  out[1] = p1sum / grid * 1e-6;        // phase 1 (mean CTA)
  out[2] = double(p2 - p1max) * 1e-6;  // barrier release after the last arrival
  out[3] = double(end - p2) * 1e-6;    // phase 2 (last CTA)
  return MJ_OK;
}

int mj_mb_info(const mj_mb* mb, int* grid, int* ctas_per_sm, int* n_tiles, int* n_chunks, int* graph) {
  MJ_CHECK_ARG(mb, "mj_mb_info: null batch");
  const MbLists& L = mb->cfg[mb->use < 0 ? 0 : mb->use];
  if (grid) *grid = L.grid;
  if (ctas_per_sm) *ctas_per_sm = L.ctas_per_sm;
  if (n_tiles) *n_tiles = L.n_work;
  if (n_chunks) *n_chunks = L.n_chunks;
  if (graph) *graph = mb->last_graph ? 1 : 0;
  return MJ_OK;
}

int mj_mb_set_config(mj_mb* mb, int threads) {
  MJ_CHECK_ARG(mb, "mj_mb_set_config: null batch");
  MJ_CHECK_ARG(threads == 0 || threads == 128 || threads == 256, "mj_mb_set_config: threads must be 0, 128 or 256");
  mb->use = threads == 0 ? -1 : threads == 256 ? 0 : 1;
  for (auto& g : mb->graph)
    if (g) {
      cudaGraphExecDestroy(g);
      g = nullptr;
    }
  return MJ_OK;
}

int mj_mb_tuning(const mj_mb* mb, int* threads, double* candidate_ms) {
  MJ_CHECK_ARG(mb, "mj_mb_tuning: null batch");
  if (threads) *threads = mb->use < 0 ? 0 : mb->cfg[mb->use].threads;
  if (candidate_ms) {
    candidate_ms[0] = mb->tune_ms[0];
    candidate_ms[1] = mb->tune_ms[1];
  }
  return MJ_OK;
}

}  // extern "C"
