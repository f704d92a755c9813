// Device kernels of the matrix-free Q_r hexahedral stiffness operator and the
// leap-frog update (sm_103a).
//
// Data layout in HBM ("tile layout").  Elements are grouped in tiles of E
// consecutive elements; one CTA processes one tile at a time with E*n*n
// threads, thread (el, j, i) owning the line of n points (i, j, k=0..n-1) of
// element el.  Every per-point array is stored so that, for a fixed k, the
// E*n*n threads of a tile read one contiguous run:
//   nodle_t[((tile*n + k)*E + el)*n*n + j*n + i]             (int32)
//   fac_t  [(((tile*6 + c)*n + k)*E + el)*n*n + j*n + i]     (c = xx,xy,xz,yy,yz,zz)
//   R      [((tile*n + k)*E + el)*n*n + j*n + i]             (element-local A*u)
// The global result is gathered per dof from R through a CSR incidence list
// (owner computes: deterministic, no atomics).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace mj {

template <typename Real, int N>
struct GMatrix {
  Real g[N * N];  // g[a*N + b] = phi_a'(x_b)
};

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
// ---------------------------------------------------------------------------
template <typename Real, int N, int E>
__global__ void __launch_bounds__(E* N* N)
    k_local_stiffness(const Real* __restrict__ x, const int* __restrict__ nodle_t,
                      const Real* __restrict__ fac_t, Real* __restrict__ R, int n_tiles,
                      const GMatrix<Real, N> G) {
  constexpr int NN = N * N;
  constexpr int TQ = E * N * NN;  // points per tile
  __shared__ Real s_u[E * N * NN];
  __shared__ Real s_vx[E * N * NN];
  __shared__ Real s_vy[E * N * NN];

  const int t = threadIdx.x;
  const int el = t / NN;
  const int ij = t - el * NN;
  const int j = ij / N;
  const int i = ij - j * N;
  // G columns/rows this thread needs with runtime indices.
  Real gci[N], gcj[N], gri[N], grj[N];
#pragma unroll
  for (int a = 0; a < N; a++) {
    gci[a] = G.g[a * N + i];
    gcj[a] = G.g[a * N + j];
    gri[a] = G.g[i * N + a];
    grj[a] = G.g[j * N + a];
  }
  // shared-memory offsets: s[((el*N + k)*N + j)*N + i]
  const int s_line_x = (el * N * N + j) * N;   // + k*NN + a   : row (j,k) along x
  const int s_line_y = el * N * NN + i;        // + k*NN + a*N : row (i,k) along y

  for (int tile = blockIdx.x; tile < n_tiles; tile += gridDim.x) {
    const size_t base = (size_t)tile * TQ + t;
    Real u[N];
#pragma unroll
    for (int k = 0; k < N; k++) {
      const int idx = __ldg(nodle_t + base + (size_t)k * E * NN);
      u[k] = __ldg(x + idx);
      s_u[(el * N + k) * NN + ij] = u[k];
    }
    __syncthreads();

    const size_t fbase = (size_t)tile * 6 * TQ + t;
    Real vz[N];
#pragma unroll
    for (int k = 0; k < N; k++) {
      Real gx = 0, gy = 0, gz = 0;
#pragma unroll
      for (int a = 0; a < N; a++) {
        gz += G.g[a * N + k] * u[a];
        gx += gci[a] * s_u[s_line_x + k * NN + a];
        gy += gcj[a] * s_u[s_line_y + k * NN + a * N];
      }
      const Real* f = fac_t + fbase + (size_t)k * E * NN;
      const Real bxx = __ldg(f), bxy = __ldg(f + TQ), bxz = __ldg(f + 2 * TQ);
      const Real byy = __ldg(f + 3 * TQ), byz = __ldg(f + 4 * TQ), bzz = __ldg(f + 5 * TQ);
      s_vx[(el * N + k) * NN + ij] = bxx * gx + bxy * gy + bxz * gz;
      s_vy[(el * N + k) * NN + ij] = bxy * gx + byy * gy + byz * gz;
      vz[k] = bxz * gx + byz * gy + bzz * gz;
    }
    __syncthreads();

#pragma unroll
    for (int k = 0; k < N; k++) {
      Real y = 0;
#pragma unroll
      for (int a = 0; a < N; a++) {
        y += gri[a] * s_vx[s_line_x + k * NN + a];
        y += grj[a] * s_vy[s_line_y + k * NN + a * N];
        y += G.g[k * N + a] * vz[a];
      }
      R[base + (size_t)k * E * NN] = y;
    }
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
