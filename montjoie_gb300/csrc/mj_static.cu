// Allocation-free stiffness product.
//
// Some callers cannot let a library allocate GPU memory.  Examples are a
// solver whose device memory is all carved out of one arena owned by another
// allocator, or a time loop that stages every buffer once at start-up and must
// not call cudaMalloc/cudaFree later, because those calls can synchronise the
// device and fragment the arena.  For them, mj_stiffness_mltadd_static computes
// the same product as mj_op_create + mj_op_mltadd_device on arrays the caller
// already owns.  Its element-local scratch is a fixed array in this file,
// allocated once per GPU when the library's code is loaded and kept until exit.
#include <cuda_runtime.h>

#include "mj_common.cuh"

namespace mj {

// Element-local values of one product: n_elt * (r+1)^3 doubles at most.
constexpr size_t kStaticScratchPoints = size_t(4) << 20;  // 4,194,304 values = 32 MiB

static __device__ __align__(256) double g_static_scratch[kStaticScratchPoints];
static __device__ int g_static_bad_index;  // set when a Nodle entry is out of [0, n_dof)

namespace {

// Local index NumDofs3D(i,j,k) of a Q_r hexahedron, in closed form
// (vertices, the 12 edges, faces x=0,y=0,z=0,z=r,y=r,x=r, interior;
// MONTJOIE/src/Quadrature/HexahedronQuadrature.cxx:51-171).
__device__ int local_index(int r, int i, int j, int k) {
  const int bi = (i == 0 || i == r), bj = (j == 0 || j == r), bk = (k == 0 || k == r);
  const int nb = bi + bj + bk, m = r - 1;
  if (nb == 3) {
    const int x = i / r, y = j / r, z = k / r;
    const int base = (x == 0) ? ((y == 0) ? 0 : 3) : ((y == 0) ? 1 : 2);
    return base + 4 * z;
  }
  const int eoff = 8, foff = 8 + 12 * m, ioff = 8 + 12 * m + 6 * m * m;
  if (nb == 2) {
    // edge e from vertex a to vertex b, parameter l counted from a
    int e, l;
    if (!bi) {  // along x at (y, z) in {0, r}^2: edges 0 (y0z0), 2 (y1z0: 3->2), 8 (y0z1), 10 (y1z1: 7->6)
      e = (j == 0) ? ((k == 0) ? 0 : 8) : ((k == 0) ? 2 : 10);
      l = i;
    } else if (!bj) {  // along y: edges 3 (x0z0: 0->3), 1 (x1z0: 1->2), 11 (x0z1: 4->7), 9 (x1z1: 5->6)
      e = (i == 0) ? ((k == 0) ? 3 : 11) : ((k == 0) ? 1 : 9);
      l = j;
    } else {  // along z: edges 4 (0->4), 5 (1->5), 6 (2->6), 7 (3->7)
      e = (i == 0) ? ((j == 0) ? 4 : 7) : ((j == 0) ? 5 : 6);
      l = k;
    }
    return eoff + e * m + (l - 1);
  }
  if (nb == 1) {
    int f, p, q;
    if (bi) { f = (i == 0) ? 0 : 5; p = j; q = k; }
    else if (bj) { f = (j == 0) ? 1 : 4; p = i; q = k; }
    else { f = (k == 0) ? 2 : 3; p = i; q = j; }
    return foff + f * m * m + (p - 1) * m + (q - 1);
  }
  return ioff + ((i - 1) * m + (j - 1)) * m + (k - 1);
}

template <int N>
struct StaticG {
  double g[N * N];  // g[a*N + b] = phi_a'(x_b)
};

// Element-local product of one element per CTA iteration, N*N threads, thread
// (i,j) owning the z-line; reference-layout inputs (Nodle rows and factors in
// local order).  Writes the element-local result into the scratch array.
template <int N>
__global__ void __launch_bounds__(N* N)
    k_static_local(const int* __restrict__ nodle, const double* __restrict__ fac, const double* __restrict__ x,
                   double* __restrict__ scratch, int n_elt, int n_dof, const StaticG<N> G) {
  constexpr int Q = N * N * N, NN = N * N;
  __shared__ double s_u[Q], s_vx[Q], s_vy[Q];
  const int i = threadIdx.x % N, j = threadIdx.x / N;
  int q[N];
#pragma unroll
  for (int k = 0; k < N; k++) q[k] = local_index(N - 1, i, j, k);
  for (int e = blockIdx.x; e < n_elt; e += gridDim.x) {
    const size_t base = (size_t)e * Q;
    double u[N];
#pragma unroll
    for (int k = 0; k < N; k++) {
      const int d = nodle[base + q[k]];
      const bool ok = (d >= 0 && d < n_dof);
      if (!ok) g_static_bad_index = 1;
      u[k] = ok ? x[d] : 0.0;
      s_u[k * NN + j * N + i] = u[k];
    }
    __syncthreads();
    double vz[N];
#pragma unroll
    for (int k = 0; k < N; k++) {
      double gx = 0, gy = 0, gz = 0;
#pragma unroll
      for (int a = 0; a < N; a++) {
        gz += G.g[a * N + k] * u[a];
        gx += G.g[a * N + i] * s_u[k * NN + j * N + a];
        gy += G.g[a * N + j] * s_u[k * NN + a * N + i];
      }
      const double* b = fac + (base + q[k]) * 6;
      s_vx[k * NN + j * N + i] = b[0] * gx + b[1] * gy + b[2] * gz;
      s_vy[k * NN + j * N + i] = b[1] * gx + b[3] * gy + b[4] * gz;
      vz[k] = b[2] * gx + b[4] * gy + b[5] * gz;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < N; k++) {
      double y = 0;
#pragma unroll
      for (int a = 0; a < N; a++) {
        y += G.g[i * N + a] * s_vx[k * NN + j * N + a];
        y += G.g[j * N + a] * s_vy[k * NN + a * N + i];
        y += G.g[k * N + a] * vz[a];
      }
      scratch[base + q[k]] = y;
    }
    __syncthreads();
  }
}

__global__ void k_static_scale(double* __restrict__ y, double beta, int n) {
  for (int d = blockIdx.x * blockDim.x + threadIdx.x; d < n; d += gridDim.x * blockDim.x)
    y[d] = (beta == 0.0) ? 0.0 : beta * y[d];
}

__global__ void k_static_scatter(const int* __restrict__ nodle, const double* __restrict__ scratch, double alpha,
                                 double* __restrict__ y, long long total, int n_dof) {
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < total;
       p += (long long)gridDim.x * blockDim.x) {
    const int d = nodle[p];
    if (d >= 0 && d < n_dof) atomicAdd(y + d, alpha * scratch[p]);
  }
}

__global__ void k_static_clear_flag() { g_static_bad_index = 0; }

template <int N>
int static_launch(int n_elt, int n_dof, const int32_t* nodle, const double* factors, double alpha, const double* x,
                  double beta, double* y, cudaStream_t s, double* scratch) {
  StaticG<N> G;
  double pts[kMaxN], wts[kMaxN], g[kMaxN * kMaxN];
  gauss_lobatto(N - 1, pts, wts);
  gl_derivative_matrix(N - 1, pts, g);
  for (int a = 0; a < N * N; a++) G.g[a] = g[a];
  const int blocks = (int)std::min<long long>(n_elt, (long long)sm_count() * 16);
  k_static_clear_flag<<<1, 1, 0, s>>>();
  k_static_local<N><<<blocks, N * N, 0, s>>>(nodle, factors, x, scratch, n_elt, n_dof, G);
  const int sb = (int)std::min<long long>((n_dof + 255) / 256, (long long)sm_count() * 16);
  k_static_scale<<<sb, 256, 0, s>>>(y, beta, n_dof);
  const long long total = (long long)n_elt * N * N * N;
  const int pb = (int)std::min<long long>((total + 255) / 256, (long long)sm_count() * 16);
  k_static_scatter<<<pb, 256, 0, s>>>(nodle, scratch, alpha, y, total, n_dof);
  count_launch(4);
  MJ_CUDA(cudaGetLastError());
  return MJ_OK;
}

}  // namespace
}  // namespace mj

using namespace mj;

extern "C" int mj_stiffness_mltadd_static(int order, int n_elt, int n_dof, const int32_t* nodle,
                                          const double* factors, double alpha, const double* x, double beta,
                                          double* y, void* stream) {
  MJ_CHECK_ARG(order >= 1 && order <= kMaxOrder, "mj_stiffness_mltadd_static: order must be in [1, 8]");
  MJ_CHECK_ARG(n_elt > 0 && n_dof > 0, "mj_stiffness_mltadd_static: empty mesh");
  MJ_CHECK_ARG(nodle && factors && x && y, "mj_stiffness_mltadd_static: null device pointer");
  const long long points = (long long)n_elt * (order + 1) * (order + 1) * (order + 1);
  if (points > (long long)kStaticScratchPoints) {
    set_error("mj_stiffness_mltadd_static: n_elt*(order+1)^3 = " + std::to_string(points) +
              " exceeds the static scratch of " + std::to_string(kStaticScratchPoints) + " values");
    return MJ_ERR_ARG;
  }
  // The device addresses of the scratch array and the flag in the current
  // device's context (the host-side symbols are only stand-ins).  Looked up on
  // every call: the lookup allocates nothing, and an address kept from an
  // earlier call would dangle once that context is destroyed (cudaDeviceReset)
  // and the library's device code is loaded again.  The first lookup on a
  // device loads that code, which is why the first call comes before any
  // stream capture.
  void* p = nullptr;
  void* f = nullptr;
  MJ_CUDA(cudaGetSymbolAddress(&p, g_static_scratch));
  MJ_CUDA(cudaGetSymbolAddress(&f, g_static_bad_index));
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  double* scratch = static_cast<double*>(p);
  int rc = MJ_OK;
  switch (order + 1) {
    case 2: rc = static_launch<2>(n_elt, n_dof, nodle, factors, alpha, x, beta, y, s, scratch); break;
    case 3: rc = static_launch<3>(n_elt, n_dof, nodle, factors, alpha, x, beta, y, s, scratch); break;
    case 4: rc = static_launch<4>(n_elt, n_dof, nodle, factors, alpha, x, beta, y, s, scratch); break;
    case 5: rc = static_launch<5>(n_elt, n_dof, nodle, factors, alpha, x, beta, y, s, scratch); break;
    case 6: rc = static_launch<6>(n_elt, n_dof, nodle, factors, alpha, x, beta, y, s, scratch); break;
    case 7: rc = static_launch<7>(n_elt, n_dof, nodle, factors, alpha, x, beta, y, s, scratch); break;
    case 8: rc = static_launch<8>(n_elt, n_dof, nodle, factors, alpha, x, beta, y, s, scratch); break;
    case 9: rc = static_launch<9>(n_elt, n_dof, nodle, factors, alpha, x, beta, y, s, scratch); break;
  }
  if (rc) return rc;
  MJ_CUDA(cudaStreamSynchronize(s));
  int bad = 0;
  MJ_CUDA(cudaMemcpy(&bad, f, sizeof(int), cudaMemcpyDeviceToHost));
  if (bad) {
    set_error("mj_stiffness_mltadd_static: a Nodle entry is outside [0, n_dof); those entries were skipped");
    return MJ_ERR_ARG;
  }
  return MJ_OK;
}
