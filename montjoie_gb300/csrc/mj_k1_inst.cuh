// Instantiation and dispatch of the single-RHS element kernel for one
// precision (included by mj_k1_f64.cu and mj_k1_f32.cu with MJ_REAL set).
#pragma once

#include "mj_internal.cuh"
#include "mj_k1.cuh"

namespace mj {
namespace {

using Real = MJ_REAL;

template <int N, int E, bool VEC>
int prepare_one(int* ctas) {
  using P = K1Plan<Real, N, E, 1, VEC>;
  int dev = 0, optin = 0;
  MJ_CUDA(cudaGetDevice(&dev));
  MJ_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  if ((int)P::total > optin) {
    set_error("element kernel variant does not fit in shared memory");
    return MJ_ERR_ARG;
  }
  MJ_CUDA(cudaFuncSetAttribute(k_local_stiffness<Real, N, E, VEC>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)P::total));
  MJ_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(ctas, k_local_stiffness<Real, N, E, VEC>, P::threads,
                                                        P::total));
  if (*ctas < 1) {
    set_error("element kernel variant cannot be resident");
    return MJ_ERR_ARG;
  }
  return MJ_OK;
}

template <int N, int E, bool VEC>
void launch_one(int grid, const void* x, const int* nodle_e, const void* fac_e, void* R, const int* slot_e,
                int n_tiles, int* err, cudaStream_t s) {
  using P = K1Plan<Real, N, E, 1, VEC>;
  k_local_stiffness<Real, N, E, VEC><<<grid, P::threads, P::total, s>>>(static_cast<const Real*>(x), nodle_e,
                                                                        static_cast<const Real*>(fac_e),
                                                                        static_cast<Real*>(R), slot_e, n_tiles, err);
}

// (n, E) table: keep in step with k1_tile_candidates.
#define MJ_K1_VARIANTS(X) \
  X(2, 30) X(2, 60) X(3, 12) X(3, 24) X(4, 8) X(4, 16) X(5, 4) X(5, 5) X(5, 8) X(5, 10) \
  X(6, 3) X(6, 4) X(6, 6) X(7, 2) X(7, 3) X(7, 4) X(7, 5) X(8, 2) X(8, 3) X(8, 4) X(9, 1) X(9, 2) X(9, 3)

int prepare_any(int n, int E, bool vec, int* ctas) {
#define MJ_X(NV, EV)                                                       \
  if (n == NV && E == EV) {                                                \
    if (vec && MJ_HAS_VEC) return prepare_one<NV, EV, MJ_HAS_VEC>(ctas);   \
    return prepare_one<NV, EV, false>(ctas);                               \
  }
  MJ_K1_VARIANTS(MJ_X)
#undef MJ_X
  set_error("no element kernel variant for this order and tile size");
  return MJ_ERR_ARG;
}

void launch_any(int n, int E, bool vec, int grid, const void* x, const int* nodle_e, const void* fac_e, void* R,
                const int* slot_e, int n_tiles, int* err, cudaStream_t s) {
#define MJ_X(NV, EV)                                                                          \
  if (n == NV && E == EV) {                                                                   \
    if (vec && MJ_HAS_VEC)                                                                    \
      launch_one<NV, EV, MJ_HAS_VEC>(grid, x, nodle_e, fac_e, R, slot_e, n_tiles, err, s);    \
    else                                                                                      \
      launch_one<NV, EV, false>(grid, x, nodle_e, fac_e, R, slot_e, n_tiles, err, s);         \
    return;                                                                                   \
  }
  MJ_K1_VARIANTS(MJ_X)
#undef MJ_X
}

int set_gmat(int n, const double* g) {
  Real v[kMaxNK * kMaxNK];
  for (int a = 0; a < n * n; a++) v[a] = Real(g[a]);
  const size_t off = sizeof(Real) * kMaxNK * kMaxNK * n;
  if (sizeof(Real) == sizeof(double)) MJ_CUDA(cudaMemcpyToSymbol(c_gmat64, v, sizeof(Real) * n * n, off));
  else MJ_CUDA(cudaMemcpyToSymbol(c_gmat32, v, sizeof(Real) * n * n, off));
  return MJ_OK;
}

}  // namespace
}  // namespace mj
