// Element kernels with one factor stage (k_local_stiffness_fs), FP32: every
// (order, tile size) of the compact layout's table, in a translation unit of
// their own so the build compiles them beside the others.
#include "mj_internal.cuh"
#include "mj_k1.cuh"

namespace mj {
namespace {

template <int N, int E>
int prepare_fs_one(int* ctas) {
  using P = K1PlanFS<float, N, E>;
  int dev = 0, optin = 0;
  MJ_CUDA(cudaGetDevice(&dev));
  MJ_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  if ((int)P::total > optin) {
    set_error("element kernel variant does not fit in shared memory");
    return MJ_ERR_ARG;
  }
  MJ_CUDA(cudaFuncSetAttribute(k_local_stiffness_fs<float, N, E>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)P::total));
  MJ_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(ctas, k_local_stiffness_fs<float, N, E>, P::threads,
                                                        P::total));
  if (*ctas < 1) {
    set_error("element kernel variant cannot be resident");
    return MJ_ERR_ARG;
  }
  return MJ_OK;
}

template <int N, int E>
void launch_fs_one(int grid, const void* x, const int* nodle_e, const void* fac_e, void* R, const int* slot_e,
                   int n_tiles, int* err, cudaStream_t s) {
  using P = K1PlanFS<float, N, E>;
  k_local_stiffness_fs<float, N, E><<<grid, P::threads, P::total, s>>>(
      static_cast<const float*>(x), nodle_e, static_cast<const float*>(fac_e), static_cast<float*>(R), slot_e,
      n_tiles, err);
}

// (n, E) table: the compact layout's (k1_tile_candidates)
#define MJ_K1FS_VARIANTS(X) \
  X(2, 30) X(2, 60) X(3, 12) X(3, 24) X(4, 8) X(4, 16) X(5, 4) X(5, 5) X(5, 8) X(5, 10) \
  X(6, 3) X(6, 4) X(6, 6) X(7, 2) X(7, 3) X(7, 4) X(7, 5) X(8, 2) X(8, 3) X(8, 4) X(9, 1) X(9, 2) X(9, 3)

}  // namespace

// The derivative matrix of order n in this unit's constant bank (each unit
// that instantiates element kernels holds its own copy).
int k1_set_gmat_fs(int n, const double* g) {
  float v[kMaxNK * kMaxNK];
  for (int a = 0; a < n * n; a++) v[a] = float(g[a]);
  MJ_CUDA(cudaMemcpyToSymbol(c_gmat32, v, sizeof(float) * n * n, sizeof(float) * kMaxNK * kMaxNK * n));
  return MJ_OK;
}

int k1_prepare_fs_f32(int n, int E, int* ctas) {
#define MJ_X(NV, EV) \
  if (n == NV && E == EV) return prepare_fs_one<NV, EV>(ctas);
  MJ_K1FS_VARIANTS(MJ_X)
#undef MJ_X
  set_error("no one-factor-stage element kernel variant for this order and tile size");
  return MJ_ERR_ARG;
}

void k1_launch_fs_f32(int n, int E, int grid, const void* x, const int* nodle_e, const void* fac_e, void* R,
                      const int* slot_e, int n_tiles, int* err, cudaStream_t s) {
#define MJ_X(NV, EV)                                                                 \
  if (n == NV && E == EV) {                                                          \
    launch_fs_one<NV, EV>(grid, x, nodle_e, fac_e, R, slot_e, n_tiles, err, s);      \
    return;                                                                          \
  }
  MJ_K1FS_VARIANTS(MJ_X)
#undef MJ_X
}

}  // namespace mj
