// Single-RHS element kernels in FP32 (the chosen form).
#define MJ_REAL float
#define MJ_HAS_VEC true  // instantiate the vector-line work layout too
#include "mj_k1_inst.cuh"

namespace mj {
int k1_set_gmat_f32(int n, const double* g) {
  const int rc = set_gmat(n, g);
  return rc ? rc : k1_set_gmat_fs(n, g);  // and the one-factor-stage unit's copy
}
int k1_prepare_f32(int n, int E, bool vec, int* ctas) { return prepare_any(n, E, vec, ctas); }
void k1_launch_f32(int n, int E, bool vec, int grid, const void* x, const int* nodle_e, const void* fac_e,
                   void* R, const int* slot_e, int n_tiles, int* err, cudaStream_t s) {
  launch_any(n, E, vec, grid, x, nodle_e, fac_e, R, slot_e, n_tiles, err, s);
}

// warp-per-element layout, order 4 (n = 5): E warps per CTA
namespace {
template <int E, bool PK>
int prepare_w_one(int* ctas) {
  using P = K1Plan<float, 5, E, 1, false>;
  auto* k = k_local_stiffness_w<float, 5, E, kSpinLimit, PK>;
  MJ_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)P::total));
  MJ_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(ctas, k, E * 32, P::total));
  if (*ctas < 1) {
    set_error("element kernel variant cannot be resident");
    return MJ_ERR_ARG;
  }
  return MJ_OK;
}
template <int E, bool PK>
void launch_w_one(int grid, const void* x, const int* nodle_e, const void* fac_e, void* R, const int* slot_e,
                  int n_tiles, int* err, cudaStream_t s) {
  using P = K1Plan<float, 5, E, 1, false>;
  k_local_stiffness_w<float, 5, E, kSpinLimit, PK><<<grid, E * 32, P::total, s>>>(
      static_cast<const float*>(x), nodle_e, static_cast<const float*>(fac_e), static_cast<float*>(R), slot_e,
      n_tiles, err);
}
}  // namespace

bool k1_launch_w_f32_waits_out(int n, int E, int grid, const void* x, const int* nodle_e, const void* fac_e,
                               void* R, const int* slot_e, int n_tiles, int* err, cudaStream_t s) {
  if (n != 5 || E != 2) return false;
  using P = K1Plan<float, 5, 2, 1, false>;
  auto* k = k_local_stiffness_w<float, 5, 2, 0>;
  if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)P::total) != cudaSuccess)
    return false;
  k<<<grid, 2 * 32, P::total, s>>>(static_cast<const float*>(x), nodle_e, static_cast<const float*>(fac_e),
                                    static_cast<float*>(R), slot_e, n_tiles, err);
  return true;
}

std::vector<int> k1_warp_tile_candidates(int n) {
  return n == 5 ? std::vector<int>{1, 2, 3, 4, 5, 6, 8, 10} : std::vector<int>{};
}

#define MJ_W_TILES(X) X(1) X(2) X(3) X(4) X(5) X(6) X(8) X(10)

int k1_prepare_w_f32(int n, int E, bool packed, int* ctas) {
#define MJ_X(EV)                                                                 \
  if (n == 5 && E == EV) return packed ? prepare_w_one<EV, true>(ctas) : prepare_w_one<EV, false>(ctas);
  MJ_W_TILES(MJ_X)
#undef MJ_X
  set_error("no warp-per-element kernel variant for this order and tile size");
  return MJ_ERR_ARG;
}

void k1_launch_w_f32(int n, int E, bool packed, int grid, const void* x, const int* nodle_e, const void* fac_e,
                     void* R, const int* slot_e, int n_tiles, int* err, cudaStream_t s) {
#define MJ_X(EV)                                                                                      \
  if (n == 5 && E == EV) {                                                                            \
    if (packed) launch_w_one<EV, true>(grid, x, nodle_e, fac_e, R, slot_e, n_tiles, err, s);          \
    else launch_w_one<EV, false>(grid, x, nodle_e, fac_e, R, slot_e, n_tiles, err, s);                \
    return;                                                                                           \
  }
  MJ_W_TILES(MJ_X)
#undef MJ_X
}
#undef MJ_W_TILES

std::vector<int> k1_tile_candidates(int n) {
  switch (n) {
    case 2: return {30, 60};
    case 3: return {12, 24};
    case 4: return {8, 16};
    case 5: return {4, 5, 8, 10};
    case 6: return {3, 4, 6};
    case 7: return {2, 3, 4, 5};
    case 8: return {2, 3, 4};
    case 9: return {1, 2, 3};
  }
  return {};
}
}  // namespace mj
