// Single-RHS element kernels in FP64 (the plain form).
#define MJ_REAL double
#define MJ_HAS_VEC false  // instantiate the vector-line work layout too
#include "mj_k1_inst.cuh"

namespace mj {
int k1_set_gmat_f64(int n, const double* g) { return set_gmat(n, g); }
int k1_prepare_f64(int n, int E, bool vec, int* ctas) { return prepare_any(n, E, vec, ctas); }
void k1_launch_f64(int n, int E, bool vec, int grid, const void* x, const int* nodle_e, const void* fac_e,
                   void* R, const int* slot_e, int n_tiles, int* err, cudaStream_t s) {
  launch_any(n, E, vec, grid, x, nodle_e, fac_e, R, slot_e, n_tiles, err, s);
}

bool k1_launch_f64_waits_out(int n, int E, int grid, const void* x, const int* nodle_e, const void* fac_e,
                             void* R, const int* slot_e, int n_tiles, int* err, cudaStream_t s) {
  if (n != 5 || E != 4) return false;
  using P = K1Plan<double, 5, 4, 1, false>;
  auto* k = k_local_stiffness<double, 5, 4, false, 0>;
  if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)P::total) != cudaSuccess)
    return false;
  k<<<grid, P::threads, P::total, s>>>(static_cast<const double*>(x), nodle_e, static_cast<const double*>(fac_e),
                                       static_cast<double*>(R), slot_e, n_tiles, err);
  return true;
}
}  // namespace mj
