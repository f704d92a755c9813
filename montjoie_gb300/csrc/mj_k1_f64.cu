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
}  // namespace mj
