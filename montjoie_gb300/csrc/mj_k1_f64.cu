// Single-RHS element kernels in FP64 (the plain form).
#define MJ_REAL double
#include "mj_k1_inst.cuh"

namespace mj {
int k1_set_gmat_f64(int n, const double* g) { return set_gmat(n, g); }
int k1_prepare_f64(int n, int E, int* ctas) { return prepare_any(n, E, ctas); }
void k1_launch_f64(int n, int E, int grid, const void* x, const int* nodle_e, const void* fac_e, void* R, int n_tiles,
                   int* err, cudaStream_t s) {
  launch_any(n, E, grid, x, nodle_e, fac_e, R, n_tiles, err, s);
}
}  // namespace mj
