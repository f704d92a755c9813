// Single-RHS element kernels in FP32 (the chosen form).
#define MJ_REAL float
#define MJ_HAS_VEC true  // instantiate the vector-line work layout too
#include "mj_k1_inst.cuh"

namespace mj {
int k1_set_gmat_f32(int n, const double* g) { return set_gmat(n, g); }
int k1_prepare_f32(int n, int E, bool vec, int* ctas) { return prepare_any(n, E, vec, ctas); }
void k1_launch_f32(int n, int E, bool vec, int grid, const void* x, const int* nodle_e, const void* fac_e,
                   void* R, const int* slot_e, int n_tiles, int* err, cudaStream_t s) {
  launch_any(n, E, vec, grid, x, nodle_e, fac_e, R, slot_e, n_tiles, err, s);
}

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
