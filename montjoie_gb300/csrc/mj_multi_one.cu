// Single-order instances of the many-mesh batch step: a batch whose meshes
// all have one order runs k_mesh_batch_step<T, n>, which holds that order's
// element code alone.  Kept in their own translation unit so they compile in
// parallel with the all-orders kernels of mj_multi.cu.
#include "mj_multi_kernel.cuh"

namespace mj {
namespace {

template <int T>
const void* one_order(int n) {
  switch (n) {
    case 2: return reinterpret_cast<const void*>(k_mesh_batch_step<T, 2>);
    case 3: return reinterpret_cast<const void*>(k_mesh_batch_step<T, 3>);
    case 4: return reinterpret_cast<const void*>(k_mesh_batch_step<T, 4>);
    case 5: return reinterpret_cast<const void*>(k_mesh_batch_step<T, 5>);
    case 6: return reinterpret_cast<const void*>(k_mesh_batch_step<T, 6>);
    case 7: return reinterpret_cast<const void*>(k_mesh_batch_step<T, 7>);
    case 8: return reinterpret_cast<const void*>(k_mesh_batch_step<T, 8>);
    case 9: return reinterpret_cast<const void*>(k_mesh_batch_step<T, 9>);
  }
  return nullptr;
}

}  // namespace

const void* mb_one_order_kernel(int threads, int n) {
  return threads == 256 ? one_order<256>(n) : threads == 128 ? one_order<128>(n) : nullptr;
}

int mb_one_order_set_gmat(int n, const float* v) {
  MJ_CUDA(cudaMemcpyToSymbol(c_gmat32, v, sizeof(float) * n * n, sizeof(float) * kMaxNK * kMaxNK * n));
  return MJ_OK;
}

}  // namespace mj
