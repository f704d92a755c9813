// The one-kernel leap-frog step with the adjoint's gradient term: the EN form
// of k_rhs_step (mj_rhs_step.cuh), in a unit of its own so that the plain
// step's unit compiles no larger.  An adjoint step of the discrete adjoint
// computes A_e lambda^{m+1} for every element; the EN form dots it with the
// forward state U^m in the same pass, in place of a second element pass over
// the mesh (the ENERGY variant of k_local_stiffness_rhs) whose sums it
// reproduces bit for bit.
#include <cuda_runtime.h>

#include "mj_rhs_step.cuh"

namespace mj {

namespace {
size_t en_smem(int base, int E, int S, int n) { return (size_t)base + (size_t)E * S * n * n * sizeof(float); }
}  // namespace

int rs_en_prepare(int n, int E, int LB, int V, int S, int* ctas) {
  *ctas = 0;
  int dev = 0, optin = 0;
  MJ_CUDA(cudaGetDevice(&dev));
  MJ_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
#define MJ_X(N_, E_, LB_, V_)                                                                                     \
  if (n == N_ && E == E_ && LB == LB_ && V == V_) {                                                               \
    using P = RsPlan<N_, E_, LB_, V_>;                                                                            \
    const size_t smem = en_smem(P::kSmem, E_, S, N_);                                                             \
    if (smem > (size_t)optin) return MJ_OK;                                                                       \
    MJ_CUDA(cudaFuncSetAttribute(k_rhs_step<N_, E_, LB_, V_, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                                 (int)smem));                                                                     \
    MJ_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(ctas, k_rhs_step<N_, E_, LB_, V_, true>, P::T, smem)); \
    return MJ_OK;                                                                                                 \
  }
  MJ_RS_VARIANTS(MJ_X)
#undef MJ_X
  set_error("no many-source step variant");
  return MJ_ERR_ARG;
}

int rs_en_launch(int n, int E, int LB, int V, int S, int grid, const RsParams& prm, const RsChunk* chunks,
                 int n_chunks, SyncState* sync, int par, int* err, cudaStream_t s) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  unsigned long long* no_stamps = nullptr;
#define MJ_X(N_, E_, LB_, V_)                                                                                     \
  if (n == N_ && E == E_ && LB == LB_ && V == V_) {                                                               \
    using P = RsPlan<N_, E_, LB_, V_>;                                                                            \
    cfg.blockDim = dim3(P::T);                                                                                    \
    cfg.dynamicSmemBytes = en_smem(P::kSmem, E_, S, N_);                                                          \
    MJ_CUDA(cudaLaunchKernelEx(&cfg, k_rhs_step<N_, E_, LB_, V_, true>, prm, chunks, n_chunks, sync, par, err,   \
                               no_stamps));                                                                       \
    count_launch();                                                                                               \
    return MJ_OK;                                                                                                 \
  }
  MJ_RS_VARIANTS(MJ_X)
#undef MJ_X
  set_error("no many-source step variant");
  return MJ_ERR_ARG;
}

int rs_en_set_gmat(int n, const float* g) {
  MJ_CUDA(cudaMemcpyToSymbol(c_gmat32, g, sizeof(float) * n * n, sizeof(float) * kMaxNK * kMaxNK * n));
  return MJ_OK;
}

}  // namespace mj
