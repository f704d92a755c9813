// Shared host/device helpers of the montjoie_gb300 library.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include "montjoie_gb300.h"

namespace mj {

// Largest supported order r (n = r + 1 points per axis).
constexpr int kMaxOrder = 8;
constexpr int kMaxN = kMaxOrder + 1;

// Element count padding of the element-major layout: a multiple of every
// tile size the element kernels use, so any of them covers the mesh with
// whole tiles of empty (zero) padding elements.
constexpr int kElemPad = 240;

// Slots per element: n^3 rounded up to 4, so per-element blocks of int32,
// float and double start on 16-byte boundaries (the bulk-copy rule).
__host__ __device__ constexpr int elem_slots(int n) { return (n * n * n + 3) / 4 * 4; }

void set_error(const std::string& msg);
std::atomic<uint64_t>& launch_counter();

inline void count_launch(uint64_t n = 1) { launch_counter().fetch_add(n, std::memory_order_relaxed); }

// Evaluates a CUDA call; on failure records the error and returns MJ_ERR_CUDA
// (MJ_ERR_NOMEM for allocation failures) from the calling function.
#define MJ_CUDA(call)                                                                       \
  do {                                                                                      \
    cudaError_t mj_err_ = (call);                                                           \
    if (mj_err_ != cudaSuccess) {                                                           \
      ::mj::set_error(std::string(#call) + ": " + cudaGetErrorString(mj_err_));             \
      return mj_err_ == cudaErrorMemoryAllocation ? MJ_ERR_NOMEM : MJ_ERR_CUDA;             \
    }                                                                                       \
  } while (0)

#define MJ_CHECK_ARG(cond, msg)            \
  do {                                     \
    if (!(cond)) {                         \
      ::mj::set_error(msg);                \
      return MJ_ERR_ARG;                   \
    }                                      \
  } while (0)

// Device buffer owned by the library (cudaMalloc/cudaFree).
struct DevBuf {
  void* ptr = nullptr;
  size_t bytes = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() { release(); }
  void release() {
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    bytes = 0;
  }
  cudaError_t alloc(size_t b) {
    release();
    bytes = b;
    if (b == 0) return cudaSuccess;
    return cudaMalloc(&ptr, b);
  }
  template <class T>
  T* as() const { return static_cast<T*>(ptr); }
};

// Local numbering NumDofs3D of a Q_r hexahedron, num[(i*n+j)*n+k] = local
// index of the node (i,j,k) (i along x): vertices, the 12 edges, the faces
// x=0, y=0, z=0, z=1, y=1, x=1, then the interior
// (MONTJOIE/src/Quadrature/HexahedronQuadrature.cxx:51-171).
std::vector<int> hex_local_numbering(int r);

// Gauss-Lobatto points and weights on [0,1] (r+1 points) and the derivative
// matrix g[a*n+b] = phi_a'(x_b) (MONTJOIE/src/Quadrature/GaussLobatto.cxx:175-191).
void gauss_lobatto(int r, double* pts, double* wts);
void gl_derivative_matrix(int r, const double* pts, double* g);

int sm_count();

// Reads a kernel's device error flag after the work on `s`; when it is set,
// clears it (so the next call starts clean), records "<what>: <message>" and
// returns MJ_ERR_CUDA.  Synchronises `s`.
int take_kernel_error(void* dev_flag, cudaStream_t s, const char* what);

}  // namespace mj
