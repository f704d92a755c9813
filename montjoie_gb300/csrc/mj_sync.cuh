// Grid-wide synchronisation of the cooperative persistent kernels (the mesh
// batch and the many-source step): a counter-and-generation barrier whose
// wait is bounded in time and in polls, reporting through an error flag.
// Only valid under a cooperative launch, which guarantees that every CTA of
// the grid is resident.
#pragma once

#include <cuda_runtime.h>

#include "mj_wait.cuh"

namespace mj {

struct SyncState {
  unsigned count;  // arrivals at the barrier
  unsigned gen;    // barrier generation
};

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Grid-wide barrier of a cooperative launch.  Thread 0 of each CTA arrives on
// a counter; the last arrival resets it and bumps the generation the others
// wait on.  The wait gives up after c_wait.barrier_ns (2 s) or
// c_wait.barrier_polls (2^26) polls, whichever comes first, unless a test
// lowered them: the CTA then sets *err = 2 and the barrier reports failure.
// The host resets the counter and generation after a failure.
__device__ __forceinline__ bool grid_barrier(SyncState* s, int* err) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    const unsigned g0 = ld_acquire(&s->gen);
    __threadfence();
    if (atomicAdd(&s->count, 1u) == gridDim.x - 1) {
      atomicExch(&s->count, 0u);
      __threadfence();
      atomicAdd(&s->gen, 1u);
    } else {
      const unsigned long long t0 = global_ns();
      for (long it = 0; ld_acquire(&s->gen) == g0; ++it) {
        if (it > c_wait.barrier_polls || global_ns() - t0 > c_wait.barrier_ns) {
          ok = 0;
          atomicExch(err, 2);
          break;
        }
        __nanosleep(100);
      }
    }
    __threadfence();
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

}  // namespace mj
