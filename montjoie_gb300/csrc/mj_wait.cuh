// Limits of the bounded waits, and the test hook that lowers them.
//
// Every wait of this library's kernels, on a bulk copy (mbarrier) or on the
// other CTAs of a cooperative launch (grid barrier), is bounded.  A wait that
// runs out sets the kernel's error flag; the CTA then waits, with the full
// limit, for its own copies still in flight and returns, and the entry point
// reports the failure with a message.
// - mbarrier waits poll at most kSpinLimit times, a compile-time bound (a
//   limit read from memory changes the register allocation of the element
//   kernels and slows them); the test hook instead switches two element-kernel
//   variants to instances compiled with a limit of 0 (mj_k1_f32.cu, mj_k1_f64.cu).
// - The grid barrier's limits live in constant memory, one copy per
//   translation unit that launches cooperative kernels; each unit registers a
//   setter at load so that mj_debug_set_wait_limits can lower them all.
// Either way a test can make a wait run out with no fault and no hang.
#pragma once

#include <cuda_runtime.h>

namespace mj {

constexpr long kSpinLimit = 1L << 22;                     // polls of an mbarrier wait
constexpr long kBarrierPolls = 1L << 26;                  // polls of a grid-barrier wait
constexpr unsigned long long kBarrierNs = 2000000000ull;  // and its time bound (2 s)

struct WaitLimits {
  long barrier_polls;
  unsigned long long barrier_ns;
};

static __constant__ WaitLimits c_wait = {kBarrierPolls, kBarrierNs};

// Host switch of the test hook: element-kernel launches use their instances
// compiled with a bulk-copy wait limit of 0 where one exists (mj_op.cu).
bool& k1_waits_run_out();

using WaitLimitSetter = int (*)(const WaitLimits&);
// Records a unit's setter (defined in mj_op.cu; safe during static initialisation).
void register_wait_limit_setter(WaitLimitSetter f);

namespace {
int set_wait_limits_here(const WaitLimits& w) {
  return cudaMemcpyToSymbol(c_wait, &w, sizeof(WaitLimits)) == cudaSuccess ? 0 : 1;
}
struct WaitLimitRegistration {
  WaitLimitRegistration() { register_wait_limit_setter(&set_wait_limits_here); }
};
static WaitLimitRegistration g_wait_limit_registration;
}  // namespace

}  // namespace mj
