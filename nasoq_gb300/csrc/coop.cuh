// Cooperative-launch helpers shared by the multi-CTA kernels of wide
// supernodes: the control block and a bounded grid-wide barrier.
#pragma once
#include <cuda_runtime.h>

#include <cstddef>

#include "plan.hpp"

namespace nqg {

struct WideCtl {
  unsigned count;
  unsigned gen;
  int abort;
  int kb;          // columns completed by the last panel launch
  int pivoted;     // any interchange in this supernode
  int stop;        // the fast panel stopped where a pivot search is needed
  int halt;        // a speculative fast panel stopped early: later queued kernels skip
  int pad;
  int kb_log[16];  // columns done by each fast panel of a speculative batch
  double cval[2][1024];
  int cidx[2][1024];
  double rval[2][1024];
  int ridx[2][1024];
  // panel exchanges: per CTA and parity, (candidate << 8) | epoch; cleared
  // before every panel launch
  unsigned long long pslot[2][1024];
  // fast panels: up to four candidate words per CTA and exchange
  unsigned long long mslot[2][4][1024];
  // polls before a cross-CTA wait gives up (0: SPIN_LIMIT); kept across the
  // per-supernode resets, which clear the fields above only
  long long spin_limit;
};

constexpr long long SPIN_LIMIT = 1ll << 26;  // default polls before a wait gives up

__device__ __forceinline__ long long wait_limit(const WideCtl *ctl) {
  const long long v = *(volatile const long long *)&ctl->spin_limit;
  return v > 0 ? v : SPIN_LIMIT;
}

// Grid-wide barrier for a cooperative launch, sense-reversing on ctl->gen.
// Returns false once any CTA has timed out (all CTAs then unwind).
__device__ __forceinline__ bool grid_sync(WideCtl *ctl, int *status) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    volatile unsigned *vgen = &ctl->gen;
    volatile int *vab = &ctl->abort;
    unsigned my = *vgen;
    __threadfence();
    unsigned arrived = atomicAdd(&ctl->count, 1u);
    if (arrived == gridDim.x - 1) {
      ctl->count = 0;
      __threadfence();
      atomicAdd(&ctl->gen, 1u);
    } else {
      long long it = 0;
      const long long lim = wait_limit(ctl);
      while (*vgen == my) {
        if (*vab) {
          ok = 0;
          break;
        }
        if (++it > lim) {
          atomicOr(status, ST_TIMEOUT);
          atomicExch(&ctl->abort, 1);
          ok = 0;
          break;
        }
        __nanosleep(32);
      }
    }
    __threadfence();
    if (*vab) ok = 0;
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}


}  // namespace nqg
