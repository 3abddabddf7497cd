// Software grid barrier for cooperative (all blocks resident) launches.
//
// Thread 0 of each block arrives on a counter; the last to arrive resets it
// and advances a generation word that the others poll.  Every wait is
// bounded: after `max_polls` polls (100 ns sleep each) the block records a
// fault and returns false; blocks that reach a barrier after a fault return
// false at once.  Callers return from the kernel on false, and the host turns
// the fault word into an error status, so a lost block never hangs the GPU.
#pragma once

#include "common.cuh"

namespace gbf {

struct GridBarrier {
  unsigned int count, gen;
  int fault, pad;
};

constexpr long long kBarrierPolls = 1LL << 24;  // ~2 s with the 100 ns sleeps

__device__ __forceinline__ bool grid_barrier(GridBarrier* bar, unsigned int nblocks,
                                             long long max_polls = kBarrierPolls) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    volatile unsigned int* vgen = &bar->gen;
    volatile int* vfault = &bar->fault;
    const unsigned int g = *vgen;
    __threadfence();
    if (atomicAdd(&bar->count, 1u) == nblocks - 1) {
      atomicExch(&bar->count, 0u);
      __threadfence();
      atomicAdd(&bar->gen, 1u);
    } else {
      long long polls = 0;
      while (*vgen == g) {
        if (*vfault != 0 || ++polls > max_polls) {
          atomicExch(&bar->fault, 1);
          ok = 0;
          break;
        }
        __nanosleep(100);
      }
    }
    __threadfence();
    if (*vfault != 0) ok = 0;
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

}  // namespace gbf
