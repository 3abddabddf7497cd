// Software grid barrier for cooperative (all blocks resident) launches.
//
// The arrival counter starts at zero (the launcher clears the barrier memory)
// and only grows within a launch: thread 0 of each block adds
// one with release semantics at GPU scope (publishing the block's writes,
// ordered before it by __syncthreads), which also tells it which barrier it
// is at -- all arrivals at barrier k return values in [k*G, (k+1)*G) for G
// blocks, since no block passes barrier k before all G have arrived -- and
// then polls the counter with acquire loads until it reaches (k+1)*G.  So the
// critical path is one atomic and one load; there is no reset, no separate
// generation word and no full fence.
//
// Every wait is bounded: after `max_polls` polls the block records a fault
// and returns false, and a waiting block that sees the fault word (checked
// every 16 polls) gives up at once.  Callers return from the kernel on false,
// and the host turns the fault word into an error status, so a lost block
// never hangs the GPU.
#pragma once

#include "common.cuh"

namespace gbf {

struct GridBarrier {
  unsigned long long count;
  int fault, pad;
};

constexpr long long kBarrierPolls = 1LL << 22;  // a few seconds of polling

__device__ __forceinline__ unsigned long long barrier_arrive(unsigned long long* c) {
  unsigned long long old;
  asm volatile("atom.add.release.gpu.u64 %0, [%1], 1;" : "=l"(old) : "l"(c) : "memory");
  return old;
}

__device__ __forceinline__ unsigned long long barrier_load(const unsigned long long* c) {
  unsigned long long v;
  asm volatile("ld.acquire.gpu.u64 %0, [%1];" : "=l"(v) : "l"(c) : "memory");
  return v;
}

__device__ __forceinline__ bool grid_barrier(GridBarrier* bar, unsigned int nblocks,
                                             long long max_polls = kBarrierPolls) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    const unsigned long long old = barrier_arrive(&bar->count);
    const unsigned long long target = (old / nblocks + 1) * nblocks;
    long long polls = 0;
    while (barrier_load(&bar->count) < target) {
      ++polls;
      if (polls > max_polls || ((polls & 15) == 0 && *(volatile int*)&bar->fault != 0)) {
        atomicExch(&bar->fault, 1);
        ok = 0;
        break;
      }
      __nanosleep(32);
    }
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

}  // namespace gbf
