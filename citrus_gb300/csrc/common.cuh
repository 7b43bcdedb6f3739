// Shared helpers of the citrus_gb300 kernels: status codes, the per-thread error message, argument checks and the
// bounded grid barrier of the persistent kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include "../../include/citrus_gb300.h"

namespace citrus {

// Records a message for citrus_last_error_string() and returns the status code.
int set_error(int code, const char* fmt, ...);

// Converts the launch status of the last kernel into a citrus status code.
int launch_status(const char* what);

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

inline int64_t cdiv(int64_t a, int64_t b) { return (a + b - 1) / b; }

// Number of SMs of the current device (cached per device).
int num_sms();

// Adds n kernel launches to the library's launch counter (citrus_launch_count).
void note_launches(int n = 1);

#define CITRUS_REQUIRE(cond, ...)                                   \
  do {                                                              \
    if (!(cond)) return ::citrus::set_error(CITRUS_EINVAL, __VA_ARGS__); \
  } while (0)

// ---- memory-ordering helpers ----------------------------------------------------------------------------------
__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void st_release_u32(unsigned* p, unsigned v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ uint64_t global_timer_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Grid-wide barrier of a cooperative (co-resident) launch with a bounded wait.
//
// sync[0] counts arrivals, sync[1] is the generation, sync[2] the error word (non-zero after a timeout anywhere).
// Every waiting block gives up after `timeout_ns` of wall time, records the error and returns false; a block that
// returns false must leave the kernel, so that no wait outlives the limit. `skip` makes this block not arrive (a
// test hook that forces the timeout path); it is -1 in normal use.
__device__ __forceinline__ bool grid_barrier(unsigned* sync, unsigned num_blocks, uint64_t timeout_ns, int skip) {
  __shared__ int ok_shared;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    const unsigned gen = ld_acquire_u32(&sync[1]);
    __threadfence();
    if ((int)blockIdx.x != skip) {
      const unsigned prev = atomicAdd(&sync[0], 1u);
      if (prev == num_blocks - 1) {
        atomicExch(&sync[0], 0u);
        __threadfence();
        st_release_u32(&sync[1], gen + 1u);
      }
    }
    const uint64_t t0 = global_timer_ns();
    while (ld_acquire_u32(&sync[1]) == gen) {
      if (ld_acquire_u32(&sync[2]) != 0u) { ok = 0; break; }
      if (global_timer_ns() - t0 > timeout_ns) {
        atomicExch(&sync[2], 1u);
        ok = 0;
        break;
      }
      __nanosleep(64);
    }
    if (ok && ld_acquire_u32(&sync[2]) != 0u) ok = 0;
    __threadfence();
    ok_shared = ok;
  }
  __syncthreads();
  return ok_shared != 0;
}

}  // namespace citrus
