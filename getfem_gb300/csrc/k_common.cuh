// Device helpers shared by the assembly kernels (sm_103a).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "plan.h"

namespace gfgpu {

constexpr int kWarp = 32;

__device__ __forceinline__ void set_err(int *err, int bit) { atomicOr(err, bit); }

// Bitonic sort of n (power of two) ints in shared memory by one warp.
__device__ __forceinline__ void warp_sort(int *a, int n) {
  const int lane = threadIdx.x & 31;
  for (int k = 2; k <= n; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = lane; i < n; i += kWarp) {
        const int ixj = i ^ j;
        if (ixj > i) {
          const int x = a[i], y = a[ixj];
          const bool up = (i & k) == 0;
          if ((x > y) == up) a[i] = y, a[ixj] = x;
        }
      }
      __syncwarp();
    }
  }
}

// In-place unique of a sorted array in shared memory; returns the length.
__device__ __forceinline__ int warp_unique(int *a, int n) {
  const int lane = threadIdx.x & 31;
  int out = 0;
  for (int base = 0; base < n; base += kWarp) {
    const int i = base + lane;
    const int x = i < n ? a[i] : 0;
    const bool first = i < n && (i == 0 || a[i - 1] != x);
    const unsigned m = __ballot_sync(0xffffffffu, first);
    __syncwarp();
    if (first) a[out + __popc(m & ((1u << lane) - 1))] = x;
    out += __popc(m);
    __syncwarp();
  }
  return out;
}

__device__ __forceinline__ int bsearch_slot(const int *s, int n, int key) {
  int lo = 0, hi = n;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (s[mid] < key) lo = mid + 1;
    else hi = mid;
  }
  return (lo < n && s[lo] == key) ? lo : -1;
}

__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
  const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem));
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
__device__ __forceinline__ void cp_async_wait1() { asm volatile("cp.async.wait_group 1;\n" ::); }
__device__ __forceinline__ void cp_async_wait2() { asm volatile("cp.async.wait_group 2;\n" ::); }

// |x| as an integer key: the bit pattern shifted left by one drops the sign
// and keeps the order of |x| (NaN above infinity).  Integer pipe only: the
// and-mask form (bits & 0x7ff...f) was compiled into an FP64 absolute-value
// add, one FP64 pipe instruction per entry tested (ncu: ~90 extra DADDs per
// element node in the row gather).
__device__ __forceinline__ unsigned long long abs_key(double x) {
  return static_cast<unsigned long long>(__double_as_longlong(x)) << 1;
}
__device__ __forceinline__ double abs_of_key(unsigned long long k) {
  return __longlong_as_double(static_cast<long long>(k >> 1));
}
// |x| > t for the key t of a threshold t >= +0
__device__ __forceinline__ bool abs_greater(double x, unsigned long long t_key) {
  return abs_key(x) > t_key;
}

}  // namespace gfgpu
