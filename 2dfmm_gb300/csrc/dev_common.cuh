// Device helpers shared by the kernels.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "internal.h"

#define T2D_CUDA_TRY(expr)                            \
  do {                                                \
    cudaError_t e_ = (expr);                          \
    if (e_ != cudaSuccess) {                          \
      ::t2d::note_cuda_error(e_, #expr);              \
      return TREE2D_ERR_CUDA;                         \
    }                                                 \
  } while (0)

namespace t2d {

__device__ __forceinline__ void set_err(DevStatus *st, int code) { atomicCAS(&st->err, 0, code); }

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }

__device__ __forceinline__ double2 shfl_d2(double2 v, int src) {
  return make_double2(__shfl_sync(0xffffffffu, v.x, src), __shfl_sync(0xffffffffu, v.y, src));
}

// Lane k of the warp receives z^k (lanes beyond `count` get junk): an
// inclusive scan over lanes of [1, z, z, ...] under complex multiplication.
__device__ __forceinline__ double2 warp_powers(double2 z, int lane) {
  double2 v = lane == 0 ? make_double2(1.0, 0.0) : z;
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    double2 o = make_double2(__shfl_up_sync(0xffffffffu, v.x, off), __shfl_up_sync(0xffffffffu, v.y, off));
    if (lane >= off) v = cmul(o, v);
  }
  return v;
}

// Number of leading base-4 digits shared by two keys (32 if equal).
__device__ __forceinline__ int common_levels(uint64_t a, uint64_t b) {
  uint64_t d = a ^ b;
  return d == 0 ? kKeyLevels : (__clzll(d) >> 1);
}

}  // namespace t2d
