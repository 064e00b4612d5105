// M2L over the V lists: for every cell c of level >= 2,
//   L[c] += sum_{s<27} T(class(c), s) M[V[c][s]],
// T(q,s)_lk = (-1)^l C(k+l,l) tau^-(k+l+1), tau the fixed offset of slot s
// for child class q (scaled expansions make T level independent).
#include "dev_common.cuh"
#include "mixed.h"

namespace t2d {
namespace {

// CUDA-core form: one warp per cell, lane l owns b_l.
__global__ void __launch_bounds__(256) k_m2l_cc(MixedView m, const float2 *__restrict__ T) {
  const int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (c >= m.ncell) return;
  if (m.level[c] < 2) return;
  const int P = m.P;
  const int cls = (m.ix[c] & 1) + 2 * (m.iy[c] & 1);
  const int *V = m.vlist + (size_t)c * 27;
  float2 acc = make_float2(0.f, 0.f);
  for (int s = 0; s < 27; s++) {
    const int src = V[s];
    if (src < 0) continue;
    const float *Ms = m.M + (size_t)src * 2 * P;
    const float2 a = lane < P ? make_float2(Ms[lane], Ms[P + lane]) : make_float2(0.f, 0.f);
    const float2 *Trow = T + (((size_t)cls * 27 + s) * P + (lane < P ? lane : 0)) * P;
    for (int k = 0; k < P; k++) {
      const float2 ak = make_float2(__shfl_sync(0xffffffffu, a.x, k), __shfl_sync(0xffffffffu, a.y, k));
      const float2 t = Trow[k];
      acc.x += t.x * ak.x - t.y * ak.y;
      acc.y += t.x * ak.y + t.y * ak.x;
    }
  }
  if (lane < P) {
    m.L[(size_t)c * 2 * P + lane] += acc.x;
    m.L[(size_t)c * 2 * P + P + lane] += acc.y;
  }
}

}  // namespace

int m2l_cuda_cores(MixedView &m, const float *tables, cudaStream_t s) {
  k_m2l_cc<<<(int)(((long)m.ncell * 32 + 255) / 256), 256, 0, s>>>(m, reinterpret_cast<const float2 *>(tables));
  g_launches.fetch_add(1, std::memory_order_relaxed);
  T2D_CUDA_TRY(cudaGetLastError());
  return TREE2D_OK;
}

}  // namespace t2d
