// Stable LSD radix sort of (uint64 key, uint32 value) pairs, 8 bits per
// pass, reduce-then-scan form:
//   upsweep   : per tile (4096 pairs) digit counts  -> counts[digit][tile]
//   scan      : exclusive scan of counts in digit-major order (one block)
//   downsweep : stable rank inside the tile (warp match + per-warp running
//               counts), scatter to counts-scan offset + rank.
// Tiles are processed warp-striped: warp w owns 512 consecutive pairs, its
// lanes take 32 consecutive pairs per step, so (warp, step, lane) is the
// input order and the ranking is stable.
#include "dev_common.cuh"

namespace t2d {
namespace {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kItems = 16;                    // per thread
constexpr int kTile = kThreads * kItems;      // 4096
constexpr int kBins = 256;

__device__ __forceinline__ unsigned lanemask_lt() {
  unsigned m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

__global__ void __launch_bounds__(kThreads) k_upsweep(const uint64_t *__restrict__ keys, int n, int shift,
                                                      unsigned *__restrict__ counts, int ntiles) {
  __shared__ unsigned hist[kBins];
  for (int i = threadIdx.x; i < kBins; i += kThreads) hist[i] = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const long base = (long)blockIdx.x * kTile;
  for (int k = threadIdx.x; k < kTile; k += kThreads) {
    long i = base + k;
    bool valid = i < n;
    unsigned d = valid ? (unsigned)((keys[i] >> shift) & 0xff) : 0x100u;
    unsigned peers = __match_any_sync(0xffffffffu, d);
    if (valid && (peers & lanemask_lt()) == 0) atomicAdd(&hist[d], (unsigned)__popc(peers));
    (void)lane;
  }
  __syncthreads();
  for (int d = threadIdx.x; d < kBins; d += kThreads) counts[(size_t)d * ntiles + blockIdx.x] = hist[d];
}

// Exclusive scan of `len` counts with one block of 1024 threads.
__global__ void __launch_bounds__(1024) k_scan_counts(unsigned *counts, long len) {
  __shared__ unsigned long long part[1024];
  const int t = threadIdx.x;
  const long per = (len + 1023) / 1024;
  const long b = t * per, e = min(len, b + per);
  unsigned long long s = 0;
  for (long i = b; i < e; i++) s += counts[i];
  part[t] = s;
  __syncthreads();
  // Hillis-Steele over 1024 partials
  for (int off = 1; off < 1024; off <<= 1) {
    unsigned long long v = t >= off ? part[t - off] : 0;
    __syncthreads();
    part[t] += v;
    __syncthreads();
  }
  unsigned long long run = t == 0 ? 0 : part[t - 1];
  for (long i = b; i < e; i++) {
    unsigned c = counts[i];
    counts[i] = (unsigned)run;
    run += c;
  }
}

__global__ void __launch_bounds__(kThreads) k_downsweep(const uint64_t *__restrict__ kin,
                                                        const uint32_t *__restrict__ vin,
                                                        uint64_t *__restrict__ kout, uint32_t *__restrict__ vout,
                                                        int n, int shift, const unsigned *__restrict__ offs,
                                                        int ntiles) {
  __shared__ unsigned wcount[kWarps][kBins];
  for (int i = threadIdx.x; i < kWarps * kBins; i += kThreads) (&wcount[0][0])[i] = 0;
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long base = (long)blockIdx.x * kTile + warp * (kItems * 32);
  uint64_t k[kItems];
  uint32_t v[kItems];
  unsigned r[kItems];
  const unsigned ltmask = lanemask_lt();
#pragma unroll
  for (int j = 0; j < kItems; j++) {
    long i = base + j * 32 + lane;
    bool valid = i < n;
    k[j] = valid ? kin[i] : 0;
    v[j] = valid ? vin[i] : 0;
    unsigned d = valid ? (unsigned)((k[j] >> shift) & 0xff) : 0x100u;
    unsigned peers = __match_any_sync(0xffffffffu, d);
    unsigned rank = __popc(peers & ltmask);
    unsigned c = valid ? wcount[warp][d] : 0;
    __syncwarp();
    if (valid && rank == 0) wcount[warp][d] = c + __popc(peers);
    __syncwarp();
    r[j] = c + rank;
  }
  __syncthreads();
  for (int d = threadIdx.x; d < kBins; d += kThreads) {
    unsigned run = offs[(size_t)d * ntiles + blockIdx.x];
#pragma unroll
    for (int w = 0; w < kWarps; w++) {
      unsigned c = wcount[w][d];
      wcount[w][d] = run;
      run += c;
    }
  }
  __syncthreads();
#pragma unroll
  for (int j = 0; j < kItems; j++) {
    long i = base + j * 32 + lane;
    if (i < n) {
      unsigned d = (unsigned)((k[j] >> shift) & 0xff);
      unsigned pos = wcount[warp][d] + r[j];
      kout[pos] = k[j];
      vout[pos] = v[j];
    }
  }
}

}  // namespace

size_t radix_sort_temp_bytes(int n) {
  long ntiles = (n + kTile - 1) / kTile;
  return (size_t)kBins * (size_t)(ntiles > 0 ? ntiles : 1) * sizeof(unsigned);
}

cudaError_t radix_sort_pairs(uint64_t *keys, uint32_t *vals, uint64_t *keys_alt, uint32_t *vals_alt, int n,
                             int end_bit, void *temp, cudaStream_t s) {
  if (n <= 1) return cudaSuccess;
  const int ntiles = (n + kTile - 1) / kTile;
  unsigned *counts = static_cast<unsigned *>(temp);
  uint64_t *ka = keys, *kb = keys_alt;
  uint32_t *va = vals, *vb = vals_alt;
  int passes = 0;
  for (int shift = 0; shift < end_bit; shift += 8, passes++) {
    k_upsweep<<<ntiles, kThreads, 0, s>>>(ka, n, shift, counts, ntiles);
    ::t2d::g_launches.fetch_add(1, std::memory_order_relaxed);
    k_scan_counts<<<1, 1024, 0, s>>>(counts, (long)kBins * ntiles);
    ::t2d::g_launches.fetch_add(1, std::memory_order_relaxed);
    k_downsweep<<<ntiles, kThreads, 0, s>>>(ka, va, kb, vb, n, shift, counts, ntiles);
    ::t2d::g_launches.fetch_add(1, std::memory_order_relaxed);
    uint64_t *tk = ka;
    ka = kb;
    kb = tk;
    uint32_t *tv = va;
    va = vb;
    vb = tv;
  }
  if (passes & 1) {
    cudaMemcpyAsync(keys, ka, sizeof(uint64_t) * (size_t)n, cudaMemcpyDeviceToDevice, s);
    cudaMemcpyAsync(vals, va, sizeof(uint32_t) * (size_t)n, cudaMemcpyDeviceToDevice, s);
  }
  return cudaGetLastError();
}

}  // namespace t2d
