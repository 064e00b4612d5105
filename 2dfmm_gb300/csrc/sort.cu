// Stable LSD radix sort of (uint64 key, uint32 value) pairs, 8 bits per
// pass, reduce-then-scan form:
//   upsweep   : per tile (4096 pairs) digit counts  -> counts[digit][tile]
//   scan      : per digit, exclusive scan of its tile counts (one block per
//               digit); digit totals are scanned inside the downsweep
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
static_assert(kThreads == kBins, "the downsweep scans the digit totals with one thread per digit");

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

// One block per digit: exclusive scan of counts[d][0..ntiles) in place,
// total -> totals[d].
__global__ void __launch_bounds__(1024) k_scan_digit(unsigned *counts, int ntiles, unsigned *totals) {
  __shared__ unsigned part[1024];
  unsigned *c = counts + (size_t)blockIdx.x * ntiles;
  const int t = threadIdx.x;
  const int per = (ntiles + 1023) / 1024;
  const int b = t * per, e = min(ntiles, b + per);
  unsigned s = 0;
  for (int i = b; i < e; i++) s += c[i];
  part[t] = s;
  __syncthreads();
  for (int off = 1; off < 1024; off <<= 1) {
    unsigned v = t >= off ? part[t - off] : 0u;
    __syncthreads();
    part[t] += v;
    __syncthreads();
  }
  unsigned run = t == 0 ? 0u : part[t - 1];
  for (int i = b; i < e; i++) {
    unsigned x = c[i];
    c[i] = run;
    run += x;
  }
  if (t == 1023) totals[blockIdx.x] = part[1023];
}

__global__ void __launch_bounds__(kThreads) k_downsweep(const uint64_t *__restrict__ kin,
                                                        const uint32_t *__restrict__ vin,
                                                        uint64_t *__restrict__ kout, uint32_t *__restrict__ vout,
                                                        int n, int shift, const unsigned *__restrict__ offs,
                                                        int ntiles, const unsigned *__restrict__ totals) {
  __shared__ unsigned wcount[kWarps][kBins];
  __shared__ unsigned dbase[kBins];
  {
    // exclusive scan of the 256 digit totals (kThreads == kBins)
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    const unsigned v = totals[t];
    unsigned incl = v;
    for (int o = 1; o < 32; o <<= 1) {
      unsigned u = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += u;
    }
    __shared__ unsigned wsum[kWarps];
    if (lane == 31) wsum[w] = incl;
    __syncthreads();
    unsigned base = 0;
    for (int k = 0; k < w; k++) base += wsum[k];
    dbase[t] = base + incl - v;
  }
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
    unsigned run = dbase[d] + offs[(size_t)d * ntiles + blockIdx.x];
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
  return (size_t)kBins * (size_t)(ntiles > 0 ? ntiles : 1) * sizeof(unsigned) + kBins * sizeof(unsigned);
}

cudaError_t radix_sort_pairs(uint64_t *keys, uint32_t *vals, uint64_t *keys_alt, uint32_t *vals_alt, int n,
                             int begin_bit, int end_bit, void *temp, cudaStream_t s) {
  if (n <= 1) return cudaSuccess;
  const int ntiles = (n + kTile - 1) / kTile;
  unsigned *counts = static_cast<unsigned *>(temp);
  unsigned *totals = counts + (size_t)kBins * ntiles;
  uint64_t *ka = keys, *kb = keys_alt;
  uint32_t *va = vals, *vb = vals_alt;
  int passes = 0;
  for (int shift = begin_bit; shift < end_bit; shift += 8, passes++) {
    k_upsweep<<<ntiles, kThreads, 0, s>>>(ka, n, shift, counts, ntiles);
    ::t2d::g_launches.fetch_add(1, std::memory_order_relaxed);
    k_scan_digit<<<kBins, 1024, 0, s>>>(counts, ntiles, totals);
    ::t2d::g_launches.fetch_add(1, std::memory_order_relaxed);
    k_downsweep<<<ntiles, kThreads, 0, s>>>(ka, va, kb, vb, n, shift, counts, ntiles, totals);
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
