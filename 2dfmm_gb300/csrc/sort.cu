// Stable LSD radix sort of (uint64 key, uint32 value) pairs, 8 bits per
// pass, reduce-then-scan form:
//   upsweep   : per tile (4096 pairs) digit counts  -> counts[digit][tile]
//   scan      : per digit, exclusive scan of its tile counts (one block per
//               digit); digit totals are scanned inside the downsweep
//   downsweep : stable rank inside the tile (warp match + per-warp running
//               counts), staged in shared memory in digit order, then
//               written to counts-scan offset + rank with coalesced stores.
// Tiles are processed warp-striped: warp w owns 512 consecutive pairs, its
// lanes take 32 consecutive pairs per step, so (warp, step, lane) is the
// input order and the ranking is stable.
//
// Packed words (key in the high 32 bits, value in the low 32) take a
// single-pass form per digit instead (radix_sort_packed): one read of the
// words forms every pass's digit histogram up front (k_hist_all), and each
// pass is one kernel (k_onesweep) in which a tile ranks its words as the
// downsweep does, publishes its per-digit counts, and finds the counts of
// all earlier tiles by looking back over their published words (decoupled
// look-back: a tile's word carries either its own count or, once known,
// the running total through it), then scatters.  Tiles are numbered in the
// order blocks start (an atomic counter), so a tile only ever waits on
// tiles that are already running.
#include "dev_common.cuh"

namespace t2d {
namespace {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kItems = 16;                    // per thread
constexpr int kTile = kThreads * kItems;      // 4096
constexpr int kBins = 256;
static_assert(kThreads == kBins, "the downsweep scans the digit totals with one thread per digit");
constexpr int kStageBytes = kTile * (8 + 4);  // the downsweep's staging of one tile (48 KB)
constexpr int kStagePackedBytes = kTile * 8;  // packed keys only (32 KB)

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

// Exclusive scan of one value per thread over the block (kThreads values,
// thread order).  `wsum` is kWarps words of shared scratch; the call
// synchronises the block before it returns.
__device__ __forceinline__ unsigned block_exclusive_scan(unsigned v, unsigned *wsum) {
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  unsigned incl = v;
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned u = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += u;
  }
  if (lane == 31) wsum[w] = incl;
  __syncthreads();
  unsigned base = 0;
  for (int k = 0; k < w; k++) base += wsum[k];
  __syncthreads();
  return base + incl - v;
}

// The tile's pairs are ranked (stable: warp, step, lane order within a
// digit), staged in shared memory in digit order, and written out from
// there: consecutive threads write consecutive positions of a digit's run,
// so the stores coalesce instead of scattering one pair per digit.
// kPacked: the keys are words whose high 32 bits are the key and whose low
// 32 bits are the value (vin unused); with `split` the pass writes them out
// as a key (low half cleared) and a value.
template <bool kPacked>
__global__ void __launch_bounds__(kThreads) k_downsweep(const uint64_t *__restrict__ kin,
                                                        const uint32_t *__restrict__ vin,
                                                        uint64_t *__restrict__ kout, uint32_t *__restrict__ vout,
                                                        int n, int shift, const unsigned *__restrict__ offs,
                                                        int ntiles, const unsigned *__restrict__ totals, int split) {
  extern __shared__ __align__(16) unsigned char stage[];
  uint64_t *sk = reinterpret_cast<uint64_t *>(stage);             // kTile keys, tile digit order
  uint32_t *sv = reinterpret_cast<uint32_t *>(stage + kTile * 8);  // kTile values (unpacked only)
  __shared__ unsigned wcount[kWarps][kBins];
  __shared__ unsigned lbase[kBins];  // tile-local start of each digit's run
  __shared__ unsigned gbase[kBins];  // global position of that start
  __shared__ unsigned wsum[kWarps];
  // digit d's global start: exclusive scan of the digit totals, plus the
  // tiles before this one (kThreads == kBins: thread t owns digit t)
  const unsigned dbase = block_exclusive_scan(totals[threadIdx.x], wsum);
  for (int i = threadIdx.x; i < kWarps * kBins; i += kThreads) (&wcount[0][0])[i] = 0;
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long tile0 = (long)blockIdx.x * kTile;
  const long base = tile0 + warp * (kItems * 32);
  uint64_t k[kItems];
  uint32_t v[kPacked ? 1 : kItems];
  unsigned r[kItems];
  const unsigned ltmask = lanemask_lt();
#pragma unroll
  for (int j = 0; j < kItems; j++) {
    long i = base + j * 32 + lane;
    bool valid = i < n;
    k[j] = valid ? kin[i] : 0;
    if (!kPacked) v[j] = valid ? vin[i] : 0;
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
  // per digit: the warps' counts become their starts inside the digit's run
  unsigned cnt = 0;
  {
    const int d = threadIdx.x;
#pragma unroll
    for (int w = 0; w < kWarps; w++) {
      const unsigned c = wcount[w][d];
      wcount[w][d] = cnt;
      cnt += c;
    }
  }
  const unsigned lb = block_exclusive_scan(cnt, wsum);
  lbase[threadIdx.x] = lb;
  gbase[threadIdx.x] = dbase + offs[(size_t)threadIdx.x * ntiles + blockIdx.x];
  __syncthreads();
#pragma unroll
  for (int j = 0; j < kItems; j++) {
    long i = base + j * 32 + lane;
    if (i < n) {
      const unsigned d = (unsigned)((k[j] >> shift) & 0xff);
      const unsigned lp = lbase[d] + wcount[warp][d] + r[j];
      sk[lp] = k[j];
      if (!kPacked) sv[lp] = v[j];
    }
  }
  __syncthreads();
  const int tile_n = (int)min((long)kTile, (long)n - tile0);
  for (int p = threadIdx.x; p < tile_n; p += kThreads) {
    const uint64_t key = sk[p];
    const unsigned d = (unsigned)((key >> shift) & 0xff);
    const unsigned pos = gbase[d] + ((unsigned)p - lbase[d]);
    if (!kPacked) {
      kout[pos] = key;
      vout[pos] = sv[p];
    } else if (split) {
      kout[pos] = key & 0xffffffff00000000ull;
      vout[pos] = (uint32_t)key;
    } else {
      kout[pos] = key;
    }
  }
}

// ---------------------------------------------------------------- single pass

constexpr int kMaxPasses = 4;                 // packed words: bits [32, 64)
constexpr unsigned kFlagAgg = 1u << 30;       // the tile's own count
constexpr unsigned kFlagPre = 2u << 30;       // the running total through the tile
constexpr unsigned kCountMask = kFlagAgg - 1u;
constexpr long kLookbackLimit = 1l << 22;     // polls; a healthy look-back ends in microseconds

// Every pass's digit histogram in one read of the words: per block in
// shared memory, then added to hist[pass][digit].
__global__ void __launch_bounds__(kThreads) k_hist_all(const uint64_t *__restrict__ words, int n, int begin_bit,
                                                       int passes, unsigned *__restrict__ hist) {
  __shared__ unsigned hw[kWarps][kMaxPasses][kBins];  // per warp: no atomics collide across warps
  for (int i = threadIdx.x; i < kWarps * kMaxPasses * kBins; i += kThreads) (&hw[0][0][0])[i] = 0;
  __syncthreads();
  unsigned (*h)[kBins] = hw[threadIdx.x >> 5];
  const long stride = (long)gridDim.x * kThreads;
  for (long i0 = (long)blockIdx.x * kThreads + (threadIdx.x & ~31); i0 < n; i0 += stride) {  // warp-uniform
    const long i = i0 + (threadIdx.x & 31);
    const bool valid = i < n;
    const uint64_t w = valid ? words[i] : 0;
    for (int p = 0; p < passes; p++) {
      // a shared-memory add per element: lanes that hit the same digit
      // serialise on it, which measured cheaper than grouping equal digits
      // with __match_any_sync first (the 4M-blob build took 0.68 against
      // 0.76 ms; the grouped form's histogram alone was 0.096 ms)
      const unsigned d = (unsigned)(w >> (begin_bit + 8 * p)) & 0xffu;
      if (valid) atomicAdd(&h[p][d], 1u);
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < passes * kBins; i += kThreads) {
    unsigned v = 0;
    for (int w = 0; w < kWarps; w++) v += (&hw[w][0][0])[i];
    if (v) atomicAdd(&hist[i], v);
  }
}

// One pass over packed words: tile ranking as in k_downsweep, the tile's
// per-digit offset from the look-back over earlier tiles' status words
// (status[tile][digit], zero before the pass), then the scatter through
// shared memory.  `hist` is this pass's digit histogram, `ctr` its tile
// counter (zero before the pass).  A look-back that polls `limit` times
// without an answer records TREE2D_ERR_TIMEOUT and takes the missing count
// as zero (the output is then wrong and the build reports the error).
__global__ void __launch_bounds__(kThreads) k_onesweep(const uint64_t *__restrict__ kin, uint64_t *__restrict__ kout,
                                                       uint32_t *__restrict__ vout, int n, int shift,
                                                       const unsigned *__restrict__ hist, unsigned *status,
                                                       unsigned *ctr, int ntiles, int split, long limit,
                                                       DevStatus *st) {
  extern __shared__ __align__(16) unsigned char stage[];
  uint64_t *sk = reinterpret_cast<uint64_t *>(stage);  // kTile words, tile digit order
  __shared__ unsigned wcount[kWarps][kBins];
  __shared__ unsigned lbase[kBins];
  __shared__ unsigned gbase[kBins];
  __shared__ unsigned wsum[kWarps];
  __shared__ int s_tile;
  if (threadIdx.x == 0) s_tile = (int)atomicAdd(ctr, 1u);
  const unsigned dbase = block_exclusive_scan(hist[threadIdx.x], wsum);  // synchronises: s_tile is set
  const int tile = s_tile;
  if (tile >= ntiles) return;  // uniform for the block (the grid is exactly ntiles blocks)
  for (int i = threadIdx.x; i < kWarps * kBins; i += kThreads) (&wcount[0][0])[i] = 0;
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long tile0 = (long)tile * kTile;
  const long base = tile0 + warp * (kItems * 32);
  uint64_t k[kItems];
  unsigned r[kItems];
  const unsigned ltmask = lanemask_lt();
#pragma unroll
  for (int j = 0; j < kItems; j++) {
    const long i = base + j * 32 + lane;
    const bool valid = i < n;
    k[j] = valid ? kin[i] : 0;
    const unsigned d = valid ? (unsigned)((k[j] >> shift) & 0xff) : 0x100u;
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    const unsigned rank = __popc(peers & ltmask);
    const unsigned c = valid ? wcount[warp][d] : 0;
    __syncwarp();
    if (valid && rank == 0) wcount[warp][d] = c + __popc(peers);
    __syncwarp();
    r[j] = c + rank;
  }
  __syncthreads();
  unsigned cnt = 0;
  {
    const int d = threadIdx.x;
#pragma unroll
    for (int w = 0; w < kWarps; w++) {
      const unsigned c = wcount[w][d];
      wcount[w][d] = cnt;
      cnt += c;
    }
  }
  // publish this tile's count of digit d, then look back for the earlier
  // tiles' total (thread d owns digit d)
  {
    const int d = threadIdx.x;
    volatile unsigned *my = status + (size_t)tile * kBins + d;
    unsigned excl = 0;
    if (tile == 0) {
      *my = kFlagPre | cnt;
    } else {
      *my = kFlagAgg | cnt;
      int t = tile - 1;
      long polls = 0;
      while (t >= 0) {
        const unsigned v = *(volatile const unsigned *)(status + (size_t)t * kBins + d);
        if ((v & ~kCountMask) == 0u) {
          if (++polls > limit) {
            set_err(st, TREE2D_ERR_TIMEOUT);
            break;
          }
          continue;
        }
        excl += v & kCountMask;
        if (v & kFlagPre) break;
        t--;
      }
      *my = kFlagPre | (excl + cnt);
    }
    gbase[d] = dbase + excl;
  }
  const unsigned lb = block_exclusive_scan(cnt, wsum);
  lbase[threadIdx.x] = lb;
  __syncthreads();
#pragma unroll
  for (int j = 0; j < kItems; j++) {
    const long i = base + j * 32 + lane;
    if (i < n) {
      const unsigned d = (unsigned)((k[j] >> shift) & 0xff);
      sk[lbase[d] + wcount[warp][d] + r[j]] = k[j];
    }
  }
  __syncthreads();
  const int tile_n = (int)min((long)kTile, (long)n - tile0);
  for (int p = threadIdx.x; p < tile_n; p += kThreads) {
    const uint64_t key = sk[p];
    const unsigned d = (unsigned)((key >> shift) & 0xff);
    const unsigned pos = gbase[d] + ((unsigned)p - lbase[d]);
    if (split) {
      kout[pos] = key & 0xffffffff00000000ull;
      vout[pos] = (uint32_t)key;
    } else {
      kout[pos] = key;
    }
  }
}

}  // namespace

static size_t onesweep_temp_bytes(int n) {
  const size_t ntiles = (size_t)(n > 0 ? (n + kTile - 1) / kTile : 1);
  return ((size_t)kMaxPasses * kBins + kMaxPasses + (size_t)kMaxPasses * ntiles * kBins) * sizeof(unsigned);
}

size_t radix_sort_temp_bytes(int n) {
  long ntiles = (n + kTile - 1) / kTile;
  const size_t classic = (size_t)kBins * (size_t)(ntiles > 0 ? ntiles : 1) * sizeof(unsigned) + kBins * sizeof(unsigned);
  const size_t single = onesweep_temp_bytes(n);
  return classic > single ? classic : single;
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
  cudaError_t e = cudaFuncSetAttribute(k_downsweep<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, kStageBytes);
  if (e != cudaSuccess) return e;
  for (int shift = begin_bit; shift < end_bit; shift += 8, passes++) {
    k_upsweep<<<ntiles, kThreads, 0, s>>>(ka, n, shift, counts, ntiles);
    ::t2d::g_launches.fetch_add(1, std::memory_order_relaxed);
    k_scan_digit<<<kBins, 1024, 0, s>>>(counts, ntiles, totals);
    ::t2d::g_launches.fetch_add(1, std::memory_order_relaxed);
    k_downsweep<false><<<ntiles, kThreads, kStageBytes, s>>>(ka, va, kb, vb, n, shift, counts, ntiles, totals, 0);
    ::t2d::g_launches.fetch_add(1, std::memory_order_relaxed);
    uint64_t *tk = ka;
    ka = kb;
    kb = tk;
    uint32_t *tv = va;
    va = vb;
    vb = tv;
  }
  if (passes & 1) {
    e = cudaMemcpyAsync(keys, ka, sizeof(uint64_t) * (size_t)n, cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(vals, va, sizeof(uint32_t) * (size_t)n, cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) return e;
  }
  return cudaGetLastError();
}

cudaError_t radix_sort_packed(uint64_t *words, uint64_t *words_alt, int n, int begin_bit, uint64_t *keys_out,
                              uint32_t *vals_out, void *temp, DevStatus *st, cudaStream_t s) {
  if (begin_bit < 32 || begin_bit >= 64 || n < 2) return cudaErrorInvalidValue;
  const int passes = (64 - begin_bit + 7) / 8;
  const int ntiles = (n + kTile - 1) / kTile;
  uint64_t *ka = words, *kb = words_alt;
  if (n < (1 << 30) && st) {
    // single pass per digit: counts up to 2^30 - 1 fit a status word
    unsigned *hist = static_cast<unsigned *>(temp);
    unsigned *ctr = hist + kMaxPasses * kBins;
    unsigned *status = ctr + kMaxPasses;
    const size_t zero = ((size_t)kMaxPasses * kBins + kMaxPasses + (size_t)passes * ntiles * kBins) * sizeof(unsigned);
    cudaError_t e = cudaMemsetAsync(temp, 0, zero, s);
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(k_onesweep, cudaFuncAttributeMaxDynamicSharedMemorySize, kStagePackedBytes);
    if (e != cudaSuccess) return e;
    const int hblocks = ntiles < 152 * 4 ? ntiles : 152 * 4;
    k_hist_all<<<hblocks, kThreads, 0, s>>>(ka, n, begin_bit, passes, hist);
    ::t2d::g_launches.fetch_add(1, std::memory_order_relaxed);
    for (int p = 0; p < passes; p++) {
      const bool last = p == passes - 1;
      k_onesweep<<<ntiles, kThreads, kStagePackedBytes, s>>>(
          ka, last ? keys_out : kb, last ? vals_out : nullptr, n, begin_bit + 8 * p, hist + p * kBins,
          status + (size_t)p * ntiles * kBins, ctr + p, ntiles, last ? 1 : 0, kLookbackLimit, st);
      ::t2d::g_launches.fetch_add(1, std::memory_order_relaxed);
      uint64_t *t = ka;
      ka = kb;
      kb = t;
    }
    return cudaGetLastError();
  }
  unsigned *counts = static_cast<unsigned *>(temp);
  unsigned *totals = counts + (size_t)kBins * ntiles;
  cudaError_t e = cudaFuncSetAttribute(k_downsweep<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       kStagePackedBytes);
  if (e != cudaSuccess) return e;
  for (int p = 0; p < passes; p++) {
    const int shift = begin_bit + 8 * p;
    const bool last = p == passes - 1;
    k_upsweep<<<ntiles, kThreads, 0, s>>>(ka, n, shift, counts, ntiles);
    k_scan_digit<<<kBins, 1024, 0, s>>>(counts, ntiles, totals);
    k_downsweep<true><<<ntiles, kThreads, kStagePackedBytes, s>>>(ka, nullptr, last ? keys_out : kb,
                                                                  last ? vals_out : nullptr, n, shift, counts,
                                                                  ntiles, totals, last ? 1 : 0);
    ::t2d::g_launches.fetch_add(3, std::memory_order_relaxed);
    uint64_t *t = ka;
    ka = kb;
    kb = t;
  }
  return cudaGetLastError();
}

}  // namespace t2d
