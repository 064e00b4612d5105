// Tree build on the device, bit-exact with the reference's recursive
// bucketing (ver-c/src/quadtree.c:81-99 root box, :29-35 quadrant test,
// :61-79 child centres, :173-251 split_cell).
//
//   1. k_bbox/k_root  root box: min/max reduction, side = max(dx,dy)+1e-4,
//                     centre = midpoint (quadtree.c:81-99)
//   2. k_keys         per blob, 32 levels of the reference's quadrant test
//                     against FP64 centres formed exactly as the reference
//                     forms them (c +- 0.25*R per level) -> 64-bit key of
//                     base-4 digits, level 1 in the top bits
//   3. radix sort     (key, blob index) pairs, stable
//   4. k_cpl          cpl[i] = levels shared by keys i and i+1;
//                     w[j]   = levels shared by keys j and j+num_p-1
//   5. k_leaf_level   a level-l cell holds >= num_p blobs iff some window of
//                     num_p consecutive keys inside it shares l levels, so the
//                     deepest split level of blob i is the max of w over the
//                     windows that contain i; its leaf sits one level below
//                     (the root is always split, quadtree.c:183-196)
//   6. cell counts    position i starts the cells of levels
//                     (cpl[i-1], leaf_level[i]]; a scan numbers all cells in
//                     depth-first pre-order (root = 0)
//   7. k_emit_cells   level, begin, leaf flag, centre (same FP64 descent),
//                     side; k_cell_end (binary search), k_children
//   8. k_leaf_order   blobs inside a leaf in ascending original index, the
//                     order the reference's stable bucketing leaves them in
//   9. k_gather       blob arrays in tree order
#include <cstdio>

#include "dev_common.cuh"

namespace t2d {
namespace {

constexpr int kBoxBlocks = 1216;  // 8 x 152 SMs: enough loads in flight to stream the positions

struct __align__(16) Box4 {
  double x, y, z, w;  // xmax, xmin, ymax, ymin
};
constexpr int kScanThreads = 256;
constexpr int kScanItems = 16;
constexpr int kScanTile = kScanThreads * kScanItems;

__device__ __forceinline__ double warp_max(double v) {
  for (int o = 16; o; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
__device__ __forceinline__ double warp_min(double v) {
  for (int o = 16; o; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// Order-preserving map of a non-NaN double to an unsigned integer (-0 is
// taken as +0, as the FP64 comparisons treat them): a >= b iff
// okey(a) >= okey(b).  Lets the key descent compare on the integer pipe.
__device__ __forceinline__ uint64_t okey(double d) {
  uint64_t u = (uint64_t)__double_as_longlong(d);
  if (u == 0x8000000000000000ull) u = 0;
  return (u >> 63) ? ~u : (u | 0x8000000000000000ull);
}
__device__ __forceinline__ double okey_inv(uint64_t k) {
  const uint64_t u = (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
  return __longlong_as_double((long long)u);
}

// Extremes of the positions as order-preserving integers (okey), so that the
// comparisons run on the integer pipe, not the slow FP64 one.
struct Extremes {
  uint64_t xmax, xmin, ymax, ymin;
  __device__ void init() {
    xmax = ymax = okey(-INFINITY);
    xmin = ymin = okey(INFINITY);
  }
  __device__ void add(double x, double y) {
    const uint64_t kx = okey(x), ky = okey(y);
    xmax = kx > xmax ? kx : xmax;
    xmin = kx < xmin ? kx : xmin;
    ymax = ky > ymax ? ky : ymax;
    ymin = ky < ymin ? ky : ymin;
  }
  __device__ void add(const Extremes &o) {
    xmax = o.xmax > xmax ? o.xmax : xmax;
    xmin = o.xmin < xmin ? o.xmin : xmin;
    ymax = o.ymax > ymax ? o.ymax : ymax;
    ymin = o.ymin < ymin ? o.ymin : ymin;
  }
  // over the block (blockDim.x <= 256); the result is valid in thread 0
  __device__ void reduce_block() {
    for (int o = 16; o; o >>= 1) {
      Extremes t;
      t.xmax = __shfl_xor_sync(0xffffffffu, xmax, o);
      t.xmin = __shfl_xor_sync(0xffffffffu, xmin, o);
      t.ymax = __shfl_xor_sync(0xffffffffu, ymax, o);
      t.ymin = __shfl_xor_sync(0xffffffffu, ymin, o);
      add(t);
    }
    __shared__ Extremes s[8];
    if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = *this;
    __syncthreads();
    if (threadIdx.x == 0)
      for (int k = 1; k < (int)(blockDim.x >> 5); k++) add(s[k]);
  }
  // as doubles (-0 as +0, which compares the same)
  __device__ Box4 box() const { return Box4{okey_inv(xmax), okey_inv(xmin), okey_inv(ymax), okey_inv(ymin)}; }
};

// Bounding box of the positions (non-finite positions are bad input; the
// circulations and core radii are checked where they are first read, in
// k_gather).
__global__ void __launch_bounds__(256) k_bbox(const double *__restrict__ xy, int n, Box4 *part, DevStatus *st) {
  Extremes ex;
  ex.init();
  bool bad = false;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const double x = xy[2 * i], y = xy[2 * i + 1];  // the caller's array: 8-byte alignment only
    bad |= !(isfinite(x) && isfinite(y));
    ex.add(x, y);
  }
  if (__syncthreads_or(bad) && threadIdx.x == 0) set_err(st, TREE2D_ERR_BAD_INPUT);
  ex.reduce_block();
  if (threadIdx.x == 0) part[blockIdx.x] = ex.box();
}

// Root box of a blob set from its coordinate extremes (quadtree.c:87-98).
__device__ __forceinline__ RootBox root_from_box(const Box4 &r) {
  const double rx = __dadd_rn(fabs(__dsub_rn(r.x, r.y)), 0.0001);
  const double ry = __dadd_rn(fabs(__dsub_rn(r.z, r.w)), 0.0001);
  RootBox b;
  b.region = rx > ry ? rx : ry;
  b.cx = __dmul_rn(0.5, __dadd_rn(r.x, r.y));
  b.cy = __dmul_rn(0.5, __dadd_rn(r.z, r.w));
  b.xmax = r.x;
  b.xmin = r.y;
  b.ymax = r.z;
  b.ymin = r.w;
  return b;
}

// One warp: the lanes reduce strided parts, then a shuffle reduction.
// The root box from the blocks' extremes: one block of kRootThreads.
constexpr int kRootThreads = 256;
__global__ void __launch_bounds__(kRootThreads) k_root(const Box4 *part, int nparts, RootBox *root) {
  uint64_t e[4] = {okey(-INFINITY), okey(INFINITY), okey(-INFINITY), okey(INFINITY)};
  for (int k = threadIdx.x; k < nparts; k += kRootThreads) {
    const Box4 p = part[k];
    const uint64_t v[4] = {okey(p.x), okey(p.y), okey(p.z), okey(p.w)};
#pragma unroll
    for (int q = 0; q < 4; q++) e[q] = (q & 1) ? (v[q] < e[q] ? v[q] : e[q]) : (v[q] > e[q] ? v[q] : e[q]);
  }
  __shared__ uint64_t s[kRootThreads / 32][4];
#pragma unroll
  for (int q = 0; q < 4; q++) {
    for (int o = 16; o; o >>= 1) {
      const uint64_t a = __shfl_xor_sync(0xffffffffu, e[q], o);
      e[q] = (q & 1) ? (a < e[q] ? a : e[q]) : (a > e[q] ? a : e[q]);
    }
    if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5][q] = e[q];
  }
  __syncthreads();
  if (threadIdx.x != 0) return;
  for (int w = 1; w < kRootThreads / 32; w++)
#pragma unroll
    for (int q = 0; q < 4; q++) e[q] = (q & 1) ? (s[w][q] < e[q] ? s[w][q] : e[q]) : (s[w][q] > e[q] ? s[w][q] : e[q]);
  *root = root_from_box(Box4{okey_inv(e[0]), okey_inv(e[1]), okey_inv(e[2]), okey_inv(e[3])});
}
// Batched sets: blocks (set, slice) reduce slice `slice` of the set's blob
// range [off[s], off[s+1]) to a partial box, check the positions and write
// the set id of each blob; k_roots_sets then forms each set's root box from its
// kSetSlices partials (the same formulas as a single set's).
constexpr int kSetSlices = 16;

__global__ void __launch_bounds__(256) k_bbox_sets(const double *__restrict__ xy, const int *__restrict__ off,
                                                   Box4 *part, int *set_of, DevStatus *st) {
  const int set = blockIdx.x;
  const int n0 = off[set], len = off[set + 1] - n0;
  const int per = (len + kSetSlices - 1) / kSetSlices;
  const int b = n0 + min(len, per * (int)blockIdx.y), e = n0 + min(len, per * ((int)blockIdx.y + 1));
  Extremes ex;
  ex.init();
  bool bad = false;
  for (int i = b + threadIdx.x; i < e; i += blockDim.x) {
    const double x = xy[2 * (long)i], y = xy[2 * (long)i + 1];
    bad |= !(isfinite(x) && isfinite(y));
    ex.add(x, y);
    set_of[i] = set;
  }
  if (__syncthreads_or(bad) && threadIdx.x == 0) set_err(st, TREE2D_ERR_BAD_INPUT);
  ex.reduce_block();
  if (threadIdx.x == 0) part[(size_t)set * kSetSlices + blockIdx.y] = ex.box();
}

__global__ void k_roots_sets(const Box4 *part, int nsets, RootBox *roots) {
  const int set = blockIdx.x * blockDim.x + threadIdx.x;
  if (set >= nsets) return;
  Box4 r = part[(size_t)set * kSetSlices];
  for (int k = 1; k < kSetSlices; k++) {
    const Box4 p = part[(size_t)set * kSetSlices + k];
    r.x = fmax(r.x, p.x);
    r.y = fmin(r.y, p.y);
    r.z = fmax(r.z, p.z);
    r.w = fmin(r.w, p.w);
  }
  roots[set] = root_from_box(r);
}

// One level of the reference's descent: digit of (x,y) against the centre,
// then the centre of that child (quadtree.c:29-35, :61-79, :236).
__device__ __forceinline__ unsigned descend(double x, double y, double &cx, double &cy, double &R) {
  unsigned q = (x >= cx ? 1u : 0u) | (y <= cy ? 2u : 0u);
  double h = __dmul_rn(0.25, R);
  cx = (q & 1u) ? __dadd_rn(cx, h) : __dsub_rn(cx, h);
  cy = (q & 2u) ? __dsub_rn(cy, h) : __dadd_rn(cy, h);
  R = __dmul_rn(0.5, R);
  return q;
}


// Centre table of the first `lt` levels: entry (l, i) of the x
// table is the x centre of the level-l cells in column i, formed by the
// same sequence of FP64 operations as the descent (c +- 0.25 R per level,
// quadtree.c:61-79), so comparing against it gives the reference's digits.
// Level l occupies entries [2^l - 1, 2^(l+1) - 1) (2^lt - 1 per axis); the
// y table follows, with row i counted from the top (bit 1 = y <= cy = lower
// half).  16 levels (1 MB) for large sets, 12 (64 KB) otherwise.
inline int centre_levels(int n) { return n > 65536 ? 16 : 12; }
inline size_t centre_entries(int lt) { return ((size_t)1 << lt) - 1; }

__global__ void __launch_bounds__(256) k_centre_table(const RootBox *__restrict__ root, uint64_t *__restrict__ tab,
                                                      int lt) {
  const int per = (1 << lt) - 1;
  root += blockIdx.y;  // batched sets: one table per set root
  tab += (size_t)blockIdx.y * 2 * per;
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= 2 * per) return;
  const int axis = g >= per;
  const int e = g - axis * per;
  const int l = 31 - __clz(e + 1);
  const unsigned i = (unsigned)(e + 1 - (1 << l));
  double c = axis ? root->cy : root->cx, R = root->region;
  for (int j = 0; j < l; j++) {
    const unsigned bit = (i >> (l - 1 - j)) & 1u;
    const double h = __dmul_rn(0.25, R);
    if (axis == 0)
      c = bit ? __dadd_rn(c, h) : __dsub_rn(c, h);
    else
      c = bit ? __dsub_rn(c, h) : __dadd_rn(c, h);
    R = __dmul_rn(0.5, R);
  }
  tab[g] = okey(c);
}

// Batched sets: the table of one set and one axis per block, built level by
// level in shared memory.  Each entry is its parent's centre plus or minus a
// quarter of the parent's side: the same FP64 operation, on the same operands,
// as the last step of k_centre_table's descent, so the values are equal
// (one operation per entry instead of one per level).
constexpr int kSetTableLevels = 12;
__global__ void __launch_bounds__(256) k_centre_table_sets(const RootBox *__restrict__ root,
                                                           uint64_t *__restrict__ tab, int lt) {
  __shared__ double c[(1 << kSetTableLevels) - 1];
  const int per = (1 << lt) - 1;
  const int set = blockIdx.x >> 1, axis = blockIdx.x & 1;
  root += set;
  tab += (size_t)set * 2 * per + (size_t)axis * per;
  double R = root->region;
  if (threadIdx.x == 0) c[0] = axis ? root->cy : root->cx;
  __syncthreads();
  for (int l = 1; l < lt; l++) {
    const double h = __dmul_rn(0.25, R);  // R = R0 * 2^-(l-1)
    const int off = (1 << l) - 1, poff = (1 << (l - 1)) - 1;
    for (int i = threadIdx.x; i < (1 << l); i += blockDim.x) {
      const double p = c[poff + (i >> 1)];
      const bool bit = i & 1;
      c[off + i] = axis == 0 ? (bit ? __dadd_rn(p, h) : __dsub_rn(p, h)) : (bit ? __dsub_rn(p, h) : __dadd_rn(p, h));
    }
    R = __dmul_rn(0.5, R);
    __syncthreads();
  }
  for (int g = threadIdx.x; g < per; g += blockDim.x) tab[g] = okey(c[g]);
}

// `levels` digits, level 1 in the top two bits, zero below the last level.
// With a centre table of `tlev` levels the first digits are integer
// compares against it; the rest continue the FP64 descent from the centre
// of the level-tlev cell.
// Batched sets (`set_of` non-null): the digits are those of the blob's own
// set root, preceded by `lev0` digits that place the set's root in tile
// (2a, 2b) of a 2^lev0 x 2^lev0 grid (set = b * 2^(lev0-1) + a): the set
// roots become the level-lev0 cells of one tree, and the empty tiles
// between them keep every set's cells from touching another set's.
__device__ __forceinline__ uint64_t set_prefix(int set, int lev0) {
  const unsigned w = 1u << (lev0 - 1);
  const unsigned tx = 2u * ((unsigned)set % w), ty = 2u * ((unsigned)set / w);
  uint64_t p = 0;
  for (int j = lev0 - 1; j >= 0; j--) p = (p << 2) | ((tx >> j) & 1u) | (((ty >> j) & 1u) << 1);
  return p;
}

// Index of the level-lt cell along one axis, from f = the position's
// fraction of the root box along it (0..1, in the direction the index grows),
// computed in FP32: |f - exact| < 2.5 * 2^-24 (a rounded offset from the
// centre, a rounded reciprocal of the side, one fused multiply-add), i.e.
// below 0.01 of a level-16 cell.  With u = f * 2^lt, the decisions of all
// levels follow from floor(u) unless u lies within kCandEps of an integer k,
// the split of exactly one level j (k an odd multiple of 2^(lt-1-j)); that
// decision is read from the table -- okey >= centre for x, okey <= centre for
// y (the reference's y >= / <= comparisons) -- and puts the cell at k or k-1.
// Deeper splits are at least half a cell away, so no other decision moves.
constexpr float kCandEps = 0.05f;

__device__ __forceinline__ unsigned axis_index(float f, int lt, uint64_t okey_pos, const uint64_t *__restrict__ tab_axis,
                                               bool le) {
  const float span = (float)(1u << lt);
  const float u = f * span;
  const float k = rintf(u);
  unsigned i = (unsigned)fminf(fmaxf(floorf(u), 0.f), span - 1.f);
  if (fabsf(u - k) < kCandEps && k > 0.f && k < span) {
    const unsigned kk = (unsigned)k;
    const int j = lt - __ffs(kk);  // level whose split is at kk
    const uint64_t c = __ldg(tab_axis + (1 << j) - 1 + (kk >> (lt - j)));
    const bool upper = le ? okey_pos <= c : okey_pos >= c;
    i = upper ? kk : kk - 1;
  }
  return i;
}

// `packed` (at most 16 digits in all): one word per blob, the key in the
// high 32 bits and the blob's index in the low 32 (vals unused).
__global__ void __launch_bounds__(256) k_keys(const double *__restrict__ xy, int n, const RootBox *__restrict__ root,
                                              const uint64_t *__restrict__ tab, int tlev, uint64_t *__restrict__ keys,
                                              uint32_t *__restrict__ vals, int levels, const int *__restrict__ set_of,
                                              int lev0, int packed) {
  long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  double x = xy[2 * i], y = xy[2 * i + 1];
  int set = 0;
  if (set_of) {
    set = set_of[i];
    root += set;
    if (tab) tab += (size_t)set * 2 * ((1 << tlev) - 1);
  }
  double cx = root->cx, cy = root->cy, R = root->region;
  uint64_t key = 0;
  int l = 0;
  if (tab) {
    const uint64_t xk = okey(x), yk = okey(y);
    const int lt = min(levels, tlev);
    const int ybase = (1 << tlev) - 1;
    // The level-lt cell from the position's fraction of the root box, in
    // FP32 (FP64 arithmetic is slow on this part): at most one level's
    // decision along each axis can differ from the reference's, the one
    // whose split passes within the FP32 error of the position; that
    // decision alone is taken from the table (axis_index).
    const float rinv = __frcp_rn((float)R);
    unsigned ix = axis_index(fmaf((float)(x - cx), rinv, 0.5f), lt, xk, tab, false);
    unsigned iy = axis_index(fmaf((float)(cy - y), rinv, 0.5f), lt, yk, tab + ybase, true);
    for (; l < lt; l++) {
      const int sh = lt - 1 - l;
      key = (key << 2) | ((ix >> sh) & 1u) | (((iy >> sh) & 1u) << 1);
    }
    if (l < levels) {
      // centre of the level-lt cell: its parent's centre +- a quarter side
      const int off = (1 << (lt - 1)) - 1;
      const double px = okey_inv(tab[off + (ix >> 1)]), py = okey_inv(tab[ybase + off + (iy >> 1)]);
      for (int j = 0; j < lt - 1; j++) R = __dmul_rn(0.5, R);
      const double h = __dmul_rn(0.25, R);
      cx = (ix & 1u) ? __dadd_rn(px, h) : __dsub_rn(px, h);
      cy = (iy & 1u) ? __dsub_rn(py, h) : __dadd_rn(py, h);
      R = __dmul_rn(0.5, R);
    }
  }
#pragma unroll 4
  for (; l < levels; l++) key = (key << 2) | descend(x, y, cx, cy, R);
  int total = levels;
  if (set_of) {
    key |= set_prefix(set, lev0) << (2 * levels);
    total += lev0;
  }
  if (packed) {
    keys[i] = (key << (64 - 2 * total)) | (uint64_t)(uint32_t)i;
    return;
  }
  keys[i] = total < kKeyLevels ? key << (64 - 2 * total) : key;
  vals[i] = (uint32_t)i;
}

__global__ void __launch_bounds__(256) k_cpl(const uint64_t *__restrict__ keys, int n, int num_p,
                                             uint8_t *__restrict__ cpl, uint8_t *__restrict__ w) {
  long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i + 1 < n) cpl[i] = (uint8_t)common_levels(keys[i], keys[i + 1]);
  if (i + num_p - 1 < n) w[i] = (uint8_t)common_levels(keys[i], keys[i + num_p - 1]);
}

// Sliding maximum of w over the num_p windows that contain position i.
// Tile of kLLTile outputs; two shared buffers hold w[tile-H .. tile+kLLTile)
// (H = num_p-1) and the log-step doubling ping-pongs between them:
// after the step of width k, buf[t] = max(w[t .. t+k-1]).
constexpr int kLLTile = 2048;
// `lev0` > 0 (batched sets): the container cells above the set roots and
// the set roots themselves are always split, as a single set's root is.
__global__ void __launch_bounds__(256) k_leaf_level(const uint8_t *__restrict__ w, int n, int num_p,
                                                    uint8_t *__restrict__ leaf_level, DevStatus *st, int levels,
                                                    int lev0) {
  extern __shared__ uint8_t sbuf[];
  const int H = num_p - 1;
  const long tile0 = (long)blockIdx.x * kLLTile;
  const int len = kLLTile + H;
  uint8_t *cur = sbuf, *nxt = sbuf + len;
  const long nw = (long)n - num_p + 1;  // number of windows
  for (int t = threadIdx.x; t < len; t += blockDim.x) {
    long j = tile0 - H + t;
    cur[t] = (j >= 0 && j < nw) ? w[j] : 0;
  }
  __syncthreads();
  const int W = num_p;
  int K = 1;
  while (K * 2 <= W) K *= 2;
  for (int k = 1; k < K; k *= 2) {
    for (int t = threadIdx.x; t < len; t += blockDim.x) {
      uint8_t a = cur[t];
      uint8_t b = (t + k < len) ? cur[t + k] : 0;
      nxt[t] = a > b ? a : b;
    }
    __syncthreads();
    uint8_t *tmp = cur;
    cur = nxt;
    nxt = tmp;
  }
  int local_max = 0;
  for (int t = threadIdx.x; t < kLLTile; t += blockDim.x) {
    long i = tile0 + t;
    if (i >= n) break;
    // window starts j in [i-H, i]  ->  buffer [t, t+H]
    uint8_t a = cur[t];
    uint8_t b = cur[t + W - K];
    int s = a > b ? a : b;
    s = s > lev0 ? s : lev0;
    if (s >= levels) {
      // a cell at the deepest key level still holds >= num_p blobs
      if (levels < kKeyLevels)
        atomicExch(&st->deeper, 1);
      else
        set_err(st, TREE2D_ERR_TOO_DEEP);
      s = levels - 1;
    }
    leaf_level[i] = (uint8_t)(s + 1);
    local_max = max(local_max, s + 1);
  }
  for (int o = 16; o; o >>= 1) local_max = max(local_max, __shfl_xor_sync(0xffffffffu, local_max, o));
  if ((threadIdx.x & 31) == 0) atomicMax(&st->depth, local_max);
}

__device__ __forceinline__ void cell_counts(const uint8_t *cpl, const uint8_t *leaf_level, long i, int n,
                                            unsigned &ncell, unsigned &isleaf) {
  ncell = 0;
  isleaf = 0;
  if (i < n) {
    int prev = i > 0 ? cpl[i - 1] : 0;
    int lam = leaf_level[i];
    if (lam > prev) {
      ncell = (unsigned)(lam - prev);
      isleaf = 1;
    }
  }
}

// pack: cells in the high 32 bits, leaves in the low 32 bits
__global__ void __launch_bounds__(kScanThreads) k_cells_reduce(const uint8_t *cpl, const uint8_t *leaf_level, int n,
                                                               unsigned long long *part) {
  unsigned long long s = 0;
  long base = (long)blockIdx.x * kScanTile;
  for (int k = threadIdx.x; k < kScanTile; k += kScanThreads) {
    unsigned c, l;
    cell_counts(cpl, leaf_level, base + k, n, c, l);
    s += ((unsigned long long)c << 32) | l;
  }
  for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  __shared__ unsigned long long ws[kScanThreads / 32];
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long t = 0;
    for (int k = 0; k < kScanThreads / 32; k++) t += ws[k];
    part[blockIdx.x] = t;
  }
}

// exclusive scan of the tile partials (one block); total -> *total
__global__ void __launch_bounds__(1024) k_scan_part(unsigned long long *part, int len, unsigned long long *total) {
  __shared__ unsigned long long s[1024];
  const int t = threadIdx.x;
  const int per = (len + 1023) / 1024;
  const int b = t * per, e = min(len, b + per);
  unsigned long long acc = 0;
  for (int i = b; i < e; i++) acc += part[i];
  s[t] = acc;
  __syncthreads();
  for (int off = 1; off < 1024; off <<= 1) {
    unsigned long long v = t >= off ? s[t - off] : 0;
    __syncthreads();
    s[t] += v;
    __syncthreads();
  }
  unsigned long long run = t == 0 ? 0 : s[t - 1];
  for (int i = b; i < e; i++) {
    unsigned long long c = part[i];
    part[i] = run;
    run += c;
  }
  if (t == 1023) *total = s[1023];
}

struct EmitArgs {
  const uint64_t *keys;
  const uint8_t *cpl;
  const uint8_t *leaf_level;
  const unsigned long long *part;
  const RootBox *root;
  int n;
  unsigned *cellbase;  // per position: id of the first cell it starts
  int *level, *begin;
  unsigned char *leaf;
  double *cx, *cy, *region;
  int *leaf_cell;
  const uint64_t *tab;  // centre table(s) of `tlev` levels (k_centre_table), one per set
  int tlev;
  int lev0;             // batched sets: levels above the set roots (0 = one set)
};

// x (even) or y (odd) bits of the top 2*l key bits, compacted: the column
// or row index of the level-l cell holding the key.
__device__ __forceinline__ unsigned key_axis(uint64_t key, int l, int axis) {
  if (l == 0) return 0u;
  uint64_t v = (key >> (64 - 2 * l) >> axis) & 0x5555555555555555ull;
  v = (v | (v >> 1)) & 0x3333333333333333ull;
  v = (v | (v >> 2)) & 0x0f0f0f0f0f0f0f0full;
  v = (v | (v >> 4)) & 0x00ff00ff00ff00ffull;
  v = (v | (v >> 8)) & 0x0000ffff0000ffffull;
  v = (v | (v >> 16)) & 0x00000000ffffffffull;
  return (unsigned)v;
}

// Set of a key in a batched tree: its first lev0 digits name tile
// (2a, 2b), set = b * 2^(lev0-1) + a (the layout k_keys writes).
__device__ __forceinline__ int set_of_key(uint64_t key, int lev0) {
  const unsigned tx = key_axis(key, lev0, 0), ty = key_axis(key, lev0, 1);
  return (int)((ty >> 1) * (1u << (lev0 - 1)) + (tx >> 1));
}

// Centre and side of the level-`lev` cell holding `key`, bit-identical to
// the reference's descent: read from the centre table up to its last level,
// then continued in FP64 (c +- 0.25 R per level).  In a batched tree the
// geometry is that of the key's own set (the container cells above the set
// roots have none: zero).
__device__ __forceinline__ void cell_geometry(const EmitArgs &a, uint64_t key, int lev, double &cx, double &cy,
                                              double &R) {
  const uint64_t *tab = a.tab;
  const RootBox *root = a.root;
  if (a.lev0 > 0) {
    if (lev < a.lev0) {
      cx = cy = R = 0.0;
      return;
    }
    const int set = set_of_key(key, a.lev0);
    root += set;
    tab += (size_t)set * 2 * ((1 << a.tlev) - 1);
    key <<= 2 * a.lev0;
    lev -= a.lev0;
  }
  const int l0 = min(lev, a.tlev - 1);
  const int off = (1 << l0) - 1, ybase = (1 << a.tlev) - 1;
  cx = okey_inv(tab[off + key_axis(key, l0, 0)]);
  cy = okey_inv(tab[ybase + off + key_axis(key, l0, 1)]);
  R = root->region;
  for (int j = 0; j < l0; j++) R = __dmul_rn(0.5, R);  // exact: R0 * 2^-l0
  for (int l = l0 + 1; l <= lev; l++) {
    const unsigned q = (unsigned)(key >> (64 - 2 * l)) & 3u;
    const double h = __dmul_rn(0.25, R);
    cx = (q & 1u) ? __dadd_rn(cx, h) : __dsub_rn(cx, h);
    cy = (q & 2u) ? __dsub_rn(cy, h) : __dadd_rn(cy, h);
    R = __dmul_rn(0.5, R);
  }
}

__global__ void __launch_bounds__(kScanThreads) k_emit_cells(EmitArgs a) {
  const long base = (long)blockIdx.x * kScanTile + (long)threadIdx.x * kScanItems;
  unsigned c[kScanItems], l[kScanItems];
  unsigned long long mine = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; k++) {
    cell_counts(a.cpl, a.leaf_level, base + k, a.n, c[k], l[k]);
    mine += ((unsigned long long)c[k] << 32) | l[k];
  }
  // block exclusive scan of `mine`
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  unsigned long long incl = mine;
  for (int o = 1; o < 32; o <<= 1) {
    unsigned long long v = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += v;
  }
  __shared__ unsigned long long wsum[kScanThreads / 32];
  if (lane == 31) wsum[warp] = incl;
  __syncthreads();
  unsigned long long woff = 0;
  for (int k = 0; k < warp; k++) woff += wsum[k];
  unsigned long long run = a.part[blockIdx.x] + woff + incl - mine;
  const double R0 = a.root->region, cx0 = a.root->cx, cy0 = a.root->cy;
#pragma unroll 1
  for (int k = 0; k < kScanItems; k++) {
    long i = base + k;
    if (i >= a.n) break;
    unsigned cell0 = 1u + (unsigned)(run >> 32);  // root is cell 0
    unsigned leaf0 = (unsigned)(run & 0xffffffffu);
    a.cellbase[i] = cell0;
    if (c[k]) {
      int prev = i > 0 ? a.cpl[i - 1] : 0;
      int lam = a.leaf_level[i];
      uint64_t key = a.keys[i];
      for (int lev = prev + 1; lev <= lam; lev++) {
        double cx, cy, R;
        cell_geometry(a, key, lev, cx, cy, R);
        {
          unsigned id = cell0 + (unsigned)(lev - prev - 1);
          a.level[id] = lev;
          a.begin[id] = (int)i;
          a.leaf[id] = (lev == lam) ? 1 : 0;
          a.cx[id] = cx;
          a.cy[id] = cy;
          a.region[id] = R;
          if (lev == lam) a.leaf_cell[leaf0] = (int)id;
        }
      }
    }
    run += ((unsigned long long)c[k] << 32) | l[k];
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    a.level[0] = 0;
    a.begin[0] = 0;
    a.leaf[0] = 0;
    a.cx[0] = a.lev0 ? 0.0 : cx0;  // a batched tree's root is a container
    a.cy[0] = a.lev0 ? 0.0 : cy0;
    a.region[0] = a.lev0 ? 0.0 : R0;
  }
}

__global__ void __launch_bounds__(256) k_cell_end(const uint64_t *__restrict__ keys, int n, int ncell,
                                                  const int *__restrict__ level, const int *__restrict__ begin,
                                                  int *__restrict__ end) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncell) return;
  if (c == 0) {
    end[0] = n;
    return;
  }
  int lev = level[c];
  int b = begin[c];
  uint64_t k = keys[b];
  int s = 64 - 2 * lev;
  uint64_t hi = (s == 0) ? k : (k | ((1ull << s) - 1));
  // first position in (b, n) whose key > hi
  int lo = b + 1, up = n;
  while (lo < up) {
    int mid = lo + ((up - lo) >> 1);
    if (keys[mid] <= hi)
      lo = mid + 1;
    else
      up = mid;
  }
  end[c] = lo;
}

__global__ void __launch_bounds__(256) k_children(const uint64_t *__restrict__ keys, const uint8_t *__restrict__ cpl,
                                                  const unsigned *__restrict__ cellbase, int ncell,
                                                  const int *__restrict__ level, const int *__restrict__ begin,
                                                  const int *__restrict__ end, const unsigned char *__restrict__ leaf,
                                                  int *__restrict__ child) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncell) return;
  int4 ch = make_int4(-1, -1, -1, -1);
  if (!leaf[c] && end[c] > begin[c]) {
    int lev = level[c] + 1;
    int pos = begin[c], e = end[c];
    int id = c + 1;
    for (int k = 0; k < 4 && pos < e; k++) {
      if (k > 0) {
        int prev = cpl[pos - 1];
        id = (int)cellbase[pos] + (lev - prev - 1);
      }
      unsigned q = (unsigned)(keys[pos] >> (64 - 2 * lev)) & 3u;
      (&ch.x)[q] = id;
      pos = end[id];
    }
  }
  reinterpret_cast<int4 *>(child)[c] = ch;
}

// A warp's 32 K values (element k * 32 + lane in v[k] of that lane) sorted
// ascending by a bitonic network: partners within a lane's column by
// shuffles, across its registers by exchanges.  Fully unrolled, so v stays
// in registers.
template <int K>
__device__ __forceinline__ void warp_bitonic_sort(uint32_t (&v)[K], int lane) {
  constexpr int N = 32 * K;
#pragma unroll
  for (int size = 2; size <= N; size <<= 1) {
#pragma unroll
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      uint32_t p[K];
#pragma unroll
      for (int k = 0; k < K; k++)
        p[k] = stride < 32 ? __shfl_xor_sync(0xffffffffu, v[k], stride) : v[k ^ (stride >> 5)];
#pragma unroll
      for (int k = 0; k < K; k++) {
        const int i = k * 32 + lane;
        const bool up = (i & size) == 0, low = (i & stride) == 0;
        v[k] = low == up ? min(v[k], p[k]) : max(v[k], p[k]);
      }
    }
  }
}

// Blobs of leaf [b, e) in ascending original index (the values are the
// indices, all different): a bitonic sort in registers for up to 32 K.
template <int K>
__device__ __forceinline__ void leaf_sort(const uint32_t *__restrict__ vals, int b, int e, int lane,
                                          int *__restrict__ perm) {
  uint32_t v[K];
#pragma unroll
  for (int k = 0; k < K; k++) {
    const int i = b + k * 32 + lane;
    v[k] = i < e ? vals[i] : 0xffffffffu;  // padding sorts last
  }
  warp_bitonic_sort<K>(v, lane);
#pragma unroll
  for (int k = 0; k < K; k++) {
    const int i = b + k * 32 + lane;
    if (i < e) perm[i] = (int)v[k];
  }
}

// One warp per leaf: blobs of the leaf in ascending original index (leaves
// of more than 128 blobs by counting, for each blob, the smaller ones).
__global__ void __launch_bounds__(256) k_leaf_order(const uint32_t *__restrict__ vals, int nleaf,
                                                    const int *__restrict__ leaf_cell, const int *__restrict__ begin,
                                                    const int *__restrict__ end, int *__restrict__ perm) {
  int wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (wid >= nleaf) return;
  int c = leaf_cell[wid];
  int b = begin[c], e = end[c];
  const int cnt = e - b;
  if (cnt <= 32) {
    leaf_sort<1>(vals, b, e, lane, perm);
  } else if (cnt <= 64) {
    leaf_sort<2>(vals, b, e, lane, perm);
  } else if (cnt <= 128) {
    leaf_sort<4>(vals, b, e, lane, perm);
  } else {
    for (int i = b + lane; i < e; i += 32) {
      uint32_t v = vals[i];
      int rank = 0;
      for (int j = b; j < e; j++) rank += vals[j] < v;
      perm[b + rank] = (int)v;
    }
  }
}

// Blob arrays in tree order, plus 1/sigma^2 for the direct pairs; a
// non-finite circulation or a NaN core radius is bad input.
__global__ void __launch_bounds__(256) k_gather(const double *__restrict__ xy, const double *__restrict__ cir,
                                                const double *__restrict__ cor, const int *__restrict__ perm, int n,
                                                double *x, double *y, double *c, double *r, double *icor2,
                                                DevStatus *st) {
  long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  int p = perm[i];
  const double g = cir[p], rc = cor[p];
  if (!isfinite(g) || isnan(rc)) set_err(st, TREE2D_ERR_BAD_INPUT);
  x[i] = xy[2 * (long)p];
  y[i] = xy[2 * (long)p + 1];
  c[i] = g;
  r[i] = rc;
  icor2[i] = 1.0 / (rc * rc);
}

}  // namespace

size_t build_blob_bytes(int n, int nsets) {
  const int ns = nsets > 1 ? nsets : 1;
  size_t need = 0;
  need += Arena::bytes_for(n, 8) * 5;  // x y cir cor icor2
  need += Arena::bytes_for(n, 4);      // perm
  need += Arena::bytes_for(n, 8);      // keys (sorted)
  need += Arena::bytes_for(n, 4);      // cellbase
  need += Arena::bytes_for(n, 1) * 2;  // cpl, leaf_level
  need += Arena::bytes_for(ns, sizeof(RootBox));
  return need;
}

size_t build_tmp_bytes(int n, int nsets) {
  const bool batched = nsets > 1;
  const int ns = batched ? nsets : 1;
  const int ntiles = (n + kScanTile - 1) / kScanTile;
  size_t tneed = 0;
  tneed += Arena::bytes_for(n, 8) + Arena::bytes_for(n, 4) * 2;  // keys_alt, vals, vals_alt
  tneed += Arena::bytes_for(n, 1);                              // w
  tneed += radix_sort_temp_bytes(n) + 256;
  tneed += Arena::bytes_for(kBoxBlocks, sizeof(Box4));
  tneed += Arena::bytes_for(ntiles + 1, 8) + 256;
  const int tlev = batched ? 12 : centre_levels(n);
  tneed += Arena::bytes_for(2 * centre_entries(tlev) * ns, 8);
  if (batched) tneed += Arena::bytes_for(n, 4) + Arena::bytes_for((size_t)nsets * kSetSlices, sizeof(Box4));
  return tneed;
}

size_t build_cell_bytes(long long ncell, long long nleaf, int nterms) {
  size_t cneed = 0;
  cneed += Arena::bytes_for(ncell, 4) * 3;           // level begin end
  cneed += Arena::bytes_for(ncell * 4, 4);           // child
  cneed += Arena::bytes_for(ncell, 1);               // leaf
  cneed += Arena::bytes_for(ncell, 8) * 3;           // cx cy region
  cneed += Arena::bytes_for(nleaf > 0 ? nleaf : 1, 4);  // leaf_cell
  cneed += Arena::bytes_for(ncell * nterms, 16);     // coef
  cneed += Arena::bytes_for(ncell, 16);              // mac
  cneed += Arena::bytes_for(ncell, 16);              // cf32
  cneed += Arena::bytes_for(ncell, 8);               // macf
  return cneed;
}

int build_tree(Workspace &ws, int n, const double *d_xy, const double *d_cir, const double *d_cor, const Params &p,
               Tree &t, cudaStream_t s, const int *d_set_off, int nsets, cudaEvent_t cir_cor_ready) {
  t.n = n;
  t.nterms = p.nterms;
  t.leaf_cap = p.num_p - 1;
  const bool batched = nsets > 1;
  int lev0 = 0;  // levels of container cells above the set roots
  if (batched) {
    lev0 = 1;
    while ((1ll << (2 * (lev0 - 1))) < (long long)nsets) lev0++;
    if (lev0 + 12 > kKeyLevels) return TREE2D_ERR_TOO_LARGE;
  }
  t.nsets = batched ? nsets : 1;
  t.lev0 = lev0;
  t.set_off = batched ? d_set_off : nullptr;
  t.set_cor = batched ? d_cor : nullptr;
  const int ntiles = (n + kScanTile - 1) / kScanTile;
  // ---- blob-sized buffers
  T2D_CUDA_TRY(ws.blob_arena.reserve(build_blob_bytes(n, nsets)));
  ws.blob_arena.reset();
  t.x = ws.blob_arena.take<double>(n);
  t.y = ws.blob_arena.take<double>(n);
  t.cir = ws.blob_arena.take<double>(n);
  t.cor = ws.blob_arena.take<double>(n);
  t.icor2 = ws.blob_arena.take<double>(n);
  t.perm = ws.blob_arena.take<int>(n);
  t.keys = ws.blob_arena.take<uint64_t>(n);
  unsigned *cellbase = ws.blob_arena.take<unsigned>(n);
  uint8_t *cpl = ws.blob_arena.take<uint8_t>(n);
  uint8_t *leaf_level = ws.blob_arena.take<uint8_t>(n);
  t.root = ws.blob_arena.take<RootBox>(t.nsets);  // one per set
  t.cpl = cpl;
  t.leaf_level = leaf_level;
  t.cellbase = cellbase;

  // ---- scratch
  const int tlev = batched ? 12 : centre_levels(n);
  T2D_CUDA_TRY(ws.tmp_arena.reserve(build_tmp_bytes(n, nsets)));
  ws.tmp_arena.reset();
  uint64_t *keys_alt = ws.tmp_arena.take<uint64_t>(n);
  uint32_t *vals = ws.tmp_arena.take<uint32_t>(n);
  uint32_t *vals_alt = ws.tmp_arena.take<uint32_t>(n);
  uint8_t *w = ws.tmp_arena.take<uint8_t>(n);
  void *sort_tmp = ws.tmp_arena.take<char>(radix_sort_temp_bytes(n));
  Box4 *bpart = ws.tmp_arena.take<Box4>(kBoxBlocks);
  unsigned long long *part = ws.tmp_arena.take<unsigned long long>(ntiles + 1);
  unsigned long long *total = ws.tmp_arena.take<unsigned long long>(1);
  uint64_t *ctab = ws.tmp_arena.take<uint64_t>(2 * centre_entries(tlev) * t.nsets);
  int *set_of = batched ? ws.tmp_arena.take<int>(n) : nullptr;
  Box4 *set_part = batched ? ws.tmp_arena.take<Box4>((size_t)nsets * kSetSlices) : nullptr;

  // Digits below the set root on the first attempt: as few as the tree is
  // likely to need (the previous tree's depth + 2, at least 16 for one set
  // and 10 per set in a batch, where the set prefix takes up to 6 more), so
  // that the keys come from the centre table alone and the sort makes fewer
  // passes (4 of 8 bits up to 16 digits in all).  A deeper tree is caught by
  // the leaf-level pass and rebuilt with the full 32-digit keys.
  const int floor_levels = batched ? 10 : 16;
  int levels = ws.last_depth - lev0 + 2;
  if (levels < floor_levels) levels = floor_levels;
  if (levels > kShortKeyLevels) levels = kShortKeyLevels;
retry:
  T2D_CUDA_TRY(cudaMemsetAsync(ws.status, 0, sizeof(DevStatus), s));

  // 1. root box (per set)
  if (batched) {
    k_bbox_sets<<<dim3((unsigned)nsets, kSetSlices), 256, 0, s>>>(d_xy, d_set_off, set_part, set_of, ws.status);
    k_roots_sets<<<(nsets + 127) / 128, 128, 0, s>>>(set_part, nsets, t.root);
    ::t2d::g_launches.fetch_add(2, std::memory_order_relaxed);
  } else {
    k_bbox<<<kBoxBlocks, 256, 0, s>>>(d_xy, n, bpart, ws.status);
    k_root<<<1, kRootThreads, 0, s>>>(bpart, kBoxBlocks, t.root);
    ::t2d::g_launches.fetch_add(2, std::memory_order_relaxed);
  }
  // 2. keys
  const int total_levels = levels + lev0;
  if (batched && tlev <= kSetTableLevels)
    k_centre_table_sets<<<2 * (unsigned)t.nsets, 256, 0, s>>>(t.root, ctab, tlev);
  else
    k_centre_table<<<dim3((unsigned)((2 * centre_entries(tlev) + 255) / 256), (unsigned)t.nsets), 256, 0, s>>>(
        t.root, ctab, tlev);
  // Up to 16 digits the key and the blob index share one word: the sort
  // then moves 8 bytes per blob and pass instead of 12, and its last pass
  // writes them out split.  The words start in the buffer that the last
  // pass does not read, so that its output lands in t.keys.
  const bool packed = 2 * total_levels <= 32 && n >= 2;
  const int passes = (2 * total_levels + 7) / 8;
  uint64_t *words = packed && (passes & 1) ? keys_alt : t.keys;
  k_keys<<<(n + 255) / 256, 256, 0, s>>>(d_xy, n, t.root, ctab, tlev, words, vals, levels, set_of, lev0,
                                         packed ? 1 : 0);
  ::t2d::g_launches.fetch_add(2, std::memory_order_relaxed);
  // 3. sort
  if (packed)
    T2D_CUDA_TRY(radix_sort_packed(words, words == t.keys ? keys_alt : t.keys, n, 64 - 2 * total_levels, t.keys,
                                   vals, sort_tmp, ws.status, s));
  else
    T2D_CUDA_TRY(radix_sort_pairs(t.keys, vals, keys_alt, vals_alt, n, 64 - 2 * total_levels, 64, sort_tmp, s));
  t.key_order = vals;
  // 4-5. leaf levels
  k_cpl<<<(n + 255) / 256, 256, 0, s>>>(t.keys, n, p.num_p, cpl, w);
  ::t2d::g_launches.fetch_add(1, std::memory_order_relaxed);
  {
    const int H = p.num_p - 1;
    size_t smem = 2 * (size_t)(kLLTile + H);
    if (smem > 48 * 1024) T2D_CUDA_TRY(cudaFuncSetAttribute(k_leaf_level, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_leaf_level<<<(n + kLLTile - 1) / kLLTile, 256, smem, s>>>(w, n, p.num_p, leaf_level, ws.status, total_levels,
                                                                lev0);
    ::t2d::g_launches.fetch_add(1, std::memory_order_relaxed);
  }
  // 6. counts and scan
  k_cells_reduce<<<ntiles, kScanThreads, 0, s>>>(cpl, leaf_level, n, part);
  ::t2d::g_launches.fetch_add(1, std::memory_order_relaxed);
  k_scan_part<<<1, 1024, 0, s>>>(part, ntiles, total);
  ::t2d::g_launches.fetch_add(1, std::memory_order_relaxed);
  T2D_CUDA_TRY(cudaGetLastError());
  T2D_CUDA_TRY(cudaMemcpyAsync(ws.h_status, ws.status, sizeof(DevStatus), cudaMemcpyDeviceToHost, s));
  unsigned long long *h_total = reinterpret_cast<unsigned long long *>(ws.h_status + 1);
  T2D_CUDA_TRY(cudaMemcpyAsync(h_total, total, 8, cudaMemcpyDeviceToHost, s));
  T2D_CUDA_TRY(cudaStreamSynchronize(s));
  if (ws.h_status->err) return ws.h_status->err;
  if (ws.h_status->deeper && total_levels < kKeyLevels) {
    levels = kKeyLevels - lev0;  // rare: a cell at the short depth still needs splitting
    goto retry;
  }
  t.key_levels = total_levels;
  ws.last_depth = ws.h_status->depth;
  unsigned long long tot = *h_total;
  long long ncell = 1 + (long long)(tot >> 32);
  long long nleaf = (long long)(tot & 0xffffffffu);
  if (ncell > (1ll << 31) - 1) return TREE2D_ERR_TOO_DEEP;
  t.ncell = (int)ncell;
  t.nleaf = (int)nleaf;
  t.depth = ws.h_status->depth;
  const int nt = p.nterms;

  // ---- cell-sized buffers
  T2D_CUDA_TRY(ws.cell_arena.reserve(build_cell_bytes(ncell, nleaf, nt)));
  ws.cell_arena.reset();
  t.level = ws.cell_arena.take<int>(ncell);
  t.begin = ws.cell_arena.take<int>(ncell);
  t.end = ws.cell_arena.take<int>(ncell);
  t.child = ws.cell_arena.take<int>(ncell * 4);
  t.leaf = ws.cell_arena.take<unsigned char>(ncell);
  t.cx = ws.cell_arena.take<double>(ncell);
  t.cy = ws.cell_arena.take<double>(ncell);
  t.region = ws.cell_arena.take<double>(ncell);
  t.leaf_cell = ws.cell_arena.take<int>(nleaf > 0 ? nleaf : 1);
  t.coef = ws.cell_arena.take<double2>(ncell * nt);
  t.mac = ws.cell_arena.take<double2>(ncell);
  t.cf32 = ws.cell_arena.take<float4>(ncell);
  t.macf = ws.cell_arena.take<float2>(ncell);
  ws.mac_theta = -1.0;

  // 7. cells
  EmitArgs ea{t.keys, cpl, leaf_level, part, t.root, n, cellbase, t.level, t.begin, t.leaf, t.cx, t.cy, t.region,
              t.leaf_cell, ctab, tlev, lev0};
  k_emit_cells<<<ntiles, kScanThreads, 0, s>>>(ea);
  ::t2d::g_launches.fetch_add(1, std::memory_order_relaxed);
  k_cell_end<<<(t.ncell + 255) / 256, 256, 0, s>>>(t.keys, n, t.ncell, t.level, t.begin, t.end);
  ::t2d::g_launches.fetch_add(1, std::memory_order_relaxed);
  k_children<<<(t.ncell + 255) / 256, 256, 0, s>>>(t.keys, cpl, cellbase, t.ncell, t.level, t.begin, t.end, t.leaf,
                                                    t.child);
  ::t2d::g_launches.fetch_add(1, std::memory_order_relaxed);
  // 8. in-leaf order, 9. gather
  if (t.nleaf > 0) {
    k_leaf_order<<<(int)(((long)t.nleaf * 32 + 255) / 256), 256, 0, s>>>(vals, t.nleaf, t.leaf_cell, t.begin, t.end,
                                                                          t.perm);
    ::t2d::g_launches.fetch_add(1, std::memory_order_relaxed);
  }
  if (cir_cor_ready) T2D_CUDA_TRY(cudaStreamWaitEvent(s, cir_cor_ready, 0));
  k_gather<<<(n + 255) / 256, 256, 0, s>>>(d_xy, d_cir, d_cor, t.perm, n, t.x, t.y, t.cir, t.cor, t.icor2,
                                           ws.status);
  ::t2d::g_launches.fetch_add(1, std::memory_order_relaxed);
  T2D_CUDA_TRY(cudaGetLastError());
  return TREE2D_OK;
}

int sort_targets(Workspace &ws, int n, const double *d_xy, const RootBox *d_root, int *d_order, cudaStream_t s) {
  if (n <= 0) return TREE2D_OK;
  size_t need = Arena::bytes_for(n, 8) * 2 + Arena::bytes_for(n, 4) + radix_sort_temp_bytes(n) + 512;
  T2D_CUDA_TRY(ws.tmp_arena.reserve(need));
  ws.tmp_arena.reset();
  uint64_t *k = ws.tmp_arena.take<uint64_t>(n);
  uint64_t *k2 = ws.tmp_arena.take<uint64_t>(n);
  uint32_t *v2 = ws.tmp_arena.take<uint32_t>(n);
  void *tmp = ws.tmp_arena.take<char>(radix_sort_temp_bytes(n));
  // order only (for coherent warps): the short key depth is enough
  k_keys<<<(n + 255) / 256, 256, 0, s>>>(d_xy, n, d_root, nullptr, 0, k, reinterpret_cast<uint32_t *>(d_order),
                                          kShortKeyLevels, nullptr, 0, 0);
  ::t2d::g_launches.fetch_add(1, std::memory_order_relaxed);
  T2D_CUDA_TRY(radix_sort_pairs(k, reinterpret_cast<uint32_t *>(d_order), k2, v2, n, 64 - 2 * kShortKeyLevels, 64,
                                tmp, s));
  return TREE2D_OK;
}

}  // namespace t2d

namespace t2d {
namespace {
__global__ void k_gather_targets(const double *__restrict__ xy, const int *__restrict__ order, int n,
                                 double *__restrict__ tx, double *__restrict__ ty, int *__restrict__ out_idx) {
  long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  int o = order ? order[i] : (int)i;
  tx[i] = xy[2 * (long)o];
  ty[i] = xy[2 * (long)o + 1];
  out_idx[i] = o;
}
}  // namespace

int gather_targets(int n, const double *d_xy, const int *d_order, double *tx, double *ty, int *out_idx,
                   cudaStream_t s) {
  if (n <= 0) return TREE2D_OK;
  k_gather_targets<<<(n + 255) / 256, 256, 0, s>>>(d_xy, d_order, n, tx, ty, out_idx);
  ::t2d::g_launches.fetch_add(1, std::memory_order_relaxed);
  T2D_CUDA_TRY(cudaGetLastError());
  return TREE2D_OK;
}
}  // namespace t2d
