// Mixed-precision FMM on the device (TREE2D_MODE_MIXED).
//
// The tree is the plain path's (same FP64 keys, same cells).  On it runs an
// adaptive FMM (Carrier-Greengard-Rokhlin lists) for the point-vortex part
// of the kernel, plus a short-range correction for the blob regularisation:
//
//   U(B)  leaf B: leaves adjacent to B (any level)       -> P2P, regularised
//   V(C)  cell C: children of parent(C)'s colleagues not
//         adjacent to C; 27 fixed offsets per child class -> M2L (dense
//         contraction over all cells of a class, m2l.cu)
//   W(B)  leaf B: descendants of B's colleagues not adjacent
//         to B whose parent is adjacent                    -> M2P at B's targets
//   X(C)  cell C: leaves coarser than C, adjacent to
//         parent(C), not adjacent to C                     -> P2L into C
//   K(B)  leaf B: leaves not adjacent to B whose box lies
//         within rc of B's box (rc = cutoff * max sigma)   -> Gaussian correction
//                                                             -G e^{-r^2/s^2}/r^2
//
// The far field treats blobs as point vortices; the exact kernel differs
// from that by -G exp(-r^2/sigma^2)/r, which K(B) adds back for every pair
// closer than rc that is not already a direct (U) pair.
//
// Expansions are scaled by the cell side h so coefficients stay O(1):
//   multipole  phi(z) = (1/h) sum_k  a_k ((z - zc)/h)^-(k+1)
//   local      psi(z) = (1/h) sum_l  b_l ((z - zc)/h)^l
// With that scaling every translation operator is level independent:
//   M2M/L2L: 4 matrices (child quadrant), M2L: 4 classes x 27 offsets.
// Formulas: M2L b_l = sum_k a_k (-1)^l C(k+l,l) tau^-(k+l+1) (the Laurent
// re-expansion of ver-fortran/src/fmm.f90:104-139, written for the C
// path's convention phi = sum_j G_j/(z - z_j), u = Im phi/2pi, v = Re phi/2pi
// of ver-c/src/fmm.c:115-117); L2L b'_k = sum_{l>=k} b_l C(l,k) s^(l-k)
// (ver-fortran/src/fmm.f90:142-168); L2P = Horner (fmm.f90:198-206).
//
// Arithmetic: FP32 throughout (positions as FP32 offsets from their leaf
// centre, formed from the FP64 centres), compensated (Kahan) sums for the
// direct and correction terms, FP64 for the final per-target reduction.
#include <cmath>
#include <type_traits>
#include <vector>

#include "dev_common.cuh"
#include "mixed.h"
#include "learn.h"
#include "tc_ptx.cuh"

namespace t2d {
namespace {

// ---------------------------------------------------------------- lookups

struct Found {
  int kind;  // 0 empty, 1 cell at the requested level, 2 coarser leaf
  int id;
};

__device__ __forceinline__ uint64_t interleave(unsigned jx, unsigned jy, int lev) {
  uint64_t p = 0;
  for (int i = lev - 1; i >= 0; i--) p = (p << 2) | ((jx >> i) & 1u) | (((jy >> i) & 1u) << 1);
  return p;
}

// The tree cell covering grid position (jx, jy) of level `lev`.
__device__ Found find_cell(const MixedView &m, int lev, unsigned jx, unsigned jy) {
  const int n = m.n;
  const uint64_t P = interleave(jx, jy, lev);
  const int sh = 64 - 2 * lev;
  const uint64_t Pk = sh >= 64 ? 0 : (P << sh);
  int lo = 0, up = n;
  while (lo < up) {
    int mid = lo + ((up - lo) >> 1);
    if (m.keys[mid] < Pk)
      lo = mid + 1;
    else
      up = mid;
  }
  const int pos = lo;
  if (pos < n && (sh >= 64 ? 0 : (m.keys[pos] >> sh)) == P) {
    int lam = m.leaf_level[pos];
    if (lam >= lev) {
      int prev = pos > 0 ? m.cpl[pos - 1] : 0;
      return {1, (int)m.cellbase[pos] + (lev - prev - 1)};
    }
    return {2, m.leaf_of[pos]};
  }
  int best = -1, nb = -1;
  if (pos > 0) {
    int c = min(common_levels(Pk, m.keys[pos - 1]), lev - 1);
    if (c > best) best = c, nb = pos - 1;
  }
  if (pos < n) {
    int c = min(common_levels(Pk, m.keys[pos]), lev - 1);
    if (c > best) best = c, nb = pos;
  }
  if (nb >= 0 && m.leaf_level[nb] <= best) return {2, m.leaf_of[nb]};
  return {0, -1};
}

// Boxes of cells a (level la) and b (level lb) touch or overlap.
__device__ __forceinline__ bool adjacent(int la, unsigned ax, unsigned ay, int lb, unsigned bx, unsigned by) {
  if (la > lb) {
    int t = la;
    la = lb;
    lb = t;
    unsigned u = ax;
    ax = bx;
    bx = u;
    u = ay;
    ay = by;
    by = u;
  }
  const long long s = 1ll << (lb - la);
  const long long x0 = (long long)ax * s, y0 = (long long)ay * s;
  return (long long)bx >= x0 - 1 && (long long)bx <= x0 + s && (long long)by >= y0 - 1 && (long long)by <= y0 + s;
}

__device__ __forceinline__ bool adj_cells(const MixedView &m, int a, int b) {
  return adjacent(m.level[a], m.ix[a], m.iy[a], m.level[b], m.ix[b], m.iy[b]);
}

// ------------------------------------------------------------ cell setup

__global__ void k_cell_info(MixedView m) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.ncell) return;
  int lev = m.level[c];
  uint64_t k = m.keys[m.begin[c]];
  unsigned ix = 0, iy = 0;
  for (int i = 1; i <= lev; i++) {
    unsigned q = (unsigned)(k >> (64 - 2 * i)) & 3u;
    ix = (ix << 1) | (q & 1u);
    iy = (iy << 1) | (q >> 1);
  }
  m.ix[c] = ix;
  m.iy[c] = iy;
  m.h[c] = (float)m.region[c];
  m.inv_h[c] = (float)(1.0 / m.region[c]);
  m.cxf[c] = (float)m.cx[c];
  m.cyf[c] = (float)m.cy[c];
  m.cxl[c] = (float)(m.cx[c] - (double)m.cxf[c]);
  m.cyl[c] = (float)(m.cy[c] - (double)m.cyf[c]);
}

// Per-position arrays of the mixed form (leaf_of, FP32 offsets from the
// leaf centre, circulation, 1/sigma^2, the near field's source records),
// one warp per leaf.  Inside a leaf the blobs are laid out by sub-cell: the
// leaf is cut into 8 x 8 sub-cells, taken in Morton order, and the blobs of
// one sub-cell keep their tree order (a stable counting sort: each 32-blob
// round groups equal sub-cells with __match_any_sync, shared-memory
// counters hold the running offsets).  Consecutive blobs are then
// neighbours, so a kChunk-blob chunk has a small bounding box (the near field
// culls correction chunks by it), and the layout depends only on the
// leaf's own blobs and geometry: a set gets the same layout alone or in a
// batch.  mperm maps each position to its original blob.  The sub-cell of a
// blob comes from its FP32 offset; the offsets and sub-cells of a leaf's
// first kSetupStage blobs are kept in shared memory between the passes
// (larger leaves form the rest again from global memory).  Each warp's leaf
// is a chain of dependent loads, so the kernel is bounded to 32 registers:
// 64 warps per SM (measured 16.36 -> 16.32 ms for the 512-set batch).
constexpr int kSubCells = 64;
constexpr int kSetupWarps = 8;
constexpr int kSetupStage = 128;

__device__ __forceinline__ unsigned spread3(unsigned v) {  // 3 bits -> even bits of 6
  v = (v | (v << 2)) & 0x13u;
  v = (v | (v << 1)) & 0x15u;
  return v;
}

__global__ void __launch_bounds__(32 * kSetupWarps, 8) k_leaf_setup(MixedView m, const double *x, const double *y,
                                                                 const double *cir, const double *cor,
                                                                 const int *perm) {
  __shared__ int s_cnt[kSetupWarps][kSubCells];
  __shared__ float2 s_lc[kSetupWarps][kSetupStage];   // offsets, in tree order
  __shared__ float2 s_out[kSetupWarps][kSetupStage];  // offsets, in the new order
  __shared__ unsigned char s_code[kSetupWarps][kSetupStage];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int wid = blockIdx.x * kSetupWarps + warp;
  if (wid >= m.nleaf) return;  // warp-uniform; nothing below syncs the block
  int *cnt = s_cnt[warp];
  const int c = m.leaf_cell[wid];
  const double cx = m.cx[c], cy = m.cy[c], side = m.region[c];
  const int b = m.begin[c], e = m.end[c];
  const float hs = (float)(0.5 * side), q = (float)(8.0 / side);
  const unsigned lt = (1u << lane) - 1u;
  auto offset_of = [&](int i) { return make_float2((float)(x[i] - cx), (float)(y[i] - cy)); };
  auto code_of = [&](float2 lc) {
    const int qx = min(max((int)(__fmul_rn(__fadd_rn(lc.x, hs), q)), 0), 7);
    const int qy = min(max((int)(__fmul_rn(__fadd_rn(lc.y, hs), q)), 0), 7);
    return (int)(spread3((unsigned)qx) | (spread3((unsigned)qy) << 1));
  };
  // pass 1: blobs per sub-cell, and whether all share the first one's core
  cnt[lane] = 0;
  cnt[lane + 32] = 0;
  __syncwarp();
  const double cor0 = cor[b];
  bool same = true;
  for (int i0 = b; i0 < e; i0 += 32) {
    const int i = i0 + lane, o = i - b;
    int code = kSubCells;
    if (i < e) {
      same = same && cor[i] == cor0;
      const float2 lc = offset_of(i);
      code = code_of(lc);
      if (o < kSetupStage) {
        s_lc[warp][o] = lc;
        s_code[warp][o] = (unsigned char)code;
      }
    }
    const unsigned grp = __match_any_sync(0xffffffffu, code);
    if (code < kSubCells && (grp & lt) == 0) cnt[code] += __popc(grp);  // one leader per sub-cell
    __syncwarp();
  }
  // s = sqrt(log2 e) / sigma from the FP32 1/sigma^2 the records carry.
  // Scaled records need a finite s whose products with the leaf's offsets
  // stay far inside FP32 (their squares too): a core radius of 0 (the
  // mirror images are point vortices) or one far below the leaf's size
  // keeps the leaf, and so the solve, on the unscaled records.
  const float sf0 = (float)cor0;
  const float s0 = sqrtf(1.44269504f * __frcp_rn(sf0 * sf0));
  const bool uniform = __all_sync(0xffffffffu, same) && s0 > 0.f && __fmul_rn(s0, (float)side) < 1e15f;
  const float sc = uniform ? s0 : 0.f;
  if (lane == 0) {
    m.lscale[c] = sc;
    if (!uniform) m.st->nonuniform = 1;
  }
  // exclusive prefix over the sub-cells (two per lane): the first position of each
  {
    const int c0 = cnt[2 * lane], c1 = cnt[2 * lane + 1];
    int incl = c0 + c1;
    for (int d = 1; d < 32; d <<= 1) {
      const int t = __shfl_up_sync(0xffffffffu, incl, d);
      if (lane >= d) incl += t;
    }
    const int excl = incl - c0 - c1;
    __syncwarp();
    cnt[2 * lane] = excl;
    cnt[2 * lane + 1] = excl + c0;
  }
  __syncwarp();
  // pass 2: place every blob
  for (int i0 = b; i0 < e; i0 += 32) {
    const int i = i0 + lane, o = i - b;
    const bool v = i < e;
    float2 lc = make_float2(0.f, 0.f);
    int code = kSubCells;
    if (v) {
      if (o < kSetupStage) {
        lc = s_lc[warp][o];
        code = s_code[warp][o];
      } else {
        lc = offset_of(i);
        code = code_of(lc);
      }
    }
    const unsigned grp = __match_any_sync(0xffffffffu, code);
    const int r = v ? cnt[code] + __popc(grp & lt) : 0;  // position within the leaf
    __syncwarp();
    if (v && (grp & lt) == 0) cnt[code] += __popc(grp);
    __syncwarp();
    if (v) {
      const int d = b + r;
      if (r < kSetupStage) s_out[warp][r] = lc;
      m.leaf_of[d] = c;
      m.loc[d] = lc;
      const float g = (float)cir[i];
      m.gam[d] = g;
      // 1/sigma^2 is only kept in FP32, so it is formed in FP32 (the FP64
      // divide is slow on this GPU and buys nothing after the rounding);
      // the correctly rounded reciprocal is 1.f / (sf * sf) exactly
      const float sf = (float)cor[i];
      const float w = __frcp_rn(sf * sf);
      m.src4[d] = make_float4(lc.x, lc.y, g, -1.44269504f * w);
      if (uniform) m.src4s[d] = make_float4(__fmul_rn(lc.x, sc), __fmul_rn(lc.y, sc), __fmul_rn(g, sc), 0.f);
      m.mperm[d] = perm[i];
    }
  }
  __syncwarp();
  // each kChunk-blob chunk's bounding box, for the near field's correction
  // cull: a warp covers 32 / kChunk chunks per round, reduced within
  // groups of kChunk lanes
  for (int i0 = b; i0 < e; i0 += 32) {  // warp-uniform
    const int i = i0 + lane, o = i - b;
    const bool v = i < e;
    const float2 lc = !v ? make_float2(0.f, 0.f) : (o < kSetupStage ? s_out[warp][o] : m.loc[i]);
    float bx0 = v ? lc.x : INFINITY, by0 = v ? lc.y : INFINITY, bx1 = v ? lc.x : -INFINITY, by1 = v ? lc.y : -INFINITY;
    for (int sh = kChunk / 2; sh; sh >>= 1) {
      bx0 = fminf(bx0, __shfl_xor_sync(0xffffffffu, bx0, sh));
      by0 = fminf(by0, __shfl_xor_sync(0xffffffffu, by0, sh));
      bx1 = fmaxf(bx1, __shfl_xor_sync(0xffffffffu, bx1, sh));
      by1 = fmaxf(by1, __shfl_xor_sync(0xffffffffu, by1, sh));
    }
    const int k = (o >> kChunkShift);  // this lane's chunk
    if ((lane & (kChunk - 1)) == 0 && v && k < m.kchunks)
      m.cbox[(size_t)c * m.kchunks + k] = make_float4(bx0, by0, bx1, by1);
  }
}

// Same-level 3x3 neighbourhood of every cell: exact cells and coarser leaves.
__global__ void k_colleagues(MixedView m) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.ncell) return;
  const int lev = m.level[c];
  const long long side = 1ll << lev;
  for (int k = 0; k < 9; k++) {
    int dx = k % 3 - 1, dy = k / 3 - 1;
    long long jx = (long long)m.ix[c] + dx, jy = (long long)m.iy[c] + dy;
    int ex = -1, co = -1;
    if (lev >= 1 && jx >= 0 && jy >= 0 && jx < side && jy < side) {
      if (dx == 0 && dy == 0) {
        ex = c;
      } else {
        Found f = find_cell(m, lev, (unsigned)jx, (unsigned)jy);
        if (f.kind == 1) ex = f.id;
        if (f.kind == 2) co = f.id;
      }
    }
    m.coll[c * 9 + k] = ex;
    m.coarse[c * 9 + k] = co;
  }
}

__constant__ signed char c_slot[4][6][6];  // [class][dy+2+qy][dx+2+qx] -> slot (or -1)

// V and X lists of every cell of level >= 2 (counted from its set root).
// One warp per internal cell p builds the lists of p's children: the four
// siblings share p's 3x3 neighbourhood, so lane k loads colleague k of p
// (its children, or itself when it is a leaf, and the coarser leaf at that
// position) once for all four, then every child takes from each lane:
//   V: the colleague's children that are not adjacent to the child, at the
//      slot of their offset (unique per offset, so the lanes write apart);
//   X: the colleague when it is a leaf, or the coarser leaf, when not
//      adjacent to the child (a position has at most one of the two; a
//      coarser leaf seen at several positions is kept once), in position
//      order.
__global__ void __launch_bounds__(256) k_vx_lists(MixedView m) {
  // the slot table in shared memory: the lanes index it divergently, which
  // constant memory would serialise
  __shared__ signed char slot[4][6][6];
  for (int i = threadIdx.x; i < 4 * 6 * 6; i += blockDim.x) (&slot[0][0][0])[i] = (&c_slot[0][0][0])[i];
  __syncthreads();
  const int p = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (p >= m.ncell) return;  // uniform over the warp
  const unsigned lt = (1u << lane) - 1u;
  if (p == 0) {  // the root is nobody's child
    if (lane < 27) m.vlist[lane] = -1;
    if (lane < 8) m.xlist[lane] = -1;
  }
  if (m.leaf[p]) return;
  const int4 chp = reinterpret_cast<const int4 *>(m.child)[p];
  // lane k < 8: position k of p's 3x3 neighbourhood (the centre skipped)
  int e = -1, co = -1, elev = 0, colev = 0;
  unsigned ex = 0, ey = 0, cox = 0, coy = 0;
  bool eleaf = false;
  int4 ech = make_int4(-1, -1, -1, -1);
  if (lane < 8) {
    const int k = lane < 4 ? lane : lane + 1;
    e = m.coll[p * 9 + k];
    co = m.coarse[p * 9 + k];
    if (e >= 0) {
      eleaf = m.leaf[e];
      elev = m.level[e];
      ex = m.ix[e];
      ey = m.iy[e];
      if (!eleaf) ech = reinterpret_cast<const int4 *>(m.child)[e];
    }
    if (co >= 0) {
      colev = m.level[co];
      cox = m.ix[co];
      coy = m.iy[co];
    }
  }
  unsigned long long nv = 0;
  for (int q = 0; q < 4; q++) {
    const int c = (&chp.x)[q];
    if (c < 0) continue;  // uniform
    int *V = m.vlist + (size_t)c * 27;
    int *X = m.xlist + (size_t)c * 8;
    if (lane < 27) V[lane] = -1;
    if (lane < 8) X[lane] = -1;
    const int lev = m.level[c];
    if (lev - m.lev0 < 2) continue;  // uniform: levels counted from the cell's set root
    __syncwarp();  // the -1 fill is done before any slot is written
    const unsigned ix = m.ix[c], iy = m.iy[c];
    const int qx = ix & 1, qy = iy & 1, cls = qx + 2 * qy;
    if (e >= 0 && !eleaf) {
      for (int qq = 0; qq < 4; qq++) {
        const int cc = (&ech.x)[qq];
        if (cc < 0) continue;
        const int jx = (int)(2 * ex + (qq & 1)), jy = (int)(2 * ey + (qq >> 1));
        const int dx = jx - (int)ix, dy = jy - (int)iy;
        if (abs(dx) <= 1 && abs(dy) <= 1) continue;
        const int sl = slot[cls][dy + 2 + qy][dx + 2 + qx];
        if (sl >= 0) {
          V[sl] = cc;
          nv++;
        }
      }
    }
    // X candidate of this position: the colleague leaf or the coarser leaf
    int xc = -1;
    if (e >= 0 && eleaf && !adjacent(elev, ex, ey, lev, ix, iy)) xc = e;
    if (co >= 0 && !adjacent(colev, cox, coy, lev, ix, iy)) xc = co;
    // a coarser leaf met at several positions is kept at its first one
    const unsigned same = __match_any_sync(0xffffffffu, xc);
    if (xc >= 0 && (same & lt) != 0 && xc == co) xc = -1;
    const unsigned bal = __ballot_sync(0xffffffffu, xc >= 0);
    if (xc >= 0) X[__popc(bal & lt)] = xc;
  }
  for (int o = 16; o; o >>= 1) nv += __shfl_xor_sync(0xffffffffu, nv, o);
  if (lane == 0 && nv) atomicAdd(&m.st->n_m2l, nv);
}

// rc = cutoff * max sigma.  |cor| is taken as the bit pattern of a
// non-negative double, whose integer order is the value order, so the
// largest is found on the integer pipe (not the slow FP64 one) and rounded
// to FP32 once; the result is stored as FP32 bits (non-negative floats order
// like their bits too, for the atomicMax).  NaN counts as 0.
__device__ __forceinline__ unsigned long long abs_bits(double v) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffull;
  return u > 0x7ff0000000000000ull ? 0ull : u;
}
__device__ __forceinline__ unsigned warp_max_as_float_bits(unsigned long long mx) {
  for (int o = 16; o; o >>= 1) {
    const unsigned long long t = __shfl_xor_sync(0xffffffffu, mx, o);
    mx = t > mx ? t : mx;
  }
  return __float_as_uint((float)__longlong_as_double((long long)mx));
}
__global__ void k_sigma_max(const double *cor, int n, unsigned *out) {
  unsigned long long mx = 0;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const unsigned long long u = abs_bits(cor[i]);
    mx = u > mx ? u : mx;
  }
  const unsigned f = warp_max_as_float_bits(mx);
  if ((threadIdx.x & 31) == 0) atomicMax(out, f);
}

__global__ void k_cutoff(unsigned *bits, float cutoff, int count) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  float s = __uint_as_float(bits[i]);
  float rc = cutoff * s * 1.0001f;  // slack for the FP32 rounding of sigma
  reinterpret_cast<float *>(bits)[i] = isfinite(rc) ? rc : 0.f;
}

// Batched sets: max sigma of each set, blocks (set, slice) over slice
// `slice` of the set's input range.
constexpr int kSigmaSlices = 16;
__global__ void k_sigma_max_sets(const double *cor, const int *off, unsigned *out) {
  const int set = blockIdx.x;
  const int n0 = off[set], len = off[set + 1] - n0;
  const int per = (len + kSigmaSlices - 1) / kSigmaSlices;
  const int b = n0 + min(len, per * (int)blockIdx.y), e = n0 + min(len, per * ((int)blockIdx.y + 1));
  unsigned long long mx = 0;
  for (int i = b + threadIdx.x; i < e; i += blockDim.x) {
    const unsigned long long u = abs_bits(cor[i]);
    mx = u > mx ? u : mx;
  }
  const unsigned f = warp_max_as_float_bits(mx);
  if ((threadIdx.x & 31) == 0) atomicMax(out + set, f);
}

// Cells grouped by level (a counting sort), so that the per-level
// expansion passes visit only their own level's cells.  level_off[l] holds
// the count of level l-1 first, then the exclusive offsets, and
// level_off[kKeyLevels + 2 + l] is the fill cursor of level l.
__global__ void k_level_hist(MixedView m) {
  __shared__ int h[kKeyLevels + 1];
  for (int i = threadIdx.x; i <= kKeyLevels; i += blockDim.x) h[i] = 0;
  __syncthreads();
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < m.ncell) atomicAdd(&h[m.level[c]], 1);
  __syncthreads();
  for (int i = threadIdx.x; i <= kKeyLevels; i += blockDim.x)
    if (h[i]) atomicAdd(&m.level_off[i + 1], h[i]);
}

__global__ void k_level_scan(MixedView m) {
  if (threadIdx.x != 0) return;
  int run = 0;
  for (int l = 0; l <= kKeyLevels; l++) {
    run += m.level_off[l + 1];
    m.level_off[l + 1] = run;
    m.level_off[kKeyLevels + 2 + l] = m.level_off[l];
  }
}

// One atomic per warp and level: lanes of equal level share a reservation.
__global__ void k_level_fill(MixedView m) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  const int lev = c < m.ncell ? m.level[c] : -1;
  const unsigned grp = __match_any_sync(0xffffffffu, lev);
  const int leader = __ffs(grp) - 1;
  int base = 0;
  if (lev >= 0 && lane == leader) base = atomicAdd(&m.level_off[kKeyLevels + 2 + lev], __popc(grp));
  base = __shfl_sync(0xffffffffu, base, leader);
  if (lev >= 0) m.by_level[base + __popc(grp & ((1u << lane) - 1u))] = c;
}

__global__ void k_parent(MixedView m) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.ncell) return;
  if (m.leaf[c]) return;
  const int4 ch = reinterpret_cast<const int4 *>(m.child)[c];
  for (int q = 0; q < 4; q++)
    if ((&ch.x)[q] >= 0) m.parent[(&ch.x)[q]] = c;
}

// Distance between the boxes of cells a and b (FP32: only compared with rc).
__device__ __forceinline__ float box_gap(const MixedView &m, int a, int b) {
  const float half = 0.5f * (m.h[a] + m.h[b]);
  const float gx = fmaxf(fabsf(m.cxf[a] - m.cxf[b]) - half, 0.f);
  const float gy = fmaxf(fabsf(m.cyf[a] - m.cyf[b]) - half, 0.f);
  return sqrtf(gx * gx + gy * gy);
}

// U, W and K lists of leaf B, one warp per leaf.
//   U: leaves adjacent to B (any level, B itself included): the coarser
//      leaves among B's neighbours, the same-level neighbours that are
//      leaves, and the adjacent leaves below the others;
//   W: cells below B's same-level neighbours that are not adjacent to B
//      but whose parent is;
//   K: leaves not adjacent to B whose box lies within rc of B's box (the
//      blob-core correction).  The correction walk descends to the walk
//      radius walk_scale * rc, and the counting passes add up the source
//      blobs of the non-adjacent leaves out to that radius (st->k_blobs:
//      the learned form's training envelope is a K-list density, counted
//      at the training radius); every pass walks the same cells, so the
//      lists keep one emission order.
// The walk keeps one stack per warp in shared memory; every round pops up
// to 8 cells and lane (entry, quadrant) classifies one child, so a leaf's
// lists take tens of rounds instead of hundreds of serial steps.  Stack
// entries of the correction walk carry kTagK.  A round pops k <= 8 and
// pushes <= 32, and the cells it pushes lie one level below the ones it
// popped, so the stack holds at most 24 entries per level plus one round:
// 24 * 32 + 32 < kWalkStack for the deepest tree (32 levels).
constexpr int kWalkWarps = 4;
constexpr int kWalkStack = 1024;
constexpr unsigned kTagK = 0x80000000u;

// kMode 0: count the entries of each list kind; 1: write the lists at the
// scanned offsets; 2: count and also store the walk's entries ((kind << 30)
// | id, in emission order) in the leaf's scratch row, which k_lists_compact
// turns into the same lists without a second walk.
template <int kMode>
__global__ void __launch_bounds__(32 * kWalkWarps) k_lists(MixedView m) {
  constexpr bool kFill = kMode == 1;
  __shared__ unsigned s_stack[kWalkWarps][kWalkStack];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int l = blockIdx.x * kWalkWarps + warp;
  if (l >= m.nleaf) return;  // uniform over the warp
  unsigned *stk = s_stack[warp];
  const unsigned lt = (1u << lane) - 1u;
  const int b = m.leaf_cell[l];
  const int lev = m.level[b];
  const unsigned bx = m.ix[b], by = m.iy[b];
  // the correction walk starts at the leaf's set root (the tree root for a
  // single set); a batched tree keeps one cutoff per set
  int root = b;
  while (m.level[root] > m.lev0) root = m.parent[root];
  float rc = *m.rc_ptr;
  if (m.rc_set) {
    const int sh = lev - m.lev0;
    const unsigned tx = bx >> sh, ty = by >> sh;
    rc = m.rc_set[(ty >> 1) * (1u << (m.lev0 - 1)) + (tx >> 1)];
  }
  const float rw = rc * m.walk_scale;
  unsigned long long kb = 0;  // this lane's K-leaf source blobs out to rw
  int base[3] = {0, 0, 0};
  if (kFill) {
    base[0] = m.u_off[l];
    base[1] = m.w_off[l];
    base[2] = m.k_off[l];
  }
  int *const dst[3] = {m.u_idx, m.w_idx, m.k_idx};
  int *const own[3] = {m.u_leaf, m.w_leaf, m.k_leaf};
  int *const row = kMode == 2 ? m.list_scratch + (size_t)l * m.list_cap : nullptr;
  // each lane offers (kind, id), kind -1 = nothing; outputs keep lane order
  auto emit = [&](int kind, int id) {
    if (kMode == 2) {
      const unsigned any = __ballot_sync(0xffffffffu, kind >= 0);
      const int pos = base[0] + base[1] + base[2] + __popc(any & lt);
      if (kind >= 0 && pos < m.list_cap) row[pos] = (int)(((unsigned)kind << 30) | (unsigned)id);
    }
#pragma unroll
    for (int k = 0; k < 3; k++) {
      const unsigned bal = __ballot_sync(0xffffffffu, kind == k);
      if (kFill && kind == k) {
        const int pos = base[k] + __popc(bal & lt);
        dst[k][pos] = id;
        if (own[k]) own[k][pos] = l;
      }
      base[k] += __popc(bal);
    }
  };
  int top = 0;
  auto push = [&](bool want, unsigned v) {
    const unsigned bal = __ballot_sync(0xffffffffu, want);
    if (want) stk[top + __popc(bal & lt)] = v;
    top += __popc(bal);
  };
  {
    // the 3x3 neighbourhood: coarser leaves (each once), same-level cells
    int co = -1, e = -1;
    if (lane < 9) {
      co = m.coarse[b * 9 + lane];
      e = m.coll[b * 9 + lane];
    }
    const unsigned same = __match_any_sync(0xffffffffu, co);
    emit(co >= 0 && (same & lt) == 0 ? 0 : -1, co);
    const bool eleaf = e >= 0 && m.leaf[e];
    emit(eleaf ? 0 : -1, e);
    push(e >= 0 && !eleaf, (unsigned)e);
    push(lane == 0 && rc > 0.f, (unsigned)root | kTagK);  // the set root, for the correction walk
  }
  __syncwarp();
  while (top > 0) {
    const int k = min(8, top);
    const int ent = lane >> 2, q = lane & 3;
    const bool act = ent < k;
    const unsigned v = act ? stk[top - 1 - ent] : 0u;
    __syncwarp();
    top -= k;
    int kind = -1, cc = -1;
    bool grow = false;
    unsigned gv = 0;
    if (act) {
      const int c = (int)(v & ~kTagK);
      cc = m.child[4 * c + q];
      if (cc >= 0) {
        if (v & kTagK) {
          const float g = box_gap(m, cc, b);
          if (g < rw) {
            if (m.leaf[cc]) {
              if (!adj_cells(m, cc, b)) {
                if (g < rc) kind = 2;
                if (!kFill) kb += (unsigned long long)(m.end[cc] - m.begin[cc]);
              }
            } else {
              grow = true;
              gv = (unsigned)cc | kTagK;
            }
          }
        } else if (adjacent(lev, bx, by, m.level[cc], m.ix[cc], m.iy[cc])) {
          if (m.leaf[cc]) {
            kind = 0;
          } else {
            grow = true;
            gv = (unsigned)cc;
          }
        } else {
          kind = 1;
        }
      }
    }
    emit(kind, cc);
    if (top + 32 > kWalkStack) {  // unreachable for trees of <= 32 levels
      if (lane == 0) set_err(m.st, TREE2D_ERR_TOO_DEEP);
      break;
    }
    push(grow, gv);
    __syncwarp();
  }
  if (!kFill) {
    for (int o = 16; o; o >>= 1) kb += __shfl_xor_sync(0xffffffffu, kb, o);
    if (lane == 0 && kb) atomicAdd(&m.st->k_blobs, kb);
  }
  if (!kFill && lane == 0) {
    m.u_off[l] = base[0];
    m.w_off[l] = base[1];
    m.k_off[l] = base[2];
    if (kMode == 2) {
      const int total = base[0] + base[1] + base[2];
      atomicMax(&m.st->list_max, total);
      if (total > m.list_cap) atomicExch(&m.st->list_overflow, 1);
    }
  }
}

// The lists from the one-walk scratch: one warp per leaf reads its row in
// emission order and writes each kind at its scanned offsets, in the order
// the filling walk would (lane order within an emission).
__global__ void __launch_bounds__(256) k_lists_compact(MixedView m) {
  const int l = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (l >= m.nleaf) return;
  const unsigned lt = (1u << lane) - 1u;
  int base[3] = {m.u_off[l], m.w_off[l], m.k_off[l]};
  const int n = (m.u_off[l + 1] - base[0]) + (m.w_off[l + 1] - base[1]) + (m.k_off[l + 1] - base[2]);
  const int *row = m.list_scratch + (size_t)l * m.list_cap;
  int *const dst[3] = {m.u_idx, m.w_idx, m.k_idx};
  int *const own[3] = {m.u_leaf, m.w_leaf, m.k_leaf};
  for (int c0 = 0; c0 < n; c0 += 32) {
    const int e = c0 + lane;
    const unsigned enc = e < n ? (unsigned)row[e] : 0u;
    const int kind = e < n ? (int)(enc >> 30) : -1, id = (int)(enc & 0x3fffffffu);
#pragma unroll
    for (int k = 0; k < 3; k++) {
      const unsigned bal = __ballot_sync(0xffffffffu, kind == k);
      if (kind == k) {
        const int pos = base[k] + __popc(bal & lt);
        dst[k][pos] = id;
        if (own[k]) own[k][pos] = l;
      }
      base[k] += __popc(bal);
    }
  }
}

// Exclusive scan of three count arrays of length len in place, totals at
// [len]: per-tile sums (kScanTile3 entries per block), a scan of the tile
// sums, then each tile scanned with its offset.
constexpr int kScan3Threads = 512, kScan3Items = 8, kScanTile3 = kScan3Threads * kScan3Items;

__device__ __forceinline__ int block_exclusive_scan(int v, int *sh, int &total) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int x = v;
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) sh[w] = x;
  __syncthreads();
  if (w == 0) {
    const int nw = blockDim.x >> 5;
    int t = lane < nw ? sh[lane] : 0;
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, t, o);
      if (lane >= o) t += y;
    }
    if (lane < nw) sh[lane] = t;
  }
  __syncthreads();
  total = sh[(blockDim.x >> 5) - 1];
  const int r = (w ? sh[w - 1] : 0) + x - v;
  __syncthreads();
  return r;
}

__global__ void __launch_bounds__(kScan3Threads) k_scan3_tiles(const int *a, const int *b, const int *c, int len,
                                                               int *tile_sums, int ntiles) {
  __shared__ int sh[32];
  const int *arr[3] = {a, b, c};
  for (int k = 0; k < 3; k++) {
    int v = 0;
    const long i0 = (long)blockIdx.x * kScanTile3 + threadIdx.x * kScan3Items;
    for (int j = 0; j < kScan3Items; j++)
      if (i0 + j < len) v += arr[k][i0 + j];
    int tot;
    block_exclusive_scan(v, sh, tot);
    if (threadIdx.x == 0) tile_sums[k * (ntiles + 1) + blockIdx.x] = tot;
  }
}

// One thread per array: 64-bit running sums over the tile sums.  List
// positions are ints, so a total beyond INT_MAX is reported as -1 (the host
// then stops before any list is filled).
__global__ void k_scan3_sums(int *tile_sums, int ntiles) {
  const int k = threadIdx.x;
  if (k >= 3) return;
  int *t = tile_sums + k * (ntiles + 1);
  long long run = 0;
  for (int i = 0; i < ntiles; i++) {
    const int v = t[i];
    t[i] = (int)(run < 2147483647ll ? run : 2147483647ll);
    run += v;
  }
  t[ntiles] = run > 2147483647ll ? -1 : (int)run;
}

__global__ void __launch_bounds__(kScan3Threads) k_scan3_apply(int *a, int *b, int *c, int len, const int *tile_sums,
                                                               int ntiles) {
  __shared__ int sh[32];
  int *arr[3] = {a, b, c};
  for (int k = 0; k < 3; k++) {
    const long i0 = (long)blockIdx.x * kScanTile3 + threadIdx.x * kScan3Items;
    int v[kScan3Items], sum = 0;
    for (int j = 0; j < kScan3Items; j++) {
      v[j] = i0 + j < len ? arr[k][i0 + j] : 0;
      sum += v[j];
    }
    int tot;
    int run = block_exclusive_scan(sum, sh, tot) + tile_sums[k * (ntiles + 1) + blockIdx.x];
    for (int j = 0; j < kScan3Items; j++) {
      if (i0 + j < len) arr[k][i0 + j] = run;
      run += v[j];
    }
    if (blockIdx.x == ntiles - 1 && threadIdx.x == 0) arr[k][len] = tile_sums[k * (ntiles + 1) + ntiles];
  }
}

// ------------------------------------------------------------ expansions
// Coefficient storage: per cell 2P floats, real parts then imaginary parts.


// Complex product with every rounding spelled out (explicit FMA and
// round-to-nearest products), so that no kernel variant can contract it
// differently: the near-field variants must agree bit for bit.
__device__ __forceinline__ float2 fmul(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, -__fmul_rn(a.y, b.y)), fmaf(a.x, b.y, __fmul_rn(a.y, b.x)));
}

// Packed FP32x2 forms for a lane's two targets: f2 broadcasts a scalar,
// C2 holds one complex value per target (x: real parts, y: imaginary), and
// cmul2 is fmul on each target with the same roundings.
__device__ __forceinline__ float2 f2(float v) { return make_float2(v, v); }
__device__ __forceinline__ float2 neg2(float2 v) { return make_float2(-v.x, -v.y); }
struct C2 {
  float2 x, y;
};
__device__ __forceinline__ C2 cmul2(C2 a, C2 b) {
  return C2{__ffma2_rn(a.x, b.x, neg2(__fmul2_rn(a.y, b.y))), __ffma2_rn(a.x, b.y, __fmul2_rn(a.y, b.x))};
}

// Coefficients are formed in chunks of kCoefChunk: every lane takes its own
// blobs and accumulates the chunk's terms for them in registers, then the
// warp sums the 32 lanes' partials through shared memory (lane t ends with
// the real (t even) or imaginary (t odd) part of coefficient t/2 of the
// chunk).  This costs one transposed reduction per chunk instead of a
// shuffle scan per blob.
constexpr int kCoefChunk = 16;
constexpr int kCoefPitch = 2 * kCoefChunk + 1;  // padded row of the reduction buffer

__device__ __forceinline__ float warp_chunk_sum(const float (&acc)[2 * kCoefChunk], float *sh, int lane) {
#pragma unroll
  for (int i = 0; i < 2 * kCoefChunk; i++) sh[lane * kCoefPitch + i] = acc[i];
  __syncwarp();
  float s = 0.f;
  for (int r = 0; r < 32; r++) s += sh[r * kCoefPitch + lane];
  __syncwarp();
  return s;
}

// S2M: one warp per leaf, a_k = sum_j G_j ((z_j - c)/h)^k.
__global__ void __launch_bounds__(256) k_s2m_f32(MixedView m) {
  __shared__ float sh[8][32 * kCoefPitch];
  const int wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (wid >= m.nleaf) return;
  float *buf = sh[threadIdx.x >> 5];
  const int c = m.leaf_cell[wid];
  const float ih = m.inv_h[c];
  const int P = m.P;
  for (int c0 = 0; c0 < P; c0 += kCoefChunk) {
    float acc[2 * kCoefChunk];
#pragma unroll
    for (int i = 0; i < 2 * kCoefChunk; i++) acc[i] = 0.f;
    for (int j = m.begin[c] + lane; j < m.end[c]; j += 32) {
      const float2 z = make_float2(m.loc[j].x * ih, m.loc[j].y * ih);
      const float g = m.gam[j];
      float2 pw = make_float2(1.f, 0.f);
      for (int k = 0; k < c0; k++) pw = fmul(pw, z);
#pragma unroll
      for (int k = 0; k < kCoefChunk; k++) {
        acc[2 * k] = fmaf(g, pw.x, acc[2 * k]);
        acc[2 * k + 1] = fmaf(g, pw.y, acc[2 * k + 1]);
        pw = fmul(pw, z);
      }
    }
    const float sum = warp_chunk_sum(acc, buf, lane);
    const int k = c0 + (lane >> 1);
    if (k < P) m.M[(size_t)c * 2 * P + ((lane & 1) ? P + k : k)] = sum;
  }
}

// The [4][P][P] block of a [4][kMaxP][kMaxP] translation table, copied
// into shared memory by the whole block.
__device__ __forceinline__ void stage_translation(const float2 *__restrict__ tab, int P, float2 *s_tab) {
  const int pp = P * P;
  for (int i = threadIdx.x; i < 4 * pp; i += blockDim.x) {
    const int q = i / pp, r = i - q * pp, row = r / P, col = r - row * P;
    s_tab[i] = tab[((size_t)q * kMaxP + row) * kMaxP + col];
  }
  __syncthreads();
}

// M2M into the internal cells of one level (grid-stride over all cells,
// one warp per cell).  The operator sits in shared memory; with P <= 16
// (kG = 16) each half-warp takes two of the four children, lane = output
// coefficient, and the halves' sums meet by one shuffle: the children's
// sums are independent chains, ((q0 + q1) + (q2 + q3)) at the end.
template <int kG>
__global__ void __launch_bounds__(256) k_m2m_f32(MixedView m, int lev) {
  extern __shared__ float2 s_tab[];  // [4][P][P]: [q][n][k]
  const int P = m.P;
  stage_translation(m.m2m, P, s_tab);
  constexpr int kCh = 4 * kG / 32;  // children per lane
  const int lane = threadIdx.x & 31, n = lane % kG, q0 = (lane / kG) * kCh, base = lane - n;
  const int *cells = m.by_level + m.level_off[lev];
  const int cnt = m.level_off[lev + 1] - m.level_off[lev];
  for (int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < cnt; i += (gridDim.x * blockDim.x) >> 5) {
    const int p = cells[i];
    if (m.leaf[p]) continue;
    const int4 ch = reinterpret_cast<const int4 *>(m.child)[p];
    float2 a[kCh], acc[kCh];
#pragma unroll
    for (int c = 0; c < kCh; c++) {
      const int cc = (&ch.x)[q0 + c];
      a[c] = cc >= 0 && n < P ? make_float2(m.M[(size_t)cc * 2 * P + n], m.M[(size_t)cc * 2 * P + P + n])
                              : make_float2(0.f, 0.f);
      acc[c] = make_float2(0.f, 0.f);
    }
#pragma unroll 4
    for (int k = 0; k < P; k++) {
#pragma unroll
      for (int c = 0; c < kCh; c++) {
        const float2 ak = make_float2(__shfl_sync(0xffffffffu, a[c].x, base + k),
                                      __shfl_sync(0xffffffffu, a[c].y, base + k));
        if (k <= n && n < P) {
          const float2 t = s_tab[((q0 + c) * P + n) * P + k];
          acc[c].x += t.x * ak.x - t.y * ak.y;
          acc[c].y += t.x * ak.y + t.y * ak.x;
        }
      }
    }
    float2 sum = make_float2(acc[0].x + acc[1].x, acc[0].y + acc[1].y);
    if (kCh == 4) sum = make_float2(sum.x + (acc[2].x + acc[3].x), sum.y + (acc[2].y + acc[3].y));
    if (kG == 16) {
      const float ox = __shfl_xor_sync(0xffffffffu, sum.x, 16), oy = __shfl_xor_sync(0xffffffffu, sum.y, 16);
      sum = make_float2(sum.x + ox, sum.y + oy);  // the same value in both halves
    }
    if (lane < P) {
      m.M[(size_t)p * 2 * P + lane] = sum.x;
      m.M[(size_t)p * 2 * P + P + lane] = sum.y;
    }
  }
}

// P2L: the blobs of cell c's X leaves (coarser leaves adjacent to its
// parent, not to c) into c's local expansion, b_l -= G w^(l+1), w = 1/z,
// z the blob's offset from c's centre in units of c's side.  One warp per
// cell, lanes over blobs, chunked coefficients as S2M.
__global__ void __launch_bounds__(256) k_p2l(MixedView m) {
  __shared__ float sh[8][32 * kCoefPitch];
  const int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (c >= m.ncell) return;
  const int *X = m.xlist + (size_t)c * 8;
  if (X[0] < 0) return;
  float *buf = sh[threadIdx.x >> 5];
  const int P = m.P;
  const float ih = m.inv_h[c];
  for (int c0 = 0; c0 < P; c0 += kCoefChunk) {
    float acc[2 * kCoefChunk];
#pragma unroll
    for (int i = 0; i < 2 * kCoefChunk; i++) acc[i] = 0.f;
    for (int e = 0; e < 8 && X[e] >= 0; e++) {
      const int d = X[e];
      const float ox = centre_offset(m.cxf, m.cxl, d, c), oy = centre_offset(m.cyf, m.cyl, d, c);
      for (int j = m.begin[d] + lane; j < m.end[d]; j += 32) {
        const float zx = (m.loc[j].x + ox) * ih, zy = (m.loc[j].y + oy) * ih;
        const float r2 = zx * zx + zy * zy;
        const float2 w = make_float2(zx / r2, -zy / r2);
        const float g = m.gam[j];
        float2 pw = w;
        for (int k = 0; k < c0; k++) pw = fmul(pw, w);
#pragma unroll
        for (int k = 0; k < kCoefChunk; k++) {
          acc[2 * k] = fmaf(-g, pw.x, acc[2 * k]);
          acc[2 * k + 1] = fmaf(-g, pw.y, acc[2 * k + 1]);
          pw = fmul(pw, w);
        }
      }
    }
    const float sum = warp_chunk_sum(acc, buf, lane);
    const int k = c0 + (lane >> 1);
    if (k < P) m.L[(size_t)c * 2 * P + ((lane & 1) ? P + k : k)] += sum;
  }
}

// M2M and L2L with four threads per parent cell, one per child quadrant q,
// for kP terms (the default 16): the coefficients sit in registers, the
// operator in shared memory (each quadrant's block padded by one entry so
// that the four quadrants' reads fall in different banks; the eight cells
// of a warp read the same addresses, a broadcast), and the passes issue one
// shared load per complex multiply-add.  M2M adds the four children's
// shifted expansions as ((q0 + q1) + (q2 + q3)) by two shuffles within the
// quad; L2L writes each child from its own thread.
constexpr int kQuadThreads = 128;

template <int kP>
__device__ __forceinline__ void stage_translation_padded(const float2 *__restrict__ tab, float2 *s_tab) {
  constexpr int pp = kP * kP;
  for (int i = threadIdx.x; i < 4 * pp; i += blockDim.x) {
    const int q = i / pp, r = i - q * pp, row = r / kP, col = r - row * kP;
    s_tab[q * (pp + 1) + r] = tab[((size_t)q * kMaxP + row) * kMaxP + col];
  }
  __syncthreads();
}

__device__ __forceinline__ int child_of(const int4 ch, int q) {
  return q == 0 ? ch.x : q == 1 ? ch.y : q == 2 ? ch.z : ch.w;
}

// One level of M2M with four threads per parent cell (thread q of a quad
// translates child q, the quad sums the four by shuffles), cells i0, i0 +
// stride, ... of level lev.  kCg: the children's multipoles are read past
// L1 (written by other blocks of the same launch in the level chain).
template <int kP, bool kCg>
__device__ __forceinline__ void m2m_quad_level(const MixedView &m, const float2 *s_tab, int lev, int i0, int stride) {
  const int lane = threadIdx.x & 31, q = lane & 3;
  const unsigned qmask = 0xfu << (lane & ~3);
  const int *cells = m.by_level + m.level_off[lev];
  const int cnt = m.level_off[lev + 1] - m.level_off[lev];
  const float2 *t = s_tab + q * (kP * kP + 1);
  for (int i = i0; i < cnt; i += stride) {
    const int p = cells[i];
    if (m.leaf[p]) continue;  // the same cell, so the same branch, for the whole quad
    const int c = child_of(reinterpret_cast<const int4 *>(m.child)[p], q);
    float2 acc[kP];
#pragma unroll
    for (int n = 0; n < kP; n++) acc[n] = make_float2(0.f, 0.f);
    if (c >= 0) {
      const float4 *src = reinterpret_cast<const float4 *>(m.M + (size_t)c * 2 * kP);
      float a[2 * kP];
#pragma unroll
      for (int j = 0; j < kP / 2; j++) {
        const float4 v = kCg ? __ldcg(src + j) : src[j];
        a[4 * j] = v.x;
        a[4 * j + 1] = v.y;
        a[4 * j + 2] = v.z;
        a[4 * j + 3] = v.w;
      }
#pragma unroll
      for (int n = 0; n < kP; n++)
#pragma unroll
        for (int k = 0; k <= n; k++) {
          const float2 tk = t[n * kP + k];
          const float ax = a[k], ay = a[kP + k];
          acc[n].x += tk.x * ax - tk.y * ay;
          acc[n].y += tk.x * ay + tk.y * ax;
        }
    }
#pragma unroll
    for (int n = 0; n < kP; n++) {
      acc[n].x += __shfl_xor_sync(qmask, acc[n].x, 1);
      acc[n].y += __shfl_xor_sync(qmask, acc[n].y, 1);
      acc[n].x += __shfl_xor_sync(qmask, acc[n].x, 2);
      acc[n].y += __shfl_xor_sync(qmask, acc[n].y, 2);
    }
    // thread q stores coefficients 4q .. 4q+3 of the kP / 4 groups it owns
    float4 *dst = reinterpret_cast<float4 *>(m.M + (size_t)p * 2 * kP);
#pragma unroll
    for (int j = 0; j < kP / 4; j++) {
      if ((j & 3) != q) continue;
      dst[j] = make_float4(acc[4 * j].x, acc[4 * j + 1].x, acc[4 * j + 2].x, acc[4 * j + 3].x);
      dst[kP / 4 + j] = make_float4(acc[4 * j].y, acc[4 * j + 1].y, acc[4 * j + 2].y, acc[4 * j + 3].y);
    }
  }
}

// One level of L2L from the internal cells of level lev-1 into their
// children, thread q of a quad for child q.  kCg: the parents' local
// expansions are read past L1 (the level chain).
template <int kP, bool kCg>
__device__ __forceinline__ void l2l_quad_level(const MixedView &m, const float2 *s_tab, int lev, int i0, int stride) {
  const int q = threadIdx.x & 3;
  const int *cells = m.by_level + m.level_off[lev - 1];
  const int cnt = m.level_off[lev] - m.level_off[lev - 1];
  const float2 *t = s_tab + q * (kP * kP + 1);
  for (int i = i0; i < cnt; i += stride) {
    const int p = cells[i];
    if (m.leaf[p]) continue;
    const int c = child_of(reinterpret_cast<const int4 *>(m.child)[p], q);
    if (c < 0) continue;
    const float4 *src = reinterpret_cast<const float4 *>(m.L + (size_t)p * 2 * kP);
    float b[2 * kP];
#pragma unroll
    for (int j = 0; j < kP / 2; j++) {
      const float4 v = kCg ? __ldcg(src + j) : src[j];
      b[4 * j] = v.x;
      b[4 * j + 1] = v.y;
      b[4 * j + 2] = v.z;
      b[4 * j + 3] = v.w;
    }
    float4 *dst = reinterpret_cast<float4 *>(m.L + (size_t)c * 2 * kP);
#pragma unroll
    for (int j = 0; j < kP / 4; j++) {
      float2 acc[4];
#pragma unroll
      for (int u = 0; u < 4; u++) {
        const int k = 4 * j + u;
        acc[u] = make_float2(0.f, 0.f);
#pragma unroll
        for (int l = k; l < kP; l++) {
          const float2 tl = t[k * kP + l];
          const float bx = b[l], by = b[kP + l];
          acc[u].x += tl.x * bx - tl.y * by;
          acc[u].y += tl.x * by + tl.y * bx;
        }
      }
      float4 re = dst[j], im = dst[kP / 4 + j];
      re.x += acc[0].x;
      re.y += acc[1].x;
      re.z += acc[2].x;
      re.w += acc[3].x;
      im.x += acc[0].y;
      im.y += acc[1].y;
      im.z += acc[2].y;
      im.w += acc[3].y;
      dst[j] = re;
      dst[kP / 4 + j] = im;
    }
  }
}

template <int kP>
__global__ void __launch_bounds__(kQuadThreads) k_m2m_quad(MixedView m, int lev) {
  __shared__ float2 s_tab[4 * (kP * kP + 1)];  // [q][n][k], padded per q
  stage_translation_padded<kP>(m.m2m, s_tab);
  m2m_quad_level<kP, false>(m, s_tab, lev, (blockIdx.x * blockDim.x + threadIdx.x) >> 2,
                            (gridDim.x * blockDim.x) >> 2);
}

template <int kP>
__global__ void __launch_bounds__(kQuadThreads) k_l2l_quad(MixedView m, int lev) {
  __shared__ float2 s_tab[4 * (kP * kP + 1)];  // [q][k][l], padded per q
  stage_translation_padded<kP>(m.l2l, s_tab);
  l2l_quad_level<kP, false>(m, s_tab, lev, (blockIdx.x * blockDim.x + threadIdx.x) >> 2,
                            (gridDim.x * blockDim.x) >> 2);
}

// Grid-wide barrier of a cooperative launch (every block resident): block
// arrivals are counted in st->bar_count (zero before the launch); the last
// block to arrive resets it and advances st->bar_gen, the others poll the
// generation, at most `limit` times (a healthy barrier ends in
// microseconds).  After a poll limit the kernel records TREE2D_ERR_TIMEOUT
// and returns false in every thread of the block; later barriers of that
// block do not wait.
__device__ bool grid_barrier(DevStatus *st, unsigned nblocks, long limit, bool &ok) {
  __syncthreads();
  if (threadIdx.x == 0 && ok) {
    volatile unsigned *gen = &st->bar_gen;
    const unsigned g = *gen;
    __threadfence();
    if (atomicAdd(&st->bar_count, 1u) + 1u == nblocks) {
      st->bar_count = 0;
      __threadfence();
      atomicAdd(&st->bar_gen, 1u);
    } else {
      long i = 0;
      while (*gen == g && i < limit) i++;
      if (*gen == g) {
        ok = false;
        set_err(st, TREE2D_ERR_TIMEOUT);
      }
    }
    __threadfence();
  }
  ok = __syncthreads_and(threadIdx.x == 0 ? ok : 1) != 0;
  return ok;
}

// The M2M chain (kUp: levels depth-1 down to lev_end) or the L2L chain
// (levels lev_end up to depth) in one cooperative launch of persistent
// blocks: each level's cells are spread over all blocks, and the blocks
// meet at the grid barrier before the next level reads what this one wrote.
template <int kP, bool kUp>
__global__ void __launch_bounds__(kQuadThreads) k_chain_quad(MixedView m, int lev_first, int lev_last, long limit) {
  __shared__ float2 s_tab[4 * (kP * kP + 1)];
  stage_translation_padded<kP>(kUp ? m.m2m : m.l2l, s_tab);
  const int i0 = (blockIdx.x * blockDim.x + threadIdx.x) >> 2, stride = (gridDim.x * blockDim.x) >> 2;
  bool ok = true;
  const int step = kUp ? -1 : 1;
  for (int lev = lev_first;; lev += step) {
    if (kUp)
      m2m_quad_level<kP, true>(m, s_tab, lev, i0, stride);
    else
      l2l_quad_level<kP, true>(m, s_tab, lev, i0, stride);
    if (lev == lev_last) break;
    if (!grid_barrier(m.st, gridDim.x, limit, ok)) return;
  }
}

// L2L from the internal cells of level lev-1 into their children (one
// warp per parent, the operator in shared memory).  With P <= 16 (kG = 16)
// each half-warp translates two of the four children, lane = coefficient.
template <int kG>
__global__ void __launch_bounds__(256) k_l2l_f32(MixedView m, int lev) {
  extern __shared__ float2 s_tab[];  // [4][P][P]: [q][k][l]
  const int P = m.P;
  stage_translation(m.l2l, P, s_tab);
  constexpr int kCh = 4 * kG / 32;
  const int lane = threadIdx.x & 31, k = lane % kG, q0 = (lane / kG) * kCh;
  const int *cells = m.by_level + m.level_off[lev - 1];
  const int cnt = m.level_off[lev] - m.level_off[lev - 1];
  for (int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < cnt; i += (gridDim.x * blockDim.x) >> 5) {
    const int p = cells[i];
    if (m.leaf[p]) continue;
    const float *src = m.L + (size_t)p * 2 * P;
    const float2 b = k < P ? make_float2(src[k], src[P + k]) : make_float2(0.f, 0.f);
    const int4 ch = reinterpret_cast<const int4 *>(m.child)[p];
    float2 acc[kCh];
#pragma unroll
    for (int c = 0; c < kCh; c++) acc[c] = make_float2(0.f, 0.f);
#pragma unroll 4
    for (int l = 0; l < P; l++) {
      const float2 bl = make_float2(__shfl_sync(0xffffffffu, b.x, l), __shfl_sync(0xffffffffu, b.y, l));
      if (l >= k && k < P) {
#pragma unroll
        for (int c = 0; c < kCh; c++) {
          const float2 t = s_tab[((q0 + c) * P + k) * P + l];
          acc[c].x += t.x * bl.x - t.y * bl.y;
          acc[c].y += t.x * bl.y + t.y * bl.x;
        }
      }
    }
    if (k < P) {
#pragma unroll
      for (int c = 0; c < kCh; c++) {
        const int cc = (&ch.x)[q0 + c];
        if (cc < 0) continue;
        m.L[(size_t)cc * 2 * P + k] += acc[c].x;
        m.L[(size_t)cc * 2 * P + P + k] += acc[c].y;
      }
    }
  }
}

__device__ __forceinline__ void kahan(float &s, float &cmp, float v) {
  float y = v - cmp;
  float t = s + y;
  cmp = (t - s) - y;
  s = t;
}

// Order of an M2P the network chose: class c >= 1 is order c + 3 (4..16),
// raised by the margin, capped at P; class 0 of a W entry keeps P.
__device__ __forceinline__ int chosen_order(int d, int margin, int P) {
  return d > 0 ? min(min(class_order(d) + margin, 16), P) : P;
}

// M2P of source leaf A at order p (terms 0..p-1) at a target offset z from
// leaf B's centre, added to phi.
__device__ __forceinline__ void m2p_order(const MixedView &m, int B, int A, int p, float2 z, float2 &phi) {
  const int P = m.P;
  const float ih = m.inv_h[A];
  const float zx = __fmul_rn(__fadd_rn(z.x, centre_offset(m.cxf, m.cxl, B, A)), ih);
  const float zy = __fmul_rn(__fadd_rn(z.y, centre_offset(m.cyf, m.cyl, B, A)), ih);
  const float ir2 = __fdiv_rn(1.f, fmaf(zx, zx, __fmul_rn(zy, zy)));
  const float2 w = make_float2(__fmul_rn(zx, ir2), -__fmul_rn(zy, ir2));
  const float *MA = m.M + (size_t)A * 2 * P;
  float2 a = make_float2(MA[p - 1], MA[P + p - 1]);
  for (int k = p - 2; k >= 0; k--) {
    a = fmul(a, w);
    a.x = __fadd_rn(a.x, MA[k]);
    a.y = __fadd_rn(a.y, MA[P + k]);
  }
  a = fmul(a, w);
  phi.x = fmaf(a.x, ih, phi.x);
  phi.y = fmaf(a.y, ih, phi.y);
}

// m2p_order for the lane's two targets (offsets za, zb from B's centre) in
// packed arithmetic: each target's value is m2p_order's, bit for bit, and
// the multipole is read once for both.
__device__ __forceinline__ void m2p_order2(const MixedView &m, int B, int A, int p, float2 za, float2 zb, float2 &pa,
                                           float2 &pb) {
  const int P = m.P;
  const float ih = m.inv_h[A];
  const float2 zx = __fmul2_rn(__fadd2_rn(make_float2(za.x, zb.x), f2(centre_offset(m.cxf, m.cxl, B, A))), f2(ih));
  const float2 zy = __fmul2_rn(__fadd2_rn(make_float2(za.y, zb.y), f2(centre_offset(m.cyf, m.cyl, B, A))), f2(ih));
  const float2 r2 = __ffma2_rn(zx, zx, __fmul2_rn(zy, zy));
  const float2 ir2 = make_float2(__fdiv_rn(1.f, r2.x), __fdiv_rn(1.f, r2.y));
  const C2 w{__fmul2_rn(zx, ir2), neg2(__fmul2_rn(zy, ir2))};
  const float *MA = m.M + (size_t)A * 2 * P;
  C2 a{f2(MA[p - 1]), f2(MA[P + p - 1])};
  for (int k = p - 2; k >= 0; k--) {
    a = cmul2(a, w);
    a.x = __fadd2_rn(a.x, f2(MA[k]));
    a.y = __fadd2_rn(a.y, f2(MA[P + k]));
  }
  a = cmul2(a, w);
  const float2 px = __ffma2_rn(a.x, f2(ih), make_float2(pa.x, pb.x));
  const float2 py = __ffma2_rn(a.y, f2(ih), make_float2(pa.y, pb.y));
  pa = make_float2(px.x, py.x);
  pb = make_float2(px.y, py.y);
}

// Evaluation: one warp per leaf; each lane owns up to two targets (chunks
// of 64 targets), so a leaf of <= 64 blobs walks its source lists once.
// Sources are read as one float4 {x, y, G, 1/sigma^2} (offsets from their
// leaf centre), the same address for the whole warp.
__device__ __forceinline__ void far_field(const MixedView &m, int l, int B, float2 zt, float2 &phi,
                                          const unsigned char *wdec = nullptr, int margin = 0) {
  const int P = m.P;
  const float ihB = m.inv_h[B];
  const float *LB = m.L + (size_t)B * 2 * P;
  const float2 zeta = make_float2(__fmul_rn(zt.x, ihB), __fmul_rn(zt.y, ihB));
  float2 acc = make_float2(LB[P - 1], LB[2 * P - 1]);
  for (int k = P - 2; k >= 0; k--) {
    acc = fmul(acc, zeta);
    acc.x = __fadd_rn(acc.x, LB[k]);
    acc.y = __fadd_rn(acc.y, LB[P + k]);
  }
  phi.x = __fmul_rn(acc.x, ihB);
  phi.y = __fmul_rn(acc.y, ihB);
  for (int e = m.w_off[l]; e < m.w_off[l + 1]; e++)
    m2p_order(m, B, m.w_idx[e], wdec ? chosen_order(wdec[e], margin, P) : P, zt, phi);
}

// far_field for the lane's two targets in packed arithmetic (each target's
// value is far_field's, bit for bit).
__device__ __forceinline__ void far_field2(const MixedView &m, int l, int B, float2 za, float2 zb, float2 &pa,
                                           float2 &pb, const unsigned char *wdec = nullptr, int margin = 0) {
  const int P = m.P;
  const float ihB = m.inv_h[B];
  const float *LB = m.L + (size_t)B * 2 * P;
  const C2 zeta{__fmul2_rn(make_float2(za.x, zb.x), f2(ihB)), __fmul2_rn(make_float2(za.y, zb.y), f2(ihB))};
  C2 acc{f2(LB[P - 1]), f2(LB[2 * P - 1])};
  for (int k = P - 2; k >= 0; k--) {
    acc = cmul2(acc, zeta);
    acc.x = __fadd2_rn(acc.x, f2(LB[k]));
    acc.y = __fadd2_rn(acc.y, f2(LB[P + k]));
  }
  const float2 px = __fmul2_rn(acc.x, f2(ihB)), py = __fmul2_rn(acc.y, f2(ihB));
  pa = make_float2(px.x, py.x);
  pb = make_float2(px.y, py.y);
  for (int e = m.w_off[l]; e < m.w_off[l + 1]; e++)
    m2p_order2(m, B, m.w_idx[e], wdec ? chosen_order(wdec[e], margin, P) : P, za, zb, pa, pb);
}

// 2^t on the SFU (PTX ex2.approx: relative error ~2^-22, FTZ).
__device__ __forceinline__ float sfu_exp2(float t) {
  float r;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(t));
  return r;
}

// 1/x on the SFU (PTX rcp.approx: relative error ~2^-23, FTZ).
__device__ __forceinline__ float sfu_rcp(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// One pair: source (x, y, G, t) with t = -log2(e)/sigma^2, target given
// negated, (ntx, nty) = (-tx, -ty).  The offset is taken source minus
// target, (nrx, nry) = -(tx - x, ty - y) exactly (round to nearest is
// symmetric), and the pair adds f nry to a and f nrx to b with f >= 0 up to
// the sign of G:
//   direct (U):     f = G (1 - exp(-r^2/s^2)) / r^2, velocity (a, -b);
//                   1 - e^-x is taken from its series x (1 - x/2) =
//                   t (-ln2 - (ln2)^2/2 t) below x = 1e-3, where the
//                   subtraction would cancel;
//   correction (K): f = G exp(-r^2/s^2) / r^2, velocity (-a, b): the
//                   correction -G exp(-r^2/s^2) / r^2 of every pair of the
//                   two leaves (the list holds the leaves within rc; pairs
//                   beyond rc add their tiny exact terms).
// The signs are applied once per source leaf, in its compensated add, so no
// pair spends an instruction on them.  r2 carries a 1e-30 floor, so a
// coincident pair has a finite factor and contributes f * (0, 0) = 0, as
// the reference skips r <= 1e-10 (fmm.c:132); nothing else sees the floor
// (it is below FP32 resolution of any r2 that matters).  The quotient is
// G (...) times the SFU reciprocal of r2.
constexpr float kSer1 = -0.69314718f;  // -ln 2
constexpr float kSer2 = -0.24022651f;  // -(ln 2)^2 / 2
constexpr float kSerT = -1.44269504e-3f;  // t at x = 1e-3

// kScaled: the records of a leaf whose blobs share one core radius, held
// scaled by s = sqrt(log2 e) / sigma, {x s, y s, G s, -} (src4s), with the
// targets' offsets scaled by the same s: the squared distance is then
// q = r^2 log2(e) / sigma^2 itself, the Gaussian exp2(-q) needs no product
// per pair, and G s / q carries the 1 / r^2 (G s / q (y s) = G / r^2 y).
// One FP32 operation fewer per pair, the same quantities up to rounding.
template <bool kCorrection, bool kScaled = false>
__device__ __forceinline__ void pair(const float4 sj, float ntx, float nty, float &a, float &b) {
  const float nrx = __fadd_rn(sj.x, ntx), nry = __fadd_rn(sj.y, nty);
  const float r2 = fmaf(nrx, nrx, fmaf(nry, nry, 1e-30f));
  // the Gaussian's exponent, base 2: t = r2 * (-log2(e)/sigma^2), or -q scaled
  const float t = kScaled ? 0.f : __fmul_rn(r2, sj.w);
  const float e = sfu_exp2(kScaled ? -r2 : t);
  const float ir2 = sfu_rcp(r2);
  float f;
  if (!kCorrection) {
    // x (1 - x/2) = t (-ln2 - (ln2)^2/2 t) = q (ln2 - (ln2)^2/2 q), the same bits
    const float ser = kScaled ? __fmul_rn(r2, fmaf(kSer2, r2, -kSer1)) : __fmul_rn(t, fmaf(kSer2, t, kSer1));
    const float ome = fmaf(-1.f, e, 1.f);
    const bool small = kScaled ? r2 < -kSerT : t > kSerT;
    f = __fmul_rn(__fmul_rn(sj.z, small ? ser : ome), ir2);
  } else {
    f = __fmul_rn(__fmul_rn(sj.z, e), ir2);
  }
  a = fmaf(f, nry, a);
  b = fmaf(f, nrx, b);
}

// The same pair for two targets at once, on packed FP32x2 arithmetic: one
// instruction forms both targets' value of every step, with the rounding
// of the scalar step (each component rounds as the scalar operation does),
// so a target's sum does not depend on how many targets its lane holds.
template <bool kCorrection, bool kScaled = false>
__device__ __forceinline__ void pair2(const float4 sj, float2 ntx, float2 nty, float2 &a, float2 &b) {
  const float2 nrx = __fadd2_rn(f2(sj.x), ntx), nry = __fadd2_rn(f2(sj.y), nty);
  const float2 r2 = __ffma2_rn(nrx, nrx, __ffma2_rn(nry, nry, f2(1e-30f)));
  const float2 t = kScaled ? f2(0.f) : __fmul2_rn(r2, f2(sj.w));
  const float2 e = kScaled ? make_float2(sfu_exp2(-r2.x), sfu_exp2(-r2.y)) : make_float2(sfu_exp2(t.x), sfu_exp2(t.y));
  const float2 ir2 = make_float2(sfu_rcp(r2.x), sfu_rcp(r2.y));
  float2 f;
  if (!kCorrection) {
    const float2 ser = kScaled ? __fmul2_rn(r2, __ffma2_rn(f2(kSer2), r2, f2(-kSer1)))
                               : __fmul2_rn(t, __ffma2_rn(f2(kSer2), t, f2(kSer1)));
    const float2 ome = __ffma2_rn(f2(-1.f), e, f2(1.f));
    const bool sx = kScaled ? r2.x < -kSerT : t.x > kSerT, sy = kScaled ? r2.y < -kSerT : t.y > kSerT;
    const float2 e1f = make_float2(sx ? ser.x : ome.x, sy ? ser.y : ome.y);
    f = __fmul2_rn(__fmul2_rn(f2(sj.z), e1f), ir2);
  } else {
    f = __fmul2_rn(__fmul2_rn(f2(sj.z), e), ir2);
  }
  a = __ffma2_rn(f, nry, a);
  b = __ffma2_rn(f, nrx, b);
}

// Source records {x, y, G, t} of one leaf, read from a stage buffer in
// shared memory (ld.shared, from its shared-window address) or from global
// memory (read-only while the kernel runs).  Two types, so that the pair
// loop issues shared or global loads, never generic ones.
struct SmemSrc {
  uint32_t base;
  __device__ __forceinline__ float4 operator[](int j) const {
    float4 v;
    asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];"
                 : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
                 : "r"(base + 16u * (uint32_t)j));
    return v;
  }
};
struct GlobalSrc {
  const float4 *__restrict__ p;
  __device__ __forceinline__ float4 operator[](int j) const { return __ldg(p + j); }
};

// Direct (U list) or correction (K list) sums of source blobs [j0, j1) for
// one target per lane (leaf_pairs1), one pack of two (leaf_pairs2) or two
// packs sharing every source record (leaf_pairs4); the targets are given
// negated (see pair).  Each source leaf is summed in plain FP32 and then
// added with compensation (leaf_add), so the compensated sum costs once per
// leaf, not once per pair.
template <bool kCorrection, bool kScaled, class S>
__device__ __forceinline__ void leaf_pairs1(const S src, int j0, int j1, float ntx, float nty, float &a, float &b) {
#pragma unroll 4
  for (int j = j0; j < j1; j++) pair<kCorrection, kScaled>(src[j], ntx, nty, a, b);
}

template <bool kCorrection, bool kScaled, int kUnroll, class S>
__device__ __forceinline__ void leaf_pairs2(const S src, int j0, int j1, float2 ntx, float2 nty, float2 &a,
                                            float2 &b) {
#pragma unroll kUnroll
  for (int j = j0; j < j1; j++) pair2<kCorrection, kScaled>(src[j], ntx, nty, a, b);
}

template <bool kCorrection, bool kScaled, int kUnroll, class S>
__device__ __forceinline__ void leaf_pairs4(const S src, int j0, int j1, float2 ntx0, float2 nty0, float2 ntx1,
                                            float2 nty1, float2 &a0, float2 &b0, float2 &a1, float2 &b1) {
#pragma unroll kUnroll
  for (int j = j0; j < j1; j++) {
    const float4 sj = src[j];
    pair2<kCorrection, kScaled>(sj, ntx0, nty0, a0, b0);
    pair2<kCorrection, kScaled>(sj, ntx1, nty1, a1, b1);
  }
}

struct Decisions {
  const unsigned char *u, *k;  // class per U / K entry; null: all direct
  int margin;
  const unsigned char *w;      // class per W entry (order of its M2P); null: all at the full order
};


// Persistent near-field warps: the grid holds as many warps as fit on the
// GPU at once, and each warp takes the next target leaf from a counter
// (DevStatus::eval_next, zeroed before each launch) until none is left.
// Leaves differ widely in work, so a warp that finishes early takes more
// instead of idling beside the slowest warp of a resident block.
__device__ __forceinline__ int next_leaf(DevStatus *st, int lane) {
  int l = 0;
  if (lane == 0) l = (int)atomicAdd(&st->eval_next, 1u);
  return __shfl_sync(0xffffffffu, l, 0);
}

// Correction radius of leaf cell B: the tree's, or in a batched tree its
// set's (the same rule as the list walk, k_lists).
__device__ __forceinline__ float leaf_cutoff(const MixedView &m, int B) {
  float rc = *m.rc_ptr;
  if (m.rc_set) {
    const int sh = m.level[B] - m.lev0;
    const unsigned tx = m.ix[B] >> sh, ty = m.iy[B] >> sh;
    rc = m.rc_set[(ty >> 1) * (1u << (m.lev0 - 1)) + (tx >> 1)];
  }
  return rc;
}

constexpr unsigned kAllChunks = 0xffffffffu;

// Pair counters of one warp, kept in shared memory by lane 0 (every count
// is warp-uniform): target-source pairs evaluated, correction pairs
// evaluated and correction pairs listed, over the current chunk of targets
// and then summed over chunks.
struct WarpCounts {
  unsigned chunk[3];
  unsigned long long total[3];
};

__device__ __forceinline__ void counts_add(WarpCounts *c, int lane, unsigned done, unsigned done_k, unsigned listed) {
  if (lane == 0) {
    c->chunk[0] += done;
    c->chunk[1] += done_k;
    c->chunk[2] += listed;
  }
}

__device__ __forceinline__ void counts_flush(WarpCounts *c, int lane, DevStatus *st) {
  if (lane == 0) {
    atomicAdd(&st->n_pairs, c->total[0]);
    atomicAdd(&st->n_pairs_k, c->total[1]);
    atomicAdd(&st->n_pairs_k_listed, c->total[2]);
  }
}

// The next run of consecutive source chunks (kChunk blobs each, bit k of a mask
// for chunk k of a leaf of cnt blobs) kept for the same target packs: r0
// and r1 are the chunks kept for pack 0 and pack 1, kAllChunks for both the
// whole leaf.  Returns blobs [s0, s1) and the packs (bit 0: pack 0, bit 1:
// pack 1); the run is removed from both masks.
__device__ __forceinline__ int next_run(unsigned &r0, unsigned &r1, int cnt, int &s0, int &s1) {
  if (r0 == kAllChunks && r1 == kAllChunks) {
    s0 = 0;
    s1 = cnt;
    r0 = r1 = 0;
    return 3;
  }
  const int a = __ffs(r0 | r1) - 1;
  const int packs = (int)((r0 >> a) & 1u) | (int)(((r1 >> a) & 1u) << 1);
  const unsigned same = ((packs & 1) ? r0 : ~r0) & ((packs & 2) ? r1 : ~r1);
  const unsigned gap = ~(same >> a);
  const int len = gap ? __ffs(gap) - 1 : 32 - a;
  s0 = a << kChunkShift;
  s1 = min(cnt, (a + len) << kChunkShift);
  const unsigned run = a + len >= 32 ? ~0u << a : ((1u << len) - 1u) << a;
  r0 &= ~run;
  r1 &= ~run;
  return packs;
}

// Chunks of correction source leaf A whose pairs with a pack of targets can
// lie within the correction radius: bit k of *m0 (*m1) for the kChunk-blob chunk
// k of A whose bounding box comes within rc of pack 0's (pack 1's) target
// box, tb[0..3] (tb[4..7]), rc^2 in tb[8]; the boxes are offsets from the
// target leaf's centre, (ox, oy) is A's centre seen from there.  Pairs
// farther than rc from every target add terms below exp(-rc^2/sigma^2) of a
// point vortex: the ones the correction list already leaves out beyond rc.
// A leaf of more than 32 chunks is not culled (kAllChunks).  Warp-uniform.
template <int kPacks>
__device__ __forceinline__ void chunk_mask(const MixedView &m, int A, float ox, float oy, const float *tb, int lane,
                                           unsigned &m0, unsigned &m1) {
  const int nch = (m.end[A] - m.begin[A] + kChunk - 1) >> kChunkShift;
  if (nch > 32 || nch > m.kchunks) {
    m0 = m1 = kAllChunks;
    return;
  }
  bool keep[2] = {false, false};
  if (lane < nch) {
    const float rc2 = tb[8];
    const float4 s = m.cbox[(size_t)A * m.kchunks + lane];
#pragma unroll
    for (int p = 0; p < kPacks; p++) {
      // pack p's box in A's frame: T + (ox, oy)
      const float4 T = make_float4(tb[4 * p], tb[4 * p + 1], tb[4 * p + 2], tb[4 * p + 3]);
      const float gx = fmaxf(fmaxf(__fsub_rn(s.x, __fadd_rn(T.z, ox)), __fsub_rn(__fadd_rn(T.x, ox), s.z)), 0.f);
      const float gy = fmaxf(fmaxf(__fsub_rn(s.y, __fadd_rn(T.w, oy)), __fsub_rn(__fadd_rn(T.y, oy), s.w)), 0.f);
      keep[p] = fmaf(gx, gx, __fmul_rn(gy, gy)) <= rc2;
    }
  }
  m0 = __ballot_sync(0xffffffffu, keep[0]);
  m1 = kPacks == 2 ? __ballot_sync(0xffffffffu, keep[1]) : m0;
}

// The persistent near-field warps take target leaves in the order of
// m.leaf_order.  Leaves differ in work by two orders of magnitude (the
// dense patch centres against the sheet), and a heavy leaf taken last
// keeps one warp busy while the rest of the GPU idles, so the schedule is
// longest first: k_leaf_cost keys each leaf by its estimated pairs
// (targets x the blobs of its U and K entries) on a half-octave scale, and
// one stable radix pass orders the keys (ties by leaf ordinal).  The order
// changes only which warp evaluates a leaf, never a result.
__global__ void k_leaf_cost(MixedView m, uint64_t *keys, uint32_t *vals) {
  const int l = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (l >= m.nleaf) return;
  const int B = m.leaf_cell[l];
  float src = 0.f;
  for (int e = m.u_off[l] + lane; e < m.u_off[l + 1]; e += 32) src += (float)(m.end[m.u_idx[e]] - m.begin[m.u_idx[e]]);
  for (int e = m.k_off[l] + lane; e < m.k_off[l + 1]; e += 32) src += (float)(m.end[m.k_idx[e]] - m.begin[m.k_idx[e]]);
  for (int o = 16; o; o >>= 1) src += __shfl_xor_sync(0xffffffffu, src, o);
  if (lane == 0) {
    const float work = src * (float)(m.end[B] - m.begin[B]) + 1.f;
    const int b = min(max((int)(2.f * __log2f(work)), 0), 127);  // half octaves, 2^63 at most
    keys[l] = (uint64_t)(255 - b) << 56;  // ascending key = descending work
    vals[l] = (uint32_t)l;
  }
}

// Near field of every leaf: one warp per target leaf.  The leaf's targets
// are taken in chunks of 128, 64 or 32 (4, 2 or 1 per lane, packed in
// twos: a leaf of 97-128 blobs walks its source lists once with four
// targets per lane instead of twice with two).  For each chunk the warp
// walks its direct entries (U list, then K list; in the learned form the
// entries the network accepted are M2P'd after the walk and skipped in it)
// and sums each source leaf's blobs for every target.  kStaged: each source
// leaf is staged in shared memory by a bulk copy (cp.async.bulk, one
// 16-byte record per blob, completion on a per-buffer mbarrier),
// double-buffered, so the next leaf is in flight while the lanes sum the
// current one; leaves larger than a stage buffer, and every leaf after a
// wait that gave up (recorded as TREE2D_ERR_TIMEOUT), are read from global
// memory instead, so the result never depends on the staging.  Otherwise
// the sources are read from global memory (through L1).  The compensated
// per-target sums live in shared memory (written once per source leaf),
// which keeps the pair loop's registers for the targets.
constexpr int kStage = 128;  // blobs per stage buffer: the largest leaf of the default leaf sizes
constexpr long kEvalWaitLimit = 1l << 22;  // polls; a healthy copy lands within microseconds

struct NearWarp {
  float4 *src;       // stage buffers [2][kStage] (kStaged)
  uint64_t *bar;     // their mbarriers [2]
  float *tbox;       // target boxes of the chunk's packs and rc^2
  float4 *acc;       // compensated sums {ax, cx, ay, cy} [4][32]
  WarpCounts *cnts;
  unsigned parity;   // bit b: parity of buffer b's next completion
  unsigned inflight; // bit b: a copy into buffer b not yet waited for
  bool staging;      // false after a wait gave up
};

// Adds one source leaf's sums (sa, sb of pair) to target slot k's
// compensated sums: velocity (a, -b) for a direct leaf, (-a, b) for a
// correction leaf.
__device__ __forceinline__ void leaf_add(float4 *acc, int k, int lane, bool corr, float a, float b) {
  float4 s = acc[32 * k + lane];
  kahan(s.x, s.y, corr ? -a : a);
  kahan(s.z, s.w, corr ? b : -b);
  acc[32 * k + lane] = s;
}

// One chunk of a target leaf's targets: 32 kT of them from t0 on, kT per
// lane (target t0 + 32 k + lane in slot k), in packs of two slots (k = 0, 1
// and k = 2, 3), each pack with its own bounding box for the correction
// cull.  The tree's in-leaf order is spatial (k_leaf_setup), so a pack of
// 64 consecutive targets is compact.
template <bool kLearned, bool kStaged, int kT, int kUnroll, bool kScaled>
__device__ __forceinline__ void near_chunk(const MixedView &m, const Decisions &dec, double *uv, const int *perm,
                                           long wait_limit, int l, int B, int t0, int lane, NearWarp &w) {
  constexpr int kPacks = kT == 4 ? 2 : 1;
  const int tend = m.end[B];
  float bx[kPacks][4];
#pragma unroll
  for (int p = 0; p < kPacks; p++) bx[p][0] = bx[p][1] = INFINITY, bx[p][2] = bx[p][3] = -INFINITY;
#pragma unroll
  for (int k = 0; k < kT; k++) {
    const int t = t0 + 32 * k + lane, p = k >> 1;
    const float2 zk = t < tend ? m.loc[t] : make_float2(0.f, 0.f);
    if (t < tend)
      bx[p][0] = fminf(bx[p][0], zk.x), bx[p][1] = fminf(bx[p][1], zk.y), bx[p][2] = fmaxf(bx[p][2], zk.x),
      bx[p][3] = fmaxf(bx[p][3], zk.y);
    w.acc[32 * k + lane] = make_float4(0.f, 0.f, 0.f, 0.f);
  }
  // each pack's target box (offsets from B's centre) and rc^2, in shared memory
#pragma unroll
  for (int p = 0; p < kPacks; p++)
    for (int o = 16; o; o >>= 1) {
      bx[p][0] = fminf(bx[p][0], __shfl_xor_sync(0xffffffffu, bx[p][0], o));
      bx[p][1] = fminf(bx[p][1], __shfl_xor_sync(0xffffffffu, bx[p][1], o));
      bx[p][2] = fmaxf(bx[p][2], __shfl_xor_sync(0xffffffffu, bx[p][2], o));
      bx[p][3] = fmaxf(bx[p][3], __shfl_xor_sync(0xffffffffu, bx[p][3], o));
    }
  if (lane == 0) {
    const float rc = leaf_cutoff(m, B);
#pragma unroll
    for (int p = 0; p < kPacks; p++)
      for (int i = 0; i < 4; i++) w.tbox[4 * p + i] = bx[p][i];
    w.tbox[8] = __fmul_rn(rc, rc);
  }
  __syncwarp();
  // target offsets from B's centre, held in registers for the chunk
  float2 zr[kT];
#pragma unroll
  for (int k = 0; k < kT; k++) {
    const int t = t0 + 32 * k + lane;
    zr[k] = t < tend ? m.loc[t] : make_float2(0.f, 0.f);
  }
  auto zof = [&](int k) { return zr[k]; };
  // valid targets of each pack (the pair counts are per target)
  const unsigned nt = (unsigned)min(tend - t0, 32 * kT);
  const unsigned vp0 = kT == 4 ? min(nt, 64u) : nt, vp1 = kT == 4 ? nt - vp0 : 0u;
  const int u0 = m.u_off[l], nu = m.u_off[l + 1] - u0;
  const int k0 = m.k_off[l], nk = m.k_off[l + 1] - k0;
  auto src_leaf = [&](int q) { return q < nu ? m.u_idx[u0 + q] : m.k_idx[k0 + q - nu]; };
  auto direct = [&](int q) {
    if (!kLearned) return true;
    return (q < nu ? dec.u[u0 + q] : dec.k[k0 + q - nu]) == 0;
  };
  // the next entry with work for these targets: a direct entry, and for a
  // correction entry at least one chunk within rc of a pack (r0, r1: its
  // chunks per pack, all for a U entry); culled correction entries are
  // counted and skipped
  auto next_work = [&](int q, unsigned &r0, unsigned &r1) {
    for (; q < nu + nk; q++) {
      if (!direct(q)) continue;
      if (q < nu) {
        r0 = r1 = kAllChunks;
        return q;
      }
      const int A = m.k_idx[k0 + q - nu];
      chunk_mask<kPacks>(m, A, centre_offset(m.cxf, m.cxl, B, A), centre_offset(m.cyf, m.cyl, B, A), w.tbox, lane,
                         r0, r1);
      if (r0 | r1) return q;
      counts_add(w.cnts, lane, 0u, 0u, (unsigned)(m.end[A] - m.begin[A]) * nt);
    }
    r0 = r1 = 0;
    return q;
  };
  // copy source leaf of position q into buffer b (warp-uniform decision)
  auto stage = [&](int q, int b) {
    if (!kStaged) return false;
    const int A = src_leaf(q);
    const int j0 = m.begin[A], cnt = m.end[A] - j0;
    if (!w.staging || cnt > kStage) return false;
    if (lane == 0) {
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      mbar_expect_tx(&w.bar[b], (uint32_t)cnt * 16u);
      bulk_g2s(w.src + b * kStage, (kScaled ? m.src4s : m.src4) + j0, (uint32_t)cnt * 16u, &w.bar[b]);
    }
    w.inflight |= 1u << b;
    return true;
  };
  unsigned r0 = 0, r1 = 0;
  int q = next_work(0, r0, r1);
  int buf = 0;
  bool staged = q < nu + nk && stage(q, buf);
  while (q < nu + nk) {
    unsigned r0n = 0, r1n = 0;
    const int qn = next_work(q + 1, r0n, r1n);
    const bool staged_next = qn < nu + nk && stage(qn, buf ^ 1);
    const int A = src_leaf(q);
    // offset of the source leaf's centre from the two-float centres: FP32
    // centres alone would carry ~3e-8 absolute error into every close pair
    const float ox = centre_offset(m.cxf, m.cxl, B, A), oy = centre_offset(m.cyf, m.cyl, B, A);
    const int j0 = m.begin[A], cnt = m.end[A] - j0;
    bool use_smem = false;
    if (staged) {
      if (mbar_wait(&w.bar[buf], (w.parity >> buf) & 1u, wait_limit)) {
        w.parity ^= 1u << buf;
        w.inflight &= ~(1u << buf);
        use_smem = true;
      } else {
        w.staging = false;  // the copy stays in flight; read global memory from now on
        if (lane == 0) set_err(m.st, TREE2D_ERR_TIMEOUT);
      }
    }
    const bool corr = q >= nu;
    // the targets' offsets from A's centre, negated (see pair), and scaled
    // by A's s with scaled records
    const float sA = kScaled ? m.lscale[A] : 1.f;
    float ntx[kT], nty[kT], sa[kT], sb[kT];
#pragma unroll
    for (int k = 0; k < kT; k++) {
      const float2 zk = zof(k);
      ntx[k] = kScaled ? __fmul_rn(-__fadd_rn(zk.x, ox), sA) : -__fadd_rn(zk.x, ox);
      nty[k] = kScaled ? __fmul_rn(-__fadd_rn(zk.y, oy), sA) : -__fadd_rn(zk.y, oy);
      sa[k] = 0.f;
      sb[k] = 0.f;
    }
    unsigned done = 0;  // pairs evaluated for the chunk's valid targets
    auto runs = [&](const auto src) {
    while (r0 | r1) {
      int s0, s1;
      const int packs = next_run(r0, r1, cnt, s0, s1);
      done += (unsigned)(s1 - s0) * ((packs & 1 ? vp0 : 0u) + (packs & 2 ? vp1 : 0u));
      if (kT == 1) {
        if (!corr)
          leaf_pairs1<false, kScaled>(src, s0, s1, ntx[0], nty[0], sa[0], sb[0]);
        else
          leaf_pairs1<true, kScaled>(src, s0, s1, ntx[0], nty[0], sa[0], sb[0]);
      } else if (kT == 2 || packs != 3) {
        // one pack: slots 0, 1, or in a four-slot chunk 2, 3 when the run is
        // pack 1's alone (constant indices keep the slots in registers)
        auto one_pack = [&](auto k_) {
          constexpr int k = decltype(k_)::value;
          const float2 tx = make_float2(ntx[k], ntx[k + 1]), ty = make_float2(nty[k], nty[k + 1]);
          float2 a = make_float2(sa[k], sa[k + 1]), b = make_float2(sb[k], sb[k + 1]);
          if (!corr)
            leaf_pairs2<false, kScaled, kUnroll>(src, s0, s1, tx, ty, a, b);
          else
            leaf_pairs2<true, kScaled, kUnroll>(src, s0, s1, tx, ty, a, b);
          sa[k] = a.x, sa[k + 1] = a.y, sb[k] = b.x, sb[k + 1] = b.y;
        };
        if (kT == 4 && packs == 2)
          one_pack(std::integral_constant<int, kT - 2>{});
        else
          one_pack(std::integral_constant<int, 0>{});
      } else {
        const float2 tx0 = make_float2(ntx[0], ntx[1]), ty0 = make_float2(nty[0], nty[1]);
        const float2 tx1 = make_float2(ntx[kT - 2], ntx[kT - 1]), ty1 = make_float2(nty[kT - 2], nty[kT - 1]);
        float2 a0 = make_float2(sa[0], sa[1]), b0 = make_float2(sb[0], sb[1]);
        float2 a1 = make_float2(sa[kT - 2], sa[kT - 1]), b1 = make_float2(sb[kT - 2], sb[kT - 1]);
        if (!corr)
          leaf_pairs4<false, kScaled, kUnroll>(src, s0, s1, tx0, ty0, tx1, ty1, a0, b0, a1, b1);
        else
          leaf_pairs4<true, kScaled, kUnroll>(src, s0, s1, tx0, ty0, tx1, ty1, a0, b0, a1, b1);
        sa[0] = a0.x, sa[1] = a0.y, sb[0] = b0.x, sb[1] = b0.y;
        sa[kT - 2] = a1.x, sa[kT - 1] = a1.y, sb[kT - 2] = b1.x, sb[kT - 1] = b1.y;
      }
    }
    };
    if (use_smem)
      runs(SmemSrc{smem_u32(w.src + buf * kStage)});
    else
      runs(GlobalSrc{(kScaled ? m.src4s : m.src4) + j0});
#pragma unroll
    for (int k = 0; k < kT; k++) leaf_add(w.acc, k, lane, corr, sa[k], sb[k]);
    counts_add(w.cnts, lane, done, corr ? done : 0u, corr ? (unsigned)cnt * nt : 0u);
    __syncwarp();  // every lane is done with this buffer before it is refilled
    q = qn;
    r0 = r0n;
    r1 = r1n;
    buf ^= 1;
    staged = staged_next;
  }
  // far field: L2P of B's local expansion and the W list's M2P, then in the
  // learned form the accepted U entries' multipoles at the chosen order
  float2 phi[kT], z[kT];
#pragma unroll
  for (int k = 0; k < kT; k++) z[k] = zof(k);
  const unsigned char *wdec = kLearned ? dec.w : nullptr;
  if (kT == 1) {
    far_field(m, l, B, z[0], phi[0], wdec, dec.margin);
  } else {
#pragma unroll
    for (int k = 0; k < kT; k += 2)
      far_field2(m, l, B, z[k], z[(k + 1) % kT], phi[k], phi[(k + 1) % kT], wdec, dec.margin);
  }
  if (kLearned) {
    for (int e = u0; e < u0 + nu; e++) {
      const int d = dec.u[e];
      if (d > 0) {
        const int A = m.u_idx[e];
        const int p = min(min(class_order(d) + dec.margin, 16), m.P);
        if (kT == 1) {
          m2p_order(m, B, A, p, z[0], phi[0]);
        } else {
#pragma unroll
          for (int k = 0; k < kT; k += 2) m2p_order2(m, B, A, p, z[k], z[(k + 1) % kT], phi[k], phi[(k + 1) % kT]);
        }
      }
    }
  }
  if (lane == 0)
    for (int c = 0; c < 3; c++) {
      w.cnts->total[c] += w.cnts->chunk[c];
      w.cnts->chunk[c] = 0;
    }
  // FP64 final reduction: u = Im(phi)/2pi + ax/2pi, v = Re(phi)/2pi + ay/2pi
  const double inv2pi = 0.15915494309189533577;
#pragma unroll
  for (int k = 0; k < kT; k++)
    if (t0 + 32 * k + lane < tend) {
      const float4 sacc = w.acc[32 * k + lane];
      const int o = perm[t0 + 32 * k + lane];
      uv[2 * (size_t)o] = ((double)phi[k].y + (double)sacc.x - (double)sacc.y) * inv2pi;
      uv[2 * (size_t)o + 1] = ((double)phi[k].x + (double)sacc.z - (double)sacc.w) * inv2pi;
    }
  __syncwarp();
}

template <bool kLearned, bool kStaged, int kWarps, bool kWide, bool kScaled>
__global__ void __launch_bounds__(32 * kWarps, (kWide ? 24 : 32) / kWarps) k_eval_near(MixedView m, double *uv, const int *perm,
                                                                         Decisions dec, long wait_limit) {
  extern __shared__ __align__(128) float4 s_src[];  // kStaged: [kWarps][2 * kStage]
  __shared__ __align__(8) uint64_t s_bar[kWarps][2];
  __shared__ float s_tb[kWarps][9];
  __shared__ __align__(16) float4 s_acc[kWarps][4 * 32];
  __shared__ WarpCounts s_cnt[kWarps];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int i = next_leaf(m.st, lane);
  if (i >= m.nleaf) return;  // uniform over the warp; nothing below syncs the block
  NearWarp w{s_src + (kStaged ? warp * 2 * kStage : 0), s_bar[warp], s_tb[warp], s_acc[warp], &s_cnt[warp], 0u, 0u,
             true};
  if (kStaged && lane == 0) {
    mbar_init(&w.bar[0], 1);
    mbar_init(&w.bar[1], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (lane == 0) *w.cnts = WarpCounts{};
  __syncwarp();
  for (; i < m.nleaf; i = next_leaf(m.st, lane)) {
    const int l = m.leaf_order ? m.leaf_order[i] : i;
    const int B = m.leaf_cell[l];
    for (int t0 = m.begin[B]; t0 < m.end[B];) {
      const int rem = m.end[B] - t0;
      if (rem > 96) {
        near_chunk<kLearned, kStaged, 4, kWide ? 4 : 2, kScaled>(m, dec, uv, perm, wait_limit, l, B, t0, lane, w);
        t0 += 128;
      } else if (rem > 32) {
        near_chunk<kLearned, kStaged, 2, kWide ? 4 : 2, kScaled>(m, dec, uv, perm, wait_limit, l, B, t0, lane, w);
        t0 += 64;
      } else {
        near_chunk<kLearned, kStaged, 1, kWide ? 4 : 2, kScaled>(m, dec, uv, perm, wait_limit, l, B, t0, lane, w);
        t0 += 32;
      }
    }
  }
  // copies still in flight after a wait gave up: wait (bounded) before the
  // shared memory is released
  if (kStaged)
    for (int b = 0; b < 2; b++)
      if (w.inflight & (1u << b)) mbar_wait(&w.bar[b], (w.parity >> b) & 1u, wait_limit);
  counts_flush(w.cnts, lane, m.st);
}

// ------------------------------------------------------------ off-blob points

// Velocity at arbitrary points (not blob positions) on a mixed tree: one
// warp per 32 points (in key order), each lane one point, the warp walking
// the union of its lanes' traversals (a LIFO of cells with the lanes still
// inside each).  A lane accepts a cell's multipole when the point is at
// least kPtMac cell sides from the cell's centre (the scaled FP32 multipole
// of order P then truncates at (sqrt(2)/2 / kPtMac)^P = 0.283^16 = 2e-9 of
// the cell's field) and farther than the correction radius rc from the
// cell's box (so the point-vortex form leaves out only exp(-rc^2/s^2)
// terms, as the near field's correction list does).  Other cells are
// descended; leaves are summed pair by pair with the regularised kernel
// (fmm.c:121-142, the near field's FP32 pair), each leaf in FP32 and added
// in FP64.  Cells without a multipole (the root and the level-1 cells above
// the upward pass) are always descended.  The FP64 point is offset from
// each cell's FP64 centre before rounding to FP32, as the near field's
// centre offsets are.
constexpr int kPtWarps = 4;
constexpr int kPtStack = 160;
constexpr double kPtMac = 2.5;

__global__ void __launch_bounds__(kPtWarps * 32) k_eval_points(MixedView m, int ntgt, const double *tx,
                                                               const double *ty, const int *out_idx, double *uv) {
  __shared__ int s_cell[kPtWarps][kPtStack];
  __shared__ unsigned s_mask[kPtWarps][kPtStack];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long i = ((long)blockIdx.x * kPtWarps + warp) * 32 + lane;
  const bool valid = i < ntgt;
  const unsigned vmask = __ballot_sync(0xffffffffu, valid);
  if (vmask == 0) return;
  const double x = valid ? tx[i] : 0.0, y = valid ? ty[i] : 0.0;
  const double rc = (double)*m.rc_ptr, rc2 = rc * rc;
  const double mac2 = kPtMac * kPtMac;
  const int P = m.P;
  double phx = 0.0, phy = 0.0, ax = 0.0, ay = 0.0;
  unsigned long long n_m2p = 0, n_pairs = 0;
  bool overflow = false;
  int top = 0;
  if (lane == 0) {
    s_cell[warp][0] = 0;
    s_mask[warp][0] = vmask;
  }
  __syncwarp();
  while (top >= 0) {
    const int c = s_cell[warp][top];
    const unsigned msk = s_mask[warp][top];
    __syncwarp();
    top--;
    const bool act = (msk >> lane) & 1u;
    const bool is_leaf = m.leaf[c] != 0;
    const bool has_mp = is_leaf || m.level[c] >= 2 + m.lev0;
    bool far = false;
    double dx = 0.0, dy = 0.0;
    if (act && c != 0) {
      dx = x - m.cx[c];
      dy = y - m.cy[c];
      const double side = m.region[c];
      const double gx = fmax(fabs(dx) - 0.5 * side, 0.0), gy = fmax(fabs(dy) - 0.5 * side, 0.0);
      far = has_mp && dx * dx + dy * dy >= mac2 * side * side && gx * gx + gy * gy > rc2;
    }
    if (far) {
      // M2P: phi = (1/h) sum_k M_k w^(k+1), w = h / (z - zc)
      const float ih = m.inv_h[c];
      const float zx = __fmul_rn((float)dx, ih), zy = __fmul_rn((float)dy, ih);
      const float ir2 = __fdiv_rn(1.f, fmaf(zx, zx, __fmul_rn(zy, zy)));
      const float2 w = make_float2(__fmul_rn(zx, ir2), -__fmul_rn(zy, ir2));
      const float *MA = m.M + (size_t)c * 2 * P;
      float2 a = make_float2(MA[P - 1], MA[2 * P - 1]);
      for (int k = P - 2; k >= 0; k--) {
        a = fmul(a, w);
        a.x = __fadd_rn(a.x, MA[k]);
        a.y = __fadd_rn(a.y, MA[P + k]);
      }
      a = fmul(a, w);
      phx += (double)__fmul_rn(a.x, ih);
      phy += (double)__fmul_rn(a.y, ih);
      n_m2p++;
    }
    if (is_leaf) {
      if (act && !far) {
        const float nfx = -(float)dx, nfy = -(float)dy;
        float sa = 0.f, sb = 0.f;  // velocity (sa, -sb), see pair
        for (int j = m.begin[c]; j < m.end[c]; j++) pair<false>(m.src4[j], nfx, nfy, sa, sb);
        ax += (double)sa;
        ay -= (double)sb;
        n_pairs += (unsigned long long)(m.end[c] - m.begin[c]);
      }
    } else {
      const unsigned dmask = __ballot_sync(0xffffffffu, act && !far);
      if (dmask) {
        const int4 ch = reinterpret_cast<const int4 *>(m.child)[c];
        for (int q = 3; q >= 0; q--) {
          const int cc = (&ch.x)[q];
          if (cc < 0) continue;
          if (top + 1 >= kPtStack) {
            overflow = true;
            break;
          }
          top++;
          if (lane == 0) {
            s_cell[warp][top] = cc;
            s_mask[warp][top] = dmask;
          }
        }
      }
      __syncwarp();
      if (overflow) break;  // warp-uniform
    }
  }
  if (overflow && lane == 0) set_err(m.st, TREE2D_ERR_TIMEOUT);
  if (valid) {
    const double inv2pi = 0.15915494309189533577;
    const long o = out_idx ? out_idx[i] : i;
    uv[2 * o] = overflow ? NAN : (phy + ax) * inv2pi;
    uv[2 * o + 1] = overflow ? NAN : (phx + ay) * inv2pi;
  }
  for (int o = 16; o; o >>= 1) {
    n_m2p += __shfl_xor_sync(0xffffffffu, n_m2p, o);
    n_pairs += __shfl_xor_sync(0xffffffffu, n_pairs, o);
  }
  if (lane == 0) {
    atomicAdd(&m.st->n_m2s, n_m2p);
    atomicAdd(&m.st->n_pairs, n_pairs);
  }
}

// ------------------------------------------------------------ host side

double binom_d(int n, int k) {
  if (k < 0 || k > n) return 0.0;
  double r = 1.0;
  for (int i = 1; i <= k; i++) r = r * (double)(n - k + i) / (double)i;
  return r;
}

struct Cplx {
  double re, im;
};
Cplx cmulh(Cplx a, Cplx b) { return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
Cplx cpowi(Cplx z, int k) {
  Cplx r{1, 0};
  for (int i = 0; i < k; i++) r = cmulh(r, z);
  return r;
}
Cplx cinv(Cplx z) {
  double d = z.re * z.re + z.im * z.im;
  return {z.re / d, -z.im / d};
}

// child centre offset from the parent centre in units of the parent side,
// quadrant q (x+ if q odd, y- if q >= 2)
Cplx quad_offset(int q) { return {(q & 1) ? 0.25 : -0.25, (q & 2) ? -0.25 : 0.25}; }

bool g_tables_ready[64] = {};

}  // namespace

// Host tables: h_m2l [4][27][P][P] complex, h_m2m / h_l2l [4][kMaxP][kMaxP]
// complex (M2M [q][n][k], L2L [q][k][l]); the slot table goes to constant
// memory of the current device.
cudaError_t mixed_tables(int P, float *h_m2l, float *h_m2m, float *h_l2l) {
  // slot table: class (qx,qy) -> 6x6 offsets around the parent's block
  static signed char slot[4][6][6];
  int cnt[4] = {0, 0, 0, 0};
  for (int cls = 0; cls < 4; cls++) {
    int qx = cls & 1, qy = cls >> 1;
    for (int a = 0; a < 6; a++)
      for (int b = 0; b < 6; b++) slot[cls][a][b] = -1;
    for (int dy = -2 - qy; dy <= 3 - qy; dy++)
      for (int dx = -2 - qx; dx <= 3 - qx; dx++) {
        if (abs(dx) <= 1 && abs(dy) <= 1) continue;
        int s = cnt[cls]++;
        slot[cls][dy + 2 + qy][dx + 2 + qx] = (signed char)s;
        if (!h_m2l) continue;
        // tau = (z_target - z_source)/h = -dx + i dy
        Cplx tau{(double)-dx, (double)dy};
        Cplx ti = cinv(tau);
        for (int l = 0; l < P; l++)
          for (int k = 0; k < P; k++) {
            Cplx v = cpowi(ti, k + l + 1);
            double f = ((l & 1) ? -1.0 : 1.0) * binom_d(k + l, l);
            float *o = h_m2l + ((((size_t)cls * 27 + s) * P + l) * P + k) * 2;
            o[0] = (float)(f * v.re);
            o[1] = (float)(f * v.im);
          }
      }
  }
  auto m2m = reinterpret_cast<float(*)[kMaxP][kMaxP][2]>(h_m2m);
  auto l2l = reinterpret_cast<float(*)[kMaxP][kMaxP][2]>(h_l2l);
  for (int q = 0; q < 4 && h_m2m && h_l2l; q++) {
    Cplx d = quad_offset(q);
    for (int n = 0; n < kMaxP; n++)
      for (int k = 0; k < kMaxP; k++) {
        // M2M: a'_n += a_k 2^-k C(n,k) d^(n-k)   (k <= n)
        Cplx v{0, 0};
        if (k <= n) {
          Cplx pw = cpowi(d, n - k);
          double f = std::ldexp(binom_d(n, k), -k);
          v = {f * pw.re, f * pw.im};
        }
        m2m[q][n][k][0] = (float)v.re;
        m2m[q][n][k][1] = (float)v.im;
        // L2L: b'_k += b_l C(l,k) d^(l-k) 2^-(k+1)   (l >= k); stored [k][l]
        Cplx w{0, 0};
        int kk = n, l = k;
        if (l >= kk) {
          Cplx pw = cpowi(d, l - kk);
          double f = std::ldexp(binom_d(l, kk), -(kk + 1));
          w = {f * pw.re, f * pw.im};
        }
        l2l[q][kk][l][0] = (float)w.re;
        l2l[q][kk][l][1] = (float)w.im;
      }
  }
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev >= 0 && dev < 64 && g_tables_ready[dev]) return cudaSuccess;
  cudaError_t e = cudaMemcpyToSymbol(c_slot, slot, sizeof(slot));
  if (e == cudaSuccess && dev >= 0 && dev < 64) g_tables_ready[dev] = true;
  return e;
}

int mixed_lists(MixedView &m, cudaStream_t s) {
  const int cb = (m.ncell + 255) / 256;
  k_cell_info<<<cb, 256, 0, s>>>(m);
  T2D_CUDA_TRY(cudaMemsetAsync(m.level_off, 0, sizeof(int) * (2 * kKeyLevels + 4), s));
  k_level_hist<<<cb, 256, 0, s>>>(m);
  k_level_scan<<<1, 32, 0, s>>>(m);
  k_level_fill<<<cb, 256, 0, s>>>(m);
  g_launches.fetch_add(3, std::memory_order_relaxed);
  k_parent<<<cb, 256, 0, s>>>(m);
  k_colleagues<<<cb, 256, 0, s>>>(m);
  k_vx_lists<<<(int)(((long)m.ncell * 32 + 255) / 256), 256, 0, s>>>(m);
  if (m.list_scratch)
    k_lists<2><<<(m.nleaf + kWalkWarps - 1) / kWalkWarps, 32 * kWalkWarps, 0, s>>>(m);
  else
    k_lists<0><<<(m.nleaf + kWalkWarps - 1) / kWalkWarps, 32 * kWalkWarps, 0, s>>>(m);
  const int ntiles = max(1, (m.nleaf + kScanTile3 - 1) / kScanTile3);
  k_scan3_tiles<<<ntiles, kScan3Threads, 0, s>>>(m.u_off, m.w_off, m.k_off, m.nleaf, m.scan_tmp, ntiles);
  k_scan3_sums<<<1, 32, 0, s>>>(m.scan_tmp, ntiles);
  k_scan3_apply<<<ntiles, kScan3Threads, 0, s>>>(m.u_off, m.w_off, m.k_off, m.nleaf, m.scan_tmp, ntiles);
  g_launches.fetch_add(8, std::memory_order_relaxed);
  T2D_CUDA_TRY(cudaGetLastError());
  return TREE2D_OK;
}

int mixed_fill_lists(MixedView &m, bool from_scratch, cudaStream_t s) {
  if (from_scratch)
    k_lists_compact<<<(int)(((long)m.nleaf * 32 + 255) / 256), 256, 0, s>>>(m);
  else
    k_lists<1><<<(m.nleaf + kWalkWarps - 1) / kWalkWarps, 32 * kWalkWarps, 0, s>>>(m);
  g_launches.fetch_add(1, std::memory_order_relaxed);
  T2D_CUDA_TRY(cudaGetLastError());
  return TREE2D_OK;
}

int mixed_leaf_setup(MixedView &m, const Tree &t, cudaStream_t s) {
  k_leaf_setup<<<(m.nleaf + kSetupWarps - 1) / kSetupWarps, 32 * kSetupWarps, 0, s>>>(m, t.x, t.y, t.cir, t.cor,
                                                                                        t.perm);
  g_launches.fetch_add(1, std::memory_order_relaxed);
  T2D_CUDA_TRY(cudaGetLastError());
  return TREE2D_OK;
}

// Blocks of 8 warps for a per-level pass over cnt cells (one warp per cell,
// grid-stride beyond 8 blocks per SM): a level of few cells gets few blocks.
static int level_blocks(const int *lev_off, int lev) {
  const int full = 152 * 8;
  if (!lev_off) return full;
  const int cnt = lev_off[lev + 1] - lev_off[lev];
  const int b = (cnt + 7) / 8;
  return b < 1 ? 1 : (b > full ? full : b);
}

// Blocks of kQuadThreads for a per-level pass with four threads per cell.
static int quad_blocks(const int *lev_off, int lev) {
  const int full = 152 * 8;
  if (!lev_off) return full;
  const int cnt = lev_off[lev + 1] - lev_off[lev];
  const int b = (cnt + kQuadThreads / 4 - 1) / (kQuadThreads / 4);
  return b < 1 ? 1 : (b > full ? full : b);
}

// The M2M or L2L level chain as one cooperative launch of persistent
// blocks (k_chain_quad), for P = 16 and at least two levels: returns false
// (nothing launched) where the device cannot co-schedule the grid, and the
// caller launches one kernel per level instead.
constexpr long kChainWaitLimit = 1l << 22;

template <bool kUp>
bool launch_chain(MixedView &m, int lev_first, int lev_last, cudaStream_t s) {
  static int blocks[2] = {0, 0};  // per direction: resident blocks, found once (the devices here are one model)
  int &nb = blocks[kUp ? 1 : 0];
  auto k = k_chain_quad<16, kUp>;
  if (nb == 0) {
    int dev = 0, sms = 0, per_sm = 0, coop = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess || !coop ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, kQuadThreads, 0) != cudaSuccess || per_sm < 1) {
      nb = -1;
    } else {
      nb = sms * (per_sm < 4 ? per_sm : 4);
    }
  }
  if (nb < 0) return false;
  if (cudaMemsetAsync(&m.st->bar_count, 0, sizeof(unsigned), s) != cudaSuccess) return false;
  long limit = kChainWaitLimit;
  void *args[] = {&m, &lev_first, &lev_last, &limit};
  if (cudaLaunchCooperativeKernel((const void *)k, dim3((unsigned)nb), dim3(kQuadThreads), args, 0, s) !=
      cudaSuccess) {
    (void)cudaGetLastError();  // not launched: clear the error, run per level
    return false;
  }
  g_launches.fetch_add(1, std::memory_order_relaxed);
  return true;
}

int mixed_upward(MixedView &m, int depth, const int *lev_off, cudaStream_t s, bool chain) {
  k_s2m_f32<<<(int)(((long)m.nleaf * 32 + 255) / 256), 256, 0, s>>>(m);
  g_launches.fetch_add(1, std::memory_order_relaxed);
  const size_t tab_bytes = 4 * sizeof(float2) * m.P * m.P;
  if (chain && m.P == 16 && depth - 1 > 2 + m.lev0 && launch_chain<true>(m, depth - 1, 2 + m.lev0, s)) {
    T2D_CUDA_TRY(cudaGetLastError());
    return TREE2D_OK;
  }
  for (int lev = depth - 1; lev >= 2 + m.lev0; lev--) {
    if (m.P == 16)
      k_m2m_quad<16><<<quad_blocks(lev_off, lev), kQuadThreads, 0, s>>>(m, lev);
    else if (m.P < 16)
      k_m2m_f32<16><<<level_blocks(lev_off, lev), 256, tab_bytes, s>>>(m, lev);
    else
      k_m2m_f32<32><<<level_blocks(lev_off, lev), 256, tab_bytes, s>>>(m, lev);
    g_launches.fetch_add(1, std::memory_order_relaxed);
  }
  T2D_CUDA_TRY(cudaGetLastError());
  return TREE2D_OK;
}

int mixed_downward(MixedView &m, int depth, const int *lev_off, cudaStream_t s, bool chain) {
  k_p2l<<<(int)(((long)m.ncell * 32 + 255) / 256), 256, 0, s>>>(m);
  g_launches.fetch_add(1, std::memory_order_relaxed);
  const size_t tab_bytes = 4 * sizeof(float2) * m.P * m.P;
  if (chain && m.P == 16 && depth > 3 + m.lev0 && launch_chain<false>(m, 3 + m.lev0, depth, s)) {
    T2D_CUDA_TRY(cudaGetLastError());
    return TREE2D_OK;
  }
  for (int lev = 3 + m.lev0; lev <= depth; lev++) {
    if (m.P == 16)
      k_l2l_quad<16><<<quad_blocks(lev_off, lev - 1), kQuadThreads, 0, s>>>(m, lev);
    else if (m.P < 16)
      k_l2l_f32<16><<<level_blocks(lev_off, lev - 1), 256, tab_bytes, s>>>(m, lev);
    else
      k_l2l_f32<32><<<level_blocks(lev_off, lev - 1), 256, tab_bytes, s>>>(m, lev);
    g_launches.fetch_add(1, std::memory_order_relaxed);
  }
  T2D_CUDA_TRY(cudaGetLastError());
  return TREE2D_OK;
}

// Near-field variants (bit-identical results): 0/1 read the source blobs
// from global memory with 4/8 warps per block, 2/3 stage them in shared
// memory by bulk copies with 4/8 warps per block, 4 stages them with 4
// warps per block of up to 80 registers per thread (6 blocks per SM) and
// the pair loops unrolled four times.  At 1M Lamb-Oseen blobs 4 is the
// fastest, at 4M two-patch + sheet blobs 2, for the 512-set batch 0.
constexpr int kEvalVariants = kEvalVariantCount;

// Blocks of a persistent near-field launch: as many as are resident on the
// device at once (the kernel's occupancy times the SM count, found once per
// kernel and kept in *resident), fewer when the leaves are fewer.
template <class K>
int persistent_blocks(K kernel, int warps_per_block, size_t smem, int nleaf, int *resident) {
  if (*resident == 0) {
    int dev = 0, sms = 0, per_sm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, 32 * warps_per_block, smem) != cudaSuccess ||
        per_sm < 1)
      return (nleaf + warps_per_block - 1) / warps_per_block;  // one warp per leaf
    *resident = sms * per_sm;
  }
  const int need = (nleaf + warps_per_block - 1) / warps_per_block;
  return need < *resident ? need : *resident;
}

// One near-field variant: kStaged sources (stage buffers in dynamic shared
// memory, 4 KB per warp), kWarps warps per block, persistent blocks.
template <bool kLearned, bool kScaled, bool kStaged, int kWarps, bool kWide = false>
cudaError_t launch_near(const MixedView &m, double *uv, const int *perm, Decisions d, cudaStream_t s, int *resident) {
  auto k = k_eval_near<kLearned, kStaged, kWarps, kWide, kScaled>;
  const size_t smem = kStaged ? (size_t)kWarps * 2 * kStage * sizeof(float4) : 0;
  if (*resident == 0 && smem > 0) {
    const cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  k<<<persistent_blocks(k, kWarps, smem, m.nleaf, resident), 32 * kWarps, smem, s>>>(m, uv, perm, d, kEvalWaitLimit);
  return cudaSuccess;
}

template <bool kLearned, bool kScaled>
cudaError_t launch_eval(int v, const MixedView &m, double *uv, const int *perm, Decisions d, cudaStream_t s) {
  static int resident[kEvalVariants] = {};  // per variant (the devices here are all one model)
  cudaError_t e = cudaMemsetAsync(&m.st->eval_next, 0, sizeof(unsigned), s);
  if (e != cudaSuccess) return e;
  switch (v) {
    case 0: e = launch_near<kLearned, kScaled, false, 4>(m, uv, perm, d, s, &resident[0]); break;
    case 1: e = launch_near<kLearned, kScaled, false, 8>(m, uv, perm, d, s, &resident[1]); break;
    case 2: e = launch_near<kLearned, kScaled, true, 4>(m, uv, perm, d, s, &resident[2]); break;
    case 3: e = launch_near<kLearned, kScaled, true, 8>(m, uv, perm, d, s, &resident[3]); break;
    default: e = launch_near<kLearned, kScaled, true, 4, true>(m, uv, perm, d, s, &resident[4]); break;
  }
  if (e != cudaSuccess) return e;
  g_launches.fetch_add(1, std::memory_order_relaxed);
  return cudaGetLastError();
}

// The near field with the variant the tuner chose for this size class: on
// the first solve of a (device, form, P, leaf-count octave) class every
// variant runs twice, in the order 0 1 2 3 3 2 1 0 (so that clocks still
// ramping up favour no variant), timed by CUDA events on the stream, and the
// one with the fastest run is kept (each run writes the same velocities, so
// the last one stands).
int near_field(Workspace &ws, const MixedParams &mp, MixedView &m, bool learned, Decisions d, double *uv,
               const int *perm, cudaStream_t s, tree2d_stats_t &st) {
  // scaled source records where every leaf's blobs share one core radius
  const bool scaled = m.src4s && !ws.h_status->nonuniform;
  auto run = [&](int v) {
    if (scaled)
      return learned ? launch_eval<true, true>(v, m, uv, perm, d, s) : launch_eval<false, true>(v, m, uv, perm, d, s);
    return learned ? launch_eval<true, false>(v, m, uv, perm, d, s) : launch_eval<false, false>(v, m, uv, perm, d, s);
  };
  int v = mp.eval_variant;
  if (v < 0 && mp.autotune) {
    int dev = 0;
    T2D_CUDA_TRY(cudaGetDevice(&dev));
    int octave = 0;
    while (octave < 40 && (1ll << (octave + 1)) <= (long long)m.nleaf) octave++;
    const uint64_t key = ((uint64_t)dev << 40) | ((uint64_t)(learned ? 1 : 0) << 32) | ((uint64_t)m.P << 16) |
                         (uint64_t)octave;
    auto it = ws.eval_tuned.find(key);
    if (it != ws.eval_tuned.end()) {
      v = it->second;
    } else {
      float best = 0.f;
      int bv = 0;
      for (int r = 0; r < 2 * kEvalVariants; r++) {
        const int c = r < kEvalVariants ? r : 2 * kEvalVariants - 1 - r;
        T2D_CUDA_TRY(cudaMemsetAsync(&ws.status->n_pairs, 0, sizeof(unsigned long long), s));
        T2D_CUDA_TRY(cudaEventRecord(ws.ev[6], s));
        T2D_CUDA_TRY(run(c));
        T2D_CUDA_TRY(cudaEventRecord(ws.ev[7], s));
        T2D_CUDA_TRY(cudaEventSynchronize(ws.ev[7]));
        float ms = 0.f;
        T2D_CUDA_TRY(cudaEventElapsedTime(&ms, ws.ev[6], ws.ev[7]));
        if (r == 0 || ms < best) {
          best = ms;
          bv = c;
        }
      }
      ws.eval_tuned[key] = bv;
      st.eval_variant = bv;
      return TREE2D_OK;
    }
  }
  if (v < 0 || v >= kEvalVariants) v = 0;
  T2D_CUDA_TRY(run(v));
  st.eval_variant = v;
  return TREE2D_OK;
}

// The tensor-core M2L with the tile the tuner chose for this size class
// (cells per CTA, 128 or 64, bit-identical results): on the first solve of
// a (device, P, cell-count octave) class both shapes run twice, in the
// order 128 64 64 128, timed by CUDA events on the stream, and the faster
// is kept (each run stores the same local expansions).
int m2l_tc_tuned(Workspace &ws, const MixedParams &mp, MixedView &m, const float *dimg, int *cls_list,
                 int *cls_count, cudaStream_t s, tree2d_stats_t &st) {
  int rows = mp.m2l_rows;
  if (rows == 0 && mp.autotune) {
    int dev = 0;
    T2D_CUDA_TRY(cudaGetDevice(&dev));
    int octave = 0;
    while (octave < 40 && (1ll << (octave + 1)) <= (long long)m.ncell) octave++;
    const uint64_t key = ((uint64_t)dev << 40) | ((uint64_t)m.P << 16) | (uint64_t)octave;
    auto it = ws.m2l_tuned.find(key);
    if (it != ws.m2l_tuned.end()) {
      rows = it->second;
    } else {
      static const int kShapes[4] = {128, 64, 64, 128};
      float best = 0.f;
      int br = 128;
      for (int r = 0; r < 4; r++) {
        T2D_CUDA_TRY(cudaEventRecord(ws.ev[6], s));
        const int rc = m2l_tensor_cores(m, dimg, cls_list, cls_count, kShapes[r], s);
        if (rc) return rc;
        T2D_CUDA_TRY(cudaEventRecord(ws.ev[7], s));
        T2D_CUDA_TRY(cudaEventSynchronize(ws.ev[7]));
        float ms = 0.f;
        T2D_CUDA_TRY(cudaEventElapsedTime(&ms, ws.ev[6], ws.ev[7]));
        if (r == 0 || ms < best) {
          best = ms;
          br = kShapes[r];
        }
      }
      ws.m2l_tuned[key] = br;
      st.m2l_rows = br;
      return TREE2D_OK;
    }
  }
  if (rows != 64) rows = 128;
  st.m2l_rows = rows;
  return m2l_tensor_cores(m, dimg, cls_list, cls_count, rows, s);
}

int mixed_eval_points(Workspace &ws, int ntgt, const double *tx, const double *ty, const int *out_idx, double *uv,
                      cudaStream_t s) {
  if (ntgt <= 0) return TREE2D_OK;
  if (!ws.mxv) return TREE2D_ERR_NO_TREE;
  const int warps = (ntgt + 31) / 32;
  k_eval_points<<<(warps + kPtWarps - 1) / kPtWarps, kPtWarps * 32, 0, s>>>(*ws.mxv, ntgt, tx, ty, out_idx, uv);
  g_launches.fetch_add(1, std::memory_order_relaxed);
  T2D_CUDA_TRY(cudaGetLastError());
  return TREE2D_OK;
}

int mixed_solve(Workspace &ws, const Tree &t, const MixedParams &mp, double *d_uv, cudaStream_t s,
                tree2d_stats_t &st) {
  const int P = mp.pterms;
  if (P < 2 || P > kMaxP) return TREE2D_ERR_BAD_PARAMS;
  const int n = t.n, nc = t.ncell, nl = t.nleaf;
  // ---- operators (per P, cached)
  const bool tc = mp.use_tensor_cores && (P % 4 == 0);
  const size_t n_m2l = (size_t)4 * 27 * P * P * 2, n_tr = (size_t)4 * kMaxP * kMaxP * 2;
  const size_t n_img = (size_t)4 * 27 * 2 * m2l_npad(P) * 2 * P;
  Arena &tab = ws.mx_tables[P];
  if (tab.capacity() == 0) {
    std::vector<float> m2l(n_m2l), m2m(n_tr), l2l(n_tr), img;
    T2D_CUDA_TRY(mixed_tables(P, m2l.data(), m2m.data(), l2l.data()));
    m2l_b_images(P, m2l.data(), img);
    size_t need = Arena::bytes_for(n_m2l, 4) + 2 * Arena::bytes_for(n_tr, 4) + Arena::bytes_for(n_img, 4);
    T2D_CUDA_TRY(tab.reserve(need));
    tab.reset();
    float *dm2l = tab.take<float>(n_m2l);
    float *dm2m = tab.take<float>(n_tr);
    float *dl2l = tab.take<float>(n_tr);
    float *dimg = tab.take<float>(n_img);
    cudaError_t e = cudaMemcpy(dm2l, m2l.data(), n_m2l * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dm2m, m2m.data(), n_tr * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dl2l, l2l.data(), n_tr * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dimg, img.data(), n_img * 4, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
      ws.mx_tables.erase(P);  // not filled: made again by the next solve at this P
      note_cuda_error(e, "mixed operator tables");
      return TREE2D_ERR_CUDA;
    }
  } else {
    T2D_CUDA_TRY(mixed_tables(P, nullptr, nullptr, nullptr));
  }
  tab.reset();
  const float *dm2l = tab.take<float>(n_m2l);
  const float *dm2m = tab.take<float>(n_tr);
  const float *dl2l = tab.take<float>(n_tr);
  const float *dimg = tab.take<float>(n_img);

  // ---- arrays
  size_t need = 0;
  need += Arena::bytes_for(nc, 4) * 5;            // ix iy h inv_h parent
  need += Arena::bytes_for(n, 4) * 3;             // leaf_of gam + pad
  need += Arena::bytes_for(n, 8);                 // loc
  need += Arena::bytes_for(n, 16) + Arena::bytes_for(nc, 4) * 4;  // src4, cxf, cyf, cxl, cyl
  need += Arena::bytes_for(n, 16) + Arena::bytes_for(nc, 4);      // src4s, lscale
  const int kchunks = t.leaf_cap > 0 ? (t.leaf_cap + kChunk - 1) / kChunk : 1;
  need += Arena::bytes_for((size_t)nc * kchunks, 16);              // chunk boxes
  need += Arena::bytes_for(n, 4);                                  // mperm
  need += Arena::bytes_for((size_t)nc * 9, 4) * 2;
  need += Arena::bytes_for((size_t)nc * 27, 4) + Arena::bytes_for((size_t)nc * 8, 4);
  need += Arena::bytes_for((size_t)nl + 1, 4) * 3;
  need += Arena::bytes_for(3 * ((size_t)nl / kScanTile3 + 2), 4);  // scan tile sums
  need += Arena::bytes_for((size_t)t.nsets, 4);                     // cutoff per set
  need += Arena::bytes_for(nc, 4) + Arena::bytes_for(2 * kKeyLevels + 4, 4);  // cells by level
  // one-walk list scratch, sized from the previous solve's largest leaf
  // (a leaf beyond it makes this solve walk twice instead); kept below 4 GB
  const int cap = ws.list_cap;
  const bool one_walk = (size_t)nl * (size_t)cap * 4 <= (size_t(4) << 30) && nc < (1 << 30);
  if (one_walk) need += Arena::bytes_for((size_t)nl * cap, 4);
  need += Arena::bytes_for((size_t)nc * 2 * P, 4) * 2;
  need += Arena::bytes_for((size_t)nc * 4, 4) + 1024;  // class lists + counts
  // near-field schedule: keys, values and their sort buffers
  need += 2 * Arena::bytes_for((size_t)nl, 8) + 2 * Arena::bytes_for((size_t)nl, 4) +
          Arena::bytes_for(radix_sort_temp_bytes(nl), 1);
  need += 256;
  T2D_CUDA_TRY(ws.mx_arena.reserve(need));
  ws.mx_arena.reset();
  MixedView m{};
  m.n = n;
  m.ncell = nc;
  m.nleaf = nl;
  m.P = P;
  m.keys = t.keys;
  m.cpl = t.cpl;
  m.leaf_level = t.leaf_level;
  m.cellbase = t.cellbase;
  m.level = t.level;
  m.begin = t.begin;
  m.end = t.end;
  m.child = t.child;
  m.leaf_cell = t.leaf_cell;
  m.leaf = t.leaf;
  m.cx = t.cx;
  m.cy = t.cy;
  m.region = t.region;
  m.ix = ws.mx_arena.take<unsigned>(nc);
  m.iy = ws.mx_arena.take<unsigned>(nc);
  m.h = ws.mx_arena.take<float>(nc);
  m.inv_h = ws.mx_arena.take<float>(nc);
  m.parent = ws.mx_arena.take<int>(nc);
  m.leaf_of = ws.mx_arena.take<int>(n);
  m.loc = ws.mx_arena.take<float2>(n);
  m.gam = ws.mx_arena.take<float>(n);
  m.src4 = ws.mx_arena.take<float4>(n);
  m.src4s = ws.mx_arena.take<float4>(n);
  m.lscale = ws.mx_arena.take<float>(nc);
  m.kchunks = kchunks;
  m.cbox = ws.mx_arena.take<float4>((size_t)nc * kchunks);
  m.mperm = ws.mx_arena.take<int>(n);
  m.cxf = ws.mx_arena.take<float>(nc);
  m.cyf = ws.mx_arena.take<float>(nc);
  m.cxl = ws.mx_arena.take<float>(nc);
  m.cyl = ws.mx_arena.take<float>(nc);
  m.coll = ws.mx_arena.take<int>((size_t)nc * 9);
  m.coarse = ws.mx_arena.take<int>((size_t)nc * 9);
  m.vlist = ws.mx_arena.take<int>((size_t)nc * 27);
  m.xlist = ws.mx_arena.take<int>((size_t)nc * 8);
  m.u_off = ws.mx_arena.take<int>((size_t)nl + 1);
  m.w_off = ws.mx_arena.take<int>((size_t)nl + 1);
  m.k_off = ws.mx_arena.take<int>((size_t)nl + 1);
  m.scan_tmp = ws.mx_arena.take<int>(3 * ((size_t)nl / kScanTile3 + 2));
  m.by_level = ws.mx_arena.take<int>(nc);
  m.list_cap = cap;
  m.list_scratch = one_walk ? ws.mx_arena.take<int>((size_t)nl * cap) : nullptr;
  m.level_off = ws.mx_arena.take<int>(2 * kKeyLevels + 4);
  m.M = ws.mx_arena.take<float>((size_t)nc * 2 * P);
  m.L = ws.mx_arena.take<float>((size_t)nc * 2 * P);
  uint64_t *ord_keys = ws.mx_arena.take<uint64_t>((size_t)nl), *ord_keys2 = ws.mx_arena.take<uint64_t>((size_t)nl);
  uint32_t *ord_vals = ws.mx_arena.take<uint32_t>((size_t)nl), *ord_vals2 = ws.mx_arena.take<uint32_t>((size_t)nl);
  void *ord_tmp = ws.mx_arena.take<char>(radix_sort_temp_bytes(nl));
  m.leaf_order = nullptr;
  unsigned *rc_bits = ws.mx_arena.take<unsigned>(1);
  unsigned *rc_set_bits = t.nsets > 1 ? ws.mx_arena.take<unsigned>((size_t)t.nsets) : nullptr;
  int *cls_list = ws.mx_arena.take<int>((size_t)nc * 4);
  int *cls_count = ws.mx_arena.take<int>(4);
  m.rc_ptr = reinterpret_cast<const float *>(rc_bits);
  m.rc_set = reinterpret_cast<const float *>(rc_set_bits);
  m.lev0 = t.lev0;
  // the learned form's envelope counts K entries at the radius its network
  // was trained with; when that is larger than the one in force, the
  // correction walk goes out to it and counts the extra leaves
  const bool envelope_walk = mp.learned && mp.lp && mp.lp->have_weights && mp.lp->k_blobs_max > 0.0 &&
                             mp.lp->cutoff_train > mp.cutoff && t.lev0 == 0;
  m.walk_scale = envelope_walk ? (float)(mp.lp->cutoff_train / mp.cutoff) : 1.f;
  m.m2m = reinterpret_cast<const float2 *>(dm2m);
  m.l2l = reinterpret_cast<const float2 *>(dl2l);
  m.st = ws.status;
  T2D_CUDA_TRY(cudaMemsetAsync(m.parent, 0xff, sizeof(int) * (size_t)nc, s));
  T2D_CUDA_TRY(cudaMemsetAsync(rc_bits, 0, 4, s));
  k_sigma_max<<<304, 256, 0, s>>>(t.cor, n, rc_bits);
  k_cutoff<<<1, 32, 0, s>>>(rc_bits, (float)mp.cutoff, 1);
  g_launches.fetch_add(2, std::memory_order_relaxed);
  if (rc_set_bits) {
    T2D_CUDA_TRY(cudaMemsetAsync(rc_set_bits, 0, 4 * (size_t)t.nsets, s));
    k_sigma_max_sets<<<dim3((unsigned)t.nsets, kSigmaSlices), 256, 0, s>>>(t.set_cor, t.set_off, rc_set_bits);
    k_cutoff<<<(t.nsets + 255) / 256, 256, 0, s>>>(rc_set_bits, (float)mp.cutoff, t.nsets);
    g_launches.fetch_add(2, std::memory_order_relaxed);
  }

  int rc = mixed_leaf_setup(m, t, s);
  if (rc) return rc;
  rc = mixed_lists(m, s);
  if (rc) return rc;
  int tot[3];
  T2D_CUDA_TRY(cudaMemcpyAsync(&tot[0], m.u_off + nl, 4, cudaMemcpyDeviceToHost, s));
  T2D_CUDA_TRY(cudaMemcpyAsync(&tot[1], m.w_off + nl, 4, cudaMemcpyDeviceToHost, s));
  T2D_CUDA_TRY(cudaMemcpyAsync(&tot[2], m.k_off + nl, 4, cudaMemcpyDeviceToHost, s));
  T2D_CUDA_TRY(cudaMemcpyAsync(ws.h_status, ws.status, sizeof(DevStatus), cudaMemcpyDeviceToHost, s));
  if (ws.h_levels)
    T2D_CUDA_TRY(cudaMemcpyAsync(ws.h_levels, m.level_off, sizeof(int) * (kKeyLevels + 2), cudaMemcpyDeviceToHost, s));
  T2D_CUDA_TRY(cudaStreamSynchronize(s));
  const bool from_scratch = one_walk && !ws.h_status->list_overflow;
  {
    // the next solve's scratch rows: 1.25 x this solve's largest leaf
    int want = ws.h_status->list_max + ws.h_status->list_max / 4 + 32;
    want = (want + 31) & ~31;
    ws.list_cap = want < 64 ? 64 : (want > 8192 ? 8192 : want);
  }
  if (tot[0] < 0 || tot[1] < 0 || tot[2] < 0) {
    // more than 2^31 - 1 entries in one list kind (int positions)
    note_cuda_error(cudaErrorMemoryAllocation, "interaction lists beyond 2^31 entries");
    return TREE2D_ERR_TOO_LARGE;
  }
  size_t lneed = 2 * Arena::bytes_for((size_t)tot[0] + 1, 4) + 2 * Arena::bytes_for((size_t)tot[1] + 1, 4) +
                 2 * Arena::bytes_for((size_t)tot[2] + 1, 4);
  T2D_CUDA_TRY(ws.mx_lists.reserve(lneed));
  ws.mx_lists.reset();
  m.u_idx = ws.mx_lists.take<int>((size_t)tot[0] + 1);
  m.w_idx = ws.mx_lists.take<int>((size_t)tot[1] + 1);
  m.k_idx = ws.mx_lists.take<int>((size_t)tot[2] + 1);
  m.u_leaf = ws.mx_lists.take<int>((size_t)tot[0] + 1);
  m.w_leaf = ws.mx_lists.take<int>((size_t)tot[1] + 1);
  m.k_leaf = ws.mx_lists.take<int>((size_t)tot[2] + 1);
  rc = mixed_fill_lists(m, from_scratch, s);
  if (rc) return rc;
  // the near field's largest-first schedule, on the second stream beside
  // the expansions (joined before the near field)
  if (nl > 1) m.leaf_order = reinterpret_cast<const int *>(ord_vals);
  auto schedule = [&](cudaStream_t q) -> cudaError_t {
    if (nl <= 1) return cudaSuccess;
    k_leaf_cost<<<(int)(((long)nl * 32 + 255) / 256), 256, 0, q>>>(m, ord_keys, ord_vals);
    g_launches.fetch_add(1, std::memory_order_relaxed);
    return radix_sort_pairs(ord_keys, ord_vals, ord_keys2, ord_vals2, nl, 56, 64, ord_tmp, q);
  };
  // keep the view for sampling (training data)
  if (!ws.mxv) ws.mxv = new MixedView();
  *ws.mxv = m;
  ws.mx_tot[0] = tot[0];
  ws.mx_tot[1] = tot[1];
  ws.mx_tot[2] = tot[2];
  // The network's decisions need only the lists and the leaves' source
  // statistics, not the expansions: they run on a second stream, forked
  // here and joined before the near field, beside the upward pass, M2L and
  // the downward pass (both chains are latency-bound and share the GPU
  // well).  On a batched tree each set has its own reference scale u_ref,
  // the one it has alone.
  // the network decides only inside its training envelope: denser lists
  // than it was trained on would add up more accepted errors per target
  // than its per-interaction budget allows for.  The density is the K
  // leaves' source blobs per leaf, counted out to the training radius: it
  // does not depend on the leaf size, which a count of entries would.
  const double k_blobs = (double)ws.h_status->k_blobs;
  const bool in_envelope = mp.lp && (mp.lp->k_blobs_max <= 0.0 || k_blobs <= mp.lp->k_blobs_max * nl);
  const bool learned = mp.learned && mp.lp && mp.lp->have_weights && in_envelope;
  st.learned_active = learned ? 1 : 0;
  st.n_list_u = tot[0];
  st.n_list_k = tot[2];
  st.n_list_k_blobs = (long long)ws.h_status->k_blobs;
  unsigned char *u_dec = nullptr, *k_dec = nullptr, *w_dec = nullptr;
  const bool side = learned || mp.learned;
  // after the fork, an early return first waits for the second stream, so
  // that no kernel of this solve still runs when its buffers are reused
  bool forked = false;
  auto drain = [&](int code) {
    if (forked) {
      cudaStreamSynchronize(ws.side);
      cudaStreamSynchronize(ws.hi);
    }
    return code;
  };
#define T2D_TRY_DRAIN(expr)                 \
  do {                                      \
    cudaError_t e_ = (expr);                \
    if (e_ != cudaSuccess) {                \
      note_cuda_error(e_, #expr);           \
      return drain(TREE2D_ERR_CUDA);        \
    }                                       \
  } while (0)
  if (side) {
    // leaf statistics and u_ref (also used by sampling), then decisions
    const size_t wim = learn_weight_image_elems();
    size_t need = Arena::bytes_for(wim, 2) + Arena::bytes_for(208, 4) + Arena::bytes_for((size_t)nc, sizeof(LeafStats)) +
                  Arena::bytes_for((size_t)tot[0] + 1, 1) + Arena::bytes_for((size_t)tot[2] + 1, 1) +
                  Arena::bytes_for((size_t)tot[1] + 1, 1) + 3 * Arena::bytes_for((size_t)t.nsets, 4) + 512;
    const size_t cap0 = ws.lr_arena.capacity();
    T2D_CUDA_TRY(ws.lr_arena.reserve(need));
    if (ws.lr_arena.capacity() != cap0) ws.lr_version = -1;  // reallocated: weights must be uploaded again
    ws.lr_arena.reset();
    uint16_t *wimg = ws.lr_arena.take<uint16_t>(wim);
    float *bias = ws.lr_arena.take<float>(208);
    LeafStats *stats = ws.lr_arena.take<LeafStats>((size_t)nc);
    u_dec = ws.lr_arena.take<unsigned char>((size_t)tot[0] + 1);
    k_dec = ws.lr_arena.take<unsigned char>((size_t)tot[2] + 1);
    w_dec = mp.lp->far_orders ? ws.lr_arena.take<unsigned char>((size_t)tot[1] + 1) : nullptr;
    float *uref = ws.lr_arena.take<float>((size_t)t.nsets);  // one per set
    int *set_lo = t.nsets > 1 ? ws.lr_arena.take<int>((size_t)t.nsets) : nullptr;
    int *set_hi = t.nsets > 1 ? ws.lr_arena.take<int>((size_t)t.nsets) : nullptr;
    if (learned && ws.lr_version != mp.lp_version) {
      std::vector<uint16_t> img;
      std::vector<float> b;
      learn_weight_images(mp.lp->theta, img, b);
      T2D_CUDA_TRY(cudaMemcpy(wimg, img.data(), img.size() * 2, cudaMemcpyHostToDevice));
      T2D_CUDA_TRY(cudaMemcpy(bias, b.data(), b.size() * 4, cudaMemcpyHostToDevice));
      ws.lr_version = mp.lp_version;
    }
    cudaStream_t s2 = ws.side;
    T2D_CUDA_TRY(cudaEventRecord(ws.fork_ev, s));
    T2D_CUDA_TRY(cudaStreamWaitEvent(s2, ws.fork_ev, 0));
    forked = true;
    rc = learned_leaf_stats(m, stats, s2);
    if (rc) return drain(rc);
    rc = t.nsets > 1 ? learned_uref_sets(m, stats, t.root, t.nsets, set_lo, set_hi, uref, s2)
                     : learned_uref(m, stats, t.root, uref, s2);
    if (rc) return drain(rc);
    if (learned) {
      rc = learned_decide(m, stats, uref, wimg, bias, mp.lp->direct_bias, tot[0], tot[2], tot[1], u_dec, k_dec,
                          w_dec, s2);
      if (rc) return drain(rc);
    }
    T2D_TRY_DRAIN(schedule(s2));
    T2D_TRY_DRAIN(cudaEventRecord(ws.join_ev, s2));
  } else {
    T2D_CUDA_TRY(cudaEventRecord(ws.fork_ev, s));
    T2D_CUDA_TRY(cudaStreamWaitEvent(ws.side, ws.fork_ev, 0));
    forked = true;
    T2D_TRY_DRAIN(schedule(ws.side));
    T2D_TRY_DRAIN(cudaEventRecord(ws.join_ev, ws.side));
  }
  // Beside the decisions, the expansions run on the highest-priority
  // stream: their chain of short per-level kernels is the critical path,
  // and the inference CTAs (low priority, a few tiles each) fill the SMs
  // around it instead of holding them.
  cudaStream_t su = s;
  if (side) {
    T2D_TRY_DRAIN(cudaEventRecord(ws.hi_fork, s));
    T2D_TRY_DRAIN(cudaStreamWaitEvent(ws.hi, ws.hi_fork, 0));
    su = ws.hi;
  }
  rc = mixed_upward(m, t.depth, ws.h_levels, su, mp.level_chain != 0);
  if (rc) return drain(rc);
  T2D_TRY_DRAIN(cudaMemsetAsync(m.L, 0, sizeof(float) * (size_t)nc * 2 * P, su));
  rc = tc ? m2l_tc_tuned(ws, mp, m, dimg, cls_list, cls_count, su, st) : m2l_cuda_cores(m, dm2l, su);
  if (rc) return drain(rc);
  st.m2l_path = tc ? 2 : 1;
  rc = mixed_downward(m, t.depth, ws.h_levels, su, mp.level_chain != 0);
  if (rc) return drain(rc);
  if (side) {
    T2D_TRY_DRAIN(cudaEventRecord(ws.hi_join, ws.hi));
    T2D_TRY_DRAIN(cudaStreamWaitEvent(s, ws.hi_join, 0));
  }
  T2D_TRY_DRAIN(cudaStreamWaitEvent(s, ws.join_ev, 0));
  T2D_CUDA_TRY(cudaEventRecord(ws.ev[4], s));
  const Decisions dec = learned ? Decisions{u_dec, k_dec, mp.lp->order_margin, w_dec}
                                : Decisions{nullptr, nullptr, 0, nullptr};
  rc = near_field(ws, mp, m, learned, dec, d_uv, m.mperm, s, st);
  if (rc) return rc;
  T2D_CUDA_TRY(cudaEventRecord(ws.ev[5], s));
#undef T2D_TRY_DRAIN
  return TREE2D_OK;
}

}  // namespace t2d
