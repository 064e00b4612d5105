// Mixed-precision FMM: device view and host entry points (mixed.cu, m2l.cu).
#pragma once

#include <vector>

#include "internal.h"

namespace t2d {

constexpr int kMaxP = 32;  // largest expansion length of the mixed form

// Everything the mixed kernels read or write, by value into each kernel.
// Blobs per chunk of a leaf for the near field's correction cull: each
// chunk has a bounding box, and a correction leaf's chunks farther than the
// correction radius from a pack of targets are skipped.
constexpr int kChunkShift = 4;
constexpr int kChunk = 1 << kChunkShift;

struct MixedView {
  int n, ncell, nleaf, P;
  const float *rc_ptr;  // device: cutoff radius of the regularisation correction
  const float *rc_set;  // batched sets: cutoff radius per set (else null)
  float walk_scale;     // correction walk radius / rc (>= 1): the counting walks also count
                        // the leaves between rc and walk_scale * rc (their blobs, into st->k_blobs)
  int lev0;             // batched sets: levels of container cells above the set roots
  // from the tree
  const uint64_t *keys;
  const uint8_t *cpl, *leaf_level;
  const unsigned *cellbase;
  const int *level, *begin, *end, *child, *leaf_cell;
  const unsigned char *leaf;
  const double *cx, *cy, *region;
  // mixed arrays
  unsigned *ix, *iy;
  float *h, *inv_h;
  int *parent;
  int *leaf_of;          // per position
  float2 *loc;           // per position, offset from its leaf centre
  float *gam;            // per position: circulation
  float4 *src4;          // per position {loc.x, loc.y, G, -log2(e)/sigma^2}
  float4 *src4s;         // per position of a leaf with one core radius: {loc.x s, loc.y s, G s, 0},
                         // s = sqrt(log2 e) / sigma (the near field's scaled records)
  float *lscale;         // per leaf cell: that s, 0 where its blobs' core radii differ
  int *mperm;            // per position: original blob index.  The per-position arrays of the
                         // mixed form hold each leaf's blobs by sub-cell (8 x 8 sub-cells in
                         // Morton order, tree order inside one), not in the tree's order
  float4 *cbox;          // per leaf cell, kchunks entries: bounding box {xmin, ymin, xmax, ymax}
                         // of each kChunk-blob chunk of the leaf (from its first blob), leaf-local
  int kchunks;           // chunk boxes per cell: ceil(most blobs per leaf / 32)
  float *cxf, *cyf;      // per cell, FP32 centre (rounded)
  float *cxl, *cyl;      // per cell, the rest: centre - (double)cxf, in FP32
  int *coll, *coarse;    // 9 per cell
  int *vlist;            // 27 per cell, slot order of the cell's class
  int *xlist;            // 8 per cell
  int *u_off, *w_off, *k_off;  // per leaf (+1)
  int *scan_tmp;               // tile sums of the list-size scan
  int *by_level;               // cell ids grouped by level (order within a level arbitrary)
  int *list_scratch;           // one-walk list build: list_cap entries per leaf (or null)
  int list_cap;
  int *level_off;              // [kKeyLevels + 2]: start of each level in by_level, then cursors
  int *u_idx, *w_idx, *k_idx;
  int *u_leaf, *w_leaf, *k_leaf;  // leaf ordinal of each U / W / K entry
  const int *leaf_order; // near-field schedule: leaf ordinals by estimated work, largest first
  float *M, *L;          // per cell, 2P floats (re[P], im[P])
  const float2 *m2m, *l2l;  // [4][kMaxP][kMaxP] translation operators
  DevStatus *st;
};

// Offset hi[b]+lo[b] - (hi[a]+lo[a]) of two cell centres in FP32, from the
// two-float form of each centre (hi = the centre rounded to FP32, lo = the
// rest, exact to ~2^-48 of the centre).  The hi difference is exact when the
// two are within a factor of two of each other (Sterbenz), as neighbouring
// cells away from the axes are, and otherwise rounded at the scale of the
// difference; the lo difference is exact to far below that.  The result is
// within about an ulp of the FP64 difference rounded to FP32, with no FP64
// arithmetic.  Without the lo parts an offset would carry up to half an
// ulp of the coordinate (~3e-8 at 0.5), too much for pairs 1e-3 apart.
__device__ __forceinline__ float centre_offset(const float *hi, const float *lo, int b, int a) {
  return __fadd_rn(__fsub_rn(hi[b], hi[a]), __fsub_rn(lo[b], lo[a]));
}

cudaError_t mixed_tables(int P, float *h_m2l, float *h_m2m, float *h_l2l);
int mixed_leaf_setup(MixedView &m, const Tree &t, cudaStream_t s);
int mixed_lists(MixedView &m, cudaStream_t s);
int mixed_fill_lists(MixedView &m, bool from_scratch, cudaStream_t s);
// lev_off: the per-level cell offsets on the host (level_off's first
// kKeyLevels + 2 entries), to size each level's grid; null = full grids.
// chain: run the P = 16 M2M (L2L) levels as one cooperative launch of
// persistent blocks where the device allows it, else one launch per level.
int mixed_upward(MixedView &m, int depth, const int *lev_off, cudaStream_t s, bool chain);
int mixed_downward(MixedView &m, int depth, const int *lev_off, cudaStream_t s, bool chain);

// M2L over the V lists (m2l.cu): L[c] += sum_s T(class(c), s) M[V[c][s]].
// `tables` is the device copy of the [4][27][P][P] complex operators.
int m2l_cuda_cores(MixedView &m, const float *tables, cudaStream_t s);
// Tensor-core form: needs P % 4 == 0.  `bimg` are the B operator images
// (m2l_b_images), cls_list/cls_count scratch of 4*ncell and 4 ints.
// rows: cells per CTA, 128 or 64 (bit-identical results)
int m2l_tensor_cores(MixedView &m, const float *bimg, int *cls_list, int *cls_count, int rows, cudaStream_t s);
int m2l_npad(int P);
void m2l_b_images(int P, const float *h_m2l, std::vector<float> &img);

// Whole mixed solve on a built tree: lists, upward, M2L, downward,
// evaluation; uv written in original blob order.  Synchronises the stream
// once (to size the interaction lists).
// Near-field kernel variants the tuner times (tree2d_set_tuning forces one).
constexpr int kEvalVariantCount = TREE2D_EVAL_VARIANTS;

int mixed_solve(Workspace &ws, const Tree &t, const MixedParams &mp, double *d_uv, cudaStream_t s,
                tree2d_stats_t &st);

// Velocity at ntgt arbitrary points (tx, ty, FP64, device; in key order for
// warp coherence) against the last mixed solve of `ws` (its view, lists and
// expansions must be intact): uv[2 * out_idx[i]] (out_idx may be null).  A
// per-point traversal that accepts a cell's multipole only far from the
// point (2.5 cell sides, beyond the correction radius) and sums the rest
// pair by pair, for points that are not blob positions.
int mixed_eval_points(Workspace &ws, int ntgt, const double *tx, const double *ty, const int *out_idx, double *uv,
                      cudaStream_t s);

}  // namespace t2d
