// Internal interfaces shared by the translation units of libtree2d_gb300.so.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <cstddef>
#include <cstdint>
#include <map>
#include <string>

#include "../../include/tree2d.h"

namespace t2d {

// Key depth: 2 bits per level in a 64-bit key.  A cell holding >= num_p
// blobs at this level cannot be split further (TREE2D_ERR_TOO_DEEP).
constexpr int kKeyLevels = 32;
// Keys are first formed to this depth (fewer FP64 steps and radix passes);
// the build falls back to kKeyLevels when a cell at this depth still holds
// >= num_p blobs.  The tree is the same either way.
constexpr int kShortKeyLevels = 20;
// Largest number of stored coefficients (nterms) the kernels support.
constexpr int kMaxTerms = 32;

struct Params {
  int nterms = 0;   // stored coefficients; M2S uses nterms-1 of them
  int num_p = 0;    // a cell with >= num_p blobs is split
  double theta = 0;
  double r_min = 0; // read and kept, unused (as in the reference)
};

struct LearnedParams;
struct MixedView;
struct LeafStats;

// Parameters of the mixed-precision form.
struct MixedParams {
  int pterms = 16;        // expansion length P (terms 0..P-1) of multipole and local
  double cutoff = 2.5;    // regularisation correction radius, in units of max sigma
  int use_tensor_cores = 1;
  int learned = 0;        // TREE2D_MODE_LEARNED: near-field decisions by the network
  const LearnedParams *lp = nullptr;
  long lp_version = 0;
  int autotune = 1;       // time the near-field variants on a new size class
  int eval_variant = -1;  // >= 0: force this near-field variant
  int leaf_blobs = -1;    // most blobs per leaf of the mixed forms' tree: -1 by set size
                          // (mixed_leaf_blobs), 0 the parameters' num_p - 1, > 0 this
  int level_chain = 0;    // M2M / L2L level chains as one cooperative launch each (P = 16)
  int m2l_rows = 0;       // tensor-core M2L cells per CTA: 0 = the tuner's choice, 64 or 128 forced
};

// Most blobs per leaf of the tree the mixed forms build (the plain form keeps
// the parameters' num_p - 1, the reference's).  By set size (n_set blobs per
// set): a leaf's near field grows with its size while the per-leaf work (lists,
// decisions, expansions, M2L) shrinks, and in larger, denser sets more of each
// leaf's list is correction entries, so larger leaves pay: 96 below 2M
// blobs, 128 from 2M (measured on GB300: the 512-set batch of 2K-200K blobs
// per set takes 16.9 ms at 96 against 17.5 at 64 and 17.4 at 112; 1M
// Lamb-Oseen blobs 2.13 ms at 96 and 128 against 2.39 at 64).
inline int mixed_leaf_blobs(const MixedParams &mp, long n_set, int num_p) {
  if (mp.leaf_blobs > 0) return mp.leaf_blobs;
  if (mp.leaf_blobs == 0) return num_p - 1;
  return n_set < (2l << 20) ? 96 : 128;
}

// Root box, written on the device (quadtree.c:81-99 semantics).
struct RootBox {
  double cx, cy, region;
  double xmin, xmax, ymin, ymax;
};

// Device-side status and work counters.
struct DevStatus {
  int err;                 // TREE2D_ERR_* (first error wins via atomicCAS)
  int depth;               // deepest leaf level
  unsigned long long n_m2s;
  unsigned long long n_pairs;
  unsigned long long n_m2l;
  unsigned long long n_fallback;  // targets whose traversal stack overflowed
  int deeper;              // build: keys of kShortKeyLevels levels do not suffice
  int list_overflow;       // mixed: a leaf's lists did not fit the one-walk scratch
  int list_max;            // mixed: most list entries (U + W + K) of one leaf
  unsigned long long k_blobs;  // mixed: source blobs of the K leaves of all leaves, out to the walk radius
  unsigned long long n_pairs_k;   // mixed: correction pairs evaluated (part of n_pairs)
  unsigned long long n_pairs_k_listed;  // mixed: correction pairs of the K entries evaluated, before the chunk cull
  unsigned eval_next;      // mixed: next target leaf of the persistent near-field warps
  unsigned bar_count;      // mixed: arrivals at the level chain's grid barrier (zeroed before a launch)
  unsigned bar_gen;        // mixed: generation of that barrier
  int nonuniform;          // mixed: some leaf's blobs have different core radii
};

// Bump allocator over one device allocation.  Buffers are 256-byte aligned.
class Arena {
 public:
  ~Arena();
  // Makes sure `bytes` are available from the start; keeps the contents
  // only if no reallocation was needed.  An arena attached to caller-owned
  // memory never allocates: it fails with cudaErrorMemoryAllocation instead.
  cudaError_t reserve(size_t bytes);
  // Uses [base, base+cap) as the arena's memory (owned by the caller).
  void attach(void *base, size_t cap) {
    base_ = static_cast<char *>(base);
    cap_ = cap;
    used_ = 0;
    fixed_ = true;
  }
  // True once reserve() was refused on attached memory.
  bool overflowed() const { return overflowed_; }
  void reset() { used_ = 0; }
  template <class T>
  T *take(size_t count) {
    size_t bytes = (count * sizeof(T) + 255) & ~size_t(255);
    if (used_ + bytes > cap_) return nullptr;
    T *p = reinterpret_cast<T *>(base_ + used_);
    used_ += bytes;
    return p;
  }
  size_t used() const { return used_; }
  size_t capacity() const { return cap_; }
  static size_t bytes_for(size_t count, size_t elem) { return (count * elem + 255) & ~size_t(255); }

 private:
  char *base_ = nullptr;
  size_t cap_ = 0, used_ = 0;
  bool fixed_ = false;
  bool overflowed_ = false;
};

// A tree on the device.  Blobs are stored in tree order (leaves in
// depth-first quadrant order, ascending original index inside a leaf);
// cells in depth-first pre-order with the root at 0.
struct Tree {
  int n = 0, ncell = 0, nleaf = 0, depth = 0, nterms = 0;
  double *x = nullptr, *y = nullptr, *cir = nullptr, *cor = nullptr;
  double *icor2 = nullptr;    // 1 / cor^2 per blob (tree order)
  int *perm = nullptr;        // tree position -> original blob index
  int *level = nullptr, *begin = nullptr, *end = nullptr;
  int *child = nullptr;       // 4 per cell, quadrant order, -1 = no blob there
  unsigned char *leaf = nullptr;
  double *cx = nullptr, *cy = nullptr, *region = nullptr;
  int *leaf_cell = nullptr;   // leaf ordinal -> cell id
  int *level_start = nullptr; // host-built cell lists per level (device copy)
  int *by_level = nullptr;    // cell ids grouped by level
  double2 *coef = nullptr;    // ncell * nterms, FP64 Laurent coefficients
  double2 *mac = nullptr;     // plain: per cell, the squared distances below / above which
                              // the opening test surely descends / accepts (k_mac_bounds)
  float4 *cf32 = nullptr;     // plain: per cell, the centre as FP32 pairs (cx hi, cx lo, cy hi, cy lo)
  float2 *macf = nullptr;     // plain: mac rounded outwards to FP32 (-1 / +inf where that is unsafe)
  RootBox *root = nullptr;    // device
  uint64_t *keys = nullptr;   // sorted keys (tree order before in-leaf sort)
  uint8_t *cpl = nullptr;     // per position: levels shared with the next key
  uint8_t *leaf_level = nullptr;  // per position: level of its leaf
  unsigned *cellbase = nullptr;   // per position: id of the first cell it starts
  int key_levels = 0;             // digits in the keys (kShortKeyLevels or kKeyLevels)
  int nsets = 1;                  // blob sets in the tree (batched solve: > 1)
  const int *set_off = nullptr;   // batched: device offsets of the sets (nsets + 1)
  const double *set_cor = nullptr;  // batched: core radii in input order (valid during the solve)
  int lev0 = 0;                   // batched: levels of container cells above the set roots
  int leaf_cap = 0;               // most blobs a leaf can hold (num_p - 1 of the build)
  const uint32_t *key_order = nullptr;  // blob indices in key order (build scratch in the tmp
                                        // arena: valid until that arena is next used)
};

// Per-solver working state (one per library instance).
struct Workspace {
  Arena blob_arena;   // N-sized buffers
  Arena cell_arena;   // cell-sized buffers
  Arena tmp_arena;    // scratch (sort buffers, scans)
  Arena mx_arena;     // mixed form: per-cell and per-position arrays
  Arena mx_lists;     // mixed form: interaction lists
  std::map<int, Arena> mx_tables;  // mixed form: translation operators, per expansion length P
                                   // (made once each: switching P between solves rebuilds nothing)
  Arena lr_arena;     // learned form: weights, leaf statistics, decisions
  long lr_version = -1;
  MixedView *mxv = nullptr;  // the last mixed solve's view (kept for sampling)
  long mx_tot[3] = {0, 0, 0};  // U, W, K list entries of that solve
  std::map<uint64_t, int> eval_tuned;  // size class -> fastest near-field variant
  std::map<uint64_t, int> m2l_tuned;   // size class -> faster M2L tile rows (64 or 128)
  int last_depth = 0;  // depth of the last tree built (sizes the next keys)
  double mac_theta = -1.0;  // theta that the tree's Tree::mac bounds were formed for (< 0: none)
  int list_cap = 256;  // entries per leaf of the one-walk list scratch (from the last solve)
  DevStatus *status = nullptr;   // device
  DevStatus *h_status = nullptr; // pinned host mirror
  int *h_levels = nullptr;        // pinned: the mixed form's per-level cell offsets (kKeyLevels + 2)
  cudaEvent_t ev[8] = {};
  cudaStream_t side = nullptr;    // second stream (learned decisions beside the expansions)
  cudaEvent_t fork_ev = nullptr, join_ev = nullptr;
  cudaStream_t hi = nullptr;      // highest-priority stream: the expansions while the decisions run
  cudaEvent_t hi_fork = nullptr, hi_join = nullptr;
  bool init = false;
};

cudaError_t workspace_init(Workspace &ws);

// --- tree build (build_tree.cu) --------------------------------------
// Builds the tree over n blobs (xy interleaved, device).  Synchronises the
// stream once to size the cell arrays.  Returns a TREE2D status.
// Batched (nsets > 1): the blobs are nsets independent sets, set k at
// [d_set_off[k], d_set_off[k+1]) (device offsets); each set gets its own root
// box and exactly the cells it would get alone, below lev0 levels of
// container cells that keep the sets apart (t.lev0, t.root[k] per set).
// `cir_cor_ready`, when given, is an event the stream waits for before the
// circulations and core radii are first read (the positions must be ready
// when the call is made); the caller may still be uploading them.
int build_tree(Workspace &ws, int n, const double *d_xy, const double *d_cir, const double *d_cor,
               const Params &p, Tree &t, cudaStream_t s, const int *d_set_off = nullptr, int nsets = 1,
               cudaEvent_t cir_cor_ready = nullptr);
// Bytes build_tree reserves in ws.blob_arena and ws.tmp_arena for n blobs in
// nsets sets (what a caller with fixed arenas must provide).
size_t build_blob_bytes(int n, int nsets);
size_t build_tmp_bytes(int n, int nsets);
// Bytes build_tree reserves in ws.cell_arena for a tree of ncell cells and
// nleaf leaves with nterms coefficients per cell.
size_t build_cell_bytes(long long ncell, long long nleaf, int nterms);

// Keys of arbitrary points against an existing root box, then sorted:
// order[i] = index of the i-th target in key order.
int sort_targets(Workspace &ws, int n, const double *d_xy, const RootBox *d_root, int *d_order,
                 cudaStream_t s);

// Targets in evaluation order: tx/ty[i] = xy[order[i]], out_idx[i] = order[i]
// (order == nullptr: identity).
int gather_targets(int n, const double *d_xy, const int *d_order, double *tx, double *ty, int *out_idx,
                   cudaStream_t s);

// --- radix sort (sort.cu) --------------------------------------------
// Stable LSD radix sort of (key, value) pairs on bits [begin_bit, end_bit)
// (the other bits must be equal in all keys or irrelevant to the order).
// Buffers *_alt are scratch of the same size.  The result ends in keys/vals.
size_t radix_sort_temp_bytes(int n);
// The same sort of packed words (key in the high 32 bits, value in the low
// 32) on bits [begin_bit, 64), begin_bit >= 32, n >= 2: 8 bytes per element
// and pass instead of 12.  The passes alternate between words and words_alt
// (their contents are scratch afterwards); the last pass writes the keys
// (low half cleared) to keys_out and the values to vals_out.  The last pass
// reads words when the pass count ceil((64 - begin_bit) / 8) is odd and
// words_alt when it is even: keys_out may be the other one.  With st, each
// pass is a single kernel (decoupled look-back; a look-back that times out
// records TREE2D_ERR_TIMEOUT in st); without, the reduce-then-scan form.
cudaError_t radix_sort_packed(uint64_t *words, uint64_t *words_alt, int n, int begin_bit, uint64_t *keys_out,
                              uint32_t *vals_out, void *temp, DevStatus *st, cudaStream_t s);
cudaError_t radix_sort_pairs(uint64_t *keys, uint32_t *vals, uint64_t *keys_alt, uint32_t *vals_alt,
                             int n, int begin_bit, int end_bit, void *temp, cudaStream_t s);

// --- plain FP64 path (plain.cu) ---------------------------------------
int plain_upward(Workspace &ws, const Tree &t, const Params &p, cudaStream_t s);
// Evaluates targets (tx,ty) in the given order, writing uv[2*out_idx[i]].
int plain_evaluate(Workspace &ws, const Tree &t, const Params &p, int ntgt, const double *tx,
                   const double *ty, const int *out_idx, double *uv, cudaStream_t s);

// --- direct sum (direct.cu) -------------------------------------------
cudaError_t direct_sum(int ntgt, const double *txy, int nsrc, const double *sxy, const double *cir,
                       const double *cor, double *uv, cudaStream_t s);

// FP64 pipe probe: blocks x 256 threads x iters x 8 FMAs (2 flops each).
cudaError_t dfma_probe(double *out, int blocks, int iters, cudaStream_t s);
cudaError_t ffma_probe(float *out, int blocks, int iters, cudaStream_t s);
cudaError_t wait_probe(long polls, int *out, cudaStream_t s);
cudaError_t advect(long n, double *xy, const double *uv, double dt, cudaStream_t s);
// Query points [b, e) (xy interleaved, 16-byte aligned, as all the arrays
// here) looked up at the nb blob positions bxy: out[i] = buv[i] where query i
// is bitwise at blob i, else NaN and i appended to miss (count in *nmiss).
cudaError_t lookup_blobs(long b, long e, const double *q, long nb, const double *bxy, const double *buv, double *out,
                         int *miss, int *nmiss, cudaStream_t s);
// Blobs followed by their images in a wall at y = d (2n entries out).
cudaError_t mirror_images(long n, const double *xy, const double *cir, const double *cor, double d, double *oxy,
                          double *ocir, double *ocor, cudaStream_t s);

// Parameters for a device solve, resolved under the library lock; `mode`
// and `mirror` (when not null) receive the mode in force and whether a
// mirror wall is set.
int params_for_device_solve(Params &out, int *mode = nullptr, bool *mirror = nullptr);
// Stores `code` as the library's last error and returns it.
int record_error(int code);

// Kernels launched by this library (for the launch count in the stats).
extern std::atomic<long long> g_launches;

// error text of the last CUDA failure (for tree2d_error_string)
void note_cuda_error(cudaError_t e, const char *what);
// replaces that text (a failure that is not a CUDA error left it stale)
void note_error_text(const char *text);

}  // namespace t2d
