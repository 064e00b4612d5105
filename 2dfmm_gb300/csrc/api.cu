// C ABI of libtree2d_gb300.so: the reference's make_tree / biot_tree
// (ver-c/src/quadtree.c:102-171, ver-c/src/fmm.c:69-118) plus extensions.
//
// State is library-global, as in the reference (quadtree.c:9-10 keeps
// `qtree` and `vors` global): make_tree replaces the tree, biot_tree reads
// it.  make_tree runs the whole pipeline on the GPU and evaluates the
// velocity at every blob position, because the reference's callers ask for
// exactly those points one call at a time (e_velo_mpi.f90:37-48): a GPU
// launch per call would be latency bound.  biot_tree answers blob positions
// from that table (matched bit for bit on x and y) and evaluates any other
// point on the GPU with the same kernel.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "dev_common.cuh"
#include "learn.h"
#include "mixed.h"

namespace t2d {

Arena::~Arena() {
  // Device memory is released at process exit; freeing here could run after
  // the CUDA runtime has been torn down.
}

cudaError_t Arena::reserve(size_t bytes) {
  if (bytes <= cap_) return cudaSuccess;
  if (fixed_) {
    overflowed_ = true;
    return cudaErrorMemoryAllocation;
  }
  if (base_) cudaFree(base_);
  base_ = nullptr;
  cap_ = 0;
  used_ = 0;
  size_t want = bytes + bytes / 8 + 4096;
  cudaError_t e = cudaMalloc(reinterpret_cast<void **>(&base_), want);
  if (e == cudaSuccess) cap_ = want;
  return e;
}

cudaError_t workspace_init(Workspace &ws) {
  if (ws.init) return cudaSuccess;
  cudaError_t e = cudaMalloc(reinterpret_cast<void **>(&ws.status), sizeof(DevStatus));
  if (e != cudaSuccess) return e;
  e = cudaMallocHost(reinterpret_cast<void **>(&ws.h_status), 4096);
  if (e != cudaSuccess) return e;
  e = cudaMallocHost(reinterpret_cast<void **>(&ws.h_levels), sizeof(int) * (kKeyLevels + 2));
  if (e != cudaSuccess) return e;
  for (auto &ev : ws.ev) {
    e = cudaEventCreate(&ev);
    if (e != cudaSuccess) return e;
  }
  e = cudaStreamCreateWithFlags(&ws.side, cudaStreamNonBlocking);
  if (e != cudaSuccess) return e;
  e = cudaEventCreateWithFlags(&ws.fork_ev, cudaEventDisableTiming);
  if (e != cudaSuccess) return e;
  e = cudaEventCreateWithFlags(&ws.join_ev, cudaEventDisableTiming);
  if (e != cudaSuccess) return e;
  int least = 0, greatest = 0;
  e = cudaDeviceGetStreamPriorityRange(&least, &greatest);
  if (e != cudaSuccess) return e;
  e = cudaStreamCreateWithPriority(&ws.hi, cudaStreamNonBlocking, greatest);
  if (e != cudaSuccess) return e;
  e = cudaEventCreateWithFlags(&ws.hi_fork, cudaEventDisableTiming);
  if (e != cudaSuccess) return e;
  e = cudaEventCreateWithFlags(&ws.hi_join, cudaEventDisableTiming);
  if (e != cudaSuccess) return e;
  ws.init = true;
  return cudaSuccess;
}

std::atomic<long long> g_launches{0};

static std::mutex g_msg_mu;
static std::string g_cuda_msg;

void note_cuda_error(cudaError_t e, const char *what) {
  std::lock_guard<std::mutex> lk(g_msg_mu);
  g_cuda_msg = std::string(cudaGetErrorString(e)) + " (" + what + ")";
}

namespace {

// Page-locked host array (grown, never shrunk), so that the device->host
// copy of the velocity table runs at full link speed.
struct PinnedTable {
  double *p = nullptr;
  size_t cap = 0;
  cudaError_t ensure(size_t elems) {
    if (elems <= cap) return cudaSuccess;
    if (p) cudaFreeHost(p);
    p = nullptr;
    cap = 0;
    cudaError_t e = cudaMallocHost(reinterpret_cast<void **>(&p), sizeof(double) * elems);
    if (e == cudaSuccess) cap = elems;
    return e;
  }
  double operator[](size_t i) const { return p[i]; }
};

// Runs f(begin, end) over [0, n) on up to hardware_concurrency() threads,
// chunks of at least `grain` items; the calling thread takes the first.
template <class F>
void parallel_chunks(long n, long grain, F f) {
  const long hw = std::max(1u, std::thread::hardware_concurrency());
  const long nt = std::min(hw, (n + grain - 1) / grain);
  if (nt <= 1) {
    if (n > 0) f(0L, n);
    return;
  }
  const long per = (n + nt - 1) / nt;
  std::vector<std::thread> th;
  for (long t = 1; t < nt; t++) {
    const long b = t * per, e = std::min(n, b + per);
    if (b < e) th.emplace_back(f, b, e);
  }
  f(0L, std::min(n, per));
  for (auto &x : th) x.join();
}

struct Solver {
  Workspace ws;
  Arena sets;     // device copy of the set offsets of a batched solve
  Tree tree;
  Arena mirror;   // blobs + images when a mirror wall is set
  bool plain_coef = false;  // FP64 coefficients present (plain upward ran)
  bool mixed_ready = false; // the last solve was a mixed/learned one: its view, lists and
                            // expansions are intact (off-blob points use them)
  Arena io;       // device copies of host inputs and outputs
  Arena targets;  // evaluation-order targets
  Arena lookup;   // query points and answers of a batch lookup
  Arena keyed;    // the blobs as targets in key order (plain evaluation)
};

struct Lib {
  std::mutex mu;
  Params params;
  bool have_params = false;
  bool params_fixed = false;
  int mode = TREE2D_MODE_PLAIN;
  MixedParams mixed;
  LearnedParams *lp = new LearnedParams();
  long lp_version = 0;
  bool mirror_on = false;
  double mirror_d = 0.0;
  std::atomic<int> last_error{0};
  cudaStream_t stream = nullptr;
  cudaStream_t copy_stream = nullptr;  // uploads and downloads beside the solve stream
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr, ev_inputs = nullptr;
  int *h_count = nullptr;              // pinned: miss count of a batch lookup
  bool stream_ready = false;
  Solver main, dev;
  // results of the last make_tree: positions and velocities on the device
  // (original order); host copies made on first need (single-point lookups,
  // batch queries the device lookup could not place)
  std::atomic<bool> valid{false};
  std::atomic<unsigned long long> generation{0};
  const double *d_xy = nullptr, *d_uv = nullptr;
  std::atomic<bool> host_ready{false};
  PinnedTable h_xy, h_uv;
  int n = 0;
  // position -> blob index, built on first need
  std::mutex hash_mu;
  std::atomic<bool> hash_ready{false};
  std::vector<int> hash_slot;
  size_t hash_mask = 0;
  tree2d_stats_t stats{};
  tree2d_stats_t dev_stats{};
  bool last_was_dev = false;
};

Lib &lib() {
  static Lib *l = new Lib();  // never destroyed (see Arena::~Arena)
  return *l;
}

int fail(int code) {
  lib().last_error.store(code);
  return code;
}

int ensure_stream(Lib &L) {
  if (L.stream_ready) return TREE2D_OK;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return TREE2D_ERR_NO_DEVICE;
  T2D_CUDA_TRY(cudaStreamCreateWithFlags(&L.stream, cudaStreamNonBlocking));
  T2D_CUDA_TRY(cudaStreamCreateWithFlags(&L.copy_stream, cudaStreamNonBlocking));
  for (cudaEvent_t *e : {&L.ev_fork, &L.ev_join, &L.ev_inputs})
    T2D_CUDA_TRY(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
  T2D_CUDA_TRY(cudaMallocHost(reinterpret_cast<void **>(&L.h_count), sizeof(int)));
  L.stream_ready = true;
  return TREE2D_OK;
}

// ../cal_cond/fmm_param.dat, read as quadtree.c:12-27 reads it.
bool read_param_file(Params &p) {
  FILE *f = std::fopen("../cal_cond/fmm_param.dat", "r");
  if (!f) {
    std::printf("Error: Could not read FMM parameters.");
    std::fflush(stdout);
    return false;
  }
  if (std::fscanf(f, "%i    nterms", &p.nterms) < 0) { /* as the reference: ignored */ }
  if (std::fscanf(f, "%i   num_p", &p.num_p) < 0) { /* ignored */ }
  if (std::fscanf(f, "%lf theta", &p.theta) < 0) { /* ignored */ }
  if (std::fscanf(f, "%lf  r_min ! for Tree", &p.r_min) < 0) { /* ignored */ }
  std::fclose(f);
  return true;
}

int check_params(const Params &p) {
  if (p.nterms < 0 || p.nterms > kMaxTerms) return TREE2D_ERR_BAD_PARAMS;
  if (p.num_p < 2 || p.num_p > 65536) return TREE2D_ERR_BAD_PARAMS;
  if (!std::isfinite(p.theta)) return TREE2D_ERR_BAD_PARAMS;
  return TREE2D_OK;
}

// Parameters in force for the next solve: the fixed ones, else the file
// (when the file cannot be read, the previous values stay in force, as the
// reference's globals do).
int resolve_params(Lib &L) {
  if (!L.params_fixed) {
    Params p = L.params;
    if (read_param_file(p)) {
      L.params = p;
      L.have_params = true;
    }
  }
  if (!L.have_params) return TREE2D_ERR_PARAM_FILE;
  return check_params(L.params);
}

float elapsed(cudaEvent_t a, cudaEvent_t b) {
  float ms = 0.f;
  cudaEventElapsedTime(&ms, a, b);
  return ms;
}

int solve_body(Lib &L, Solver &S, int n, const double *d_xy, const double *d_cir, const double *d_cor,
               double *d_uv, cudaStream_t s, tree2d_stats_t &st, const int *d_set_off = nullptr, int nsets = 1,
               cudaEvent_t cir_cor_ready = nullptr);

// Whole pipeline over n device-resident blobs; uv (interleaved, original
// order) on the device.  With a mirror wall the images are appended as
// blobs n..2n-1 and only the first n velocities are returned.
// `cir_cor_ready`: an event to wait for before the circulations and core
// radii are read (they may still be on their way to the device).
int solve(Lib &L, Solver &S, int n, const double *d_xy, const double *d_cir, const double *d_cor, double *d_uv,
          cudaStream_t s, tree2d_stats_t &st, cudaEvent_t cir_cor_ready = nullptr) {
  if (!L.mirror_on || n == 0)
    return solve_body(L, S, n, d_xy, d_cir, d_cor, d_uv, s, st, nullptr, 1, cir_cor_ready);
  if (cir_cor_ready) T2D_CUDA_TRY(cudaStreamWaitEvent(s, cir_cor_ready, 0));
  const size_t n2 = 2 * (size_t)n;
  T2D_CUDA_TRY(S.mirror.reserve(Arena::bytes_for(2 * n2, 8) * 2 + Arena::bytes_for(n2, 8) * 2));
  S.mirror.reset();
  double *mxy = S.mirror.take<double>(2 * n2);
  double *muv = S.mirror.take<double>(2 * n2);
  double *mcir = S.mirror.take<double>(n2);
  double *mcor = S.mirror.take<double>(n2);
  T2D_CUDA_TRY(mirror_images(n, d_xy, d_cir, d_cor, L.mirror_d, mxy, mcir, mcor, s));
  int rc = solve_body(L, S, (int)n2, mxy, mcir, mcor, muv, s, st);
  if (rc) return rc;
  T2D_CUDA_TRY(cudaMemcpyAsync(d_uv, muv, sizeof(double) * 2 * (size_t)n, cudaMemcpyDeviceToDevice, s));
  T2D_CUDA_TRY(cudaStreamSynchronize(s));
  return TREE2D_OK;
}

int solve_body(Lib &L, Solver &S, int n, const double *d_xy, const double *d_cir, const double *d_cor,
               double *d_uv, cudaStream_t s, tree2d_stats_t &st, const int *d_set_off, int nsets,
               cudaEvent_t cir_cor_ready) {
  T2D_CUDA_TRY(workspace_init(S.ws));
  std::memset(&st, 0, sizeof(st));
  st.n_blobs = n;
  st.mode = L.mode;
  if (n == 0) {
    S.tree = Tree();
    return TREE2D_OK;
  }
  Workspace &ws = S.ws;
  const long long launches0 = g_launches.load();
  T2D_CUDA_TRY(cudaEventRecord(ws.ev[0], s));
  // the mixed forms build their own leaf size (the plain form the reference's)
  Params bp = L.params;
  if (L.mode != TREE2D_MODE_PLAIN) bp.num_p = mixed_leaf_blobs(L.mixed, n / (nsets > 0 ? nsets : 1), L.params.num_p) + 1;
  st.leaf_blobs = bp.num_p - 1;
  S.mixed_ready = false;
  int rc = build_tree(ws, n, d_xy, d_cir, d_cor, bp, S.tree, s, d_set_off, nsets, cir_cor_ready);
  if (rc) return rc;
  T2D_CUDA_TRY(cudaEventRecord(ws.ev[1], s));
  S.plain_coef = false;
  if (L.mode == TREE2D_MODE_PLAIN) {
    rc = plain_upward(ws, S.tree, L.params, s);
    if (rc) return rc;
    S.plain_coef = true;
    T2D_CUDA_TRY(cudaEventRecord(ws.ev[2], s));
    // The blobs as targets in full-key order, so that a warp's 32 targets
    // are neighbours (inside a leaf the tree order is the reference's index
    // order, spread over the whole leaf) and their traversals coincide.  A
    // target's result does not depend on its warp: each lane meets its own
    // cells in its own LIFO order.
    T2D_CUDA_TRY(S.keyed.reserve(Arena::bytes_for(n, 8) * 2 + Arena::bytes_for(n, 4)));
    S.keyed.reset();
    double *ktx = S.keyed.take<double>(n);
    double *kty = S.keyed.take<double>(n);
    int *kout = S.keyed.take<int>(n);
    rc = gather_targets(n, d_xy, reinterpret_cast<const int *>(S.tree.key_order), ktx, kty, kout, s);
    if (rc) return rc;
    rc = plain_evaluate(ws, S.tree, L.params, n, ktx, kty, kout, d_uv, s);
    if (rc) return rc;
  } else {
    T2D_CUDA_TRY(cudaEventRecord(ws.ev[2], s));
    MixedParams mp = L.mixed;
    mp.learned = L.mode == TREE2D_MODE_LEARNED;
    mp.lp = L.lp;
    mp.lp_version = L.lp_version;
    rc = mixed_solve(ws, S.tree, mp, d_uv, s, st);
    if (rc) return rc;
    S.mixed_ready = nsets <= 1;
  }
  T2D_CUDA_TRY(cudaEventRecord(ws.ev[3], s));
  T2D_CUDA_TRY(cudaMemcpyAsync(ws.h_status, ws.status, sizeof(DevStatus), cudaMemcpyDeviceToHost, s));
  T2D_CUDA_TRY(cudaStreamSynchronize(s));
  if (ws.h_status->err) return ws.h_status->err;
  const int m2l_path = st.m2l_path;
  st.n_cells = S.tree.ncell;
  st.n_leaves = S.tree.nleaf;
  st.depth = S.tree.depth;
  st.n_m2s = (long long)ws.h_status->n_m2s;
  st.n_pairs = (long long)ws.h_status->n_pairs;
  st.n_pairs_k = (long long)ws.h_status->n_pairs_k;
  st.n_pairs_k_listed = (long long)ws.h_status->n_pairs_k_listed;
  st.n_m2l = (long long)ws.h_status->n_m2l;
  st.ms_build = elapsed(ws.ev[0], ws.ev[1]);
  if (L.mode == TREE2D_MODE_PLAIN) {
    st.ms_upward = elapsed(ws.ev[1], ws.ev[2]);
    st.ms_eval = elapsed(ws.ev[2], ws.ev[3]);
  } else {
    // mixed: lists + upward + M2L + downward, then the evaluation kernel
    st.ms_upward = elapsed(ws.ev[1], ws.ev[4]);
    st.ms_eval = elapsed(ws.ev[4], ws.ev[5]);
  }
  st.ms_total = elapsed(ws.ev[0], ws.ev[3]);
  st.n_launches = g_launches.load() - launches0;
  st.m2l_path = m2l_path;
  return TREE2D_OK;
}

uint64_t mix64(uint64_t x) {
  x += 0x9e3779b97f4a7c15ull;
  x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
  x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
  return x ^ (x >> 31);
}

uint64_t pos_hash(double x, double y) {
  uint64_t a, b;
  std::memcpy(&a, &x, 8);
  std::memcpy(&b, &y, 8);
  return mix64(a ^ mix64(b));
}

bool same_bits(double a, double b) { return std::memcmp(&a, &b, 8) == 0; }

// Host copies of the last make_tree's positions and velocities (the
// single-point lookup's table), downloaded on first need.  L.mu held.
int ensure_host_tables(Lib &L) {
  if (L.host_ready.load(std::memory_order_acquire)) return TREE2D_OK;
  const size_t m = 2 * (size_t)L.n;
  if (m > 0) {
    T2D_CUDA_TRY(L.h_xy.ensure(m));
    T2D_CUDA_TRY(L.h_uv.ensure(m));
    T2D_CUDA_TRY(cudaMemcpyAsync(L.h_xy.p, L.d_xy, sizeof(double) * m, cudaMemcpyDeviceToHost, L.stream));
    T2D_CUDA_TRY(cudaMemcpyAsync(L.h_uv.p, L.d_uv, sizeof(double) * m, cudaMemcpyDeviceToHost, L.stream));
    T2D_CUDA_TRY(cudaStreamSynchronize(L.stream));
  }
  L.host_ready.store(true, std::memory_order_release);
  return TREE2D_OK;
}

void ensure_hash(Lib &L) {
  if (L.hash_ready.load(std::memory_order_acquire)) return;
  std::lock_guard<std::mutex> lk(L.hash_mu);
  if (L.hash_ready.load(std::memory_order_relaxed)) return;
  size_t cap = 16;
  while (cap < 2 * (size_t)L.n) cap <<= 1;
  L.hash_slot.assign(cap, 0);
  L.hash_mask = cap - 1;
  for (int i = 0; i < L.n; i++) {
    double x = L.h_xy[2 * (size_t)i], y = L.h_xy[2 * (size_t)i + 1];
    size_t h = pos_hash(x, y) & L.hash_mask;
    while (true) {
      int s = L.hash_slot[h];
      if (s == 0) {
        L.hash_slot[h] = i + 1;
        break;
      }
      if (same_bits(L.h_xy[2 * (size_t)(s - 1)], x) && same_bits(L.h_xy[2 * (size_t)(s - 1) + 1], y)) break;
      h = (h + 1) & L.hash_mask;
    }
  }
  L.hash_ready.store(true, std::memory_order_release);
}

// Index of a blob at exactly (x,y), or -1.  `hint` is the index found by
// the previous lookup of the caller: the blob after it (and then it) is
// tried first, so a sweep over the blobs in order costs one compare each.
long find_blob_from(Lib &L, double x, double y, long &hint) {
  const long n = L.n;
  for (long c : {hint + 1, hint}) {
    if (c >= 0 && c < n && same_bits(L.h_xy[2 * c], x) && same_bits(L.h_xy[2 * c + 1], y)) {
      hint = c;
      return c;
    }
  }
  ensure_hash(L);
  size_t h = pos_hash(x, y) & L.hash_mask;
  while (true) {
    int s = L.hash_slot[h];
    if (s == 0) return -1;
    if (same_bits(L.h_xy[2 * (size_t)(s - 1)], x) && same_bits(L.h_xy[2 * (size_t)(s - 1) + 1], y)) {
      hint = s - 1;
      return s - 1;
    }
    h = (h + 1) & L.hash_mask;
  }
}

// As find_blob_from, with the hint kept per calling thread (biot_tree).
long find_blob(Lib &L, double x, double y) {
  thread_local unsigned long long gen = ~0ull;
  thread_local long hint = -1;
  unsigned long long g = L.generation.load(std::memory_order_acquire);
  if (gen != g) {
    gen = g;
    hint = -1;
  }
  return find_blob_from(L, x, y, hint);
}

// GPU evaluation of m arbitrary points (host xy) into host uv; L.mu held.
int eval_points(Lib &L, int m, const double *xy, double *uv) {
  Solver &S = L.main;
  if (L.n == 0) {
    for (int i = 0; i < 2 * m; i++) uv[i] = 0.0;
    return TREE2D_OK;
  }
  cudaStream_t s = L.stream;
  size_t need = Arena::bytes_for(2 * (size_t)m, 8) * 2 + Arena::bytes_for(m, 8) * 2 + Arena::bytes_for(m, 4) * 2;
  T2D_CUDA_TRY(S.targets.reserve(need));
  S.targets.reset();
  double *d_xy = S.targets.take<double>(2 * (size_t)m);
  double *d_uv = S.targets.take<double>(2 * (size_t)m);
  double *tx = S.targets.take<double>(m);
  double *ty = S.targets.take<double>(m);
  int *order = S.targets.take<int>(m);
  int *out = S.targets.take<int>(m);
  T2D_CUDA_TRY(cudaMemcpyAsync(d_xy, xy, sizeof(double) * 2 * (size_t)m, cudaMemcpyHostToDevice, s));
  int rc;
  // Points off the blobs: after a plain make_tree the plain FP64 treecode
  // (the reference's method); after a mixed or learned one a traversal of
  // the mixed tree with its own expansions, to the mixed form's accuracy.
  const bool mixed = S.mixed_ready;
  if (!mixed && !S.plain_coef) {
    rc = plain_upward(S.ws, S.tree, L.params, s);
    if (rc) return rc;
    S.plain_coef = true;
  }
  if (m > 1024) {
    rc = sort_targets(S.ws, m, d_xy, S.tree.root, order, s);
    if (rc) return rc;
    rc = gather_targets(m, d_xy, order, tx, ty, out, s);
  } else {
    rc = gather_targets(m, d_xy, nullptr, tx, ty, out, s);
  }
  if (rc) return rc;
  T2D_CUDA_TRY(cudaMemsetAsync(S.ws.status, 0, sizeof(DevStatus), s));
  rc = mixed ? mixed_eval_points(S.ws, m, tx, ty, out, d_uv, s)
             : plain_evaluate(S.ws, S.tree, L.params, m, tx, ty, out, d_uv, s);
  if (rc) return rc;
  T2D_CUDA_TRY(cudaMemcpyAsync(uv, d_uv, sizeof(double) * 2 * (size_t)m, cudaMemcpyDeviceToHost, s));
  T2D_CUDA_TRY(cudaMemcpyAsync(S.ws.h_status, S.ws.status, sizeof(DevStatus), cudaMemcpyDeviceToHost, s));
  T2D_CUDA_TRY(cudaStreamSynchronize(s));
  return S.ws.h_status->err;
}

}  // namespace

// Batch lookup on the device: the queries go up in chunks on two streams
// (one chunk's upload overlaps the previous chunk's download), query i is
// matched against blob i, and the answers come back into uv.  Queries that
// do not sit bitwise on their blob are returned in `miss` (ascending), with
// NaN in uv.  L.mu held.
int lookup_on_device(Lib &L, int n, const double *xy, double *uv, std::vector<int> &miss) {
  miss.clear();
  if (L.n == 0) {
    miss.resize(n);
    for (int i = 0; i < n; i++) miss[i] = i;
    return TREE2D_OK;
  }
  Solver &S = L.main;
  T2D_CUDA_TRY(S.lookup.reserve(Arena::bytes_for(2 * (size_t)n, 8) * 2 + Arena::bytes_for(n, 4) +
                                Arena::bytes_for(1, 4)));
  S.lookup.reset();
  double *q = S.lookup.take<double>(2 * (size_t)n);
  double *out = S.lookup.take<double>(2 * (size_t)n);
  int *midx = S.lookup.take<int>(n);
  int *cnt = S.lookup.take<int>(1);
  cudaStream_t st[2] = {L.stream, L.copy_stream};
  T2D_CUDA_TRY(cudaMemsetAsync(cnt, 0, sizeof(int), st[0]));
  T2D_CUDA_TRY(cudaEventRecord(L.ev_fork, st[0]));
  T2D_CUDA_TRY(cudaStreamWaitEvent(st[1], L.ev_fork, 0));
  const long chunk = std::max(1L << 20, ((long)n + 3) / 4);
  int k = 0;
  for (long b = 0; b < n; b += chunk, k ^= 1) {
    const long e = std::min((long)n, b + chunk);
    const size_t bytes = sizeof(double) * 2 * (size_t)(e - b);
    T2D_CUDA_TRY(cudaMemcpyAsync(q + 2 * b, xy + 2 * b, bytes, cudaMemcpyHostToDevice, st[k]));
    T2D_CUDA_TRY(lookup_blobs(b, e, q, L.n, L.d_xy, L.d_uv, out, midx, cnt, st[k]));
    T2D_CUDA_TRY(cudaMemcpyAsync(uv + 2 * b, out + 2 * b, bytes, cudaMemcpyDeviceToHost, st[k]));
  }
  T2D_CUDA_TRY(cudaEventRecord(L.ev_join, st[1]));
  T2D_CUDA_TRY(cudaStreamWaitEvent(st[0], L.ev_join, 0));
  T2D_CUDA_TRY(cudaMemcpyAsync(L.h_count, cnt, sizeof(int), cudaMemcpyDeviceToHost, st[0]));
  T2D_CUDA_TRY(cudaStreamSynchronize(st[0]));
  const int nm = *L.h_count;
  if (nm > 0) {
    miss.resize(nm);
    T2D_CUDA_TRY(cudaMemcpyAsync(miss.data(), midx, sizeof(int) * (size_t)nm, cudaMemcpyDeviceToHost, st[0]));
    T2D_CUDA_TRY(cudaStreamSynchronize(st[0]));
    std::sort(miss.begin(), miss.end());
  }
  return TREE2D_OK;
}

// Parameters in force for a device solve (as tree2d_solve_device resolves
// them), with the mode and whether a mirror wall is set, taken under the
// library lock.
int params_for_device_solve(Params &out, int *mode, bool *mirror) {
  Lib &L = lib();
  std::lock_guard<std::mutex> lk(L.mu);
  int rc = resolve_params(L);
  if (rc) return fail(rc);
  out = L.params;
  if (mode) *mode = L.mode;
  if (mirror) *mirror = L.mirror_on;
  return TREE2D_OK;
}

void note_error_text(const char *text) {
  std::lock_guard<std::mutex> lk(g_msg_mu);
  g_cuda_msg = text;
}

int record_error(int code) { return fail(code); }

}  // namespace t2d

using namespace t2d;

extern "C" {

void make_tree(int nvor_b, const double *vor_b, const double *cir_b, const double *cor_b) {
  Lib &L = lib();
  std::lock_guard<std::mutex> lk(L.mu);
  L.valid.store(false);
  L.host_ready.store(false);
  L.hash_ready.store(false);
  L.generation.fetch_add(1);
  L.last_error.store(TREE2D_OK);
  int rc = resolve_params(L);
  if (rc) {
    fail(rc);
    return;
  }
  if (nvor_b < 0 || (nvor_b > 0 && (!vor_b || !cir_b || !cor_b))) {
    fail(TREE2D_ERR_BAD_INPUT);
    return;
  }
  rc = ensure_stream(L);
  if (rc) {
    fail(rc);
    return;
  }
  const int n = nvor_b;
  Solver &S = L.main;
  double *d_xy = nullptr, *d_cir = nullptr, *d_cor = nullptr, *d_uv = nullptr;
  cudaEvent_t cir_cor_ready = nullptr;
  if (n > 0) {
    size_t need = Arena::bytes_for(2 * (size_t)n, 8) * 2 + Arena::bytes_for(n, 8) * 2;
    cudaError_t e = S.io.reserve(need);
    if (e != cudaSuccess) {
      note_cuda_error(e, "make_tree input buffers");
      fail(TREE2D_ERR_CUDA);
      return;
    }
    S.io.reset();
    d_xy = S.io.take<double>(2 * (size_t)n);
    d_uv = S.io.take<double>(2 * (size_t)n);
    d_cir = S.io.take<double>(n);
    d_cor = S.io.take<double>(n);
    // The positions go up on the solve's stream; the circulations and core
    // radii on the copy stream, landing while the keys are formed and
    // sorted (the build waits for them only before its gather).
    cudaStream_t s = L.stream, c = L.copy_stream;
    if (cudaEventRecord(L.ev_fork, s) != cudaSuccess || cudaStreamWaitEvent(c, L.ev_fork, 0) != cudaSuccess ||
        cudaMemcpyAsync(d_xy, vor_b, sizeof(double) * 2 * (size_t)n, cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaMemcpyAsync(d_cir, cir_b, sizeof(double) * (size_t)n, cudaMemcpyHostToDevice, c) != cudaSuccess ||
        cudaMemcpyAsync(d_cor, cor_b, sizeof(double) * (size_t)n, cudaMemcpyHostToDevice, c) != cudaSuccess ||
        cudaEventRecord(L.ev_inputs, c) != cudaSuccess) {
      note_cuda_error(cudaGetLastError(), "make_tree upload");
      cudaStreamSynchronize(c);
      fail(TREE2D_ERR_CUDA);
      return;
    }
    cir_cor_ready = L.ev_inputs;
  }
  rc = solve(L, S, n, d_xy, d_cir, d_cor, d_uv, L.stream, L.stats, cir_cor_ready);
  L.last_was_dev = false;
  // the copy stream is idle before the buffers can be reused
  if (n > 0) {
    cudaError_t e = cudaStreamSynchronize(L.copy_stream);
    if (e != cudaSuccess && rc == TREE2D_OK) {
      note_cuda_error(e, "make_tree upload");
      rc = TREE2D_ERR_CUDA;
    }
  }
  if (rc) {
    fail(rc);
    return;
  }
  L.d_xy = d_xy;
  L.d_uv = d_uv;
  L.n = n;
  L.valid.store(true);
}

void biot_tree(double x, double y, double *u, double *v) {
  Lib &L = lib();
  if (!L.valid.load(std::memory_order_acquire)) {
    *u = NAN;
    *v = NAN;
    L.last_error.store(TREE2D_ERR_NO_TREE);
    return;
  }
  if (!L.host_ready.load(std::memory_order_acquire)) {
    std::lock_guard<std::mutex> lk(L.mu);
    int rc = ensure_host_tables(L);
    if (rc) {
      fail(rc);
      *u = NAN;
      *v = NAN;
      return;
    }
  }
  long k = find_blob(L, x, y);
  if (k >= 0) {
    *u = L.h_uv[2 * k];
    *v = L.h_uv[2 * k + 1];
    return;
  }
  std::lock_guard<std::mutex> lk(L.mu);
  double xy[2] = {x, y}, uv[2];
  int rc = eval_points(L, 1, xy, uv);
  if (rc) {
    fail(rc);
    *u = NAN;
    *v = NAN;
    return;
  }
  *u = uv[0];
  *v = uv[1];
}

int biot_tree_batch(int n, const double *xy, double *uv) {
  Lib &L = lib();
  if (n < 0 || (n > 0 && (!xy || !uv))) return fail(TREE2D_ERR_BAD_INPUT);
  if (!L.valid.load(std::memory_order_acquire)) {
    for (long i = 0; i < 2 * (long)n; i++) uv[i] = NAN;
    return fail(TREE2D_ERR_NO_TREE);
  }
  if (n == 0) return TREE2D_OK;
  std::lock_guard<std::mutex> lk(L.mu);
  std::vector<int> miss;
  int rc = lookup_on_device(L, n, xy, uv, miss);
  if (rc) {
    // no copy into uv may still be in flight
    cudaStreamSynchronize(L.stream);
    cudaStreamSynchronize(L.copy_stream);
    for (long i = 0; i < 2 * (long)n; i++) uv[i] = NAN;
    return fail(rc);
  }
  if (miss.empty()) return TREE2D_OK;
  // Queries the device could not place: the host table (hash over the
  // positions), then the treecode for points off the blobs.
  rc = ensure_host_tables(L);
  if (rc) {
    for (int i : miss) uv[2 * (size_t)i] = uv[2 * (size_t)i + 1] = NAN;
    return fail(rc);
  }
  const long nm = (long)miss.size();
  const long grain = 1 << 14;
  const long nparts = (nm + grain - 1) / grain;
  std::vector<std::vector<int>> off_part(nparts);
  parallel_chunks(nparts, 1, [&](long pb, long pe) {
    for (long c = pb; c < pe; c++) {
      long hint = -1;
      for (long j = c * grain; j < std::min(nm, (c + 1) * grain); j++) {
        const size_t i = (size_t)miss[j];
        long k = find_blob_from(L, xy[2 * i], xy[2 * i + 1], hint);
        if (k >= 0) {
          uv[2 * i] = L.h_uv[2 * k];
          uv[2 * i + 1] = L.h_uv[2 * k + 1];
        } else {
          off_part[c].push_back((int)i);
        }
      }
    }
  });
  std::vector<int> off;
  for (auto &m : off_part) off.insert(off.end(), m.begin(), m.end());
  if (off.empty()) return TREE2D_OK;
  std::vector<double> mxy(2 * off.size()), muv(2 * off.size());
  for (size_t j = 0; j < off.size(); j++) {
    mxy[2 * j] = xy[2 * (size_t)off[j]];
    mxy[2 * j + 1] = xy[2 * (size_t)off[j] + 1];
  }
  rc = eval_points(L, (int)off.size(), mxy.data(), muv.data());
  for (size_t j = 0; j < off.size(); j++) {
    uv[2 * (size_t)off[j]] = rc ? NAN : muv[2 * j];
    uv[2 * (size_t)off[j] + 1] = rc ? NAN : muv[2 * j + 1];
  }
  return rc ? fail(rc) : TREE2D_OK;
}

int tree2d_last_error(void) { return lib().last_error.load(); }

const char *tree2d_error_string(int code) {
  switch (code) {
    case TREE2D_OK: return "ok";
    case TREE2D_ERR_PARAM_FILE: return "could not read ../cal_cond/fmm_param.dat and no parameters were set";
    case TREE2D_ERR_BAD_PARAMS:
      return "invalid parameters: an argument outside the range its call documents (tree2d_set_params: "
             "0<=nterms<=32, 2<=num_p<=65536, finite theta)";
    case TREE2D_ERR_BAD_INPUT: return "invalid input (negative count, null array, or non-finite value)";
    case TREE2D_ERR_TOO_DEEP: return "tree deeper than 32 levels (>= num_p coincident blobs?)";
    case TREE2D_ERR_CUDA: {
      std::lock_guard<std::mutex> lk(g_msg_mu);
      static thread_local std::string s;
      s = "CUDA error: " + g_cuda_msg;
      return s.c_str();
    }
    case TREE2D_ERR_NO_TREE: return "no valid tree (make_tree not called or failed)";
    case TREE2D_ERR_NO_DEVICE: return "no CUDA device";
    case TREE2D_ERR_TIMEOUT: return "a bounded device loop gave up (a traversal stack overflow or a wait past its limit)";
    case TREE2D_ERR_MODE: return "unknown mode, or a call the mode or settings in force do not support";
    case TREE2D_ERR_FILE: return "could not read the file, or it is not a weights file of this version";
    case TREE2D_ERR_TOO_LARGE:
      return "problem too large for this path (the fixed scratch of tree2d_solve_device_static: 65536 blobs, "
             "32 MiB; or more than 2^31 - 1 interaction-list entries)";
    default: return "unknown error";
  }
}

int tree2d_set_params(int nterms, int num_p, double theta, double r_min) {
  Lib &L = lib();
  std::lock_guard<std::mutex> lk(L.mu);
  Params p;
  p.nterms = nterms;
  p.num_p = num_p;
  p.theta = theta;
  p.r_min = r_min;
  int rc = check_params(p);
  if (rc) return fail(rc);
  L.params = p;
  L.have_params = true;
  L.params_fixed = true;
  return TREE2D_OK;
}

void tree2d_clear_params(void) {
  Lib &L = lib();
  std::lock_guard<std::mutex> lk(L.mu);
  L.params_fixed = false;
}

void tree2d_get_params(int *nterms, int *num_p, double *theta, double *r_min) {
  Lib &L = lib();
  std::lock_guard<std::mutex> lk(L.mu);
  if (nterms) *nterms = L.params.nterms;
  if (num_p) *num_p = L.params.num_p;
  if (theta) *theta = L.params.theta;
  if (r_min) *r_min = L.params.r_min;
}

int tree2d_set_mode(int mode) {
  Lib &L = lib();
  std::lock_guard<std::mutex> lk(L.mu);
  if (mode != TREE2D_MODE_PLAIN && mode != TREE2D_MODE_MIXED && mode != TREE2D_MODE_LEARNED)
    return fail(TREE2D_ERR_MODE);
  L.mode = mode;
  return TREE2D_OK;
}

int tree2d_get_mode(void) { return lib().mode; }

int tree2d_set_tuning(int autotune, int eval_variant) {
  Lib &L = lib();
  std::lock_guard<std::mutex> lk(L.mu);
  if (eval_variant < -1 || eval_variant >= kEvalVariantCount) return fail(TREE2D_ERR_BAD_PARAMS);
  L.mixed.autotune = autotune ? 1 : 0;
  L.mixed.eval_variant = eval_variant;
  return TREE2D_OK;
}

int tree2d_set_level_chain(int on) {
  Lib &L = lib();
  std::lock_guard<std::mutex> lk(L.mu);
  L.mixed.level_chain = on ? 1 : 0;
  return TREE2D_OK;
}

int tree2d_set_m2l_rows(int rows) {
  Lib &L = lib();
  std::lock_guard<std::mutex> lk(L.mu);
  if (rows != 0 && rows != 64 && rows != 128) return fail(TREE2D_ERR_BAD_PARAMS);
  L.mixed.m2l_rows = rows;
  return TREE2D_OK;
}

int tree2d_set_mixed_leaf(int max_blobs) {
  Lib &L = lib();
  std::lock_guard<std::mutex> lk(L.mu);
  if (max_blobs < -1 || max_blobs > 65535) return fail(TREE2D_ERR_BAD_PARAMS);
  L.mixed.leaf_blobs = max_blobs;
  return TREE2D_OK;
}

int tree2d_set_mixed_params(int pterms, double cutoff_sigmas, int use_tensor_cores) {
  Lib &L = lib();
  std::lock_guard<std::mutex> lk(L.mu);
  if (pterms < 2 || pterms > kMaxP || !(cutoff_sigmas >= 0.0) || !std::isfinite(cutoff_sigmas))
    return fail(TREE2D_ERR_BAD_PARAMS);
  L.mixed.pterms = pterms;
  L.mixed.cutoff = cutoff_sigmas;
  L.mixed.use_tensor_cores = use_tensor_cores ? 1 : 0;
  return TREE2D_OK;
}

int tree2d_solve_device(int n, const double *d_xy, const double *d_cir, const double *d_cor, double *d_uv,
                        void *stream) {
  Lib &L = lib();
  std::lock_guard<std::mutex> lk(L.mu);
  int rc = resolve_params(L);
  if (rc) return fail(rc);
  if (n < 0) return fail(TREE2D_ERR_BAD_INPUT);
  rc = ensure_stream(L);
  if (rc) return fail(rc);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  rc = solve(L, L.dev, n, d_xy, d_cir, d_cor, d_uv, s, L.dev_stats);
  L.last_was_dev = true;
  if (rc) return fail(rc);
  return TREE2D_OK;
}

int tree2d_solve_sets(int nsets, const int *set_offsets, const double *d_xy, const double *d_cir,
                      const double *d_cor, double *d_uv, void *stream) {
  Lib &L = lib();
  std::lock_guard<std::mutex> lk(L.mu);
  int rc = resolve_params(L);
  if (rc) return fail(rc);
  if (nsets < 1 || !set_offsets || set_offsets[0] != 0) return fail(TREE2D_ERR_BAD_INPUT);
  for (int k = 0; k < nsets; k++)
    if (set_offsets[k + 1] < set_offsets[k]) return fail(TREE2D_ERR_BAD_INPUT);
  const int n = set_offsets[nsets];
  if (n > 0 && (!d_xy || !d_cir || !d_cor || !d_uv)) return fail(TREE2D_ERR_BAD_INPUT);
  // one tree over all sets: the mixed form only (the plain treecode's
  // traversal starts at the tree root), and no mirror wall
  if (L.mode == TREE2D_MODE_PLAIN || L.mirror_on) return fail(TREE2D_ERR_MODE);
  rc = ensure_stream(L);
  if (rc) return fail(rc);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  Solver &S = L.dev;
  const int *d_off = nullptr;
  if (nsets > 1) {
    cudaError_t e = S.sets.reserve(Arena::bytes_for((size_t)nsets + 1, 4));
    int *d = nullptr;
    if (e == cudaSuccess) {
      S.sets.reset();
      d = S.sets.take<int>((size_t)nsets + 1);
      e = cudaMemcpyAsync(d, set_offsets, sizeof(int) * ((size_t)nsets + 1), cudaMemcpyHostToDevice, s);
    }
    if (e != cudaSuccess) {
      note_cuda_error(e, "solve_sets offsets");
      return fail(TREE2D_ERR_CUDA);
    }
    d_off = d;
  }
  rc = solve_body(L, S, n, d_xy, d_cir, d_cor, d_uv, s, L.dev_stats, d_off, nsets);
  L.last_was_dev = true;
  if (rc) return fail(rc);
  return TREE2D_OK;
}

int tree2d_get_stats(tree2d_stats_t *out) {
  Lib &L = lib();
  std::lock_guard<std::mutex> lk(L.mu);
  if (!out) return TREE2D_ERR_BAD_INPUT;
  *out = L.last_was_dev ? L.dev_stats : L.stats;  // the most recent solve
  return TREE2D_OK;
}

long long tree2d_export_tree(int *perm, long long cap, int *level, int *begin, int *end, int *leaf, double *cx,
                             double *cy, double *region, double *coef) {
  Lib &L = lib();
  std::lock_guard<std::mutex> lk(L.mu);
  if (!L.valid.load()) return -1;
  const Tree &t = L.main.tree;
  if (t.n == 0) return 0;
  long long nc = t.ncell - 1;
  if (cap <= 0) return nc;
  if (cap < nc) return -1;
  const int nt = t.nterms;
  if (perm && cudaMemcpy(perm, t.perm, sizeof(int) * (size_t)t.n, cudaMemcpyDeviceToHost) != cudaSuccess) return -1;
  std::vector<unsigned char> lf(nc);
  if (level) cudaMemcpy(level, t.level + 1, sizeof(int) * nc, cudaMemcpyDeviceToHost);
  if (begin) cudaMemcpy(begin, t.begin + 1, sizeof(int) * nc, cudaMemcpyDeviceToHost);
  if (end) cudaMemcpy(end, t.end + 1, sizeof(int) * nc, cudaMemcpyDeviceToHost);
  if (leaf) {
    cudaMemcpy(lf.data(), t.leaf + 1, nc, cudaMemcpyDeviceToHost);
    for (long long i = 0; i < nc; i++) leaf[i] = lf[i];
  }
  if (cx) cudaMemcpy(cx, t.cx + 1, sizeof(double) * nc, cudaMemcpyDeviceToHost);
  if (cy) cudaMemcpy(cy, t.cy + 1, sizeof(double) * nc, cudaMemcpyDeviceToHost);
  if (region) cudaMemcpy(region, t.region + 1, sizeof(double) * nc, cudaMemcpyDeviceToHost);
  if (coef && nt > 0) cudaMemcpy(coef, t.coef + nt, sizeof(double2) * nc * nt, cudaMemcpyDeviceToHost);
  if (cudaGetLastError() != cudaSuccess) return -1;
  return nc;
}

int tree2d_direct_device(int ntgt, const double *d_txy, int nsrc, const double *d_sxy, const double *d_cir,
                         const double *d_cor, double *d_uv, void *stream) {
  cudaError_t e = direct_sum(ntgt, d_txy, nsrc, d_sxy, d_cir, d_cor, d_uv, static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) {
    note_cuda_error(e, "direct_sum");
    return fail(TREE2D_ERR_CUDA);
  }
  return TREE2D_OK;
}

int tree2d_fp64_probe(int blocks, int iters, void *stream, double *ms) {
  return tree2d_pipe_probe(64, blocks, iters, stream, ms);
}

int tree2d_wait_probe(long long polls, int *status) {
  if (polls < 1 || !status) return fail(TREE2D_ERR_BAD_INPUT);
  int *d = nullptr;
  if (cudaMalloc(reinterpret_cast<void **>(&d), sizeof(int)) != cudaSuccess) return fail(TREE2D_ERR_CUDA);
  cudaError_t e = wait_probe((long)polls, d, nullptr);
  if (e == cudaSuccess) e = cudaMemcpy(status, d, sizeof(int), cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (e != cudaSuccess) {
    note_cuda_error(e, "wait_probe");
    return fail(TREE2D_ERR_CUDA);
  }
  return TREE2D_OK;
}

int tree2d_pipe_probe(int bits, int blocks, int iters, void *stream, double *ms) {
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  double *buf = nullptr;
  cudaEvent_t a, b;
  if (bits != 32 && bits != 64) return fail(TREE2D_ERR_BAD_INPUT);
  if (cudaMalloc(reinterpret_cast<void **>(&buf), 64) != cudaSuccess) return fail(TREE2D_ERR_CUDA);
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  auto run = [&](int it) {
    return bits == 64 ? dfma_probe(buf, blocks, it, s) : ffma_probe(reinterpret_cast<float *>(buf), blocks, it, s);
  };
  run(iters / 8 + 1);  // warm-up
  cudaEventRecord(a, s);
  cudaError_t e = run(iters);
  cudaEventRecord(b, s);
  cudaEventSynchronize(b);
  float f = 0.f;
  cudaEventElapsedTime(&f, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaFree(buf);
  if (e != cudaSuccess) {
    note_cuda_error(e, "pipe_probe");
    return fail(TREE2D_ERR_CUDA);
  }
  if (ms) *ms = f;
  return TREE2D_OK;
}

// ---------------------------------------------------------------- learned form

int tree2d_learn_set_weights(const float *theta, int n) {
  Lib &L = lib();
  std::lock_guard<std::mutex> lk(L.mu);
  if (n != kMlpParams || !theta) return fail(TREE2D_ERR_BAD_INPUT);
  for (int i = 0; i < n; i++)
    if (!std::isfinite(theta[i])) return fail(TREE2D_ERR_BAD_INPUT);
  std::memcpy(L.lp->theta, theta, sizeof(float) * n);
  L.lp->have_weights = true;
  L.lp_version++;
  return TREE2D_OK;
}

int tree2d_learn_get_weights(float *theta, int n) {
  Lib &L = lib();
  std::lock_guard<std::mutex> lk(L.mu);
  if (n != kMlpParams || !theta) return fail(TREE2D_ERR_BAD_INPUT);
  if (!L.lp->have_weights) return fail(TREE2D_ERR_NO_TREE);
  std::memcpy(theta, L.lp->theta, sizeof(float) * n);
  return TREE2D_OK;
}

int tree2d_learn_set_options(float direct_bias, int order_margin, double budget) {
  Lib &L = lib();
  std::lock_guard<std::mutex> lk(L.mu);
  if (!std::isfinite(direct_bias) || order_margin < 0 || order_margin > 12 || !(budget > 0.0))
    return fail(TREE2D_ERR_BAD_PARAMS);
  L.lp->direct_bias = direct_bias;
  L.lp->order_margin = order_margin;
  L.lp->budget = budget;
  return TREE2D_OK;
}

int tree2d_learn_set_far_orders(int on) {
  Lib &L = lib();
  std::lock_guard<std::mutex> lk(L.mu);
  L.lp->far_orders = on ? 1 : 0;
  return TREE2D_OK;
}

int tree2d_learn_set_envelope(double k_blobs_per_leaf_max, double cutoff_sigmas) {
  Lib &L = lib();
  std::lock_guard<std::mutex> lk(L.mu);
  if (!(k_blobs_per_leaf_max >= 0.0) || !std::isfinite(k_blobs_per_leaf_max)) return fail(TREE2D_ERR_BAD_PARAMS);
  if (!(cutoff_sigmas >= 0.0) || !std::isfinite(cutoff_sigmas) || cutoff_sigmas > 64.0)
    return fail(TREE2D_ERR_BAD_PARAMS);
  L.lp->k_blobs_max = k_blobs_per_leaf_max;
  L.lp->cutoff_train = cutoff_sigmas;
  return TREE2D_OK;
}

int tree2d_learn_param_count(void) { return kMlpParams; }

// Weights file (little-endian): "T2DW", uint32 version 1, uint32 parameter
// count, uint32 header bytes (32), float64 envelope limit (K-list source
// blobs per leaf; 0 = none), float64 the correction radius it is counted at
// (units of max sigma), then the parameters as float32.
int tree2d_learn_load(const char *path) {
  if (!path) return fail(TREE2D_ERR_BAD_INPUT);
  FILE *f = std::fopen(path, "rb");
  if (!f) return fail(TREE2D_ERR_FILE);
  unsigned char hdr[32];
  const bool got = std::fread(hdr, 1, sizeof(hdr), f) == sizeof(hdr);
  uint32_t version = 0, count = 0, hbytes = 0;
  double limit = 0.0, cutoff = 0.0;
  if (got) {
    std::memcpy(&version, hdr + 4, 4);
    std::memcpy(&count, hdr + 8, 4);
    std::memcpy(&hbytes, hdr + 12, 4);
    std::memcpy(&limit, hdr + 16, 8);
    std::memcpy(&cutoff, hdr + 24, 8);
  }
  if (!got || std::memcmp(hdr, "T2DW", 4) != 0 || version != 1 || count != (uint32_t)kMlpParams || hbytes != 32) {
    std::fclose(f);
    return fail(TREE2D_ERR_FILE);
  }
  std::vector<float> theta(kMlpParams);
  const bool body = std::fread(theta.data(), sizeof(float), theta.size(), f) == theta.size();
  std::fclose(f);
  if (!body) return fail(TREE2D_ERR_FILE);
  int rc = tree2d_learn_set_envelope(limit, cutoff);
  if (rc) return rc;
  return tree2d_learn_set_weights(theta.data(), kMlpParams);
}

// ---------------------------------------------------------------- extensions

int tree2d_set_mirror(int enable, double d_mirror) {
  Lib &L = lib();
  std::lock_guard<std::mutex> lk(L.mu);
  if (enable && !std::isfinite(d_mirror)) return fail(TREE2D_ERR_BAD_PARAMS);
  L.mirror_on = enable != 0;
  L.mirror_d = d_mirror;
  return TREE2D_OK;
}

int tree2d_advect_device(int n, double *d_xy, const double *d_uv, double dt, void *stream) {
  if (n < 0 || !std::isfinite(dt)) return fail(TREE2D_ERR_BAD_INPUT);
  cudaError_t e = advect(n, d_xy, d_uv, dt, static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) {
    note_cuda_error(e, "advect");
    return fail(TREE2D_ERR_CUDA);
  }
  return TREE2D_OK;
}

int tree2d_learn_collect(int max_samples, unsigned seed, float *features, int *labels) {
  Lib &L = lib();
  std::lock_guard<std::mutex> lk(L.mu);
  Workspace &ws = L.dev.ws;
  if (!ws.mxv || max_samples <= 0 || !features || !labels) return -fail(TREE2D_ERR_NO_TREE);
  MixedView &m = *ws.mxv;
  if (m.lev0 > 0) return -fail(TREE2D_ERR_MODE);  // samples come from a solve of one set
  const long nu = ws.mx_tot[0], nk = ws.mx_tot[2];
  if (nu + nk <= 0) return 0;
  std::vector<int> uoff(m.nleaf + 1), koff(m.nleaf + 1);
  cudaStream_t s = L.stream;
  if (cudaMemcpy(uoff.data(), m.u_off, sizeof(int) * (m.nleaf + 1), cudaMemcpyDeviceToHost) != cudaSuccess ||
      cudaMemcpy(koff.data(), m.k_off, sizeof(int) * (m.nleaf + 1), cudaMemcpyDeviceToHost) != cudaSuccess)
    return -fail(TREE2D_ERR_CUDA);
  const int ns = (int)std::min<long>(max_samples, nu + nk);
  std::vector<int> smp(3 * (size_t)ns);
  uint64_t st = 0x9e3779b97f4a7c15ull * (seed + 1);
  for (int i = 0; i < ns; i++) {
    st = mix64(st);
    const long g = (long)(st % (uint64_t)(nu + nk));
    const int kind = g < nu ? 0 : 1;
    const int e = (int)(kind == 0 ? g : g - nu);
    const std::vector<int> &off = kind == 0 ? uoff : koff;
    const int l = (int)(std::upper_bound(off.begin(), off.end(), e) - off.begin()) - 1;
    smp[3 * (size_t)i] = l;
    smp[3 * (size_t)i + 1] = kind;
    smp[3 * (size_t)i + 2] = e;
  }
  int *d_smp = nullptr, *d_lab = nullptr;
  float *d_feat = nullptr, *d_uref = nullptr;
  LeafStats *d_stats = nullptr;
  auto cleanup = [&]() {
    cudaFree(d_smp);
    cudaFree(d_lab);
    cudaFree(d_feat);
    cudaFree(d_uref);
    cudaFree(d_stats);
  };
  if (cudaMalloc(reinterpret_cast<void **>(&d_smp), sizeof(int) * smp.size()) != cudaSuccess ||
      cudaMalloc(reinterpret_cast<void **>(&d_lab), sizeof(int) * (size_t)ns) != cudaSuccess ||
      cudaMalloc(reinterpret_cast<void **>(&d_feat), sizeof(float) * (size_t)ns * kMlpIn) != cudaSuccess ||
      cudaMalloc(reinterpret_cast<void **>(&d_uref), sizeof(float)) != cudaSuccess ||
      cudaMalloc(reinterpret_cast<void **>(&d_stats), sizeof(LeafStats) * (size_t)m.ncell) != cudaSuccess) {
    cleanup();
    note_cuda_error(cudaErrorMemoryAllocation, "learn_collect");
    return -fail(TREE2D_ERR_CUDA);
  }
  int rc = TREE2D_OK;
  float uref = 0.f;
  if (cudaMemcpy(d_smp, smp.data(), sizeof(int) * smp.size(), cudaMemcpyHostToDevice) != cudaSuccess) rc = TREE2D_ERR_CUDA;
  if (!rc) rc = learned_leaf_stats(m, d_stats, s);
  if (!rc) rc = learned_uref(m, d_stats, L.dev.tree.root, d_uref, s);
  if (!rc && cudaMemcpyAsync(&uref, d_uref, 4, cudaMemcpyDeviceToHost, s) != cudaSuccess) rc = TREE2D_ERR_CUDA;
  if (!rc && cudaStreamSynchronize(s) != cudaSuccess) rc = TREE2D_ERR_CUDA;
  if (!rc) rc = learned_labels(m, d_stats, d_uref, L.lp->budget * (double)uref, ns, d_smp, d_feat, d_lab, s);
  if (!rc && cudaStreamSynchronize(s) != cudaSuccess) rc = TREE2D_ERR_CUDA;
  if (!rc && cudaMemcpy(features, d_feat, sizeof(float) * (size_t)ns * kMlpIn, cudaMemcpyDeviceToHost) != cudaSuccess)
    rc = TREE2D_ERR_CUDA;
  if (!rc && cudaMemcpy(labels, d_lab, sizeof(int) * (size_t)ns, cudaMemcpyDeviceToHost) != cudaSuccess)
    rc = TREE2D_ERR_CUDA;
  cleanup();
  if (rc) return -fail(rc);
  return ns;
}

// Host arrays in; weights updated in place (initialised from `seed` when
// none are loaded).
int tree2d_learn_train(int n, const float *X, const int *y, int steps, int batch, float lr, unsigned seed,
                       float *loss) {
  Lib &L = lib();
  std::lock_guard<std::mutex> lk(L.mu);
  if (n <= 0 || !X || !y || steps <= 0 || batch <= 0 || !(lr > 0.f)) return fail(TREE2D_ERR_BAD_INPUT);
  int rc = ensure_stream(L);
  if (rc) return fail(rc);
  if (!L.lp->have_weights) {
    // He-style initialisation from a seeded generator, biases zero
    uint64_t st = 0x243f6a8885a308d3ull ^ seed;
    const int fan[8] = {16, 0, 64, 0, 64, 0, 64, 0};
    const int sz[8] = {1024, 64, 4096, 64, 4096, 64, 1024, 16};
    int o = 0;
    for (int b = 0; b < 8; b++)
      for (int i = 0; i < sz[b]; i++, o++) {
        if (!fan[b]) {
          L.lp->theta[o] = 0.f;
          continue;
        }
        st = mix64(st);
        const double u1 = ((st >> 11) + 1.0) / 9007199254740993.0;
        st = mix64(st);
        const double u2 = (st >> 11) / 9007199254740992.0;
        const double g = std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
        L.lp->theta[o] = (float)(g * std::sqrt(2.0 / fan[b]));
      }
  }
  float *d_X = nullptr, *d_th = nullptr, *d_m = nullptr, *d_v = nullptr;
  int *d_y = nullptr;
  auto cleanup = [&]() {
    cudaFree(d_X);
    cudaFree(d_th);
    cudaFree(d_m);
    cudaFree(d_v);
    cudaFree(d_y);
  };
  if (cudaMalloc(reinterpret_cast<void **>(&d_X), sizeof(float) * (size_t)n * kMlpIn) != cudaSuccess ||
      cudaMalloc(reinterpret_cast<void **>(&d_y), sizeof(int) * (size_t)n) != cudaSuccess ||
      cudaMalloc(reinterpret_cast<void **>(&d_th), sizeof(float) * kMlpParams) != cudaSuccess ||
      cudaMalloc(reinterpret_cast<void **>(&d_m), sizeof(float) * kMlpParams) != cudaSuccess ||
      cudaMalloc(reinterpret_cast<void **>(&d_v), sizeof(float) * kMlpParams) != cudaSuccess) {
    cleanup();
    note_cuda_error(cudaErrorMemoryAllocation, "learn_train");
    return fail(TREE2D_ERR_CUDA);
  }
  cudaMemcpy(d_X, X, sizeof(float) * (size_t)n * kMlpIn, cudaMemcpyHostToDevice);
  cudaMemcpy(d_y, y, sizeof(int) * (size_t)n, cudaMemcpyHostToDevice);
  cudaMemcpy(d_th, L.lp->theta, sizeof(float) * kMlpParams, cudaMemcpyHostToDevice);
  cudaMemset(d_m, 0, sizeof(float) * kMlpParams);
  cudaMemset(d_v, 0, sizeof(float) * kMlpParams);
  rc = mlp_train(n, d_X, d_y, d_th, d_m, d_v, steps, batch, lr, seed, loss, L.stream);
  if (!rc && cudaMemcpy(L.lp->theta, d_th, sizeof(float) * kMlpParams, cudaMemcpyDeviceToHost) != cudaSuccess)
    rc = TREE2D_ERR_CUDA;
  cleanup();
  if (rc) return fail(rc);
  L.lp->have_weights = true;
  L.lp_version++;
  return TREE2D_OK;
}

int tree2d_mlp_grad(int n, const float *X, const int *y, const float *theta, float *grad, float *loss) {
  Lib &L = lib();
  std::lock_guard<std::mutex> lk(L.mu);
  int rc = ensure_stream(L);
  if (rc) return fail(rc);
  float *d_X = nullptr, *d_th = nullptr, *d_g = nullptr;
  int *d_y = nullptr;
  cudaMalloc(reinterpret_cast<void **>(&d_X), sizeof(float) * (size_t)n * kMlpIn);
  cudaMalloc(reinterpret_cast<void **>(&d_y), sizeof(int) * (size_t)n);
  cudaMalloc(reinterpret_cast<void **>(&d_th), sizeof(float) * kMlpParams);
  cudaMalloc(reinterpret_cast<void **>(&d_g), sizeof(float) * kMlpParams);
  if (!d_X || !d_y || !d_th || !d_g) rc = TREE2D_ERR_CUDA;
  if (!rc) {
    cudaMemcpy(d_X, X, sizeof(float) * (size_t)n * kMlpIn, cudaMemcpyHostToDevice);
    cudaMemcpy(d_y, y, sizeof(int) * (size_t)n, cudaMemcpyHostToDevice);
    cudaMemcpy(d_th, theta, sizeof(float) * kMlpParams, cudaMemcpyHostToDevice);
    rc = mlp_grad(n, d_X, d_y, d_th, d_g, loss, L.stream);
  }
  if (!rc && cudaMemcpy(grad, d_g, sizeof(float) * kMlpParams, cudaMemcpyDeviceToHost) != cudaSuccess)
    rc = TREE2D_ERR_CUDA;
  cudaFree(d_X);
  cudaFree(d_y);
  cudaFree(d_th);
  cudaFree(d_g);
  return rc ? fail(rc) : TREE2D_OK;
}

int tree2d_mlp_forward(int n, const float *X, const float *theta, float *logits, int tensor_cores) {
  Lib &L = lib();
  std::lock_guard<std::mutex> lk(L.mu);
  int rc = ensure_stream(L);
  if (rc) return fail(rc);
  T2D_CUDA_TRY(workspace_init(L.dev.ws));
  float *d_X = nullptr, *d_th = nullptr, *d_out = nullptr, *d_b = nullptr;
  uint16_t *d_img = nullptr;
  cudaMalloc(reinterpret_cast<void **>(&d_X), sizeof(float) * (size_t)n * kMlpIn);
  cudaMalloc(reinterpret_cast<void **>(&d_th), sizeof(float) * kMlpParams);
  cudaMalloc(reinterpret_cast<void **>(&d_out), sizeof(float) * (size_t)n * kMlpOut);
  cudaMalloc(reinterpret_cast<void **>(&d_b), sizeof(float) * 208);
  cudaMalloc(reinterpret_cast<void **>(&d_img), 2 * learn_weight_image_elems());
  if (!d_X || !d_th || !d_out || !d_b || !d_img) rc = TREE2D_ERR_CUDA;
  if (!rc) {
    cudaMemcpy(d_X, X, sizeof(float) * (size_t)n * kMlpIn, cudaMemcpyHostToDevice);
    cudaMemcpy(d_th, theta, sizeof(float) * kMlpParams, cudaMemcpyHostToDevice);
    if (tensor_cores) {
      std::vector<uint16_t> img;
      std::vector<float> b;
      learn_weight_images(theta, img, b);
      cudaMemcpy(d_img, img.data(), img.size() * 2, cudaMemcpyHostToDevice);
      cudaMemcpy(d_b, b.data(), b.size() * 4, cudaMemcpyHostToDevice);
      cudaMemsetAsync(L.dev.ws.status, 0, sizeof(DevStatus), L.stream);
      rc = mlp_forward_tc(n, d_X, d_img, d_b, d_out, L.dev.ws.status, L.stream);
      if (!rc && cudaStreamSynchronize(L.stream) != cudaSuccess) rc = TREE2D_ERR_CUDA;
    } else {
      rc = mlp_forward_cc(n, d_X, d_th, d_out, L.stream);
    }
  }
  if (!rc && cudaMemcpy(logits, d_out, sizeof(float) * (size_t)n * kMlpOut, cudaMemcpyDeviceToHost) != cudaSuccess)
    rc = TREE2D_ERR_CUDA;
  cudaFree(d_X);
  cudaFree(d_th);
  cudaFree(d_out);
  cudaFree(d_b);
  cudaFree(d_img);
  return rc ? fail(rc) : TREE2D_OK;
}

const char *tree2d_version(void) { return "tree2d-gb300 0.1 (sm_103a)"; }

}  // extern "C"
