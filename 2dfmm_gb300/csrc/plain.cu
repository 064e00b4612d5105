// Plain FP64 treecode on the device: the reference's numerics
// (ver-c/src/fmm.c) with GPU-shaped control flow.
//
//  k_s2m       one warp per leaf, lane k owns coefficient k; blobs are
//              summed in the leaf's order (ascending original index), the
//              order fmm.c:24-29 sums them; powers by a warp product scan.
//  k_m2m       one warp per internal cell of one level, deepest level first;
//              children in quadrant order 3,2,1,0 (fmm.c:41-56); the
//              level-1 -> root shift is skipped as in the reference.
//  k_eval      one warp per 32 consecutive targets (tree order, so the warp's
//              targets are neighbours).  The warp walks the UNION of its
//              lanes' traversals with a shared LIFO of (cell, lane mask):
//              restricted to one lane, the visit order is that lane's own
//              LIFO order in fmm.c:90-112, so every lane accumulates M2S and
//              direct terms in the reference's order.  The opening test uses
//              round-to-nearest FP64 operations without contraction
//              (r = sqrt(dx*dx + dy*dy); region > theta*r), so each lane
//              takes exactly the reference's branch.  M2S (fmm.c:60-67) is
//              evaluated by Horner in w = 1/(z - zc), from a per-lane queue
//              of accepted cells that the warp empties in rounds (all lanes
//              busy); P2P is fmm.c:121-142.
#include "dev_common.cuh"

namespace t2d {
namespace {

// 1/x for a positive normal x: the SFU's approximate reciprocal refined by
// two Newton-Raphson steps for f(y) = 1/y - x, y <- y + y (1 - x y), each
// with the residual 1 - x y formed by one FMA.  Every step squares the
// relative error, so the ~2^-20 seed ends within an ulp or so of the
// correctly rounded 1/x, which is all the 1e-12 bar needs; it replaces the
// IEEE division of the pair and M2S terms (the FP64 pipe is this kernel's
// bound).
__device__ __forceinline__ double rcp_nr(double x) {
  double y;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
  y = fma(y, fma(-x, y, 1.0), y);
  y = fma(y, fma(-x, y, 1.0), y);
  return y;
}

// a b + c for complex values as FMAs only: Re = a.x b.x + (c.x - a.y b.y),
// Im = a.x b.y + (c.y + a.y b.x), each inner term one FMA and each outer one
// another (explicit, so the rounding does not depend on how the compiler
// contracts the code around it).
__device__ __forceinline__ double2 cfma(double2 a, double2 b, double2 c) {
  return make_double2(__fma_rn(a.x, b.x, __fma_rn(-a.y, b.y, c.x)), __fma_rn(a.x, b.y, __fma_rn(a.y, b.x, c.y)));
}

__constant__ double c_binom[kMaxTerms][kMaxTerms];

constexpr double kPi = 3.14159265358979323846;
constexpr double kInv2Pi = 0.15915494309189533577;  // 1 / (2 pi), rounded

__global__ void __launch_bounds__(256) k_s2m(Tree t, int nt) {
  const int wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (wid >= t.nleaf) return;
  const int c = t.leaf_cell[wid];
  const int b = t.begin[c], e = t.end[c];
  const double cx = t.cx[c], cy = t.cy[c];
  double2 acc = make_double2(0.0, 0.0);
  for (int j = b; j < e; j++) {
    double2 z = make_double2(t.x[j] - cx, t.y[j] - cy);
    double2 pw = warp_powers(z, lane);
    double g = t.cir[j];
    acc.x += g * pw.x;
    acc.y += g * pw.y;
  }
  if (lane < nt) t.coef[(size_t)c * nt + lane] = acc;
}

__global__ void __launch_bounds__(256) k_zero_internal(Tree t, int nt) {
  long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= (long)t.ncell * nt) return;
  int c = (int)(i / nt);
  if (!t.leaf[c]) t.coef[i] = make_double2(0.0, 0.0);
}

__global__ void __launch_bounds__(256) k_m2m(Tree t, int nt, int lev) {
  const int p = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (p >= t.ncell) return;
  if (t.level[p] != lev || t.leaf[p]) return;
  const double px = t.cx[p], py = t.cy[p];
  double2 acc = make_double2(0.0, 0.0);
  const int4 ch = reinterpret_cast<const int4 *>(t.child)[p];
  for (int q = 3; q >= 0; q--) {
    const int c = (&ch.x)[q];
    if (c < 0) continue;
    // -(z_p - z_c), fmm.c:50
    double2 dz = make_double2(t.cx[c] - px, t.cy[c] - py);
    double2 pw = warp_powers(dz, lane);
    double2 a = lane < nt ? t.coef[(size_t)c * nt + lane] : make_double2(0.0, 0.0);
    double2 s = make_double2(0.0, 0.0);
    for (int k = 0; k < nt; k++) {
      double2 ak = shfl_d2(a, k);
      double2 pk = shfl_d2(pw, (lane - k) & 31);
      if (k <= lane) {
        double bin = c_binom[lane & (kMaxTerms - 1)][k];
        s = cadd(s, cmul(make_double2(ak.x * bin, ak.y * bin), pk));
      }
    }
    acc = cadd(acc, s);
  }
  if (lane < nt) t.coef[(size_t)p * nt + lane] = acc;
}

constexpr int kEvalWarps = 4;
constexpr int kStackCap = 160;
constexpr int kQueue = 32;  // deferred M2S cells per lane
static_assert((kQueue & (kQueue - 1)) == 0, "the M2S queues are rings indexed by a mask");
constexpr int kLeafQueue = 16;  // deferred direct (P2P) leaves per lane

struct EvalArgs {
  Tree t;
  int nt;
  double theta;
  int ntgt;
  const double *tx, *ty;
  const int *out_idx;
  double *uv;
  DevStatus *st;
};

__global__ void __launch_bounds__(kEvalWarps * 32) k_eval(EvalArgs a) {
  __shared__ int s_cell[kEvalWarps][kStackCap];
  __shared__ unsigned s_mask[kEvalWarps][kStackCap];
  __shared__ int s_queue[kEvalWarps][kQueue][32];
  __shared__ int s_leaves[kEvalWarps][kLeafQueue][32];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long i = ((long)blockIdx.x * kEvalWarps + warp) * 32 + lane;
  const bool valid = i < a.ntgt;
  const unsigned vmask = __ballot_sync(0xffffffffu, valid);
  if (vmask == 0) return;
  const Tree &t = a.t;
  const int nt = a.nt;
  const double x = valid ? a.tx[i] : 0.0, y = valid ? a.ty[i] : 0.0;
  const double theta = a.theta;
  // the target as FP32 pairs, for the opening pre-test (x - xh is exact)
  const float xh = __double2float_rn(x), yh = __double2float_rn(y);
  const float xl = __double2float_rn(x - (double)xh), yl = __double2float_rn(y - (double)yh);
  const float sxy = __fadd_rn(fabsf(xh), fabsf(yh));
  double2 phi = make_double2(0.0, 0.0);
  double ud0 = 0.0, ud1 = 0.0;
  unsigned long long n_m2s = 0, n_pairs = 0;
  bool overflow = false;

  // The lanes accept cells at different depths, so an M2S evaluated where
  // it is accepted runs with the warp's other lanes idle.  Each lane
  // instead queues its accepted cells (s_queue[warp][k][lane], in the order
  // it accepts them) and the warp evaluates the queues together, one entry
  // per lane per round, when a lane's queue could overflow and at the end.
  // A lane's M2S terms still reach phi in its own acceptance order, each
  // with the same operations (dx, dy, d2 formed again from the cell's
  // centre, bit for bit); the direct terms are deferred too (below).
  // The queues are rings (head qh, count nq).  A flush when some lane's
  // queue could overflow evaluates only as many rounds as every lane can
  // fill, or as the fullest lane needs to make room for four entries, if
  // that is more; the end of the traversal empties them all.
  int qh = 0, nq = 0;
  auto flush = [&](bool all) {
    int hi = nq, lo = nq;
    for (int o = 16; o; o >>= 1) {
      hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
      lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    }
    const int rounds = all ? hi : max(lo, hi - (kQueue - 4));
    for (int r = 0; r < rounds; r++) {
      if (r < nq) {
        // M2S, fmm.c:60-67: sum_{k<nt-1} a_k w^{k+1}, w = 1/(z - zc)
        const int cc = s_queue[warp][(qh + r) & (kQueue - 1)][lane];
        const double dx = __dsub_rn(x, t.cx[cc]);
        const double dy = __dsub_rn(y, t.cy[cc]);
        const double d2 = __dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy));
        const double inv = rcp_nr(d2);
        const double2 w = make_double2(__dmul_rn(dx, inv), -__dmul_rn(dy, inv));
        const double2 *cf = t.coef + (size_t)cc * nt;
        // Horner, each step acc <- acc w + a_k as two FMAs per component
        // (four per term against six for a product and a sum), and the
        // last product added into phi the same way
        double2 acc = cf[nt - 2];
        for (int k = nt - 3; k >= 0; k--) acc = cfma(acc, w, cf[k]);
        phi = cfma(acc, w, phi);
      }
    }
    const int done = min(rounds, nq);
    qh = (qh + done) & (kQueue - 1);
    nq -= done;
  };

  // The direct sums are deferred the same way: a leaf reached by some of
  // the warp's lanes would keep the others idle for its whole pair loop,
  // and on this GPU an FP64 warp instruction takes the pipe for its full
  // width whatever the lanes.  Each lane queues its leaves
  // (s_leaves[warp][k][lane]) and the warp walks the queues together, one
  // pair per lane per step, each lane through its own leaves in its own
  // order.  A lane's pairs reach ax/ay and its leaf sums reach ud0/ud1 in
  // the order and with the operations of an immediate evaluation, so the
  // results are the same bit for bit.
  int nl = 0;
  auto flush_leaves = [&]() {
    int q = 0, j = 0, e = 0;
    double ax = 0.0, ay = 0.0;
    if (nl > 0) {
      const int c0 = s_leaves[warp][0][lane];
      j = t.begin[c0];
      e = t.end[c0];
    }
    // closes the leaves whose pairs are done (empty ones too) and opens the
    // next: the reference adds 0.5 ax / pi per leaf (fmm.c:140-141); a
    // product by 1/(2 pi) instead of the FP64 division (an ulp apart)
    auto settle = [&]() {
      while (q < nl && j >= e) {
        ud0 = __dadd_rn(ud0, __dmul_rn(ax, kInv2Pi));
        ud1 = __dadd_rn(ud1, __dmul_rn(ay, kInv2Pi));
        ax = 0.0;
        ay = 0.0;
        if (++q < nl) {
          const int cq = s_leaves[warp][q][lane];
          j = t.begin[cq];
          e = t.end[cq];
        }
      }
    };
    settle();
    while (__any_sync(0xffffffffu, q < nl)) {
      if (q < nl) {
        // direct_evaluate, fmm.c:121-142
        const double rx = __dsub_rn(x, t.x[j]);
        const double ry = __dsub_rn(y, t.y[j]);
        // The reference forms r = sqrt(r2), (r/sigma)^2 and 1/(r*r); here
        // r2 and r2/sigma^2 (with 1/sigma^2 precomputed per blob) give the
        // same quantities within an ulp or two and save the square root
        // and a division per pair.  r > 1e-10 <=> r2 > 1e-20.
        const double r2 = __dadd_rn(__dmul_rn(rx, rx), __dmul_rn(ry, ry));
        if (r2 > 1.0e-20) {
          const double rv2 = rcp_nr(r2);
          const double x2 = __dmul_rn(r2, t.icor2[j]);
          // 1 - exp(-x2) rounds to exactly 1.0 once exp(-x2) < 2^-54
          // (x2 > 37.4); the shortcut keeps the result bit-identical.
          const double e1 = x2 > 40.0 ? 1.0 : 1.0 - exp(-x2);
          // G (1 - e) / r^2 once, then one FMA per component
          const double f = __dmul_rn(__dmul_rn(t.cir[j], e1), rv2);
          ax = __fma_rn(-f, ry, ax);
          ay = __fma_rn(f, rx, ay);
        }
        n_pairs++;
        j++;
        settle();
      }
    }
    nl = 0;
  };

  int top = 0;
  if (lane == 0) {
    s_cell[warp][0] = 0;
    s_mask[warp][0] = vmask;
  }
  __syncwarp();
  while (top >= 0) {
    const int c = s_cell[warp][top];
    const unsigned m = s_mask[warp][top];
    __syncwarp();
    top--;
    const bool act = (m >> lane) & 1u;
    if (t.leaf[c]) {
      if (__any_sync(0xffffffffu, nl == kLeafQueue)) flush_leaves();
      if (act) s_leaves[warp][nl++][lane] = c;
    } else {
      // a cell's four children can add four entries to a lane's queue
      if (__any_sync(0xffffffffu, nq > kQueue - 4)) flush(false);
      const int4 ch = reinterpret_cast<const int4 *>(t.child)[c];
#pragma unroll 1
      for (int q = 0; q < 4; q++) {
        const int cc = (&ch.x)[q];
        if (cc < 0) continue;
        bool desc = false;
        if (act) {
          // The reference's test is region > theta * sqrt(d2), each step
          // rounded.  Squared, region^2 > theta^2 d2, it needs no square
          // root: below the cell's bound mb.x (region^2 / (theta^2 (1 +
          // 2e-13))) it surely descends, above mb.y (the same with 1 -
          // 2e-13) it surely accepts (the roundings of either side and of
          // the bounds are below 1e-15 relative); only a d2 between the two
          // takes the exact rounded path.
          //
          // An FP64 instruction costs this GPU's SM sub-partition about 64
          // issue cycles, an FP32 one 1, so d2 is first formed in FP32 from
          // the hi/lo pairs: dxf = (xh - cxh) + (xl - cxl).  Its error is at
          // most 2^-23 |dx| + 2^-46 (|x| + |cx|), and so
          //   |d2f - d2| <= 3 2^-23 d2 + 2^-45 S (|dxf| + |dyf|) + (...)^2,
          // S = |x| + |y| + |cx| + |cy|.  err below takes 2^-20 d2f and
          // 2^-44 S, over twice that, so d2f + err < the FP32 lower bound
          // (rounded down from mb.x) means d2 < mb.x, and d2f - err > the
          // upper one (rounded up from mb.y) d2 > mb.y: the FP64 test would
          // decide the same.  Anything else (and any infinity or NaN on the
          // way, where a comparison fails) takes the FP64 test as before.
          const float4 cf = t.cf32[cc];
          const float2 mf = t.macf[cc];
          const float dxf = __fadd_rn(__fsub_rn(xh, cf.x), __fsub_rn(xl, cf.y));
          const float dyf = __fadd_rn(__fsub_rn(yh, cf.z), __fsub_rn(yl, cf.w));
          const float d2f = __fmaf_rn(dxf, dxf, __fmul_rn(dyf, dyf));
          const float ef = __fmul_rn(0x1p-44f, __fadd_rn(sxy, __fadd_rn(fabsf(cf.x), fabsf(cf.z))));
          const float err = __fmaf_rn(0x1p-20f, d2f, __fmul_rn(ef, __fadd_rn(__fadd_rn(fabsf(dxf), fabsf(dyf)), ef)));
          if (__fadd_ru(d2f, err) < mf.x) {
            desc = true;
          } else if (__fsub_rd(d2f, err) > mf.y && d2f <= 3.0e38f) {
            desc = false;
          } else {
            const double2 mb = t.mac[cc];
            const double dx = __dsub_rn(x, t.cx[cc]);
            const double dy = __dsub_rn(y, t.cy[cc]);
            const double d2 = __dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy));
            if (d2 < mb.x) {
              desc = true;
            } else if (d2 > mb.y) {
              desc = false;
            } else {
              desc = t.region[cc] > __dmul_rn(theta, __dsqrt_rn(d2));
            }
          }
        }
        const unsigned dmask = __ballot_sync(0xffffffffu, desc);
        if (act && !desc && nt >= 2) s_queue[warp][(qh + nq++) & (kQueue - 1)][lane] = cc;
        if (act && !desc) n_m2s++;
        if (dmask) {
          if (top + 1 >= kStackCap) {
            overflow = true;
            break;
          }
          top++;
          if (lane == 0) {
            s_cell[warp][top] = cc;
            s_mask[warp][top] = dmask;
          }
        }
        __syncwarp();
      }
      if (__any_sync(0xffffffffu, overflow)) break;
    }
  }
  flush(true);
  flush_leaves();
  if (__any_sync(0xffffffffu, overflow)) {
    if (lane == 0) set_err(a.st, TREE2D_ERR_TIMEOUT);
  }
  if (valid) {
    // fmm.c:115-117
    const double pre = (0.5 * -phi.y) / kPi;
    const double pim = (0.5 * phi.x) / kPi;
    const double u = -pre + ud0;
    const double v = pim + ud1;
    const long o = a.out_idx ? a.out_idx[i] : i;
    a.uv[2 * o] = overflow ? NAN : u;
    a.uv[2 * o + 1] = overflow ? NAN : v;
  }
  for (int o = 16; o; o >>= 1) {
    n_m2s += __shfl_xor_sync(0xffffffffu, n_m2s, o);
    n_pairs += __shfl_xor_sync(0xffffffffu, n_pairs, o);
  }
  if (lane == 0) {
    atomicAdd(&a.st->n_m2s, n_m2s);
    atomicAdd(&a.st->n_pairs, n_pairs);
  }
}

// The opening test's bounds per cell for a given theta: squared distances
// d2 with d2 < lo surely have region > theta sqrt(d2) (the cell is opened),
// d2 > hi surely not (it is accepted), with a relative margin of 2e-13 that
// covers the roundings of the reference's test and of the bounds.  With
// theta <= 0 the reference's test opens every cell (region > 0 >= theta r):
// both bounds are +inf.
//
// For the FP32 pre-test of k_eval: the centre as two FP32 pairs (hi = the
// nearest float, lo = the rest, rounded) and the bounds rounded outwards to
// FP32; a lower bound below 1e-30 becomes -1 and an upper one below 1e-30
// +inf (no sure answer: the FP32 error bound does not cover subnormals).
__global__ void k_mac_bounds(Tree t, double theta) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= t.ncell) return;
  const double r2 = t.region[c] * t.region[c], th2 = theta * theta;
  const double2 mb = theta > 0.0 ? make_double2(r2 / (th2 * (1.0 + 2e-13)), r2 / (th2 * (1.0 - 2e-13)))
                                 : make_double2(INFINITY, INFINITY);
  t.mac[c] = mb;
  const double cx = t.cx[c], cy = t.cy[c];
  const float cxh = __double2float_rn(cx), cyh = __double2float_rn(cy);
  t.cf32[c] = make_float4(cxh, __double2float_rn(cx - (double)cxh), cyh, __double2float_rn(cy - (double)cyh));
  t.macf[c] = make_float2(mb.x >= 1e-30 ? __double2float_rd(mb.x) : -1.0f,
                          mb.y >= 1e-30 ? __double2float_ru(mb.y) : INFINITY);
}

cudaError_t mac_bounds(Workspace &ws, const Tree &t, double theta, cudaStream_t s) {
  if (ws.mac_theta == theta || t.ncell <= 0) return cudaSuccess;
  k_mac_bounds<<<(t.ncell + 255) / 256, 256, 0, s>>>(t, theta);
  ::t2d::g_launches.fetch_add(1, std::memory_order_relaxed);
  const cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) ws.mac_theta = theta;
  return e;
}

// Binomial table, uploaded once per device (the table lives in each
// device's copy of the module).
bool g_binom_ready[64] = {};

cudaError_t upload_binom() {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev >= 0 && dev < 64 && g_binom_ready[dev]) return cudaSuccess;
  static double h[kMaxTerms][kMaxTerms];
  for (int n = 0; n < kMaxTerms; n++) {
    h[n][0] = 1.0;
    for (int k = 1; k < kMaxTerms; k++) h[n][k] = k > n ? 0.0 : h[n][k - 1] * (double)(n - k + 1) / (double)k;
  }
  // exact: every C(n,k), n < 32, is an integer below 2^53 and the running
  // product above stays integral (C(n,k-1)*(n-k+1) is divisible by k).
  e = cudaMemcpyToSymbol(c_binom, h, sizeof(h));
  if (e == cudaSuccess && dev >= 0 && dev < 64) g_binom_ready[dev] = true;
  return e;
}

}  // namespace

int plain_upward(Workspace &ws, const Tree &t, const Params &p, cudaStream_t s) {
  T2D_CUDA_TRY(upload_binom());
  const int nt = p.nterms;
  long tot = (long)t.ncell * nt;
  if (tot == 0) return TREE2D_OK;
  k_zero_internal<<<(int)((tot + 255) / 256), 256, 0, s>>>(t, nt);
  ::t2d::g_launches.fetch_add(1, std::memory_order_relaxed);
  if (t.nleaf > 0) k_s2m<<<(int)(((long)t.nleaf * 32 + 255) / 256), 256, 0, s>>>(t, nt);
  ::t2d::g_launches.fetch_add(1, std::memory_order_relaxed);
  const int blocks = (int)(((long)t.ncell * 32 + 255) / 256);
  for (int lev = t.depth - 1; lev >= 1; lev--) k_m2m<<<blocks, 256, 0, s>>>(t, nt, lev);
  ::t2d::g_launches.fetch_add(1, std::memory_order_relaxed);
  T2D_CUDA_TRY(cudaGetLastError());
  return TREE2D_OK;
}

int plain_evaluate(Workspace &ws, const Tree &t, const Params &p, int ntgt, const double *tx, const double *ty,
                   const int *out_idx, double *uv, cudaStream_t s) {
  if (ntgt <= 0) return TREE2D_OK;
  T2D_CUDA_TRY(mac_bounds(ws, t, p.theta, s));
  EvalArgs a{t, p.nterms, p.theta, ntgt, tx, ty, out_idx, uv, ws.status};
  const int warps = (ntgt + 31) / 32;
  k_eval<<<(warps + kEvalWarps - 1) / kEvalWarps, kEvalWarps * 32, 0, s>>>(a);
  ::t2d::g_launches.fetch_add(1, std::memory_order_relaxed);
  T2D_CUDA_TRY(cudaGetLastError());
  return TREE2D_OK;
}

}  // namespace t2d
