// Learned order selection: features, labels, and the training kernels of
// the MLP (BF16 weights and layer inputs, FP32 accumulation).
//
// What the network decides.  In the mixed FMM the near field of a leaf B is
// its U list (adjacent leaves, exact regularised P2P) and its K list (leaves
// within the cutoff, Gaussian correction).  For each such interaction the
// network picks the cheapest treatment whose error stays under a budget:
// direct evaluation (class 0), or the source leaf's multipole at order
// p = 4..16 (classes 1..13; for a K interaction this means the correction
// is skipped because the far field already covers the point-vortex part).
// The fixed form (all interactions direct) is the fallback when no trained
// weights are loaded.
//
// Labels come from the FMM itself against the FP64 exact contribution of
// the interaction (the direct sum restricted to it): `k_labels`.  Training
// runs on the GPU: tiled FP32 GEMMs over BF16-rounded operands, GELU,
// softmax cross-entropy and Adam, one kernel each; gradients are checked
// against the CPU oracle (oracle/mlp_oracle.py).
#include <cuda_bf16.h>

#include <cmath>
#include <cstring>

#include "dev_common.cuh"
#include "learn.h"

namespace t2d {

namespace {

__global__ void k_leaf_stats(MixedView m, LeafStats *out) {
  const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (w >= m.nleaf) return;
  const int c = m.leaf_cell[w];
  const float ih = m.inv_h[c];
  float ga = 0.f, mx = 0.f, my = 0.f, m2 = 0.f, sg = 0.f;
  for (int j = m.begin[c] + lane; j < m.end[c]; j += 32) {
    const float4 s = m.src4[j];
    const float g = fabsf(s.z);
    const float zx = s.x * ih, zy = s.y * ih;
    ga += g;
    mx += s.z * zx;
    my += s.z * zy;
    m2 += g * (zx * zx + zy * zy);
    sg = fmaxf(sg, rsqrtf(fmaxf(-s.w * 0.69314718f, 1e-30f)));  // s.w = -log2(e)/sigma^2
  }
  for (int o = 16; o; o >>= 1) {
    ga += __shfl_xor_sync(0xffffffffu, ga, o);
    mx += __shfl_xor_sync(0xffffffffu, mx, o);
    my += __shfl_xor_sync(0xffffffffu, my, o);
    m2 += __shfl_xor_sync(0xffffffffu, m2, o);
    sg = fmaxf(sg, __shfl_xor_sync(0xffffffffu, sg, o));
  }
  if (lane == 0) {
    LeafStats r;
    r.g_abs = ga;
    r.m1 = ga > 0.f ? sqrtf(mx * mx + my * my) / ga : 0.f;
    r.m2 = ga > 0.f ? m2 / ga : 0.f;
    r.sig = sg;
    out[c] = r;
  }
}

__device__ __forceinline__ float2 cmulf(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// One warp per sampled interaction.  samples[3*i] = leaf ordinal,
// [3*i+1] = kind (0 U, 1 K), [3*i+2] = entry index in that list.
__global__ void k_labels(MixedView m, const LeafStats *st, const float *u_ref_ptr, double tol, int ns,
                         const int *samples, float *features, int *labels) {
  const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (w >= ns) return;
  const int l = samples[3 * w], kind = samples[3 * w + 1], e = samples[3 * w + 2];
  const int B = m.leaf_cell[l];
  const int A = kind == 0 ? m.u_idx[e] : m.k_idx[e];
  const float u_ref = *u_ref_ptr;
  const int P = m.P;
  const double ox = m.cx[B] - m.cx[A], oy = m.cy[B] - m.cy[A];
  const float oxf = centre_offset(m.cxf, m.cxl, B, A), oyf = centre_offset(m.cyf, m.cyl, B, A);
  const float ihA = m.inv_h[A];
  const float *MA = m.M + (size_t)A * 2 * P;
  double err[14];
  // orders beyond the stored expansion cannot be used
  for (int c = 0; c < 14; c++) err[c] = (kind == 0 && class_order(c) > P) ? 1e300 : 0.0;
  for (int t0 = m.begin[B]; t0 < m.end[B]; t0 += 32) {
    const int t = t0 + lane;
    const bool valid = t < m.end[B];
    const float2 zt = valid ? m.loc[t] : make_float2(0.f, 0.f);
    // exact contribution in FP64
    double ex = 0.0, ey = 0.0;
    for (int j = m.begin[A]; j < m.end[A]; j++) {
      const float4 s = m.src4[j];
      const double rx = ((double)zt.x - (double)s.x) + ox, ry = ((double)zt.y - (double)s.y) + oy;
      const double r2 = rx * rx + ry * ry;
      const double r = sqrt(r2);
      // s.w = -log2(e)/sigma^2, so exp(-r^2/sigma^2) = 2^(r^2 s.w)
      if (kind == 0) {
        if (r > 1e-10) {
          const double f = (double)s.z * (1.0 - exp2(r2 * (double)s.w)) / r2;
          ex -= f * ry;
          ey += f * rx;
        }
      } else if (r > 1e-10) {
        const double f = -(double)s.z * exp2(r2 * (double)s.w) / r2;
        ex -= f * ry;
        ey += f * rx;
      }
    }
    if (kind == 1) {
      // skipping the correction leaves exactly this out
      const double em = valid ? sqrt(ex * ex + ey * ey) : 0.0;
      for (int c = 1; c < 14; c++) err[c] = fmax(err[c], em);
    } else {
      // the source leaf's multipole at order p (FP32, as the evaluation does)
      const float zx = (zt.x + oxf) * ihA, zy = (zt.y + oyf) * ihA;
      const float ir2 = 1.f / (zx * zx + zy * zy);
      const float2 wv = make_float2(zx * ir2, -zy * ir2);
      float2 pw = wv;       // w^(k+1)
      float2 phi = make_float2(0.f, 0.f);
      for (int k = 0; k < 16 && k < P; k++) {
        const float2 a = make_float2(MA[k], MA[P + k]);
        const float2 t2 = cmulf(a, pw);
        phi.x += t2.x * ihA;
        phi.y += t2.y * ihA;
        pw = cmulf(pw, wv);
        const int p = k + 1;  // terms 0..k used
        if (p >= 4) {
          const double dx = (double)phi.y - ex, dy = (double)phi.x - ey;
          const double em = (valid && isfinite(dx) && isfinite(dy)) ? sqrt(dx * dx + dy * dy) : (valid ? 1e300 : 0.0);
          err[p - 3] = fmax(err[p - 3], em);
        }
      }
      if (A == B) for (int c = 1; c < 14; c++) err[c] = valid ? 1e300 : err[c];
    }
  }
  for (int c = 1; c < 14; c++)
    for (int o = 16; o; o >>= 1) err[c] = fmax(err[c], __shfl_xor_sync(0xffffffffu, err[c], o));
  if (lane == 0) {
    int label = 0;
    if (kind == 1) {
      label = err[1] <= tol ? 1 : 0;
    } else {
      for (int c = 1; c < 14; c++)
        if (err[c] <= tol) {
          label = c;
          break;
        }
    }
    labels[w] = label;
    float f[kMlpIn];
    interaction_features(m, st, B, A, kind, u_ref, f);
    for (int k = 0; k < kMlpIn; k++) features[(size_t)w * kMlpIn + k] = f[k];
  }
}

// ------------------------------------------------------------ training

__device__ __forceinline__ float bf16r(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }

__device__ __forceinline__ float gelu_f(float z) {
  const float c = 0.7978845608028654f;
  return 0.5f * z * (1.f + tanhf(c * (z + 0.044715f * z * z * z)));
}
__device__ __forceinline__ float gelu_grad_f(float z) {
  const float c = 0.7978845608028654f;
  const float t = tanhf(c * (z + 0.044715f * z * z * z));
  return 0.5f * (1.f + t) + 0.5f * z * (1.f - t * t) * c * (1.f + 3.f * 0.044715f * z * z);
}

// C(i,j) = beta*C(i,j) + sum_k A(i,k) B(k,j) (+ bias[j]); A(i,k) =
// A[i*sa0 + k*sa1], B(k,j) = B[k*sb0 + j*sb1], C row-major ldc.  32x32 tiles.
__global__ void __launch_bounds__(256) k_gemm(int M, int N, int K, const float *A, long sa0, long sa1, const float *Bm,
                                              long sb0, long sb1, float *C, int ldc, const float *bias, int beta) {
  __shared__ float As[32][33], Bs[32][33];
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8
  const int i0 = blockIdx.y * 32, j0 = blockIdx.x * 32;
  float acc[4] = {0.f, 0.f, 0.f, 0.f};
  for (int k0 = 0; k0 < K; k0 += 32) {
    for (int r = ty; r < 32; r += 8) {
      const int i = i0 + r, k = k0 + tx;
      As[r][tx] = (i < M && k < K) ? A[(long)i * sa0 + (long)k * sa1] : 0.f;
      const int kk = k0 + r, j = j0 + tx;
      Bs[r][tx] = (kk < K && j < N) ? Bm[(long)kk * sb0 + (long)j * sb1] : 0.f;
    }
    __syncthreads();
    for (int k = 0; k < 32; k++) {
      const float b = Bs[k][tx];
      for (int q = 0; q < 4; q++) acc[q] = fmaf(As[ty + 8 * q][k], b, acc[q]);
    }
    __syncthreads();
  }
  const int j = j0 + tx;
  if (j >= N) return;
  for (int q = 0; q < 4; q++) {
    const int i = i0 + ty + 8 * q;
    if (i >= M) continue;
    float v = acc[q] + (bias ? bias[j] : 0.f);
    C[(long)i * ldc + j] = beta ? C[(long)i * ldc + j] + v : v;
  }
}

// mode 0: A = bf16(gelu(Z)); mode 1: D = D * gelu'(Z)
__global__ void k_act(int n, const float *Z, float *out, int mode) {
  long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (mode == 0)
    out[i] = bf16r(gelu_f(Z[i]));
  else
    out[i] *= gelu_grad_f(Z[i]);
}

__device__ __forceinline__ uint32_t hash32(uint32_t x) {
  x ^= x >> 16;
  x *= 0x7feb352du;
  x ^= x >> 15;
  x *= 0x846ca68bu;
  x ^= x >> 16;
  return x;
}

// Mini-batch rows: X rows (BF16-rounded) and labels, drawn uniformly.
__global__ void k_gather_batch(int n, const float *X, const int *y, int bt, unsigned seed, float *A0, int *yb) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= bt) return;
  const int r = seed == 0xffffffffu ? i : (int)(hash32(seed * 2654435761u + (unsigned)i) % (unsigned)n);
  for (int k = 0; k < kMlpIn; k++) A0[(long)i * kMlpIn + k] = bf16r(X[(long)r * kMlpIn + k]);
  yb[i] = y[r];
}

// D4 = (softmax(Z4[:, :14]) - onehot) / bt, loss summed into *loss.
__global__ void k_softmax_ce(int bt, const float *Z4, const int *yb, float *D4, float *loss) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= bt) return;
  const float *z = Z4 + (long)i * kMlpOut;
  float mx = z[0];
  for (int c = 1; c < kMlpClasses; c++) mx = fmaxf(mx, z[c]);
  float p[kMlpClasses], s = 0.f;
  for (int c = 0; c < kMlpClasses; c++) {
    p[c] = expf(z[c] - mx);
    s += p[c];
  }
  const int y = yb[i];
  for (int c = 0; c < kMlpOut; c++) {
    float d = c < kMlpClasses ? p[c] / s : 0.f;
    if (c == y) d -= 1.f;
    D4[(long)i * kMlpOut + c] = d / (float)bt;
  }
  atomicAdd(loss, -logf(fmaxf(p[y] / s, 1e-30f)) / (float)bt);
}

__global__ void k_colsum(int rows, int cols, const float *D, float *out) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= cols) return;
  float s = 0.f;
  for (int i = 0; i < rows; i++) s += D[(long)i * cols + j];
  out[j] = s;
}

__global__ void k_round_weights(int n, const float *theta, float *wb) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) wb[i] = bf16r(theta[i]);
}

__global__ void k_adam(int n, float *theta, float *m1, float *v1, const float *g, float lr, float b1c, float b2c) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float b1 = 0.9f, b2 = 0.999f;
  const float mi = b1 * m1[i] + (1.f - b1) * g[i];
  const float vi = b2 * v1[i] + (1.f - b2) * g[i] * g[i];
  m1[i] = mi;
  v1[i] = vi;
  theta[i] -= lr * (mi / b1c) / (sqrtf(vi / b2c) + 1e-8f);
}

struct Offs {
  int W1, b1, W2, b2, W3, b3, W4, b4;
};
constexpr Offs kOff{0, 1024, 1088, 5184, 5248, 9344, 9408, 10432};

// Scratch of one mini-batch pass.
struct Pass {
  float *A0, *Z1, *A1, *Z2, *A2, *Z3, *A3, *Z4, *D4, *D3, *D2, *D1;
  int *yb;
};

void gemm(cudaStream_t s, int M, int N, int K, const float *A, long sa0, long sa1, const float *B, long sb0, long sb1,
          float *C, int ldc, const float *bias, int beta) {
  dim3 g((N + 31) / 32, (M + 31) / 32);
  k_gemm<<<g, 256, 0, s>>>(M, N, K, A, sa0, sa1, B, sb0, sb1, C, ldc, bias, beta);
  g_launches.fetch_add(1, std::memory_order_relaxed);
}

void forward_pass(cudaStream_t s, int bt, const float *wb, const float *theta, Pass &p) {
  const int H = kMlpHidden;
  gemm(s, bt, H, kMlpIn, p.A0, kMlpIn, 1, wb + kOff.W1, 1, kMlpIn, p.Z1, H, theta + kOff.b1, 0);
  k_act<<<(bt * H + 255) / 256, 256, 0, s>>>(bt * H, p.Z1, p.A1, 0);
  gemm(s, bt, H, H, p.A1, H, 1, wb + kOff.W2, 1, H, p.Z2, H, theta + kOff.b2, 0);
  k_act<<<(bt * H + 255) / 256, 256, 0, s>>>(bt * H, p.Z2, p.A2, 0);
  gemm(s, bt, H, H, p.A2, H, 1, wb + kOff.W3, 1, H, p.Z3, H, theta + kOff.b3, 0);
  k_act<<<(bt * H + 255) / 256, 256, 0, s>>>(bt * H, p.Z3, p.A3, 0);
  gemm(s, bt, kMlpOut, H, p.A3, H, 1, wb + kOff.W4, 1, H, p.Z4, kMlpOut, theta + kOff.b4, 0);
  g_launches.fetch_add(3, std::memory_order_relaxed);
}

void backward_pass(cudaStream_t s, int bt, const float *wb, Pass &p, float *g) {
  const int H = kMlpHidden;
  // layer 4
  gemm(s, kMlpOut, H, bt, p.D4, 1, kMlpOut, p.A3, H, 1, g + kOff.W4, H, nullptr, 0);
  k_colsum<<<1, 64, 0, s>>>(bt, kMlpOut, p.D4, g + kOff.b4);
  gemm(s, bt, H, kMlpOut, p.D4, kMlpOut, 1, wb + kOff.W4, H, 1, p.D3, H, nullptr, 0);
  k_act<<<(bt * H + 255) / 256, 256, 0, s>>>(bt * H, p.Z3, p.D3, 1);
  // layer 3
  gemm(s, H, H, bt, p.D3, 1, H, p.A2, H, 1, g + kOff.W3, H, nullptr, 0);
  k_colsum<<<1, 64, 0, s>>>(bt, H, p.D3, g + kOff.b3);
  gemm(s, bt, H, H, p.D3, H, 1, wb + kOff.W3, H, 1, p.D2, H, nullptr, 0);
  k_act<<<(bt * H + 255) / 256, 256, 0, s>>>(bt * H, p.Z2, p.D2, 1);
  // layer 2
  gemm(s, H, H, bt, p.D2, 1, H, p.A1, H, 1, g + kOff.W2, H, nullptr, 0);
  k_colsum<<<1, 64, 0, s>>>(bt, H, p.D2, g + kOff.b2);
  gemm(s, bt, H, H, p.D2, H, 1, wb + kOff.W2, H, 1, p.D1, H, nullptr, 0);
  k_act<<<(bt * H + 255) / 256, 256, 0, s>>>(bt * H, p.Z1, p.D1, 1);
  // layer 1
  gemm(s, H, kMlpIn, bt, p.D1, 1, H, p.A0, kMlpIn, 1, g + kOff.W1, kMlpIn, nullptr, 0);
  k_colsum<<<1, 64, 0, s>>>(bt, H, p.D1, g + kOff.b1);
  g_launches.fetch_add(7, std::memory_order_relaxed);
}

size_t pass_floats(int bt) { return (size_t)bt * (kMlpIn + 11 * kMlpHidden + 3 * kMlpOut) + 4 * 256; }

void carve(float *base, int bt, Pass &p) {
  const size_t H = (size_t)bt * kMlpHidden;
  float *q = base;
  p.A0 = q, q += (size_t)bt * kMlpIn;
  p.Z1 = q, q += H;
  p.A1 = q, q += H;
  p.Z2 = q, q += H;
  p.A2 = q, q += H;
  p.Z3 = q, q += H;
  p.A3 = q, q += H;
  p.Z4 = q, q += (size_t)bt * kMlpOut;
  p.D4 = q, q += (size_t)bt * kMlpOut;
  p.D3 = q, q += H;
  p.D2 = q, q += H;
  p.D1 = q, q += H;
  p.yb = reinterpret_cast<int *>(q);
}

}  // namespace

// u_ref = sum |G| / R0 (deterministic: fixed per-thread ranges, tree sum).
__global__ void __launch_bounds__(1024) k_uref(MixedView m, const LeafStats *st, const RootBox *root, float *out) {
  __shared__ float part[1024];
  const int t = threadIdx.x;
  const int per = (m.nleaf + 1023) / 1024;
  float s = 0.f;
  for (int l = t * per; l < min(m.nleaf, (t + 1) * per); l++) s += st[m.leaf_cell[l]].g_abs;
  part[t] = s;
  __syncthreads();
  for (int o = 512; o; o >>= 1) {
    if (t < o) part[t] += part[t + o];
    __syncthreads();
  }
  if (t == 0) *out = part[0] / (float)root->region;
}

// The leaves of each set of a batched tree: one contiguous range of the
// leaf order (a set's cells are the subtree of its root), [lo[k], hi[k]).
__global__ void k_set_leaf_ranges(MixedView m, int *lo, int *hi) {
  const int l = blockIdx.x * blockDim.x + threadIdx.x;
  if (l >= m.nleaf) return;
  const int k = set_of_cell(m, m.leaf_cell[l]);
  if (l == 0 || set_of_cell(m, m.leaf_cell[l - 1]) != k) lo[k] = l;
  if (l == m.nleaf - 1 || set_of_cell(m, m.leaf_cell[l + 1]) != k) hi[k] = l + 1;
}

// k_uref for each set of a batched tree, one block per set: the set's leaves
// in order, split over the threads as k_uref splits a single tree's, so that
// a set's u_ref is the one it gets alone, bit for bit.
__global__ void __launch_bounds__(1024) k_uref_sets(MixedView m, const LeafStats *st, const RootBox *root,
                                                    const int *lo, const int *hi, float *out) {
  __shared__ float part[1024];
  const int k = blockIdx.x, t = threadIdx.x;
  const int l0 = lo[k], cnt = max(hi[k] - l0, 0);
  const int per = (cnt + 1023) / 1024;
  float s = 0.f;
  for (int l = t * per; l < min(cnt, (t + 1) * per); l++) s += st[m.leaf_cell[l0 + l]].g_abs;
  part[t] = s;
  __syncthreads();
  for (int o = 512; o; o >>= 1) {
    if (t < o) part[t] += part[t + o];
    __syncthreads();
  }
  if (t == 0) out[k] = part[0] / (float)root[k].region;
}

int learned_uref_sets(MixedView &m, const LeafStats *stats, const RootBox *roots, int nsets, int *leaf_lo,
                      int *leaf_hi, float *out, cudaStream_t s) {
  if (nsets <= 0) return TREE2D_OK;
  T2D_CUDA_TRY(cudaMemsetAsync(leaf_lo, 0, sizeof(int) * (size_t)nsets, s));
  T2D_CUDA_TRY(cudaMemsetAsync(leaf_hi, 0, sizeof(int) * (size_t)nsets, s));
  if (m.nleaf > 0) k_set_leaf_ranges<<<(m.nleaf + 255) / 256, 256, 0, s>>>(m, leaf_lo, leaf_hi);
  k_uref_sets<<<nsets, 1024, 0, s>>>(m, stats, roots, leaf_lo, leaf_hi, out);
  g_launches.fetch_add(2, std::memory_order_relaxed);
  T2D_CUDA_TRY(cudaGetLastError());
  return TREE2D_OK;
}

int learned_uref(MixedView &m, const LeafStats *stats, const RootBox *root, float *out, cudaStream_t s) {
  k_uref<<<1, 1024, 0, s>>>(m, stats, root, out);
  g_launches.fetch_add(1, std::memory_order_relaxed);
  T2D_CUDA_TRY(cudaGetLastError());
  return TREE2D_OK;
}

int learned_leaf_stats(MixedView &m, LeafStats *stats, cudaStream_t s) {
  k_leaf_stats<<<(int)(((long)m.nleaf * 32 + 255) / 256), 256, 0, s>>>(m, stats);
  g_launches.fetch_add(1, std::memory_order_relaxed);
  T2D_CUDA_TRY(cudaGetLastError());
  return TREE2D_OK;
}

int learned_labels(MixedView &m, const LeafStats *stats, const float *u_ref_ptr, double tol, int ns,
                   const int *samples, float *features, int *labels, cudaStream_t s) {
  if (ns <= 0) return TREE2D_OK;
  k_labels<<<(int)(((long)ns * 32 + 255) / 256), 256, 0, s>>>(m, stats, u_ref_ptr, tol, ns, samples, features,
                                                               labels);
  g_launches.fetch_add(1, std::memory_order_relaxed);
  T2D_CUDA_TRY(cudaGetLastError());
  return TREE2D_OK;
}

int mlp_train(int n, const float *X, const int *y, float *theta, float *m1, float *v1, int steps, int batch,
              float lr, unsigned seed, float *loss_out, cudaStream_t s) {
  if (n <= 0 || steps <= 0 || batch <= 0) return TREE2D_ERR_BAD_INPUT;
  float *buf = nullptr;
  const size_t nf = pass_floats(batch) + 2 * kMlpParams + 1;
  T2D_CUDA_TRY(cudaMalloc(reinterpret_cast<void **>(&buf), nf * sizeof(float)));
  Pass p;
  carve(buf, batch, p);
  float *wb = buf + pass_floats(batch);
  float *g = wb + kMlpParams;
  float *loss = g + kMlpParams;
  T2D_CUDA_TRY(cudaMemsetAsync(loss, 0, sizeof(float), s));
  const int pb = (kMlpParams + 255) / 256;
  for (int it = 0; it < steps; it++) {
    k_round_weights<<<pb, 256, 0, s>>>(kMlpParams, theta, wb);
    k_gather_batch<<<(batch + 255) / 256, 256, 0, s>>>(n, X, y, batch, seed + (unsigned)it * 7919u, p.A0, p.yb);
    forward_pass(s, batch, wb, theta, p);
    if (it == steps - 1) T2D_CUDA_TRY(cudaMemsetAsync(loss, 0, sizeof(float), s));
    k_softmax_ce<<<(batch + 255) / 256, 256, 0, s>>>(batch, p.Z4, p.yb, p.D4, loss);
    backward_pass(s, batch, wb, p, g);
    const float b1c = 1.f - powf(0.9f, (float)(it + 1)), b2c = 1.f - powf(0.999f, (float)(it + 1));
    k_adam<<<pb, 256, 0, s>>>(kMlpParams, theta, m1, v1, g, lr, b1c, b2c);
    g_launches.fetch_add(4, std::memory_order_relaxed);
  }
  T2D_CUDA_TRY(cudaGetLastError());
  if (loss_out) T2D_CUDA_TRY(cudaMemcpyAsync(loss_out, loss, sizeof(float), cudaMemcpyDeviceToHost, s));
  cudaError_t e = cudaStreamSynchronize(s);
  cudaFree(buf);
  T2D_CUDA_TRY(e);
  return TREE2D_OK;
}

int mlp_grad(int n, const float *X, const int *y, const float *theta, float *grad, float *loss_out, cudaStream_t s) {
  if (n <= 0) return TREE2D_ERR_BAD_INPUT;
  float *buf = nullptr;
  const size_t nf = pass_floats(n) + kMlpParams + 1;
  T2D_CUDA_TRY(cudaMalloc(reinterpret_cast<void **>(&buf), nf * sizeof(float)));
  Pass p;
  carve(buf, n, p);
  float *wb = buf + pass_floats(n);
  float *loss = wb + kMlpParams;
  T2D_CUDA_TRY(cudaMemsetAsync(loss, 0, sizeof(float), s));
  k_round_weights<<<(kMlpParams + 255) / 256, 256, 0, s>>>(kMlpParams, theta, wb);
  k_gather_batch<<<(n + 255) / 256, 256, 0, s>>>(n, X, y, n, 0xffffffffu, p.A0, p.yb);
  forward_pass(s, n, wb, theta, p);
  k_softmax_ce<<<(n + 255) / 256, 256, 0, s>>>(n, p.Z4, p.yb, p.D4, loss);
  backward_pass(s, n, wb, p, grad);
  g_launches.fetch_add(3, std::memory_order_relaxed);
  T2D_CUDA_TRY(cudaMemcpyAsync(loss_out, loss, sizeof(float), cudaMemcpyDeviceToHost, s));
  cudaError_t e = cudaStreamSynchronize(s);
  cudaFree(buf);
  T2D_CUDA_TRY(e);
  return TREE2D_OK;
}

int mlp_forward_cc(int n, const float *X, const float *theta, float *logits, cudaStream_t s) {
  if (n <= 0) return TREE2D_OK;
  float *buf = nullptr;
  const size_t nf = pass_floats(n) + kMlpParams;
  T2D_CUDA_TRY(cudaMalloc(reinterpret_cast<void **>(&buf), nf * sizeof(float)));
  Pass p;
  carve(buf, n, p);
  float *wb = buf + pass_floats(n);
  int *yz = p.yb;
  T2D_CUDA_TRY(cudaMemsetAsync(yz, 0, sizeof(int) * (size_t)n, s));
  k_round_weights<<<(kMlpParams + 255) / 256, 256, 0, s>>>(kMlpParams, theta, wb);
  // rows in order, labels unused
  k_gather_batch<<<(n + 255) / 256, 256, 0, s>>>(n, X, yz, n, 0xffffffffu, p.A0, p.yb);
  forward_pass(s, n, wb, theta, p);
  T2D_CUDA_TRY(cudaMemcpyAsync(logits, p.Z4, sizeof(float) * (size_t)n * kMlpOut, cudaMemcpyDeviceToDevice, s));
  g_launches.fetch_add(2, std::memory_order_relaxed);
  cudaError_t e = cudaStreamSynchronize(s);
  cudaFree(buf);
  T2D_CUDA_TRY(e);
  return TREE2D_OK;
}

}  // namespace t2d
