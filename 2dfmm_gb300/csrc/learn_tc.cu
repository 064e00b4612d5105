// Inference of the order-selection MLP on the tensor cores.
//
// A CTA (128 threads) loads the BF16 weight images once (bulk copy) and
// then, for each of its few tiles of 128 interactions, computes the features of
// its rows, and runs the four layers as tcgen05.mma kind::f16 (BF16 A and B,
// FP32 accumulator in TMEM, M = 128, N = 64/64/64/16, K = 16 per
// instruction): layer input tile in shared memory (no-swizzle K-major core
// matrices), accumulator read back with tcgen05.ld, bias + GELU in
// registers, BF16 store as the next layer's input.  The output is the class
// per interaction (argmax over 14 logits, with a bias towards direct
// evaluation), or the raw logits on the checking path.
#include <cuda_bf16.h>

#include <cstring>
#include <vector>

#include "dev_common.cuh"
#include "learn.h"
#include "tc_ptx.cuh"

namespace t2d {
namespace {

constexpr int kTile = 128;
constexpr long kTilesPerCta = 4;
constexpr uint32_t kW1Bytes = 64 * 16 * 2, kW2Bytes = 64 * 64 * 2, kW4Bytes = 16 * 64 * 2;
constexpr uint32_t kWBytes = kW1Bytes + 2 * kW2Bytes + kW4Bytes;  // 20480
constexpr uint32_t kActBytes = kTile * 64 * 2;                     // 16384

struct InferArgs {
  MixedView m;
  const LeafStats *st;
  const float *u_ref_ptr;
  const uint16_t *wimg;
  const float *bias;  // b1[64] b2[64] b3[64] b4[16]
  float direct_bias;
  long n_u, n_k, n_w;
  unsigned char *u_dec, *k_dec, *w_dec;
  const float *X;  // checking path: explicit features [nx][16]
  long nx;
  float *logits;   // checking path output [nx][16]
  long wait_limit;
};

// Two floats rounded to BF16 (round to nearest even), a in the low half.
__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
  const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
  return *reinterpret_cast<const uint32_t *>(&h);
}

// Twice the GELU (tanh form) of two values, returned as the BF16 pair of
// the next layer's input.  The pre-activations are rounded to BF16 and the
// whole GELU runs in packed BF16x2 arithmetic (FMA pipe) with the tanh on
// the SFU (one instruction for both values): the result is stored in BF16
// anyway, and every step rounds at that same 2^-9 relative level.
//   u = z (c0 + c1 z^2),  c0 = sqrt(2/pi), c1 = 0.044715 sqrt(2/pi)
//   2 g = z + z tanh(u)
// The factor 2 is taken out of the next layer's weights (their images are
// halved, learn_weight_images), which is exact in binary floating point:
// z + z t rounds to exactly twice (z/2) + (z/2) t, and each product of a
// halved weight with a doubled input is the same FP32 number as before.
__device__ __forceinline__ uint32_t gelu2x_bf16(float z0, float z1) {
  const uint32_t z = pack_bf16(z0, z1);
  const uint32_t c0 = 0x3F4C3F4Cu;  // 0.797... in both halves (BF16 0x3F4C)
  const uint32_t c1 = 0x3D123D12u;  // 0.0357 in both halves (BF16 0x3D12)
  uint32_t z2, p, u, t, g;
  asm("mul.rn.bf16x2 %0, %1, %1;" : "=r"(z2) : "r"(z));
  asm("fma.rn.bf16x2 %0, %1, %2, %3;" : "=r"(p) : "r"(z2), "r"(c1), "r"(c0));
  asm("mul.rn.bf16x2 %0, %1, %2;" : "=r"(u) : "r"(z), "r"(p));
  asm("tanh.approx.bf16x2 %0, %1;" : "=r"(t) : "r"(u));
  asm("fma.rn.bf16x2 %0, %1, %2, %1;" : "=r"(g) : "r"(z), "r"(t));
  return g;
}

// Row r of the activation tile, K = 8*nk elements: element k at
// (r/8)*SBO + (k/8)*128 + (r%8)*16 + (k%8)*2, SBO = nk*128.
__device__ __forceinline__ void store_row(unsigned char *tile, int r, const float *v, int K) {
  const uint32_t sbo = (uint32_t)(K / 8) * 128;
  unsigned char *base = tile + (uint32_t)(r >> 3) * sbo + (uint32_t)(r & 7) * 16;
  for (int k8 = 0; k8 < K / 8; k8++) {
    uint4 q;
    q.x = pack_bf16(v[8 * k8 + 0], v[8 * k8 + 1]);
    q.y = pack_bf16(v[8 * k8 + 2], v[8 * k8 + 3]);
    q.z = pack_bf16(v[8 * k8 + 4], v[8 * k8 + 5]);
    q.w = pack_bf16(v[8 * k8 + 6], v[8 * k8 + 7]);
    *reinterpret_cast<uint4 *>(base + (uint32_t)k8 * 128) = q;
  }
}

__global__ void __launch_bounds__(kTile) k_mlp_infer(InferArgs a) {
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ uint64_t bar_w, bar_mma;
  __shared__ uint32_t s_tmem;
  __shared__ int s_fail;
  __shared__ __align__(16) float s_bias[64 * 3 + 16];
  unsigned char *wsm = smem;
  unsigned char *act = smem + kWBytes;
  const int tid = threadIdx.x, warp = tid >> 5;
  const long total = a.X ? a.nx : a.n_u + a.n_k + a.n_w;
  const long ntiles = (total + kTile - 1) / kTile;
  if ((long)blockIdx.x >= ntiles) return;

  if (tid == 0) {
    mbar_init(&bar_w, 1);
    mbar_init(&bar_mma, 1);
    s_fail = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  for (int i = tid; i < 64 * 3 + 16; i += kTile) s_bias[i] = a.bias[i];
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&s_tmem)), "r"(64)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = s_tmem;
  bool w_inflight = false;
  if (tid == 0) {
    mbar_expect_tx(&bar_w, kWBytes);
    bulk_g2s(wsm, a.wimg, kWBytes, &bar_w);
    w_inflight = !mbar_wait(&bar_w, 0, a.wait_limit);
    if (w_inflight) s_fail = 1;
  }
  __syncthreads();

  const uint32_t w1 = smem_u32(wsm), w2 = w1 + kW1Bytes, w3 = w2 + kW2Bytes, w4 = w3 + kW2Bytes;
  const uint32_t aaddr = smem_u32(act);
  const uint32_t id64 = (1u << 4) | (1u << 7) | (1u << 10) | ((64u >> 3) << 17) | ((uint32_t)(kTile >> 4) << 24);
  const uint32_t id16 = (1u << 4) | (1u << 7) | (1u << 10) | ((16u >> 3) << 17) | ((uint32_t)(kTile >> 4) << 24);
  const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16);
  uint32_t phase = 0;
  const MixedView &m = a.m;

  bool mma_inflight = false;
  for (long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    if (__syncthreads_or(s_fail)) break;  // uniform exit after a wait gave up
    const long gi = tile * kTile + tid;
    const bool valid = gi < total;
    int kind = 0;
    long e = 0;
    float v[kMlpIn];
    if (!valid) {
      for (int k = 0; k < kMlpIn; k++) v[k] = 0.f;
    } else if (a.X) {
      for (int k = 0; k < kMlpIn; k++) v[k] = a.X[gi * kMlpIn + k];
    } else {
      // U entries, then K entries, then W entries (kind 2), whose source
      // cell's multipole the network sees as a U entry's: an M2P at order p
      // into the target leaf, with the same per-interaction error budget
      kind = gi < a.n_u ? 0 : (gi < a.n_u + a.n_k ? 1 : 2);
      e = kind == 0 ? gi : (kind == 1 ? gi - a.n_u : gi - a.n_u - a.n_k);
      const int l = (kind == 0 ? m.u_leaf : (kind == 1 ? m.k_leaf : m.w_leaf))[e];
      const int B = m.leaf_cell[l];
      const int A = kind == 0 ? m.u_idx[e] : (kind == 1 ? m.k_idx[e] : m.w_idx[e]);
      interaction_features(m, a.st, B, A, kind == 1 ? 1 : 0, a.u_ref_ptr ? uref_of(m, a.u_ref_ptr, B) : 1.f, v);
    }
    store_row(act, tid, v, 16);
    // layer 1 .. 4
    for (int layer = 0; layer < 4; layer++) {
      const int K = layer == 0 ? 16 : 64;
      const int N = layer == 3 ? 16 : 64;
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncthreads();
      if (tid == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t wb = layer == 0 ? w1 : (layer == 1 ? w2 : (layer == 2 ? w3 : w4));
        const uint32_t sbo = (uint32_t)(K / 8) * 128;
        for (int t = 0; t < K / 16; t++) {
          const uint64_t ad = smem_desc(aaddr + (uint32_t)t * 256, 128, sbo);
          const uint64_t bd = smem_desc(wb + (uint32_t)t * 256, 128, sbo);
          mma_bf16(tmem, ad, bd, N == 64 ? id64 : id16, t > 0 ? 1u : 0u);
        }
        mma_commit(&bar_mma);
      }
      if (mbar_wait(&bar_mma, phase, a.wait_limit)) {
        phase ^= 1;
      } else {
        s_fail = 1;
        mma_inflight = true;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      // accumulator row -> bias + GELU -> BF16 row of the next layer's input
      // (32 columns per TMEM load), or bias -> logits after the last layer
      const float *bs = s_bias + layer * 64;
      if (layer < 3) {
        unsigned char *rowp = act + (uint32_t)(tid >> 3) * 1024u + (uint32_t)(tid & 7) * 16u;  // SBO = 8*128
        for (int c0 = 0; c0 < 64; c0 += 32) {
          uint32_t r[32];
          tmem_ld32(taddr + (uint32_t)c0, r);
          tmem_wait();
#pragma unroll
          for (int q = 0; q < 4; q++) {
            uint4 w;
            const int c = c0 + 8 * q;
            const float4 b0 = *reinterpret_cast<const float4 *>(bs + c);
            const float4 b1 = *reinterpret_cast<const float4 *>(bs + c + 4);
            w.x = gelu2x_bf16(__uint_as_float(r[8 * q + 0]) + b0.x, __uint_as_float(r[8 * q + 1]) + b0.y);
            w.y = gelu2x_bf16(__uint_as_float(r[8 * q + 2]) + b0.z, __uint_as_float(r[8 * q + 3]) + b0.w);
            w.z = gelu2x_bf16(__uint_as_float(r[8 * q + 4]) + b1.x, __uint_as_float(r[8 * q + 5]) + b1.y);
            w.w = gelu2x_bf16(__uint_as_float(r[8 * q + 6]) + b1.z, __uint_as_float(r[8 * q + 7]) + b1.w);
            *reinterpret_cast<uint4 *>(rowp + (uint32_t)(c / 8) * 128u) = w;
          }
        }
      } else {
        uint32_t r[16];
        tmem_ld16(taddr, r);
        tmem_wait();
        for (int j = 0; j < 16; j += 4) {
          const float4 b = *reinterpret_cast<const float4 *>(bs + j);
          v[j] = __uint_as_float(r[j]) + b.x;
          v[j + 1] = __uint_as_float(r[j + 1]) + b.y;
          v[j + 2] = __uint_as_float(r[j + 2]) + b.z;
          v[j + 3] = __uint_as_float(r[j + 3]) + b.w;
        }
      }
    }
    if (valid) {
      if (a.X) {
        for (int c = 0; c < kMlpOut; c++) a.logits[gi * kMlpOut + c] = v[c];
      } else {
        v[0] += a.direct_bias;
        int best = 0;
        for (int c = 1; c < kMlpClasses; c++)
          if (v[c] > v[best]) best = c;
        if (kind == 2 && !m.leaf[m.w_idx[e]]) best = 0;  // statistics exist for leaf sources only: full order
        (kind == 0 ? a.u_dec : (kind == 1 ? a.k_dec : a.w_dec))[e] = (unsigned char)best;
      }
    }
  }
  if (s_fail) {
    // one more bounded wait for work still in flight before TMEM and shared
    // memory are released
    if (mma_inflight) mbar_wait(&bar_mma, phase, a.wait_limit);
    if (w_inflight) mbar_wait(&bar_w, 0, a.wait_limit);
    if (tid == 0) set_err(m.st, TREE2D_ERR_TIMEOUT);
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(64) : "memory");
}

uint16_t bf16_host(float x) {
  uint32_t b;
  std::memcpy(&b, &x, 4);
  const uint32_t r = b + 0x7FFFu + ((b >> 16) & 1u);
  return (uint16_t)(r >> 16);
}

// scale * W [N][K] row-major -> core-matrix image (rows = N, K contiguous in
// 16-byte chunks; SBO = K/8*128).  scale is a power of two, so the BF16
// image is exactly scale times the BF16 rounding of W.
void image_of(const float *W, int N, int K, float scale, uint16_t *out) {
  const int sbo = K / 8 * 128;
  for (int j = 0; j < N; j++)
    for (int k = 0; k < K; k++) {
      const size_t byte = (size_t)(j / 8) * sbo + (size_t)(k / 8) * 128 + (size_t)(j % 8) * 16 + (size_t)(k % 8) * 2;
      out[byte / 2] = bf16_host(scale * W[(size_t)j * K + k]);
    }
}

}  // namespace

size_t learn_weight_image_elems() { return kWBytes / 2; }

void learn_weight_images(const float *theta, std::vector<uint16_t> &img, std::vector<float> &bias) {
  img.assign(kWBytes / 2, 0);
  // layers 2-4 read twice the GELU (gelu2x_bf16): their weights are halved
  image_of(theta + 0, 64, 16, 1.0f, img.data());
  image_of(theta + 1088, 64, 64, 0.5f, img.data() + kW1Bytes / 2);
  image_of(theta + 5248, 64, 64, 0.5f, img.data() + (kW1Bytes + kW2Bytes) / 2);
  image_of(theta + 9408, 16, 64, 0.5f, img.data() + (kW1Bytes + 2 * kW2Bytes) / 2);
  bias.assign(64 * 3 + 16, 0.f);
  std::memcpy(bias.data(), theta + 1024, 64 * 4);
  std::memcpy(bias.data() + 64, theta + 5184, 64 * 4);
  std::memcpy(bias.data() + 128, theta + 9344, 64 * 4);
  std::memcpy(bias.data() + 192, theta + 10432, 16 * 4);
}

static int launch_infer(InferArgs &a, long total, cudaStream_t s) {
  if (total <= 0) return TREE2D_OK;
  const size_t smem = kWBytes + kActBytes;
  T2D_CUDA_TRY(cudaFuncSetAttribute(k_mlp_infer, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const long ntiles = (total + kTile - 1) / kTile;
  // four tiles per CTA: the CTAs are short-lived, so the expansion kernels
  // (on a higher-priority stream) get SMs as soon as they are launched
  // instead of waiting for CTAs that would hold every SM to the end
  // (3% off the 4M learned solve against one CTA per resident slot; 2, 8
  // and 16 tiles measured 11.15, 11.05 and 11.05 ms against 11.02 ms)
  const long grid = (ntiles + kTilesPerCta - 1) / kTilesPerCta;
  a.wait_limit = 1l << 22;
  k_mlp_infer<<<(unsigned)grid, kTile, smem, s>>>(a);
  g_launches.fetch_add(1, std::memory_order_relaxed);
  T2D_CUDA_TRY(cudaGetLastError());
  return TREE2D_OK;
}

int learned_decide(MixedView &m, const LeafStats *stats, const float *u_ref_ptr, const uint16_t *wimg,
                   const float *bias, float direct_bias, long n_u, long n_k, long n_w, unsigned char *u_dec,
                   unsigned char *k_dec, unsigned char *w_dec, cudaStream_t s) {
  InferArgs a{};
  a.m = m;
  a.st = stats;
  a.u_ref_ptr = u_ref_ptr;
  a.wimg = wimg;
  a.bias = bias;
  a.direct_bias = direct_bias;
  a.n_u = n_u;
  a.n_k = n_k;
  a.n_w = w_dec ? n_w : 0;
  a.u_dec = u_dec;
  a.k_dec = k_dec;
  a.w_dec = w_dec;
  return launch_infer(a, n_u + n_k + a.n_w, s);
}

int mlp_forward_tc(int n, const float *X, const uint16_t *wimg, const float *bias, float *logits, DevStatus *st,
                   cudaStream_t s) {
  InferArgs a{};
  a.m.st = st;
  a.wimg = wimg;
  a.bias = bias;
  a.X = X;
  a.nx = n;
  a.logits = logits;
  return launch_infer(a, n, s);
}

}  // namespace t2d
