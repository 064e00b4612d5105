// Learned order selection (TREE2D_MODE_LEARNED): interfaces shared by
// learn.cu, learn_tc.cu, mixed.cu and api.cu.
#pragma once

#include "mixed.h"

namespace t2d {

// Network: 16 inputs -> 64 -> 64 -> 64 -> 16 logits (14 classes used),
// GELU (tanh form) on the hidden layers, BF16 weights and layer inputs,
// FP32 accumulation.  Flat parameter order: W1[64][16] b1[64] W2[64][64]
// b2[64] W3[64][64] b3[64] W4[16][64] b4[16].
constexpr int kMlpIn = 16, kMlpHidden = 64, kMlpOut = 16, kMlpClasses = 14;
constexpr int kMlpParams = 64 * 16 + 64 + 64 * 64 + 64 + 64 * 64 + 64 + 16 * 64 + 16;  // 10448
constexpr int kNumFeatures = 12;

// Classes: 0 = direct evaluation; c >= 1 = the multipole of the source leaf
// at order p = c + 3 (4..16).  For a correction (K) interaction any c >= 1
// means the correction is skipped.
__host__ __device__ inline int class_order(int c) { return c + 3; }

struct LearnedParams {
  bool have_weights = false;
  float theta[kMlpParams];   // FP32 master copy (the network uses it rounded to BF16)
  float direct_bias = 1.0f;  // added to the direct logit: leans towards exact evaluation
  int order_margin = 1;      // chosen order raised by this much (capped at 16)
  double budget = 3e-7;      // label budget: per-interaction error / (sum|G| / R0)
  double k_blobs_max = 0;    // training envelope: mean source blobs of the K leaves per leaf; 0 = none
  double cutoff_train = 0;   // correction radius (units of max sigma) the envelope was counted at; 0 = the one in force
  int far_orders = 0;        // the network also sets the order of each W-list M2P (leaf sources)
};

// Per-leaf source statistics for the features.
struct LeafStats {
  float g_abs;   // sum |G|
  float m1;      // |sum G (z - c)| / (h sum |G|)
  float m2;      // sum |G| |z - c|^2 / (h^2 sum |G|)
  float sig;     // max sigma
};

// u_ref of the set that leaf cell B belongs to: one per tree, or on a
// batched tree (m.lev0 > 0) one per set, indexed as the sets' correction
// radii are (set k of a batch sits in tile (2a, 2b) of the level-lev0 grid,
// k = b 2^(lev0-1) + a).
__device__ __forceinline__ int set_of_cell(const MixedView &m, int B) {
  const int sh = m.level[B] - m.lev0;
  const unsigned tx = m.ix[B] >> sh, ty = m.iy[B] >> sh;
  return (int)((ty >> 1) * (1u << (m.lev0 - 1)) + (tx >> 1));
}
__device__ __forceinline__ float uref_of(const MixedView &m, const float *uref, int B) {
  return m.lev0 > 0 ? uref[set_of_cell(m, B)] : uref[0];
}

// Feature vector of the interaction target leaf B <- source leaf A
// (kMlpIn floats).  `type` 0 = direct (U) list, 1 = correction (K) list;
// u_ref = sum|G| / R0.  Features: log distance over the source side, log
// box gap over the source's core radius, offset direction, the source's
// |G| moments of order 0 (against u_ref), 1 and 2, occupancies, list kind,
// size ratio, self flag.  The network reads them rounded to BF16 (2^-9), so
// the SFU's logarithm and approximate quotients (~2^-22) are used; every
// argument of a logarithm is a positive normal number.
__device__ __forceinline__ void interaction_features(const MixedView &m, const LeafStats *st, int B, int A, int type, float u_ref,
                                     float *f) {
  const float dx = m.cxf[B] - m.cxf[A], dy = m.cyf[B] - m.cyf[A];
  const float dc = sqrtf(dx * dx + dy * dy);
  const float hA = m.h[A], hB = m.h[B];
  const float half = 0.5f * (hA + hB);
  const float gx = fmaxf(fabsf(dx) - half, 0.f), gy = fmaxf(fabsf(dy) - half, 0.f);
  const float gap = sqrtf(gx * gx + gy * gy);
  const LeafStats s = st[A];
  const float sig = fmaxf(s.sig, 1e-30f);
  const int nA = m.end[A] - m.begin[A], nB = m.end[B] - m.begin[B];
  f[0] = __log2f(__fdividef(fmaxf(dc, 1e-3f * hA), hA)) * 0.25f;
  f[1] = __log2f(__fdividef(fmaxf(gap, 1e-3f * sig), sig)) * 0.25f;
  f[2] = dc > 0.f ? __fdividef(dx, dc) : 0.f;
  f[3] = dc > 0.f ? __fdividef(dy, dc) : 0.f;
  const float scale = __fdividef(s.g_abs, 6.2831853f * fmaxf(dc, hA) * fmaxf(u_ref, 1e-30f));
  f[4] = fminf(fmaxf(__log2f(scale + 1e-30f), -60.f), 10.f) * (1.f / 16.f);
  f[5] = s.m1;
  f[6] = 2.f * s.m2;
  f[7] = __log2f((float)nA + 1.f) * (1.f / 6.f);
  f[8] = __log2f((float)nB + 1.f) * (1.f / 6.f);
  f[9] = (float)type;
  f[10] = __log2f(__fdividef(hB, hA)) * 0.25f;
  f[11] = A == B ? 1.f : 0.f;
  for (int k = kNumFeatures; k < kMlpIn; k++) f[k] = 0.f;
}


int learned_leaf_stats(MixedView &m, LeafStats *stats, cudaStream_t s);
int learned_uref(MixedView &m, const LeafStats *stats, const RootBox *root, float *out, cudaStream_t s);
// u_ref of every set of a batched tree (roots[k], out[k] for set k; leaf_lo
// and leaf_hi are nsets-entry scratch): for each set the same sum, in the
// same order, that learned_uref forms for the set solved alone.
int learned_uref_sets(MixedView &m, const LeafStats *stats, const RootBox *roots, int nsets, int *leaf_lo,
                      int *leaf_hi, float *out, cudaStream_t s);

// Decisions (class per list entry) for all U, K and (w_dec non-null) W
// entries of every leaf, by the tensor-core network (learn_tc.cu).  A W
// entry is presented as a U entry (an M2P of its source into the target
// leaf); its class c >= 1 sets that M2P's order as for a U entry, class 0
// keeps the full order, and so does every W entry whose source is not a
// leaf (the source statistics are per leaf).  `wimg` holds the BF16
// weights in the kernel's operand layout (learn_weight_images).
int learned_decide(MixedView &m, const LeafStats *stats, const float *u_ref_ptr, const uint16_t *wimg,
                   const float *bias, float direct_bias, long n_u, long n_k, long n_w, unsigned char *u_dec,
                   unsigned char *k_dec, unsigned char *w_dec, cudaStream_t s);
void learn_weight_images(const float *theta, std::vector<uint16_t> &img, std::vector<float> &bias);
size_t learn_weight_image_elems();

// Training data: for `ns` sampled interactions (leaf ordinal, list kind,
// entry index), features and the cheapest acceptable class against the FP64
// exact contribution (label generator, learn.cu).
int learned_labels(MixedView &m, const LeafStats *stats, const float *u_ref_ptr, double tol, int ns,
                   const int *samples, float *features, int *labels, cudaStream_t s);

// Training (learn.cu): `steps` Adam steps on mini-batches of `batch`
// samples from (X, y); theta/m/v FP32 on the device.
int mlp_train(int n, const float *X, const int *y, float *theta, float *m1, float *v1, int steps, int batch,
              float lr, unsigned seed, float *loss_out, cudaStream_t s);
// One forward + backward on n samples (for gradient checks).
int mlp_grad(int n, const float *X, const int *y, const float *theta, float *grad, float *loss, cudaStream_t s);
// Forward of the training path (CUDA cores) and of the inference path
// (tensor cores) on n feature vectors: logits [n][16].
int mlp_forward_cc(int n, const float *X, const float *theta, float *logits, cudaStream_t s);
int mlp_forward_tc(int n, const float *X, const uint16_t *wimg, const float *bias, float *logits, DevStatus *st,
                   cudaStream_t s);

}  // namespace t2d
