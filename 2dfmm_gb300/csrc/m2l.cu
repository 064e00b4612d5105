// M2L over the V lists: for every cell c of level >= 2,
//   L[c] += sum_{s<27} T(class(c), s) M[V[c][s]],
// T(q,s)_lk = (-1)^l C(k+l,l) tau^-(k+l+1), tau the fixed offset of slot s
// for child class q (scaled expansions make T level independent).
//
// Tensor-core form (k_m2l_tc): per child class the V-list M2L of all cells
// is one dense contraction
//     D[r, o] = sum_K A[r, K] B_q[K, o],   K = 27 slots x 2P, o < 2P,
// rows r = target cells of the class, A[r, s*2P + j] = M[V[c_r][s]][j]
// (gathered, zero where the slot is empty), B_q the real form of the 27
// complex operators.  One CTA (128 threads) owns 128 rows, or 64 (the
// tile shape the tuner may pick: the MMA's other 64 rows are zero, so
// twice the CTAs share a class's cells; a row's sums are its own either
// way, bit for bit); per slot it
// gathers its A chunk into shared memory, the B chunk arrives by a bulk
// copy (cp.async.bulk, the B images are pre-laid out in global memory),
// and one thread issues tcgen05.mma kind::tf32 (M=128, N=2P padded to 16,
// K=8 per instruction) with the FP32 accumulator in TMEM.  Operands are
// split into TF32 hi + lo parts and three products (hi*hi, hi*lo, lo*hi)
// keep ~21 bits.  Shared-memory operands use the no-swizzle K-major layout
// of 8-row x 16-byte core matrices (LBO = 128 B between K neighbours,
// SBO = 2P/4 * 128 B between 8-row groups).
#include <cstdio>
#include <cstring>
#include <vector>

#include "dev_common.cuh"
#include "mixed.h"
#include "tc_ptx.cuh"

namespace t2d {
namespace {

// ------------------------------------------------------------- CUDA cores

// One warp per cell, lane l owns b_l.  The reference form for checking.
__global__ void __launch_bounds__(256) k_m2l_cc(MixedView m, const float2 *__restrict__ T) {
  const int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (c >= m.ncell) return;
  if (m.level[c] - m.lev0 < 2) return;
  const int P = m.P;
  const int cls = (m.ix[c] & 1) + 2 * (m.iy[c] & 1);
  const int *V = m.vlist + (size_t)c * 27;
  float2 acc = make_float2(0.f, 0.f);
  for (int s = 0; s < 27; s++) {
    const int src = V[s];
    if (src < 0) continue;
    const float *Ms = m.M + (size_t)src * 2 * P;
    const float2 a = lane < P ? make_float2(Ms[lane], Ms[P + lane]) : make_float2(0.f, 0.f);
    const float2 *Trow = T + (((size_t)cls * 27 + s) * P + (lane < P ? lane : 0)) * P;
    for (int k = 0; k < P; k++) {
      const float2 ak = make_float2(__shfl_sync(0xffffffffu, a.x, k), __shfl_sync(0xffffffffu, a.y, k));
      const float2 t = Trow[k];
      acc.x += t.x * ak.x - t.y * ak.y;
      acc.y += t.x * ak.y + t.y * ak.x;
    }
  }
  if (lane < P) {
    m.L[(size_t)c * 2 * P + lane] += acc.x;
    m.L[(size_t)c * 2 * P + P + lane] += acc.y;
  }
}

// ------------------------------------------------------------ tensor cores

constexpr int kRows = 128;        // M of the MMA, rows per CTA
constexpr int kThreadsTC = 128;

struct TcArgs {
  MixedView m;
  const int *cls_list;   // [4][ncell]
  const int *cls_count;  // [4]
  const float *bimg;     // [4][27][2 (hi,lo)][Npad x Kc] core-matrix images
  int P, Kc, Npad, tmem_cols, ngroups;
  int nbs;               // B stages: 3 (slot i+1's images prefetched) or 2
  int rows;              // cells per CTA: kRows, or kRows / 2 (the MMA's other rows zero)
  long wait_limit;
};

constexpr int kMaxKc4 = 2 * kMaxP / 4;  // float4s in one multipole row (2P floats)

// Shared memory: the tile's V lists [27][128], 2 A stages x {A_hi, A_lo}
// (128 x Kc each) and nbs B stages x {B_hi, B_lo} (Npad x Kc each).
//
// The slots any row of the tile uses are found once (a block-wide OR of the
// rows' masks), and the walk over them is software-pipelined: while slot i
// is split into TF32 hi/lo and multiplied, each thread already holds slot
// i+1's multipole row in registers, and (with 3 B stages) slot i+1's
// operator images are in flight by bulk copy, so the gather latency is
// paid once per tile rather than once per slot.
__global__ void __launch_bounds__(kThreadsTC) k_m2l_tc(TcArgs a) {
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ uint64_t bar_mma[2], bar_b[3];
  __shared__ uint32_t s_tmem;
  __shared__ int s_fail;
  __shared__ unsigned s_mask;

  const int cls = blockIdx.y;
  const int count = a.cls_count[cls];
  const int row0 = blockIdx.x * a.rows;
  if (row0 >= count) return;  // uniform for the block
  const MixedView &m = a.m;
  const int P = a.P, Kc = a.Kc, Npad = a.Npad, nbs = a.nbs;
  const uint32_t a_bytes = kRows * Kc * 4, b_bytes = Npad * Kc * 4;
  const uint32_t sbo_a = (Kc / 4) * 128, sbo_b = sbo_a, lbo = 128;
  const int tid = threadIdx.x, warp = tid >> 5;
  int *sV = reinterpret_cast<int *>(smem);                       // [27][kRows]
  unsigned char *astage = smem + 27 * kRows * 4;                 // 2 x (hi, lo)
  unsigned char *bstage = astage + 2 * 2 * a_bytes;              // nbs x (hi, lo)

  if (tid == 0) {
    mbar_init(&bar_mma[0], 1);
    mbar_init(&bar_mma[1], 1);
    for (int k = 0; k < 3; k++) mbar_init(&bar_b[k], 1);
    s_fail = 0;
    s_mask = 0u;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&s_tmem)),
                 "r"(a.tmem_cols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = s_tmem;

  const int row = row0 + tid;
  const bool valid = tid < a.rows && row < count;
  const int cell = valid ? a.cls_list[(size_t)cls * m.ncell + row] : -1;
  {
    unsigned mine = 0u;
    const int *V = valid ? m.vlist + (size_t)cell * 27 : nullptr;
    for (int s = 0; s < 27; s++) {
      const int src = valid ? V[s] : -1;
      sV[s * kRows + tid] = src;
      if (src >= 0) mine |= 1u << s;
    }
    atomicOr(&s_mask, mine);
  }
  __syncthreads();
  const unsigned mask = s_mask;
  const int nslots = __popc(mask);
  // M = 128, N = Npad, A/B TF32 K-major, D FP32
  const uint32_t idesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(Npad >> 3) << 17) | ((uint32_t)(kRows >> 4) << 24);
  const float *bbase = a.bimg + (size_t)cls * 27 * 2 * (Npad * Kc);

  uint32_t phase_mma[2] = {0, 0}, phase_b[3] = {0, 0, 0};
  bool pending[2] = {false, false};
  bool b_inflight[3] = {false, false, false};  // thread 0: bulk copy issued, not yet waited for
  // Slots are spread over `ngroups` accumulators (TMEM column blocks of
  // Npad) by slot number, slot % ngroups; each accumulates few MMAs and the
  // partial sums are added in FP32 registers at the end, in group order,
  // which keeps the accumulation error small.  A row's sums depend only on
  // its own slots (a slot another row of the tile uses adds exact zeros),
  // so the result does not depend on which cells share the tile.
  bool gfirst[8] = {true, true, true, true, true, true, true, true};
  int issued = 0;  // steps whose MMAs were committed (or attempted)
  auto slot_at = [&](unsigned rest) { return __ffs(rest) - 1; };  // lowest remaining slot
  auto copy_b = [&](int slot, int bs) {
    if (tid != 0) return;
    mbar_expect_tx(&bar_b[bs], 2 * b_bytes);
    bulk_g2s(bstage + (size_t)bs * 2 * b_bytes, bbase + (size_t)slot * 2 * (Npad * Kc), 2 * b_bytes, &bar_b[bs]);
    b_inflight[bs] = true;
  };
  auto load_row = [&](int slot, float4 (&r)[kMaxKc4]) {
    const int src = sV[slot * kRows + tid];
    const float4 *msrc = src >= 0 ? reinterpret_cast<const float4 *>(m.M + (size_t)src * 2 * P) : nullptr;
#pragma unroll
    for (int kk = 0; kk < kMaxKc4; kk++)
      r[kk] = (msrc && kk < Kc / 4) ? msrc[kk] : make_float4(0.f, 0.f, 0.f, 0.f);
  };

  // One processed slot: the multipole rows of `slot` are in `use`; the rows
  // of the next slot are loaded into `fill` (consumed one step later, so
  // their latency overlaps a whole step).  A single block barrier per slot
  // (after the A stage is written) also carries the failure flag: a thread
  // that saw a wait give up stops the walk for the whole block at the next
  // barrier.
  auto step = [&](int i, int slot, int next, float4 (&use)[kMaxKc4], float4 (&fill)[kMaxKc4]) -> bool {
    const int ast = i & 1, bs = i % nbs;
    if (next >= 0) load_row(next, fill);
    // the MMAs that last read this A stage (and, with 3 B stages, the B
    // stage of the next slot) must be done before they are rewritten
    if (pending[ast]) {
      if (mbar_wait(&bar_mma[ast], phase_mma[ast], a.wait_limit)) {
        phase_mma[ast] ^= 1;
        pending[ast] = false;
      } else {
        s_fail = 1;
      }
    }
    if (nbs == 3 && next >= 0) copy_b(next, (i + 1) % 3);
    if (nbs == 2 && i > 0) copy_b(slot, bs);  // slot 0's copy went out before the walk
    {
      float *Ahi = reinterpret_cast<float *>(astage + (size_t)ast * 2 * a_bytes);
      float *Alo = reinterpret_cast<float *>(astage + (size_t)ast * 2 * a_bytes + a_bytes);
      const uint32_t rbase = (uint32_t)(tid >> 3) * sbo_a + (uint32_t)(tid & 7) * 16;
#pragma unroll
      for (int kk = 0; kk < kMaxKc4; kk++) {
        if (kk >= Kc / 4) break;
        const float4 v = use[kk];
        float4 h, l;
        h.x = __uint_as_float(tf32_bits(v.x));
        h.y = __uint_as_float(tf32_bits(v.y));
        h.z = __uint_as_float(tf32_bits(v.z));
        h.w = __uint_as_float(tf32_bits(v.w));
        l.x = v.x - h.x;
        l.y = v.y - h.y;
        l.z = v.z - h.z;
        l.w = v.w - h.w;
        const uint32_t off = rbase + (uint32_t)kk * lbo;
        *reinterpret_cast<float4 *>(reinterpret_cast<unsigned char *>(Ahi) + off) = h;
        *reinterpret_cast<float4 *>(reinterpret_cast<unsigned char *>(Alo) + off) = l;
      }
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    if (__syncthreads_or(s_fail)) return false;
    if (tid == 0) {
      if (mbar_wait(&bar_b[bs], phase_b[bs], a.wait_limit)) {
        phase_b[bs] ^= 1;
        b_inflight[bs] = false;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t ah = smem_u32(astage + (size_t)ast * 2 * a_bytes), al = ah + a_bytes;
        const uint32_t bh = smem_u32(bstage + (size_t)bs * 2 * b_bytes), bl = bh + b_bytes;
        const int g = slot % a.ngroups;
        const uint32_t dcol = tmem + (uint32_t)(g * Npad);
        for (int t = 0; t < Kc / 8; t++) {
          const uint32_t ko = (uint32_t)t * 2 * lbo;
          const uint64_t dah = smem_desc(ah + ko, lbo, sbo_a), dal = smem_desc(al + ko, lbo, sbo_a);
          const uint64_t dbh = smem_desc(bh + ko, lbo, sbo_b), dbl = smem_desc(bl + ko, lbo, sbo_b);
          mma_tf32(dcol, dah, dbh, idesc, gfirst[g] ? 0u : 1u);
          gfirst[g] = false;
          mma_tf32(dcol, dah, dbl, idesc, 1u);
          mma_tf32(dcol, dal, dbh, idesc, 1u);
        }
        mma_commit(&bar_mma[ast]);
      } else {
        // no MMAs for this stage: the others find out at the next barrier
        // (their wait on this stage gives up too, bounded)
        s_fail = 1;
      }
    }
    pending[ast] = true;
    issued = i + 1;
    return true;
  };

  unsigned rest = mask;
  float4 buf0[kMaxKc4], buf1[kMaxKc4];
  int slot = -1;
  if (nslots > 0) {
    slot = slot_at(rest);
    rest &= rest - 1;
    load_row(slot, buf0);
    copy_b(slot, 0);
  }
  for (int i = 0; i < nslots; i += 2) {
    // two steps per turn so that the row buffers swap roles statically
    int next = rest ? slot_at(rest) : -1;
    if (!step(i, slot, next, buf0, buf1)) break;
    if (next < 0) break;
    slot = next;
    rest &= rest - 1;
    next = rest ? slot_at(rest) : -1;
    if (!step(i + 1, slot, next, buf1, buf0)) break;
    if (next < 0) break;
    slot = next;
    rest &= rest - 1;
  }
  // drain: every stage with MMAs in flight (bounded; a failed wait is
  // retried once more below before TMEM and shared memory are released)
  for (int st = 0; st < 2; st++) {
    if (pending[st]) {
      if (mbar_wait(&bar_mma[st], phase_mma[st], a.wait_limit)) {
        phase_mma[st] ^= 1;
        pending[st] = false;
      } else {
        s_fail = 1;
      }
    }
  }
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  __syncthreads();
  if (issued > 0 && !s_fail) {
    // Row `tid` lives in TMEM lane tid; warp w reads lanes 32w..32w+31.  All
    // lanes of the warp execute the loads (they are warp-collective); only
    // lanes with a row write.
    // The local expansions are still zero here (P2L and L2L run after
    // M2L, and each cell is one row of one class), so the row is stored,
    // not added; 32 accumulator columns per TMEM load.
    const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16);
    float *dst = valid ? m.L + (size_t)cell * 2 * P : nullptr;
    unsigned gmask = 0u;  // groups that received MMAs
    for (unsigned r = mask; r; r &= r - 1) gmask |= 1u << ((__ffs(r) - 1) % a.ngroups);
    for (int c0 = 0; c0 < 2 * P; c0 += 32) {
      float acc[32];
#pragma unroll
      for (int j = 0; j < 32; j++) acc[j] = 0.f;
      for (int g = 0; g < a.ngroups; g++) {
        if (!((gmask >> g) & 1u)) continue;
        uint32_t r[32];
        tmem_ld32(taddr + (uint32_t)(g * Npad + c0), r);
        tmem_wait();
#pragma unroll
        for (int j = 0; j < 32; j++) acc[j] += __uint_as_float(r[j]);
      }
      if (dst) {
        if (c0 + 32 <= 2 * P) {
#pragma unroll
          for (int j = 0; j < 32; j += 4)
            *reinterpret_cast<float4 *>(dst + c0 + j) = make_float4(acc[j], acc[j + 1], acc[j + 2], acc[j + 3]);
        } else {
          for (int j = 0; c0 + j < 2 * P; j++) dst[c0 + j] = acc[j];
        }
      }
    }
  }
  if (s_fail) {
    // a wait gave up: give MMAs and copies still in flight one more bounded
    // wait before the TMEM and shared memory are released
    for (int st = 0; st < 2; st++)
      if (pending[st]) mbar_wait(&bar_mma[st], phase_mma[st], a.wait_limit);
    for (int bs = 0; bs < 3; bs++)
      if (tid == 0 && b_inflight[bs]) mbar_wait(&bar_b[bs], phase_b[bs], a.wait_limit);
  }
  if (s_fail && tid == 0) set_err(m.st, TREE2D_ERR_TIMEOUT);
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(a.tmem_cols) : "memory");
}

// Cells of level >= 2 (below their set root), grouped by child class (order within a class is
// irrelevant: every row's sum is its own, k_m2l_tc).
// One atomic per warp and class (the lanes of a class take consecutive
// positions in ballot order).
__global__ void k_class_lists(MixedView m, int *list, int *count) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  const bool in = c < m.ncell && m.level[c] - m.lev0 >= 2;
  const int cls = in ? (int)((m.ix[c] & 1) + 2 * (m.iy[c] & 1)) : -1;
  for (int k = 0; k < 4; k++) {
    const unsigned bal = __ballot_sync(0xffffffffu, cls == k);
    if (!bal) continue;
    const int leader = __ffs(bal) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(&count[k], __popc(bal));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (cls == k) list[(size_t)k * m.ncell + base + __popc(bal & ((1u << lane) - 1u))] = c;
  }
}

uint32_t tf32_round_host(float x) {
  uint32_t b;
  std::memcpy(&b, &x, 4);
  if ((b & 0x7f800000u) != 0x7f800000u) b = (b + 0x1000u) & 0xffffe000u;  // to nearest, ties away
  return b;
}

}  // namespace

int m2l_cuda_cores(MixedView &m, const float *tables, cudaStream_t s) {
  k_m2l_cc<<<(int)(((long)m.ncell * 32 + 255) / 256), 256, 0, s>>>(m, reinterpret_cast<const float2 *>(tables));
  g_launches.fetch_add(1, std::memory_order_relaxed);
  T2D_CUDA_TRY(cudaGetLastError());
  return TREE2D_OK;
}

int m2l_npad(int P) { return ((2 * P + 15) / 16) * 16; }

void m2l_b_images(int P, const float *h_m2l, std::vector<float> &img) {
  const int Kc = 2 * P, Npad = m2l_npad(P);
  const size_t chunk = (size_t)Npad * Kc;
  img.assign((size_t)4 * 27 * 2 * chunk, 0.f);
  const uint32_t sbo = (uint32_t)(Kc / 4) * 128;
  for (int q = 0; q < 4; q++)
    for (int s = 0; s < 27; s++) {
      const float *T = h_m2l + ((size_t)q * 27 + s) * P * P * 2;  // [l][k] complex
      float *hi = img.data() + ((size_t)q * 27 + s) * 2 * chunk;
      float *lo = hi + chunk;
      for (int k = 0; k < Kc; k++)
        for (int o = 0; o < Npad; o++) {
          // B[k][o]: rows k<P take a_re, k>=P a_im; columns o<P give b_re, o>=P b_im
          float v = 0.f;
          if (o < 2 * P) {
            const int kk = k % P, l = o % P;
            const float tre = T[((size_t)l * P + kk) * 2], tim = T[((size_t)l * P + kk) * 2 + 1];
            const bool kim = k >= P, oim = o >= P;
            v = !kim ? (!oim ? tre : tim) : (!oim ? -tim : tre);
          }
          const uint32_t hb = tf32_round_host(v);
          float h;
          std::memcpy(&h, &hb, 4);
          const float l = v - h;
          const size_t off = ((size_t)(o >> 3) * sbo + (size_t)(k >> 2) * 128 + (size_t)(o & 7) * 16 + (size_t)(k & 3) * 4) / 4;
          hi[off] = h;
          lo[off] = l;
        }
    }
}

int m2l_tensor_cores(MixedView &m, const float *bimg, int *cls_list, int *cls_count, int rows, cudaStream_t s) {
  if (rows != kRows && rows != kRows / 2) return TREE2D_ERR_BAD_PARAMS;
  const int P = m.P, Kc = 2 * P, Npad = m2l_npad(P);
  if (Kc % 8 != 0) return TREE2D_ERR_BAD_PARAMS;  // K of one MMA is 8 TF32 elements
  T2D_CUDA_TRY(cudaMemsetAsync(cls_count, 0, 4 * sizeof(int), s));
  k_class_lists<<<(m.ncell + 255) / 256, 256, 0, s>>>(m, cls_list, cls_count);
  TcArgs a;
  a.m = m;
  a.cls_list = cls_list;
  a.cls_count = cls_count;
  a.bimg = bimg;
  a.P = P;
  a.Kc = Kc;
  a.Npad = Npad;
  a.tmem_cols = 256;                            // two CTAs per SM fill the 512 columns
  a.ngroups = 256 / Npad < 8 ? 256 / Npad : 8;
  a.rows = rows;
  a.wait_limit = 1l << 22;  // polls; a healthy wait ends within microseconds
  const size_t fixed = (size_t)27 * kRows * 4 + 2 * (2 * (size_t)kRows * Kc * 4);
  const size_t bst = 2 * (size_t)Npad * Kc * 4;
  a.nbs = fixed + 3 * bst <= 110 * 1024 ? 3 : 2;  // 3 B stages while two CTAs still fit an SM
  const size_t smem = fixed + (size_t)a.nbs * bst;
  T2D_CUDA_TRY(cudaFuncSetAttribute(k_m2l_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  dim3 grid((m.ncell + rows - 1) / rows, 4);
  k_m2l_tc<<<grid, kThreadsTC, smem, s>>>(a);
  g_launches.fetch_add(2, std::memory_order_relaxed);
  T2D_CUDA_TRY(cudaGetLastError());
  return TREE2D_OK;
}

}  // namespace t2d
