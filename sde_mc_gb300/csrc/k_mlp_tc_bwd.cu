// k_mlp_tc_bwd.cu — K6 on tcgen05: gradient of the control-variate loss.
//
// The loss of train_adapted_control_variates (sde_mc/varred.py:134-199) is
// Var(Gamma) over a minibatch, Gamma_p = payoff_p + sum_k e^{-r t_k} f(t_k, X_k) . m_k
// (m = Brownian increments for f, marks minus compensator for g), so
// dL/df(row) = 2 (Gamma_p - mean) / (n - 1) e^{-r t_k} m_k.  A CTA of 128
// threads takes 128 paths (one per thread) over a range of 32 steps; at each
// step the 128 rows go through
//
//   forward   F1: A1 (inputs, split) x W1 -> H1;  F2: H1 x W2 -> H2;  F3: H2 x W3 -> H3
//   layer 4   dZ3 = (dO W4) [H3 > 0], dW4 += dO^T H3 (FP32, warp reduce-scatter)
//   dgrad     G3: dZ3 x W3 -> dH2, dZ2 = dH2 [H2 > 0];  G2: dZ2 x W2 -> dH1,
//             dZ1 = dH1 [H1 > 0]
//   wgrad     W:  [dZ3 | dZ2]^T x [H2 1 | H1 1]  (M = 128, N = 160, K = the 128 rows)
//             W1: [dZ1 high | dZ1 low]^T x A1    (M = 128, N = 16)
//
// All seven products are tcgen05.mma kind::f16 (BF16 operands, FP32
// accumulators in tensor memory) issued by one thread.  The weight-gradient
// products accumulate in tensor memory over every row the CTA processes;
// their diagonal blocks are dW3 | db3 and dW2 | db2 (the off-diagonal blocks
// are spare work), W1's rows give dW1 | db1 from the split parts.  The dgrad
// and weight-gradient products read the tiles in place: an activation tile
// stored K-major for the forward product (rows x features) is the MN-major
// operand of the transposed product (features x rows), and a K-major weight
// tile is the MN-major operand of its transpose.  One gradient partial per
// CTA in torch parameter order; grad_reduce_tc_kernel adds them in CTA order.
//
// Every wait is bounded; a CTA whose wait gives up writes NaN partials and
// SDEMC_ETIMEOUT, issues nothing more and frees its tensor memory.
#include "mlp_tc.cuh"
#include "sdemc_host.cuh"

namespace sdemc {
namespace tcb {

using tc::kH;
using tc::kK1;
using tc::kKH;
using tc::kRows;
using tc::core_offset;

constexpr int kHW = 160;          // HH: H2 | 1 1 0.. (80) | H1 | 1 1 0.. (80)
constexpr int kH1Col = 80;        // first column of H1 in HH
constexpr int kDW = 128;          // DZ: dZ3 | dZ2, later dZ1 high | dZ1 low
constexpr uint32_t kCols = 256;   // tensor-memory columns per CTA
constexpr uint32_t kColS = 0, kColW = 64, kColW1 = 224;
constexpr int kRangeLen = 32;     // steps per work unit
constexpr int kRed = 128 + 4;     // per-warp dW4 | db4 slots

// row-group strides (bytes) of the K-major tiles; 128 B between K-adjacent
// core matrices everywhere
constexpr uint32_t kCm = 128;
constexpr uint32_t kSboHH = (kHW / 8) * kCm, kSboDZ = (kDW / 8) * kCm, kSboA1 = (kK1 / 8) * kCm,
                   kSboB = (kKH / 8) * kCm;

constexpr uint32_t kIdFwd = tc::make_idesc(128, 64, false, false);
constexpr uint32_t kIdDgrad = tc::make_idesc(128, 64, false, true);
constexpr uint32_t kIdW = tc::make_idesc(128, 160, true, true);
constexpr uint32_t kIdW1 = tc::make_idesc(128, 16, true, true);

struct BwdSmem {
  unsigned char HH[kRows * kHW * 2];
  unsigned char DZ[kRows * kDW * 2];
  unsigned char A1[2][kRows * kK1 * 2];
  unsigned char B1[kH * kK1 * 2];
  unsigned char B2[kH * kKH * 2];
  unsigned char B3[kH * kKH * 2];
  float w4[2][kH];
  float red[4][kRed];
  float lo[kH][4];
  double gpart[kRows];
  float gmean;
  unsigned long long mbar;
  uint32_t tmem;
  // keeps every operand read inside the allocation even if the MN-major
  // strides were read the other way round (largest overhang: the transposed
  // W3 view, 7 x 1280 + 255 bytes past a slice start)
  unsigned char guard[4096];
};

SDEMC_DI bool sync_or(bool bad) {
  tc::fence_async_smem();
  tc::fence_before_sync();
  return __syncthreads_or(bad) != 0;
}

SDEMC_DI bool wait_phase(BwdSmem& sm, uint32_t& phase) {
  const bool ok = tc::mbar_wait(tc::saddr_of(&sm.mbar), phase);
  phase ^= 1u;
  tc::fence_after_sync();
  return ok;
}

// K-major A x K-major B, nk slices of K = 16 (256 B apart in both tiles).
SDEMC_DI void issue_kk(uint32_t d, uint32_t a, uint32_t sbo_a, uint32_t b, uint32_t sbo_b, int nk, uint32_t id) {
  for (int s = 0; s < nk; ++s)
    tc::mma_f16_id(d, tc::smem_desc_lbo(a + 256u * s, kCm, sbo_a), tc::smem_desc_lbo(b + 256u * s, kCm, sbo_b), id,
                   s > 0 ? 1u : 0u);
}
// K-major A x MN-major view of a K-major weight tile (its transpose).
SDEMC_DI void issue_dgrad(uint32_t d, uint32_t a, uint32_t b) {
  for (int s = 0; s < kH / 16; ++s)
    tc::mma_f16_id(d, tc::smem_desc_lbo(a + 256u * s, kCm, kSboDZ),
                   tc::smem_desc_lbo(b + 2u * kSboB * s, kSboB, kCm), kIdDgrad, s > 0 ? 1u : 0u);
}
// MN-major A x MN-major B over the tile's 128 rows (K), accumulating.
SDEMC_DI void issue_rows(uint32_t d, uint32_t a, uint32_t lbo_a, uint32_t b, uint32_t lbo_b, uint32_t id,
                         uint32_t acc) {
  for (int s = 0; s < kRows / 16; ++s)
    tc::mma_f16_id(d, tc::smem_desc_lbo(a + 2u * lbo_a * s, lbo_a, kCm), tc::smem_desc_lbo(b + 2u * lbo_b * s, lbo_b, kCm),
                   id, (acc | (uint32_t)s) ? 1u : 0u);
}

// Accumulator row -> ReLU -> BF16 into HH at column c0; mask bit f = (H_f > 0).
SDEMC_DI void relu_to_hh(uint32_t ts, unsigned char* HH, int c0, uint32_t* mask) {
  mask[0] = mask[1] = 0u;
  float v[kH];
  tc::tmem_ld64(ts, v);
#pragma unroll
  for (int j = 0; j < kH; ++j)
    if (v[j] > 0.f) mask[j >> 5] |= 1u << (j & 31);
#pragma unroll
  for (int c = 0; c < kH / 8; ++c) {
    uint4 q;
    q.x = tc::pack2(fmaxf(v[8 * c + 0], 0.f), fmaxf(v[8 * c + 1], 0.f));
    q.y = tc::pack2(fmaxf(v[8 * c + 2], 0.f), fmaxf(v[8 * c + 3], 0.f));
    q.z = tc::pack2(fmaxf(v[8 * c + 4], 0.f), fmaxf(v[8 * c + 5], 0.f));
    q.w = tc::pack2(fmaxf(v[8 * c + 6], 0.f), fmaxf(v[8 * c + 7], 0.f));
    *reinterpret_cast<uint4*>(HH + core_offset(threadIdx.x, c0 + 8 * c, kHW)) = q;
  }
}

// Masked accumulator row -> BF16 into DZ at column c0.
SDEMC_DI void masked_to_dz(uint32_t ts, unsigned char* DZ, int c0, const uint32_t* mask) {
  float v[kH];
  tc::tmem_ld64(ts, v);
#pragma unroll
  for (int j = 0; j < kH; ++j)
    if (!((mask[j >> 5] >> (j & 31)) & 1u)) v[j] = 0.f;
#pragma unroll
  for (int c = 0; c < kH / 8; ++c) {
    uint4 q;
    q.x = tc::pack2(v[8 * c + 0], v[8 * c + 1]);
    q.y = tc::pack2(v[8 * c + 2], v[8 * c + 3]);
    q.z = tc::pack2(v[8 * c + 4], v[8 * c + 5]);
    q.w = tc::pack2(v[8 * c + 6], v[8 * c + 7]);
    *reinterpret_cast<uint4*>(DZ + core_offset(threadIdx.x, c0 + 8 * c, kDW)) = q;
  }
}

// Masked accumulator row split into BF16 high and low parts: DZ columns
// [0, 64) and [64, 128).
SDEMC_DI void masked_split_to_dz(uint32_t ts, unsigned char* DZ, const uint32_t* mask) {
  float vall[kH];
  tc::tmem_ld64(ts, vall);
#pragma unroll
  for (int c = 0; c < kH / 16; ++c) {
    const float* v = vall + 16 * c;
    __nv_bfloat16 hi[16], lo[16];
#pragma unroll
    for (int j = 0; j < 16; ++j) {
      const float z = ((mask[c >> 1] >> ((16 * c + j) & 31)) & 1u) ? v[j] : 0.f;
      tc::split(z, hi[j], lo[j]);
    }
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      uint4 qh, ql;
      qh.x = tc::pack2b(hi[8 * h + 0], hi[8 * h + 1]); ql.x = tc::pack2b(lo[8 * h + 0], lo[8 * h + 1]);
      qh.y = tc::pack2b(hi[8 * h + 2], hi[8 * h + 3]); ql.y = tc::pack2b(lo[8 * h + 2], lo[8 * h + 3]);
      qh.z = tc::pack2b(hi[8 * h + 4], hi[8 * h + 5]); ql.z = tc::pack2b(lo[8 * h + 4], lo[8 * h + 5]);
      qh.w = tc::pack2b(hi[8 * h + 6], hi[8 * h + 7]); ql.w = tc::pack2b(lo[8 * h + 6], lo[8 * h + 7]);
      *reinterpret_cast<uint4*>(DZ + core_offset(threadIdx.x, 16 * c + 8 * h, kDW)) = qh;
      *reinterpret_cast<uint4*>(DZ + core_offset(threadIdx.x, kH + 16 * c + 8 * h, kDW)) = ql;
    }
  }
}

// Warp reduce-scatter of 32 values: lane l returns the sum over the warp of
// v[l] (fixed butterfly order).
SDEMC_DI float reduce_scatter32(float* v) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int s = 0; s < 5; ++s) {
    const int o = 16 >> s;
    const bool up = (lane & o) != 0;
#pragma unroll
    for (int i = 0; i < (16 >> s); ++i) {
      const float send = up ? v[i] : v[i + (16 >> s)];
      const float keep = up ? v[i + (16 >> s)] : v[i];
      v[i] = keep + __shfl_xor_sync(kFull, send, o);
    }
  }
  return v[0];
}

// Layer 4 backward on the H3 accumulator row: dZ3 = (dO W4) [H3 > 0] into DZ
// columns [0, 64); dW4 contributions reduce-scattered over the warp (lane l
// of chunk c holds W4[l >> 4][16 c + (l & 15)]).
template <int D>
SDEMC_DI void layer4_backward(BwdSmem& sm, uint32_t ts, const float* dO, float* acc4) {
  float vall[kH];
  tc::tmem_ld64(ts, vall);
#pragma unroll
  for (int c = 0; c < kH / 16; ++c) {
    const float* v = vall + 16 * c;
    float dz[16], w[32];
#pragma unroll
    for (int j = 0; j < 16; ++j) {
      const float h = fmaxf(v[j], 0.f);
      float s = 0.f;
#pragma unroll
      for (int i = 0; i < D; ++i) s = __fmaf_rn(dO[i], sm.w4[i][16 * c + j], s);
      dz[j] = h > 0.f ? s : 0.f;
      w[j] = __fmul_rn(dO[0], h);
      w[16 + j] = D > 1 ? __fmul_rn(dO[D > 1 ? 1 : 0], h) : 0.f;
    }
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      uint4 q;
      q.x = tc::pack2(dz[8 * h + 0], dz[8 * h + 1]);
      q.y = tc::pack2(dz[8 * h + 2], dz[8 * h + 3]);
      q.z = tc::pack2(dz[8 * h + 4], dz[8 * h + 5]);
      q.w = tc::pack2(dz[8 * h + 6], dz[8 * h + 7]);
      *reinterpret_cast<uint4*>(sm.DZ + core_offset(threadIdx.x, 16 * c + 8 * h, kDW)) = q;
    }
    acc4[c] = __fadd_rn(acc4[c], reduce_scatter32(w));
  }
}

template <int D>
__global__ void __launch_bounds__(kRows)
cv_backward_tc_kernel(const float* __restrict__ prm, const float* __restrict__ time, const float* __restrict__ paths,
                      const float* __restrict__ mult, const int64_t* idx, int64_t n, int S, float rate,
                      const float* __restrict__ gamma, int nranges, float* __restrict__ partials,
                      int32_t* status) {
  extern __shared__ unsigned char smem_raw[];
  BwdSmem& sm = *reinterpret_cast<BwdSmem*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                            ~static_cast<uintptr_t>(1023));
  using L = tc::TcLayout<D>;
  const int t = threadIdx.x, lane = t & 31, wid = t >> 5;
  tc::fill_weights<D>(sm.B1, sm.B2, sm.B3, prm);
  {
    const __nv_bfloat16 one = __float2bfloat16_rn(1.f), zero = __float2bfloat16_rn(0.f);
    for (int e = t; e < kRows * 16; e += blockDim.x) {  // bias and padding columns of HH
      const int r = e / 16, k = e % 16;
      const __nv_bfloat16 v = k < 2 ? one : zero;
      tc::put_bf16(sm.HH, r, kH + k, kHW, v);
      tc::put_bf16(sm.HH, r, kH1Col + kH + k, kHW, v);
    }
  }
  for (int j = t; j < kH; j += blockDim.x) {
    sm.w4[0][j] = prm[L::W4 + j];
    sm.w4[1][j] = D > 1 ? prm[L::W4 + (D > 1 ? kH : 0) + j] : 0.f;
  }
  // minibatch mean of Gamma, fixed order (every CTA computes the same bits)
  {
    double a = 0.0;
    for (int64_t q = t; q < n; q += blockDim.x) a += (double)gamma[q];
    sm.gpart[t] = a;
    __syncthreads();
    for (int o = kRows / 2; o > 0; o >>= 1) {
      if (t < o) sm.gpart[t] += sm.gpart[t + o];
      __syncthreads();
    }
    if (t == 0) sm.gmean = (float)(sm.gpart[0] / (double)n);
  }
  if (t == 0) {
    tc::mbar_init(tc::saddr_of(&sm.mbar));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  tc::fence_async_smem();
  if (t < 32) tc::tmem_alloc(tc::saddr_of(&sm.tmem), kCols);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const float gmean = sm.gmean;
  const float scale = 2.0f / (float)(n > 1 ? n - 1 : 1);
  const uint32_t tbase = sm.tmem + tc::lane_base();
  const uint32_t tS = sm.tmem + kColS, tW = sm.tmem + kColW, tW1 = sm.tmem + kColW1;
  const uint32_t aHH = tc::saddr_of(sm.HH), aDZ = tc::saddr_of(sm.DZ), aB1 = tc::saddr_of(sm.B1),
                 aB2 = tc::saddr_of(sm.B2), aB3 = tc::saddr_of(sm.B3);
  uint32_t phase = 0, accw = 0, acc1 = 0;
  int buf = 0;
  bool fail = false;
  float acc4[kH / 16] = {0.f, 0.f, 0.f, 0.f};
  float bsum[2] = {0.f, 0.f};
  const int64_t units = ((n + kRows - 1) / kRows) * nranges;
  for (int64_t u = blockIdx.x; u < units && !fail; u += gridDim.x) {  // uniform over the CTA
    const int64_t g = u / nranges;
    const int r = (int)(u % nranges);
    const int64_t q = g * kRows + t;
    const bool has = q < n;
    const int64_t p = has ? (idx ? idx[q] : q) : 0;
    const float dgam = has ? __fmul_rn(scale, __fsub_rn(gamma[q], gmean)) : 0.f;
    const int k0 = r * kRangeLen, k1 = min(S, k0 + kRangeLen);
    float tn = time[p * (S + 1) + k0], xn[D], mn[D];
#pragma unroll
    for (int i = 0; i < D; ++i) {
      xn[i] = paths[(p * (S + 1) + k0) * D + i];
      mn[i] = mult[(p * S + k0) * D + i];
    }
    for (int k = k0; k < k1; ++k) {
      const float tk = tn;
      float x[D], m[D];
#pragma unroll
      for (int i = 0; i < D; ++i) { x[i] = xn[i]; m[i] = mn[i]; }
      if (k + 1 < k1) {
        tn = time[p * (S + 1) + k + 1];
#pragma unroll
        for (int i = 0; i < D; ++i) {
          xn[i] = paths[(p * (S + 1) + k + 1) * D + i];
          mn[i] = mult[(p * S + k + 1) * D + i];
        }
      }
      float dO[2] = {0.f, 0.f};
      {
        const float e = __fmul_rn(dgam, expf(-tk * rate));
#pragma unroll
        for (int i = 0; i < D; ++i) dO[i] = __fmul_rn(e, m[i]);
      }
      uint32_t mask1[2], mask2[2];
      // F1: inputs -> H1 (this tile's A1 buffer; the previous tile's W1 reads the other)
      unsigned char* A1 = sm.A1[buf];
      const uint32_t aA1 = tc::saddr_of(A1);
      tc::inputs_to_tile<D>(A1, tk, x);
      if (sync_or(fail)) { fail = true; break; }
      if (t == 0) {
        tc::fence_after_sync();
        issue_kk(tS, aA1, kSboA1, aB1, kSboA1, 1, kIdFwd);
        tc::mma_commit(tc::saddr_of(&sm.mbar));
      }
      bool ok = wait_phase(sm, phase);
      if (ok) relu_to_hh(tbase + kColS, sm.HH, kH1Col, mask1);
      if (sync_or(!ok)) { fail = true; break; }
      // F2: H1 -> H2
      if (t == 0) {
        tc::fence_after_sync();
        issue_kk(tS, aHH + (kH1Col / 8) * kCm, kSboHH, aB2, kSboB, kKH / 16, kIdFwd);
        tc::mma_commit(tc::saddr_of(&sm.mbar));
      }
      ok = wait_phase(sm, phase);
      if (ok) relu_to_hh(tbase + kColS, sm.HH, 0, mask2);
      if (sync_or(!ok)) { fail = true; break; }
      // F3: H2 -> H3; layer 4 backward
      if (t == 0) {
        tc::fence_after_sync();
        issue_kk(tS, aHH, kSboHH, aB3, kSboB, kKH / 16, kIdFwd);
        tc::mma_commit(tc::saddr_of(&sm.mbar));
      }
      ok = wait_phase(sm, phase);
      if (ok) layer4_backward<D>(sm, tbase + kColS, dO, acc4);
#pragma unroll
      for (int i = 0; i < D; ++i) bsum[i] = __fadd_rn(bsum[i], warp_sum(dO[i]));
      if (sync_or(!ok)) { fail = true; break; }
      // G3: dH2 = dZ3 W3
      if (t == 0) {
        tc::fence_after_sync();
        issue_dgrad(tS, aDZ, aB3);
        tc::mma_commit(tc::saddr_of(&sm.mbar));
      }
      ok = wait_phase(sm, phase);
      if (ok) masked_to_dz(tbase + kColS, sm.DZ, kH, mask2);
      if (sync_or(!ok)) { fail = true; break; }
      // G2: dH1 = dZ2 W2, and W: [dZ3 | dZ2]^T [H2 1 | H1 1]
      if (t == 0) {
        tc::fence_after_sync();
        issue_dgrad(tS, aDZ + (kH / 8) * kCm, aB2);
        issue_rows(tW, aDZ, kSboDZ, aHH, kSboHH, kIdW, accw);
        tc::mma_commit(tc::saddr_of(&sm.mbar));
      }
      accw = 1u;
      ok = wait_phase(sm, phase);
      if (ok) masked_split_to_dz(tbase + kColS, sm.DZ, mask1);
      if (sync_or(!ok)) { fail = true; break; }
      // W1: [dZ1 high | dZ1 low]^T A1; completion is covered by the next commit
      if (t == 0) {
        tc::fence_after_sync();
        issue_rows(tW1, aDZ, kSboDZ, aA1, kSboA1, kIdW1, acc1);
      }
      acc1 = 1u;
      buf ^= 1;
    }
  }
  // the last W1
  if (!sync_or(fail)) {
    if (t == 0) {
      tc::fence_after_sync();
      tc::mma_commit(tc::saddr_of(&sm.mbar));
    }
    if (!wait_phase(sm, phase)) fail = true;
  }
  fail = sync_or(fail);
  float* out = partials + (size_t)blockIdx.x * L::N;
  const float nanv = __int_as_float(0x7fc00000);
  if (!fail && accw) {
    // row t of W: dZ3 feature t (t < 64) against [H2 1], dZ2 feature t - 64 against [H1 1]
    const int j = t & (kH - 1);
    const int c0 = t < kH ? 0 : kH1Col;
#pragma unroll
    for (int c = 0; c < 5; ++c) {
      float v[16];
      tc::tmem_ld16(tbase + kColW + c0 + 16 * c, v);
#pragma unroll
      for (int jj = 0; jj < 16; ++jj) {
        const int i = 16 * c + jj;
        if (i < kH) out[(t < kH ? L::W3 : L::W2) + j * kH + i] = v[jj];
        else if (i == kH) out[(t < kH ? L::B3 : L::B2) + j] = v[jj];
      }
    }
    float v1[16];
    tc::tmem_ld16(tbase + kColW1, v1);
    float g1[4];  // dW1[j][0..D], db1[j] of this row's part
#pragma unroll
    for (int f = 0; f <= D; ++f) g1[f] = __fadd_rn(v1[3 * f], v1[3 * f + 1]);
    g1[D + 1] = v1[3 * (D + 1)];
    if (t >= kH) {
#pragma unroll
      for (int f = 0; f <= D + 1; ++f) sm.lo[j][f] = g1[f];
    }
    __syncthreads();
    if (t < kH) {
#pragma unroll
      for (int f = 0; f <= D; ++f) out[L::W1 + j * L::IN + f] = __fadd_rn(g1[f], sm.lo[j][f]);
      out[L::B1 + j] = __fadd_rn(g1[D + 1], sm.lo[j][D + 1]);
    }
  } else {
    __syncthreads();
    for (int e = t; e < L::B4; e += blockDim.x)
      if (e < L::W4) out[e] = fail ? nanv : 0.f;
  }
  // dW4 | db4: warps in order
#pragma unroll
  for (int c = 0; c < kH / 16; ++c) sm.red[wid][32 * c + lane] = acc4[c];
  if (lane == 0) {
    sm.red[wid][128] = bsum[0];
    sm.red[wid][129] = bsum[1];
  }
  __syncthreads();
  {
    const int c = t >> 5, l = t & 31, i = l >> 4, jj = 16 * c + (l & 15);
    if (i < D) {
      const float s = __fadd_rn(__fadd_rn(__fadd_rn(sm.red[0][t], sm.red[1][t]), sm.red[2][t]), sm.red[3][t]);
      out[L::W4 + i * kH + jj] = fail ? nanv : s;
    }
    if (t < D) {
      const float s = __fadd_rn(__fadd_rn(__fadd_rn(sm.red[0][128 + t], sm.red[1][128 + t]), sm.red[2][128 + t]),
                                sm.red[3][128 + t]);
      out[L::B4 + t] = fail ? nanv : s;
    }
  }
  if (fail && t == 0) atomicOr(status, SDEMC_ETIMEOUT);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  if (t < 32) tc::tmem_dealloc(sm.tmem, kCols);
}

__global__ void grad_reduce_tc_kernel(const float* __restrict__ partials, int nparts, int nparam,
                                      float* __restrict__ grad) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nparam) return;
  float s = 0.f;
  for (int c = 0; c < nparts; ++c) s += partials[(size_t)c * nparam + e];
  grad[e] = s;
}

constexpr size_t kSmemBytes = sizeof(BwdSmem) + 1024;

// Kernel attributes and resident CTAs per SM on device dev.
template <int D>
int per_sm_for(int dev, int* out) {
  auto kern = cv_backward_tc_kernel<D>;
  int rc = check_cuda(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemBytes),
                      "smem attribute");
  if (rc) return rc;
  if ((rc = check_cuda(cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout,
                                            (int)cudaSharedmemCarveoutMaxShared), "carveout attribute")))
    return rc;
  cudaFuncAttributes fa;
  int smem_sm = 0;
  if ((rc = check_cuda(cudaFuncGetAttributes(&fa, kern), "function attributes"))) return rc;
  if ((rc = check_cuda(cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev),
                       "smem per SM")))
    return rc;
  // resident CTAs per SM from registers, shared memory and tensor memory
  // (kCols of 512 columns each, so that no allocation ever waits)
  const int regs_cta = ((fa.numRegs + 7) / 8 * 8) * kRows;
  int per_sm = 65536 / (regs_cta > 0 ? regs_cta : 1);
  const int by_smem = smem_sm / (int)(kSmemBytes + 1024);
  if (per_sm > by_smem) per_sm = by_smem;
  if (per_sm > (int)(512 / kCols)) per_sm = (int)(512 / kCols);
  if (per_sm < 1) per_sm = 1;
  *out = per_sm;
  return SDEMC_OK;
}

// CTAs the backward launches for n paths of S steps (at most nparts).  The
// kernel attributes and the resident CTAs per SM are set up once per device,
// so a call inside a CUDA graph capture only launches.
template <int D>
int grid_for(int64_t n, int S, int nparts, int* grid) {
  static int per_sm_of[64] = {};  // per device ordinal; 0 = not set up yet
  int dev = 0;
  int rc = check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
  if (rc) return rc;
  int per_sm = dev < 64 ? per_sm_of[dev] : 0;
  if (per_sm < 1) {
    if ((rc = per_sm_for<D>(dev, &per_sm))) return rc;
    if (dev < 64) per_sm_of[dev] = per_sm;
  }
  const int64_t units = ((n + kRows - 1) / kRows) * ((S + kRangeLen - 1) / kRangeLen);
  int64_t ctas = (int64_t)num_sms() * per_sm;
  if (ctas > units) ctas = units;
  if (ctas > nparts) ctas = nparts;
  *grid = (int)(ctas < 1 ? 1 : ctas);
  return SDEMC_OK;
}

template <int D>
int launch_bwd(const float* prm, const float* time, const float* paths, const float* mult, const int64_t* idx,
               int64_t n, int S, float rate, const float* gamma, float* partials, int nparts, float* grad,
               int32_t* status, cudaStream_t s) {
  int grid = 1;
  int rc = grid_for<D>(n, S, nparts, &grid);
  if (rc) return rc;
  const int nranges = (S + kRangeLen - 1) / kRangeLen;
  cv_backward_tc_kernel<D><<<(unsigned)grid, kRows, kSmemBytes, s>>>(prm, time, paths, mult, idx, n, S, rate, gamma,
                                                                    nranges, partials, status);
  if ((rc = check_cuda(cudaGetLastError(), "cv_backward_tc_kernel launch"))) return rc;
  const int np = tc::TcLayout<D>::N;
  grad_reduce_tc_kernel<<<(np + 255) / 256, 256, 0, s>>>(partials, grid, np, grad);
  return check_cuda(cudaGetLastError(), "grad_reduce_tc_kernel launch");
}

}  // namespace tcb
}  // namespace sdemc

using namespace sdemc;

extern "C" int sdemc_cv_backward_tc(int dim, const float* d_params, const float* d_time, const float* d_paths,
                                    const float* d_mult, const int64_t* d_index, int64_t n, int steps,
                                    float disc_rate, const float* d_gamma, float* d_partials, int nparts,
                                    float* d_grad, int32_t* d_status, void* stream) {
  if (n < 1 || steps < 1 || nparts < 1 || !d_params || !d_time || !d_paths || !d_mult || !d_gamma ||
      !d_partials || !d_grad || !d_status)
    return fail(SDEMC_EINVAL, "bad cv_backward_tc arguments");
  cudaStream_t s = (cudaStream_t)stream;
  switch (dim) {
    case 1: return tcb::launch_bwd<1>(d_params, d_time, d_paths, d_mult, d_index, n, steps, disc_rate, d_gamma,
                                      d_partials, nparts, d_grad, d_status, s);
    case 2: return tcb::launch_bwd<2>(d_params, d_time, d_paths, d_mult, d_index, n, steps, disc_rate, d_gamma,
                                      d_partials, nparts, d_grad, d_status, s);
    default: return fail(SDEMC_EUNSUPPORTED, "control-variate network for dim %d (supported: 1, 2)", dim);
  }
}
