// k_mlp.cu — K5/K6: the control-variate network on the GPU.
//
// The reference's adapted control variate (sde_mc/varred.py:98-199) is
//   Gamma_p = payoff_p + sum_k e^{-r t_k} sum_i f_i(t_k, X_k) dW_{k,i}
// with f = Mlp(1+d, [64, 64, 64], d) (ReLU, no batch norm, sde_mc/nets.py:39-93)
// and the loss Var(Gamma) over a minibatch of paths (unbiased), minimised by
// Adam.  Here:
//   * cv_forward_kernel — one warp per path, 16-step tiles: layer 1 (1+d -> 64)
//     and layer 4 (64 -> d) in FP32 on CUDA cores, the two 64x64 layers on BF16
//     tensor cores (mma.sync m16n8k16, FP32 accumulation; a layer's output
//     fragments are the next layer's input fragments, no data movement), then
//     Gamma_p.  Optionally writes f per row.
//   * cv_backward_kernel — CTAs of four warps stepping through their four
//     paths' tiles together: forward recompute, dgrad of the chain on tensor
//     cores, weight gradients of the 64x64 layers as tensor-core products over
//     the CTA's 64 rows (transposed operands staged in shared memory), the
//     small layers in FP32; one gradient partial per CTA.
//   * grad_reduce_kernel (fixed order over CTAs) and adam_kernel (torch.optim.Adam
//     semantics, FP32 master weights).
// Parameters are one FP32 vector in torch's order: W1 (64, 1+d), b1, W2 (64,64),
// b2, W3 (64,64), b3, W4 (d, 64), b4.
#include "sdemc_device.cuh"
#include "sdemc_host.cuh"
#include <cuda_bf16.h>

namespace sdemc {

constexpr int kH = 64;       // hidden width
constexpr int kWs = 72;      // padded row stride (bf16) of 64-wide smem matrices
constexpr int kTile = 16;    // rows (steps) per warp tile

template <int D> struct MlpLayout {
  static constexpr int IN = D + 1;
  static constexpr int W1 = 0, B1 = W1 + kH * IN, W2 = B1 + kH, B2 = W2 + kH * kH, W3 = B2 + kH,
                       B3 = W3 + kH * kH, W4 = B3 + kH, B4 = W4 + D * kH, N = B4 + D;
};

SDEMC_DI uint32_t pack_bf16(float lo, float hi) {
  const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<const uint32_t*>(&v);
}

SDEMC_DI void mma_bf16(float* c, const uint32_t* a, uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

SDEMC_DI uint32_t lds32(const __nv_bfloat16* p) { return *reinterpret_cast<const uint32_t*>(p); }

// Shared weights of the two tensor-core layers (bf16): row-major W (out, in)
// for forward B fragments and its transpose for dgrad B fragments.
struct SmemWeights {
  __nv_bfloat16 w2[kH * kWs], w3[kH * kWs], w2t[kH * kWs], w3t[kH * kWs];
};

SDEMC_DI void load_weights(SmemWeights& s, const float* prm, int off_w2, int off_w3, bool transposed) {
  for (int e = threadIdx.x; e < kH * kH; e += blockDim.x) {
    const int n = e / kH, k = e % kH;
    s.w2[n * kWs + k] = __float2bfloat16_rn(prm[off_w2 + e]);
    s.w3[n * kWs + k] = __float2bfloat16_rn(prm[off_w3 + e]);
    if (transposed) {
      s.w2t[k * kWs + n] = __float2bfloat16_rn(prm[off_w2 + e]);
      s.w3t[k * kWs + n] = __float2bfloat16_rn(prm[off_w3 + e]);
    }
  }
}

// acc (8 n-tiles x 4) = A (4 k-tiles of a 16x64 bf16 operand) x B, where B
// fragments come from a row-major (n, k) bf16 matrix in shared memory.
SDEMC_DI void gemm_16x64x64(float (*acc)[4], const uint32_t (*a)[4], const __nv_bfloat16* w) {
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
#pragma unroll
  for (int nt = 0; nt < 8; ++nt) {
#pragma unroll
    for (int kt = 0; kt < 4; ++kt) {
      const __nv_bfloat16* row = w + (nt * 8 + g) * kWs + kt * 16 + 2 * t;
      mma_bf16(acc[nt], a[kt], lds32(row), lds32(row + 8));
    }
  }
}

// C fragments (8 n-tiles) -> A fragments (4 k-tiles) of the next product.
SDEMC_DI void c_to_a(const float (*c)[4], uint32_t (*a)[4]) {
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    a[j][0] = pack_bf16(c[2 * j][0], c[2 * j][1]);
    a[j][1] = pack_bf16(c[2 * j][2], c[2 * j][3]);
    a[j][2] = pack_bf16(c[2 * j + 1][0], c[2 * j + 1][1]);
    a[j][3] = pack_bf16(c[2 * j + 1][2], c[2 * j + 1][3]);
  }
}

// Column of C element (n-tile nt, slot e): rows g (e<2) or g+8, cols 8nt+2t+(e&1).
SDEMC_DI int ccol(int nt, int e) { return nt * 8 + 2 * (threadIdx.x & 3) + (e & 1); }

// Per-row inputs of a tile: t_k, X_k (d), dW_k (d) and validity.
template <int D>
struct RowIn {
  float t, x[D], dw[D];
  bool valid;
};

template <int D>
SDEMC_DI RowIn<D> load_row(const float* time, const float* paths, const float* normals, int S, int64_t p,
                           int k) {
  RowIn<D> r;
  r.valid = k < S;
  const int kk = r.valid ? k : S - 1;
  r.t = time[p * (S + 1) + kk];
#pragma unroll
  for (int i = 0; i < D; ++i) {
    r.x[i] = paths[(p * (S + 1) + kk) * D + i];
    r.dw[i] = r.valid ? normals[(p * S + kk) * D + i] : 0.f;
  }
  return r;
}

// Forward of one 16-row tile.  Fills H1/H2 A fragments, H3 (fp32 C layout)
// and the outputs O for rows g and g+8 (every lane of the group holds them).
template <int D>
SDEMC_DI void tile_forward(const float* prm, const SmemWeights& sw, const RowIn<D>& r0, const RowIn<D>& r1,
                           uint32_t (*h1a)[4], uint32_t (*h2a)[4], float (*h3)[4], float* o0, float* o1) {
  using ML = MlpLayout<D>;
  float c[8][4];
  // layer 1 in FP32: rows g (slots 0,1) and g+8 (slots 2,3)
#pragma unroll
  for (int nt = 0; nt < 8; ++nt)
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const int n = ccol(nt, e);
      const RowIn<D>& r = e < 2 ? r0 : r1;
      float z = __fmaf_rn(prm[ML::W1 + n * ML::IN + 0], r.t, prm[ML::B1 + n]);
#pragma unroll
      for (int i = 0; i < D; ++i) z = __fmaf_rn(prm[ML::W1 + n * ML::IN + 1 + i], r.x[i], z);
      c[nt][e] = fmaxf(z, 0.f);
    }
  c_to_a(c, h1a);
  // layer 2 (tensor cores)
#pragma unroll
  for (int nt = 0; nt < 8; ++nt)
#pragma unroll
    for (int e = 0; e < 4; ++e) c[nt][e] = prm[ML::B2 + ccol(nt, e)];
  gemm_16x64x64(c, h1a, sw.w2);
#pragma unroll
  for (int nt = 0; nt < 8; ++nt)
#pragma unroll
    for (int e = 0; e < 4; ++e) c[nt][e] = fmaxf(c[nt][e], 0.f);
  c_to_a(c, h2a);
  // layer 3
#pragma unroll
  for (int nt = 0; nt < 8; ++nt)
#pragma unroll
    for (int e = 0; e < 4; ++e) h3[nt][e] = prm[ML::B3 + ccol(nt, e)];
  gemm_16x64x64(h3, h2a, sw.w3);
#pragma unroll
  for (int nt = 0; nt < 8; ++nt)
#pragma unroll
    for (int e = 0; e < 4; ++e) h3[nt][e] = fmaxf(h3[nt][e], 0.f);
  // layer 4 in FP32: partial dot products over the lane's 16 columns, then
  // the 4 lanes of the group (xor 1, 2) complete them
#pragma unroll
  for (int i = 0; i < D; ++i) {
    float s0 = 0.f, s1 = 0.f;
#pragma unroll
    for (int nt = 0; nt < 8; ++nt)
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const float w = prm[ML::W4 + i * kH + ccol(nt, e)];
        if (e < 2) s0 = __fmaf_rn(w, h3[nt][e], s0);
        else s1 = __fmaf_rn(w, h3[nt][e], s1);
      }
    s0 += __shfl_xor_sync(kFull, s0, 1);
    s0 += __shfl_xor_sync(kFull, s0, 2);
    s1 += __shfl_xor_sync(kFull, s1, 1);
    s1 += __shfl_xor_sync(kFull, s1, 2);
    o0[i] = s0 + prm[ML::B4 + i];
    o1[i] = s1 + prm[ML::B4 + i];
  }
}

// Sum over a tile of e^{-r t} f . dW for the valid rows (same value in all lanes).
template <int D>
SDEMC_DI float tile_cv(const RowIn<D>& r0, const RowIn<D>& r1, const float* o0, const float* o1, float rate) {
  const int t = threadIdx.x & 3;
  float v = 0.f;
  if (t == 0) {
    float a = 0.f, b = 0.f;
#pragma unroll
    for (int i = 0; i < D; ++i) {
      a = __fmaf_rn(o0[i], r0.dw[i], a);
      b = __fmaf_rn(o1[i], r1.dw[i], b);
    }
    if (r0.valid) v = __fmul_rn(expf(-r0.t * rate), a);
    if (r1.valid) v = __fadd_rn(v, __fmul_rn(expf(-r1.t * rate), b));
  }
  return warp_sum(v);
}

// Gamma_p for paths idx[0..n): one warp per path.
template <int D>
__global__ void __launch_bounds__(128)
cv_forward_kernel(const float* __restrict__ prm, const float* __restrict__ time, const float* __restrict__ paths,
                  const float* __restrict__ normals, const float* __restrict__ payoffs, const int64_t* idx,
                  int64_t n, int S, float rate, float* __restrict__ gamma, float* __restrict__ fout) {
  __shared__ SmemWeights sw;
  using ML = MlpLayout<D>;
  load_weights(sw, prm, ML::W2, ML::W3, false);
  __syncthreads();
  const int lane = threadIdx.x & 31, g = lane >> 2;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t q = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); q < n; q += warps) {
    const int64_t p = idx ? idx[q] : q;
    float acc = 0.f;
    for (int k0 = 0; k0 < S; k0 += kTile) {
      const RowIn<D> r0 = load_row<D>(time, paths, normals, S, p, k0 + g);
      const RowIn<D> r1 = load_row<D>(time, paths, normals, S, p, k0 + g + 8);
      uint32_t h1a[4][4], h2a[4][4];
      float h3[8][4], o0[D], o1[D];
      tile_forward<D>(prm, sw, r0, r1, h1a, h2a, h3, o0, o1);
      acc = __fadd_rn(acc, tile_cv<D>(r0, r1, o0, o1, rate));
      if (fout && (lane & 3) == 0) {
#pragma unroll
        for (int i = 0; i < D; ++i) {
          if (r0.valid) fout[(p * S + k0 + g) * D + i] = o0[i];
          if (r1.valid) fout[(p * S + k0 + g + 8) * D + i] = o1[i];
        }
      }
    }
    if (lane == 0) gamma[q] = __fadd_rn(payoffs[p], acc);
  }
}

// ------------------------------------------------------------ backward ----
constexpr int kBwdWarps = 4;
constexpr int kRows = kBwdWarps * kTile;  // 64 rows per CTA step
constexpr int kTs = kRows + 8;            // stride of the transposed buffers
constexpr int kRedLen = 512;              // FP32 small-layer gradient slots per warp

struct SmemBwd {
  SmemWeights w;
  // transposed operands of the tensor-core weight gradients: [feature][row]
  __nv_bfloat16 h1t[(kH + 8) * kTs], h2t[(kH + 8) * kTs];  // row kH = ones (bias column)
  __nv_bfloat16 dz2t[kH * kTs], dz3t[kH * kTs];
  float red[kBwdWarps][kRedLen];                          // per-warp small-layer accumulators
  float gmean;
};

template <int D>
__global__ void __launch_bounds__(128, 1)
cv_backward_kernel(const float* __restrict__ prm, const float* __restrict__ time, const float* __restrict__ paths,
                   const float* __restrict__ normals, const int64_t* idx, int64_t n, int S, float rate,
                   const float* __restrict__ gamma, float* __restrict__ partials) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  SmemBwd& sm = *reinterpret_cast<SmemBwd*>(smem_raw);
  using ML = MlpLayout<D>;
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3, wid = threadIdx.x >> 5;
  load_weights(sm.w, prm, ML::W2, ML::W3, true);
  // ones row (bias column) of the activation buffers; zero pad rows
  for (int e = threadIdx.x; e < 8 * kTs; e += blockDim.x) {
    const int row = kH + e / kTs;
    const __nv_bfloat16 v = __float2bfloat16_rn(row == kH ? 1.f : 0.f);
    sm.h1t[row * kTs + e % kTs] = v;
    sm.h2t[row * kTs + e % kTs] = v;
  }
  for (int e = threadIdx.x; e < kBwdWarps * kRedLen; e += blockDim.x) sm.red[e / kRedLen][e % kRedLen] = 0.f;
  // minibatch mean of Gamma, fixed order (every CTA computes the same bits)
  {
    __shared__ double part[128];
    double a = 0.0;
    for (int64_t q = threadIdx.x; q < n; q += blockDim.x) a += (double)gamma[q];
    part[threadIdx.x] = a;
    __syncthreads();
    for (int o = 64; o > 0; o >>= 1) {
      if ((int)threadIdx.x < o) part[threadIdx.x] += part[threadIdx.x + o];
      __syncthreads();
    }
    if (threadIdx.x == 0) sm.gmean = (float)(part[0] / (double)n);
  }
  __syncthreads();
  const float gmean = sm.gmean;
  const float scale = 2.0f / (float)(n > 1 ? n - 1 : 1);
  // tensor-core weight-gradient accumulators: rows [16w, 16w+16) of dW2 and
  // dW3, 9 column tiles (64 inputs + bias column)
  float acc2[9][4], acc3[9][4];
#pragma unroll
  for (int j = 0; j < 9; ++j)
#pragma unroll
    for (int e = 0; e < 4; ++e) { acc2[j][e] = 0.f; acc3[j][e] = 0.f; }
  float* red = sm.red[wid];  // [0, 64*IN) dW1, [64*IN, 64*IN+64) db1, then dW4 (D*64), db4 (D)
  constexpr int R_B1 = kH * ML::IN, R_W4 = R_B1 + kH, R_B4 = R_W4 + D * kH;
  static_assert(R_B4 + D <= kRedLen, "accumulator space");
  const int64_t groups = (n + kBwdWarps - 1) / kBwdWarps;
  for (int64_t grp = blockIdx.x; grp < groups; grp += gridDim.x) {
    const int64_t q = grp * kBwdWarps + wid;
    const bool has = q < n;
    const int64_t p = has ? (idx ? idx[q] : q) : 0;
    const float dgam = has ? __fmul_rn(scale, __fsub_rn(gamma[q], gmean)) : 0.f;
    for (int k0 = 0; k0 < S; k0 += kTile) {
      RowIn<D> r0 = load_row<D>(time, paths, normals, S, p, k0 + g);
      RowIn<D> r1 = load_row<D>(time, paths, normals, S, p, k0 + g + 8);
      if (!has) { r0.valid = false; r1.valid = false; }
      uint32_t h1a[4][4], h2a[4][4];
      float h3[8][4], o0[D], o1[D];
      tile_forward<D>(prm, sm.w, r0, r1, h1a, h2a, h3, o0, o1);
      // dO = dGamma e^{-rt} dW (zero on padded rows)
      float d0[D], d1[D];
      const float e0 = r0.valid ? __fmul_rn(dgam, expf(-r0.t * rate)) : 0.f;
      const float e1 = r1.valid ? __fmul_rn(dgam, expf(-r1.t * rate)) : 0.f;
#pragma unroll
      for (int i = 0; i < D; ++i) { d0[i] = __fmul_rn(e0, r0.dw[i]); d1[i] = __fmul_rn(e1, r1.dw[i]); }
      // layer 4 backward (FP32): dZ3 = (dO W4) * [H3 > 0]; dW4 += dO^T H3
      float dz[8][4];
#pragma unroll
      for (int nt = 0; nt < 8; ++nt)
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          const int col = ccol(nt, e);
          float s = 0.f;
#pragma unroll
          for (int i = 0; i < D; ++i) s = __fmaf_rn(e < 2 ? d0[i] : d1[i], prm[ML::W4 + i * kH + col], s);
          dz[nt][e] = h3[nt][e] > 0.f ? s : 0.f;
        }
#pragma unroll
      for (int i = 0; i < D; ++i) {
#pragma unroll
        for (int nt = 0; nt < 8; ++nt)
#pragma unroll
          for (int c2 = 0; c2 < 2; ++c2) {
            float v = __fmaf_rn(d0[i], h3[nt][c2], __fmul_rn(d1[i], h3[nt][2 + c2]));
            v += __shfl_xor_sync(kFull, v, 4);
            v += __shfl_xor_sync(kFull, v, 8);
            v += __shfl_xor_sync(kFull, v, 16);
            if (g == 0) red[R_W4 + i * kH + nt * 8 + 2 * t + c2] += v;
          }
        float b = __fadd_rn(d0[i], d1[i]);
        b += __shfl_xor_sync(kFull, b, 4);
        b += __shfl_xor_sync(kFull, b, 8);
        b += __shfl_xor_sync(kFull, b, 16);
        if (lane == 0) red[R_B4 + i] += b;
      }
      // stage dZ3^T and H2^T for dW3; dH2 = dZ3 W3 on tensor cores
      uint32_t dza[4][4];
      c_to_a(dz, dza);
#pragma unroll
      for (int nt = 0; nt < 8; ++nt)
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          const int col = ccol(nt, e), row = wid * kTile + g + (e < 2 ? 0 : 8);
          sm.dz3t[col * kTs + row] = __float2bfloat16_rn(dz[nt][e]);
        }
      // H2 values (bf16) from its A fragments: element (row, col) order as C
#pragma unroll
      for (int j = 0; j < 4; ++j)
#pragma unroll
        for (int r = 0; r < 4; ++r) {
          const __nv_bfloat162 v = *reinterpret_cast<const __nv_bfloat162*>(&h2a[j][r]);
          const int col = j * 16 + (r >> 1) * 8 + 2 * t, row = wid * kTile + g + ((r & 1) ? 8 : 0);
          sm.h2t[col * kTs + row] = v.x;
          sm.h2t[(col + 1) * kTs + row] = v.y;
        }
      float c[8][4];
#pragma unroll
      for (int nt = 0; nt < 8; ++nt)
#pragma unroll
        for (int e = 0; e < 4; ++e) c[nt][e] = 0.f;
      gemm_16x64x64(c, dza, sm.w.w3t);
      // dZ2 = dH2 * [H2 > 0]
#pragma unroll
      for (int j = 0; j < 4; ++j)
#pragma unroll
        for (int r = 0; r < 4; ++r) {
          const __nv_bfloat162 v = *reinterpret_cast<const __nv_bfloat162*>(&h2a[j][r]);
          const int nt = 2 * j + (r >> 1), e = (r & 1) * 2;
          if (!(__bfloat162float(v.x) > 0.f)) c[nt][e] = 0.f;
          if (!(__bfloat162float(v.y) > 0.f)) c[nt][e + 1] = 0.f;
        }
#pragma unroll
      for (int nt = 0; nt < 8; ++nt)
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          const int col = ccol(nt, e), row = wid * kTile + g + (e < 2 ? 0 : 8);
          sm.dz2t[col * kTs + row] = __float2bfloat16_rn(c[nt][e]);
        }
#pragma unroll
      for (int j = 0; j < 4; ++j)
#pragma unroll
        for (int r = 0; r < 4; ++r) {
          const __nv_bfloat162 v = *reinterpret_cast<const __nv_bfloat162*>(&h1a[j][r]);
          const int col = j * 16 + (r >> 1) * 8 + 2 * t, row = wid * kTile + g + ((r & 1) ? 8 : 0);
          sm.h1t[col * kTs + row] = v.x;
          sm.h1t[(col + 1) * kTs + row] = v.y;
        }
      // dH1 = dZ2 W2; dZ1 = dH1 * [H1 > 0]
      uint32_t dz2a[4][4];
      c_to_a(c, dz2a);
#pragma unroll
      for (int nt = 0; nt < 8; ++nt)
#pragma unroll
        for (int e = 0; e < 4; ++e) dz[nt][e] = 0.f;
      gemm_16x64x64(dz, dz2a, sm.w.w2t);
#pragma unroll
      for (int j = 0; j < 4; ++j)
#pragma unroll
        for (int r = 0; r < 4; ++r) {
          const __nv_bfloat162 v = *reinterpret_cast<const __nv_bfloat162*>(&h1a[j][r]);
          const int nt = 2 * j + (r >> 1), e = (r & 1) * 2;
          if (!(__bfloat162float(v.x) > 0.f)) dz[nt][e] = 0.f;
          if (!(__bfloat162float(v.y) > 0.f)) dz[nt][e + 1] = 0.f;
        }
      // layer 1 weight gradient (FP32): dW1 += dZ1^T [t, X], db1 += sum dZ1
#pragma unroll
      for (int nt = 0; nt < 8; ++nt)
#pragma unroll
        for (int c2 = 0; c2 < 2; ++c2) {
          const int col = nt * 8 + 2 * t + c2;
          const float a = dz[nt][c2], b = dz[nt][2 + c2];
#pragma unroll
          for (int f = 0; f <= D; ++f) {
            const float x0 = f == 0 ? r0.t : r0.x[f > 0 ? f - 1 : 0];
            const float x1 = f == 0 ? r1.t : r1.x[f > 0 ? f - 1 : 0];
            float v = __fmaf_rn(a, x0, __fmul_rn(b, x1));
            v += __shfl_xor_sync(kFull, v, 4);
            v += __shfl_xor_sync(kFull, v, 8);
            v += __shfl_xor_sync(kFull, v, 16);
            if (g == 0) red[col * ML::IN + f] += v;
          }
          float s = __fadd_rn(a, b);
          s += __shfl_xor_sync(kFull, s, 4);
          s += __shfl_xor_sync(kFull, s, 8);
          s += __shfl_xor_sync(kFull, s, 16);
          if (g == 0) red[R_B1 + col] += s;
        }
      __syncthreads();
      // tensor-core weight gradients over the CTA's 64 rows: this warp owns
      // output rows [16w, 16w+16) of dW2 (dZ2^T H1) and dW3 (dZ3^T H2)
#pragma unroll
      for (int ks = 0; ks < kRows / 16; ++ks) {
        uint32_t a2[4], a3[4];
        const int m = wid * 16 + g, kk = ks * 16 + 2 * t;
        a2[0] = lds32(&sm.dz2t[m * kTs + kk]);
        a2[1] = lds32(&sm.dz2t[(m + 8) * kTs + kk]);
        a2[2] = lds32(&sm.dz2t[m * kTs + kk + 8]);
        a2[3] = lds32(&sm.dz2t[(m + 8) * kTs + kk + 8]);
        a3[0] = lds32(&sm.dz3t[m * kTs + kk]);
        a3[1] = lds32(&sm.dz3t[(m + 8) * kTs + kk]);
        a3[2] = lds32(&sm.dz3t[m * kTs + kk + 8]);
        a3[3] = lds32(&sm.dz3t[(m + 8) * kTs + kk + 8]);
#pragma unroll
        for (int j = 0; j < 9; ++j) {
          const int nn = j * 8 + g;
          mma_bf16(acc2[j], a2, lds32(&sm.h1t[nn * kTs + kk]), lds32(&sm.h1t[nn * kTs + kk + 8]));
          mma_bf16(acc3[j], a3, lds32(&sm.h2t[nn * kTs + kk]), lds32(&sm.h2t[nn * kTs + kk + 8]));
        }
      }
      __syncthreads();
    }
  }
  // write this CTA's gradient partial (torch parameter order)
  float* out = partials + (size_t)blockIdx.x * ML::N;
#pragma unroll
  for (int j = 0; j < 9; ++j)
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const int row = wid * 16 + g + (e < 2 ? 0 : 8), col = j * 8 + 2 * t + (e & 1);
      if (col < kH) {
        out[ML::W2 + row * kH + col] = acc2[j][e];
        out[ML::W3 + row * kH + col] = acc3[j][e];
      } else if (col == kH) {
        out[ML::B2 + row] = acc2[j][e];
        out[ML::B3 + row] = acc3[j][e];
      }
    }
  __syncthreads();
  for (int e = threadIdx.x; e < R_B4 + D; e += blockDim.x) {
    const float v = ((sm.red[0][e] + sm.red[1][e]) + sm.red[2][e]) + sm.red[3][e];
    if (e < R_B1) out[ML::W1 + e] = v;
    else if (e < R_W4) out[ML::B1 + (e - R_B1)] = v;
    else if (e < R_B4) out[ML::W4 + (e - R_W4)] = v;
    else out[ML::B4 + (e - R_B4)] = v;
  }
}

__global__ void grad_reduce_kernel(const float* __restrict__ partials, int nparts, int nparam,
                                   float* __restrict__ grad) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nparam) return;
  float s = 0.f;
  for (int c = 0; c < nparts; ++c) s += partials[(size_t)c * nparam + e];
  grad[e] = s;
}

// torch.optim.Adam (no weight decay, no amsgrad): m = b1 m + (1-b1) g,
// v = b2 v + (1-b2) g^2, p -= lr/(1-b1^t) * m / (sqrt(v)/sqrt(1-b2^t) + eps).
SDEMC_DI void adam_update(int e, float* __restrict__ prm, const float* __restrict__ grad, float* __restrict__ m,
                          float* __restrict__ v, float lr, float b1, float b2, float eps, float bc1,
                          float bc2_sqrt) {
  const float gr = grad[e];
  const float mm = b1 * m[e] + (1.f - b1) * gr;
  const float vv = b2 * v[e] + (1.f - b2) * gr * gr;
  m[e] = mm;
  v[e] = vv;
  prm[e] -= (lr / bc1) * mm / (sqrtf(vv) / bc2_sqrt + eps);
}

__global__ void adam_kernel(float* __restrict__ prm, const float* __restrict__ grad, float* __restrict__ m,
                            float* __restrict__ v, int nparam, float lr, float b1, float b2, float eps,
                            float bc1, float bc2_sqrt) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e < nparam) adam_update(e, prm, grad, m, v, lr, b1, b2, eps, bc1, bc2_sqrt);
}

// The same step with the bias corrections read from device memory (bc[0] =
// 1 - b1^t, bc[1] = sqrt(1 - b2^t)), so a captured graph of many steps takes
// each step's corrections from a table the host refills between replays.
__global__ void adam_dev_kernel(float* __restrict__ prm, const float* __restrict__ grad, float* __restrict__ m,
                                float* __restrict__ v, int nparam, float lr, float b1, float b2, float eps,
                                const float* __restrict__ bc) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e < nparam) adam_update(e, prm, grad, m, v, lr, b1, b2, eps, bc[0], bc[1]);
}

template <int D>
static int launch_cv_forward(const float* prm, const float* time, const float* paths, const float* normals,
                             const float* payoffs, const int64_t* idx, int64_t n, int S, float rate, float* gamma,
                             float* fout, cudaStream_t s) {
  const int threads = 128;
  int64_t ctas = (n + 3) / 4;
  const int64_t cap = (int64_t)num_sms() * 16;
  if (ctas > cap) ctas = cap;
  if (ctas < 1) ctas = 1;
  cv_forward_kernel<D><<<(unsigned)ctas, threads, 0, s>>>(prm, time, paths, normals, payoffs, idx, n, S, rate,
                                                        gamma, fout);
  return check_cuda(cudaGetLastError(), "cv_forward_kernel launch");
}

template <int D>
static int launch_cv_backward(const float* prm, const float* time, const float* paths, const float* normals,
                              const int64_t* idx, int64_t n, int S, float rate, const float* gamma,
                              float* partials, int nparts, cudaStream_t s) {
  const size_t smem = sizeof(SmemBwd);
  int rc = check_cuda(cudaFuncSetAttribute(cv_backward_kernel<D>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)smem), "smem attribute");
  if (rc) return rc;
  cv_backward_kernel<D><<<nparts, kBwdWarps * 32, smem, s>>>(prm, time, paths, normals, idx, n, S, rate, gamma,
                                                            partials);
  return check_cuda(cudaGetLastError(), "cv_backward_kernel launch");
}

}  // namespace sdemc

using namespace sdemc;

extern "C" int sdemc_cv_nparams(int dim) {
  switch (dim) {
    case 1: return MlpLayout<1>::N;
    case 2: return MlpLayout<2>::N;
    default: return 0;
  }
}

extern "C" int sdemc_cv_forward(int dim, const float* d_params, const float* d_time, const float* d_paths,
                                const float* d_normals, const float* d_payoffs, const int64_t* d_index, int64_t n,
                                int steps, float disc_rate, float* d_gamma, float* d_fout, void* stream) {
  if (n < 0 || steps < 1 || !d_params || !d_time || !d_paths || !d_normals || !d_payoffs || !d_gamma)
    return fail(SDEMC_EINVAL, "bad cv_forward arguments");
  if (n == 0) return SDEMC_OK;
  cudaStream_t s = (cudaStream_t)stream;
  switch (dim) {
    case 1: return launch_cv_forward<1>(d_params, d_time, d_paths, d_normals, d_payoffs, d_index, n, steps,
                                        disc_rate, d_gamma, d_fout, s);
    case 2: return launch_cv_forward<2>(d_params, d_time, d_paths, d_normals, d_payoffs, d_index, n, steps,
                                        disc_rate, d_gamma, d_fout, s);
    default: return fail(SDEMC_EUNSUPPORTED, "control-variate network for dim %d (supported: 1, 2)", dim);
  }
}

extern "C" int sdemc_cv_backward(int dim, const float* d_params, const float* d_time, const float* d_paths,
                                 const float* d_normals, const int64_t* d_index, int64_t n, int steps,
                                 float disc_rate, const float* d_gamma, float* d_partials, int nparts,
                                 float* d_grad, void* stream) {
  if (n < 1 || steps < 1 || nparts < 1 || !d_params || !d_time || !d_paths || !d_normals || !d_gamma ||
      !d_partials || !d_grad)
    return fail(SDEMC_EINVAL, "bad cv_backward arguments");
  cudaStream_t s = (cudaStream_t)stream;
  int rc;
  switch (dim) {
    case 1: rc = launch_cv_backward<1>(d_params, d_time, d_paths, d_normals, d_index, n, steps, disc_rate, d_gamma,
                                       d_partials, nparts, s); break;
    case 2: rc = launch_cv_backward<2>(d_params, d_time, d_paths, d_normals, d_index, n, steps, disc_rate, d_gamma,
                                       d_partials, nparts, s); break;
    default: return fail(SDEMC_EUNSUPPORTED, "control-variate network for dim %d (supported: 1, 2)", dim);
  }
  if (rc) return rc;
  const int np = sdemc_cv_nparams(dim);
  grad_reduce_kernel<<<(np + 255) / 256, 256, 0, s>>>(d_partials, nparts, np, d_grad);
  return check_cuda(cudaGetLastError(), "grad_reduce_kernel launch");
}

extern "C" int sdemc_adam_bias(int step, float beta1, float beta2, float* h_bc) {
  if (step < 1 || !h_bc) return fail(SDEMC_EINVAL, "bad adam_bias args");
  h_bc[0] = 1.f - powf(beta1, (float)step);
  h_bc[1] = sqrtf(1.f - powf(beta2, (float)step));
  return SDEMC_OK;
}

extern "C" int sdemc_adam_step(float* d_params, const float* d_grad, float* d_m, float* d_v, int nparam, int step,
                               float lr, float beta1, float beta2, float eps, void* stream) {
  if (nparam < 1 || step < 1 || !d_params || !d_grad || !d_m || !d_v) return fail(SDEMC_EINVAL, "bad adam args");
  float bc[2];
  sdemc_adam_bias(step, beta1, beta2, bc);
  adam_kernel<<<(nparam + 255) / 256, 256, 0, (cudaStream_t)stream>>>(d_params, d_grad, d_m, d_v, nparam, lr, beta1,
                                                                      beta2, eps, bc[0], bc[1]);
  return check_cuda(cudaGetLastError(), "adam_kernel launch");
}

extern "C" int sdemc_adam_step_dev(float* d_params, const float* d_grad, float* d_m, float* d_v, int nparam,
                                   const float* d_bc, float lr, float beta1, float beta2, float eps, void* stream) {
  if (nparam < 1 || !d_params || !d_grad || !d_m || !d_v || !d_bc) return fail(SDEMC_EINVAL, "bad adam args");
  adam_dev_kernel<<<(nparam + 255) / 256, 256, 0, (cudaStream_t)stream>>>(d_params, d_grad, d_m, d_v, nparam, lr,
                                                                          beta1, beta2, eps, d_bc);
  return check_cuda(cudaGetLastError(), "adam_dev_kernel launch");
}
