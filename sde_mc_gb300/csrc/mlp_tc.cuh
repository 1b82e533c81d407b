// mlp_tc.cuh — the control-variate network on 5th-generation tensor cores.
//
// One CTA of 128 threads evaluates the network on 128 rows at a time, one row
// per thread (a path's (t_k, X_k) at one step): layer 1 (1+d -> 64) in FP32 on
// the CUDA cores, written as a BF16 A tile to shared memory in the canonical
// no-swizzle K-major layout (8-row x 16-byte core matrices); the two 64x64
// layers as tcgen05.mma kind::f16 (M = 128, N = 64, K = 16 x 4) issued by one
// thread with FP32 accumulators in tensor memory (64 columns), completion
// signalled on an mbarrier; tcgen05.ld brings each thread its row back for
// bias + ReLU; layer 4 (64 -> d) in FP32.  The weights of the 64x64 layers
// stay in shared memory (BF16, the same layout, B operands K-major).
//
// Every wait on the mbarrier is bounded; a CTA that gives up records
// SDEMC_ETIMEOUT and stops issuing work, and always frees its tensor memory.
#pragma once
#include "sdemc_device.cuh"
#include <cuda_bf16.h>

namespace sdemc {
namespace tc {

constexpr int kRows = 128;        // M: rows per tile = threads per CTA
constexpr int kH = 64;            // hidden width (N and K of the 64x64 layers)
constexpr int kTmemCols = 64;     // FP32 accumulator columns
constexpr uint32_t kCoreRowBytes = 16;                   // one core-matrix row: 8 bf16
constexpr uint32_t kLbo = 128;                           // K-adjacent core matrices (8 rows x 16 B)
constexpr uint32_t kSbo = (kH / 8) * 128;                // M/N-adjacent core-matrix rows: 1024 B
constexpr uint32_t kTileBytesA = kRows * kH * 2;         // 16 KB
constexpr uint32_t kTileBytesB = kH * kH * 2;            // 8 KB
constexpr int kMaxSpins = 1 << 22;                       // bound of one mbarrier wait

// instruction descriptor, kind::f16: D = F32 (bits 4-5 = 1), A = B = BF16
// (bits 7-9 = 1, 10-12 = 1), both K-major (bits 15, 16 = 0), N >> 3 in bits
// 17-22, M >> 4 in bits 24-28.
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kH >> 3) << 17) |
                            ((uint32_t)(kRows >> 4) << 24);

// Byte offset of element (r, k) of a K-major bf16 matrix with 64 columns in
// the canonical no-swizzle layout.
SDEMC_HDI uint32_t core_offset(int r, int k) {
  return (uint32_t)(r >> 3) * kSbo + (uint32_t)(k >> 3) * kLbo + (uint32_t)(r & 7) * kCoreRowBytes +
         (uint32_t)(k & 7) * 2u;
}

// Shared-memory matrix descriptor: start >> 4 (bits 0-13), LBO >> 4 (16-29),
// SBO >> 4 (32-45), version 1 (bits 46-47), no swizzle (bits 61-63 = 0).
SDEMC_DI uint64_t smem_desc(uint32_t saddr) {
  return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)(kLbo >> 4) << 16) | ((uint64_t)(kSbo >> 4) << 32) |
         (1ull << 46);
}

SDEMC_DI uint32_t saddr_of(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

SDEMC_DI void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
SDEMC_DI void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
SDEMC_DI void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

SDEMC_DI void tmem_alloc(uint32_t slot_saddr) {  // whole warp
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(slot_saddr),
               "r"((uint32_t)kTmemCols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
SDEMC_DI void tmem_dealloc(uint32_t taddr) {  // whole warp
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"((uint32_t)kTmemCols)
               : "memory");
}

SDEMC_DI void mbar_init(uint32_t addr) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(addr) : "memory");
}

// Bounded wait for the phase with the given parity to complete.
SDEMC_DI bool mbar_wait(uint32_t addr, uint32_t parity) {
  for (int it = 0; it < kMaxSpins; ++it) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(addr), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// D (tmem) [+]= A (smem desc) x B (smem desc), one K = 16 slice.
SDEMC_DI void mma_f16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(kIdesc), "r"(accumulate)
      : "memory");
}
SDEMC_DI void mma_commit(uint32_t mbar_saddr) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar_saddr)
               : "memory");
}

SDEMC_DI void tmem_ld_wait() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

SDEMC_DI uint32_t pack2(float lo, float hi) {
  const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<const uint32_t*>(&v);
}

// Shared memory of one CTA (placed at a 1024-byte aligned address).
template <int D>
struct TcSmem {
  unsigned char A[kTileBytesA];   // activations, 128 x 64 bf16
  unsigned char B2[kTileBytesB];  // W2 (out x in), bf16, K-major
  unsigned char B3[kTileBytesB];  // W3
  float w1[kH * (D + 1)], b1[kH], b2[kH], b3[kH], w4[D * kH], b4[D];
  unsigned long long mbar;
  uint32_t tmem;
};

// Parameter vector offsets (torch order: W1, b1, W2, b2, W3, b3, W4, b4).
template <int D> struct TcLayout {
  static constexpr int IN = D + 1;
  static constexpr int W1 = 0, B1 = W1 + kH * IN, W2 = B1 + kH, B2 = W2 + kH * kH, W3 = B2 + kH,
                       B3 = W3 + kH * kH, W4 = B3 + kH, B4 = W4 + D * kH, N = B4 + D;
};

// CTA-wide setup: weights into shared memory, mbarrier, tensor memory.
template <int D>
SDEMC_DI void setup(TcSmem<D>& sm, const float* prm) {
  using L = TcLayout<D>;
  const int t = threadIdx.x;
  for (int e = t; e < kH * kH; e += blockDim.x) {
    const int n = e / kH, k = e % kH;
    *reinterpret_cast<__nv_bfloat16*>(sm.B2 + core_offset(n, k)) = __float2bfloat16_rn(prm[L::W2 + e]);
    *reinterpret_cast<__nv_bfloat16*>(sm.B3 + core_offset(n, k)) = __float2bfloat16_rn(prm[L::W3 + e]);
  }
  for (int e = t; e < kH * L::IN; e += blockDim.x) sm.w1[e] = prm[L::W1 + e];
  for (int e = t; e < kH; e += blockDim.x) {
    sm.b1[e] = prm[L::B1 + e];
    sm.b2[e] = prm[L::B2 + e];
    sm.b3[e] = prm[L::B3 + e];
  }
  for (int e = t; e < D * kH; e += blockDim.x) sm.w4[e] = prm[L::W4 + e];
  if (t < D) sm.b4[t] = prm[L::B4 + t];
  if (t == 0) {
    mbar_init(saddr_of(&sm.mbar));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  fence_async_smem();  // B tiles: generic-proxy stores, read by the tensor cores
  if (t < 32) tmem_alloc(saddr_of(&sm.tmem));
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
}

template <int D>
SDEMC_DI void teardown(TcSmem<D>& sm) {
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  if (threadIdx.x < 32) tmem_dealloc(sm.tmem);
}

// One 64x64 layer for the CTA's 128 rows: A (already in smem, fenced and
// synchronised) x W -> TMEM; returns false if the wait gave up.
template <int D>
SDEMC_DI bool layer_mma(TcSmem<D>& sm, const unsigned char* B, uint32_t& phase) {
  if (threadIdx.x == 0) {
    fence_after_sync();
    const uint32_t a0 = saddr_of(sm.A), b0 = saddr_of(B);
#pragma unroll
    for (int kk = 0; kk < kH / 16; ++kk)
      mma_f16(sm.tmem, smem_desc(a0 + kk * 2 * kLbo), smem_desc(b0 + kk * 2 * kLbo), kk > 0 ? 1u : 0u);
    mma_commit(saddr_of(&sm.mbar));
  }
  const bool ok = mbar_wait(saddr_of(&sm.mbar), phase);
  phase ^= 1u;
  fence_after_sync();
  return ok;
}

// 16 consecutive FP32 columns of this thread's TMEM lane.
SDEMC_DI void tmem_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

SDEMC_DI uint32_t lane_base() { return (uint32_t)((threadIdx.x >> 5) * 32) << 16; }

// Accumulator row + bias, ReLU, as the next layer's BF16 A row; 16 columns
// at a time so that few values are live.
template <int D>
SDEMC_DI void relu_to_A(TcSmem<D>& sm, const float* bias) {
  const uint32_t base = sm.tmem + lane_base();
#pragma unroll
  for (int c = 0; c < kH / 16; ++c) {
    float v[16];
    tmem_ld16(base + 16 * c, v);
    tmem_ld_wait();
#pragma unroll
    for (int j = 0; j < 16; ++j) v[j] = fmaxf(__fadd_rn(v[j], bias[16 * c + j]), 0.f);
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      uint4 q;
      q.x = pack2(v[8 * h + 0], v[8 * h + 1]);
      q.y = pack2(v[8 * h + 2], v[8 * h + 3]);
      q.z = pack2(v[8 * h + 4], v[8 * h + 5]);
      q.w = pack2(v[8 * h + 6], v[8 * h + 7]);
      *reinterpret_cast<uint4*>(sm.A + core_offset(threadIdx.x, 16 * c + 8 * h)) = q;
    }
  }
}

// Accumulator row + bias, ReLU, then layer 4 (64 -> d) in FP32.
template <int D>
SDEMC_DI void relu_layer4(TcSmem<D>& sm, float* out) {
  const uint32_t base = sm.tmem + lane_base();
  float o[D];
#pragma unroll
  for (int i = 0; i < D; ++i) o[i] = 0.f;
#pragma unroll
  for (int c = 0; c < kH / 16; ++c) {
    float v[16];
    tmem_ld16(base + 16 * c, v);
    tmem_ld_wait();
#pragma unroll
    for (int j = 0; j < 16; ++j) {
      const float h = fmaxf(__fadd_rn(v[j], sm.b3[16 * c + j]), 0.f);
#pragma unroll
      for (int i = 0; i < D; ++i) o[i] = __fmaf_rn(sm.w4[i * kH + 16 * c + j], h, o[i]);
    }
  }
#pragma unroll
  for (int i = 0; i < D; ++i) out[i] = __fadd_rn(o[i], sm.b4[i]);
}

// Layer 1 (FP32) of this thread's row, written as the BF16 A row.
template <int D>
SDEMC_DI void layer1_to_A(TcSmem<D>& sm, float t, const float* x) {
  using L = TcLayout<D>;
#pragma unroll
  for (int c = 0; c < kH / 8; ++c) {
    float h[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int j = 8 * c + u;
      float z = __fmaf_rn(sm.w1[j * L::IN], t, sm.b1[j]);
#pragma unroll
      for (int i = 0; i < D; ++i) z = __fmaf_rn(sm.w1[j * L::IN + 1 + i], x[i], z);
      h[u] = fmaxf(z, 0.f);
    }
    uint4 q;
    q.x = pack2(h[0], h[1]);
    q.y = pack2(h[2], h[3]);
    q.z = pack2(h[4], h[5]);
    q.w = pack2(h[6], h[7]);
    *reinterpret_cast<uint4*>(sm.A + core_offset(threadIdx.x, 8 * c)) = q;
  }
}

// The network on the CTA's 128 rows (this thread: row threadIdx.x with
// inputs t, x); out[D] = f(t, x).  All 128 threads call it together, the same
// number of times.  `fail` carries a gave-up wait from call to call: the
// barriers agree on it (__syncthreads_or), so once any thread's wait gave up
// every thread returns false from then on without touching the tensor cores.
template <int D>
SDEMC_DI bool forward_rows(TcSmem<D>& sm, float t, const float* x, float* out, uint32_t& phase, bool& fail) {
  layer1_to_A(sm, t, x);
  fence_async_smem();
  fence_before_sync();
  if (__syncthreads_or(fail)) { fail = true; return false; }
  bool ok = layer_mma(sm, sm.B2, phase);
  if (ok) relu_to_A(sm, sm.b2);
  fence_async_smem();
  fence_before_sync();
  if (__syncthreads_or(!ok)) { fail = true; return false; }
  ok = layer_mma(sm, sm.B3, phase);
  if (!ok) { fail = true; return false; }
  relu_layer4(sm, out);
  return true;
}

}  // namespace tc
}  // namespace sdemc
