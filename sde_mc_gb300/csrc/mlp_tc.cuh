// mlp_tc.cuh — the control-variate network on 5th-generation tensor cores.
//
// One CTA of 128 threads evaluates the network on 128 rows at a time, one row
// per thread (a path's (t_k, X_k) at one step).  Three tcgen05.mma kind::f16
// products (M = 128, issued by one thread, FP32 accumulators in 64 columns of
// tensor memory, completion on an mbarrier) carry the first three layers:
//
//   layer 1 (1+d -> 64): K = 16.  FP32 accuracy from BF16 operands by
//     splitting inputs and weights into high and low BF16 parts:
//     x w ~ xh wh + xl wh + xh wl (the dropped xl wl is ~2^-16 relative), the
//     bias as bh + bl against two ones columns;
//   layers 2, 3 (64 -> 64): K = 80 = 64 activations + the bias (high, low)
//     against two ones columns + 14 zero columns.
//
// Operands sit in shared memory in the canonical no-swizzle K-major layout
// (8-row x 16-byte core matrices; K-adjacent core matrices 128 B apart, row
// groups K/8 x 128 B apart).  After each product every thread reads its own
// row back with tcgen05.ld, applies ReLU and writes the BF16 row of the next
// A tile; layer 4 (64 -> d) stays in FP32 on the CUDA cores.
//
// Every wait on the mbarrier is bounded; a CTA that gives up records
// SDEMC_ETIMEOUT, stops issuing work and always frees its tensor memory.
#pragma once
#include "sdemc_device.cuh"
#include <cuda_bf16.h>

namespace sdemc {
namespace tc {

constexpr int kRows = 128;        // M: rows per tile = threads per CTA
constexpr int kH = 64;            // hidden width (N of every product)
constexpr int kK1 = 16;           // K of layer 1 (split inputs, bias)
constexpr int kKH = 80;           // K of layers 2, 3 (64 + bias + padding)
constexpr int kTmemCols = 64;     // FP32 accumulator columns
constexpr uint32_t kLbo = 128;    // K-adjacent core matrices
constexpr int kMaxSpins = 1 << 22;  // bound of one mbarrier wait

// instruction descriptor, kind::f16: D = F32 (bits 4-5 = 1), A = B = BF16
// (bits 7-9 = 1, 10-12 = 1), both K-major (bits 15, 16 = 0), N >> 3 in bits
// 17-22, M >> 4 in bits 24-28.
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kH >> 3) << 17) |
                            ((uint32_t)(kRows >> 4) << 24);

// Byte offset of element (r, k) of a K-major bf16 matrix with K columns in
// the canonical no-swizzle layout.
SDEMC_HDI uint32_t core_offset(int r, int k, int K) {
  return (uint32_t)(r >> 3) * (uint32_t)(K / 8) * 128u + (uint32_t)(k >> 3) * kLbo + (uint32_t)(r & 7) * 16u +
         (uint32_t)(k & 7) * 2u;
}

// Shared-memory matrix descriptor: start >> 4 (bits 0-13), LBO >> 4 (16-29),
// SBO >> 4 (32-45), version 1 (bits 46-47), no swizzle (bits 61-63 = 0).
SDEMC_DI uint64_t smem_desc(uint32_t saddr, uint32_t sbo) {
  return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)(kLbo >> 4) << 16) | ((uint64_t)(sbo >> 4) << 32) |
         (1ull << 46);
}

// The same with an explicit leading-dimension byte offset.  K-major: LBO =
// distance of K-adjacent core matrices, SBO = of 8-row groups.  MN-major (8
// MN-contiguous elements x 8 K rows per core matrix): LBO = distance of 8-row
// K groups, SBO = of MN-adjacent core matrices.
SDEMC_DI uint64_t smem_desc_lbo(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)(lbo >> 4) << 16) | ((uint64_t)(sbo >> 4) << 32) |
         (1ull << 46);
}

// kind::f16 instruction descriptor for M x N, BF16 operands, FP32 accumulator;
// a_mn / b_mn select MN-major operands (bits 15, 16).
constexpr uint32_t make_idesc(int M, int N, bool a_mn, bool b_mn) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((a_mn ? 1u : 0u) << 15) | ((b_mn ? 1u : 0u) << 16) |
         ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

SDEMC_DI uint32_t saddr_of(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

SDEMC_DI void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
SDEMC_DI void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
SDEMC_DI void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

SDEMC_DI void tmem_alloc(uint32_t slot_saddr, uint32_t ncols = kTmemCols) {  // whole warp
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(slot_saddr),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
SDEMC_DI void tmem_dealloc(uint32_t taddr, uint32_t ncols = kTmemCols) {  // whole warp
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols)
               : "memory");
}

SDEMC_DI void mbar_init(uint32_t addr) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(addr) : "memory");
}

// Bounded wait for the phase with the given parity to complete; false after
// `limit` polls.
SDEMC_DI bool mbar_wait(uint32_t addr, uint32_t parity, int limit = kMaxSpins) {
  for (int it = 0; it < limit; ++it) {
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
SDEMC_DI void mma_f16_id(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}
SDEMC_DI void mma_commit(uint32_t mbar_saddr) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar_saddr)
               : "memory");
}

// 16 consecutive FP32 columns of this thread's TMEM lane; the wait for the
// load is in the same asm statement, so no use of the values can be
// scheduled before they have arrived.
SDEMC_DI void tmem_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "{\n tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15}, [%16];\n tcgen05.wait::ld.sync.aligned;\n}\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// 64 consecutive FP32 columns of this thread's TMEM lane in one load; the
// wait is in the same asm statement, so no use of the values can be
// scheduled before the data has arrived.
SDEMC_DI void tmem_ld64(uint32_t taddr, float* v) {
  uint32_t r[64];
  asm volatile(
      "{\n tcgen05.ld.sync.aligned.32x32b.x64.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31, %32, %33, %34, %35, %36, %37, %38, %39, %40, %41, %42, %43, %44, %45, %46, %47, %48, %49, %50, %51, %52, %53, %54, %55, %56, %57, %58, %59, %60, %61, %62, %63}, [%64];\n"
      " tcgen05.wait::ld.sync.aligned;\n}\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31]), "=r"(r[32]), "=r"(r[33]), "=r"(r[34]), "=r"(r[35]), "=r"(r[36]), "=r"(r[37]), "=r"(r[38]), "=r"(r[39]), "=r"(r[40]), "=r"(r[41]), "=r"(r[42]), "=r"(r[43]), "=r"(r[44]), "=r"(r[45]), "=r"(r[46]), "=r"(r[47]), "=r"(r[48]), "=r"(r[49]), "=r"(r[50]), "=r"(r[51]), "=r"(r[52]), "=r"(r[53]), "=r"(r[54]), "=r"(r[55]), "=r"(r[56]), "=r"(r[57]), "=r"(r[58]), "=r"(r[59]), "=r"(r[60]), "=r"(r[61]), "=r"(r[62]), "=r"(r[63])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int i = 0; i < 64; ++i) v[i] = __uint_as_float(r[i]);
}

SDEMC_DI uint32_t lane_base() { return (uint32_t)((threadIdx.x >> 5) * 32) << 16; }

SDEMC_DI uint32_t pack2(float lo, float hi) {
  const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<const uint32_t*>(&v);
}
SDEMC_DI uint32_t pack2b(__nv_bfloat16 lo, __nv_bfloat16 hi) {
  return (uint32_t)__bfloat16_as_ushort(lo) | ((uint32_t)__bfloat16_as_ushort(hi) << 16);
}
SDEMC_HDI void split(float v, __nv_bfloat16& h, __nv_bfloat16& l) {
  h = __float2bfloat16_rn(v);
  l = __float2bfloat16_rn(v - __bfloat162float(h));
}

// Shared memory of one CTA (placed at a 1024-byte aligned address).
struct TcSmem {
  unsigned char A[kRows * kKH * 2];   // activations of layers 2, 3 (+ ones columns)
  unsigned char A1[kRows * kK1 * 2];  // split inputs of layer 1
  unsigned char B1[kH * kK1 * 2];     // split W1 and b1
  unsigned char B2[kH * kKH * 2];     // W2 | b2 (high, low), K-major
  unsigned char B3[kH * kKH * 2];
  float2 w4[kH];                      // W4 columns (d <= 2)
  float b4[2];
  unsigned long long mbar;
  uint32_t tmem;
};

// Parameter vector offsets (torch order: W1, b1, W2, b2, W3, b3, W4, b4).
template <int D> struct TcLayout {
  static constexpr int IN = D + 1;
  static constexpr int W1 = 0, B1 = W1 + kH * IN, W2 = B1 + kH, B2 = W2 + kH * kH, W3 = B2 + kH,
                       B3 = W3 + kH * kH, W4 = B3 + kH, B4 = W4 + D * kH, N = B4 + D;
};

SDEMC_DI void put_bf16(unsigned char* M, int r, int k, int K, __nv_bfloat16 v) {
  *reinterpret_cast<__nv_bfloat16*>(M + core_offset(r, k, K)) = v;
}

// The weight operands of layers 1-3 (BF16, K-major): B1 (64 x 16: W1 and b1
// split into high and low parts), B2, B3 (64 x 80: W | b high | b low | 0).
template <int D>
SDEMC_DI void fill_weights(unsigned char* B1, unsigned char* B2, unsigned char* B3, const float* prm) {
  using L = TcLayout<D>;
  const int t = threadIdx.x;
  const __nv_bfloat16 zero = __float2bfloat16_rn(0.f);
  for (int e = t; e < kH * kKH; e += blockDim.x) {
    const int n = e / kKH, k = e % kKH;
    __nv_bfloat16 v2 = zero, v3 = zero;
    if (k < kH) {
      v2 = __float2bfloat16_rn(prm[L::W2 + n * kH + k]);
      v3 = __float2bfloat16_rn(prm[L::W3 + n * kH + k]);
    } else if (k < kH + 2) {
      __nv_bfloat16 h, l;
      split(prm[L::B2 + n], h, l);
      v2 = k == kH ? h : l;
      split(prm[L::B3 + n], h, l);
      v3 = k == kH ? h : l;
    }
    put_bf16(B2, n, k, kKH, v2);
    put_bf16(B3, n, k, kKH, v3);
  }
  // layer 1: columns 3i, 3i+1, 3i+2 of input i = (xh, xl, xh) against
  // (wh, wh, wl); columns 3(D+1), +1 = ones against (bh, bl)
  for (int e = t; e < kH * kK1; e += blockDim.x) {
    const int n = e / kK1, k = e % kK1;
    __nv_bfloat16 v = zero;
    if (k < 3 * (D + 1)) {
      __nv_bfloat16 h, l;
      split(prm[L::W1 + n * L::IN + k / 3], h, l);
      v = (k % 3 == 2) ? l : h;
    } else if (k < 3 * (D + 1) + 2) {
      __nv_bfloat16 h, l;
      split(prm[L::B1 + n], h, l);
      v = k == 3 * (D + 1) ? h : l;
    }
    put_bf16(B1, n, k, kK1, v);
  }
}

// CTA-wide setup: operands into shared memory, mbarrier, tensor memory.
template <int D>
SDEMC_DI void setup(TcSmem& sm, const float* prm) {
  using L = TcLayout<D>;
  const int t = threadIdx.x;
  const __nv_bfloat16 one = __float2bfloat16_rn(1.f), zero = __float2bfloat16_rn(0.f);
  fill_weights<D>(sm.B1, sm.B2, sm.B3, prm);
  // the A tile's bias and padding columns never change: ones, then zeros
  for (int e = t; e < kRows * (kKH - kH); e += blockDim.x) {
    const int r = e / (kKH - kH), k = kH + e % (kKH - kH);
    put_bf16(sm.A, r, k, kKH, k < kH + 2 ? one : zero);
  }
  for (int j = t; j < kH; j += blockDim.x)
    sm.w4[j] = make_float2(prm[L::W4 + j], D > 1 ? prm[L::W4 + kH + j] : 0.f);
  if (t < D) sm.b4[t] = prm[L::B4 + t];
  if (t == 0) {
    mbar_init(saddr_of(&sm.mbar));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  fence_async_smem();  // generic-proxy stores, read by the tensor cores
  if (t < 32) tmem_alloc(saddr_of(&sm.tmem));
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
}

SDEMC_DI void teardown(TcSmem& sm) {
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  if (threadIdx.x < 32) tmem_dealloc(sm.tmem);
}

// One product for the CTA's 128 rows: A (already in smem, fenced and
// synchronised) x B -> TMEM over K columns; false if the wait gave up.
SDEMC_DI bool product(TcSmem& sm, const unsigned char* A, const unsigned char* B, int K, uint32_t& phase) {
  if (threadIdx.x == 0) {
    fence_after_sync();
    const uint32_t a0 = saddr_of(A), b0 = saddr_of(B), sbo = (uint32_t)(K / 8) * 128u;
    for (int kk = 0; kk < K / 16; ++kk)
      mma_f16(sm.tmem, smem_desc(a0 + kk * 2 * kLbo, sbo), smem_desc(b0 + kk * 2 * kLbo, sbo), kk > 0 ? 1u : 0u);
    mma_commit(saddr_of(&sm.mbar));
  }
  const bool ok = mbar_wait(saddr_of(&sm.mbar), phase);
  phase ^= 1u;
  fence_after_sync();
  return ok;
}

// Accumulator row (bias included), ReLU, as the next A row (BF16).
SDEMC_DI void relu_to_A(TcSmem& sm) {
  const uint32_t base = sm.tmem + lane_base();
#pragma unroll
  for (int c = 0; c < kH / 16; ++c) {
    float v[16];
    tmem_ld16(base + 16 * c, v);
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      uint4 q;
      q.x = pack2(fmaxf(v[8 * h + 0], 0.f), fmaxf(v[8 * h + 1], 0.f));
      q.y = pack2(fmaxf(v[8 * h + 2], 0.f), fmaxf(v[8 * h + 3], 0.f));
      q.z = pack2(fmaxf(v[8 * h + 4], 0.f), fmaxf(v[8 * h + 5], 0.f));
      q.w = pack2(fmaxf(v[8 * h + 6], 0.f), fmaxf(v[8 * h + 7], 0.f));
      *reinterpret_cast<uint4*>(sm.A + core_offset(threadIdx.x, 16 * c + 8 * h, kKH)) = q;
    }
  }
}

// Accumulator row (bias included), ReLU, then layer 4 (64 -> d) in FP32.
template <int D>
SDEMC_DI void relu_layer4(TcSmem& sm, float* out) {
  const uint32_t base = sm.tmem + lane_base();
  float o0 = 0.f, o1 = 0.f;
#pragma unroll
  for (int c = 0; c < kH / 16; ++c) {
    float v[16];
    tmem_ld16(base + 16 * c, v);
#pragma unroll
    for (int j = 0; j < 16; ++j) {
      const float h = fmaxf(v[j], 0.f);
      const float2 w = sm.w4[16 * c + j];
      o0 = __fmaf_rn(w.x, h, o0);
      if (D > 1) o1 = __fmaf_rn(w.y, h, o1);
    }
  }
  out[0] = __fadd_rn(o0, sm.b4[0]);
  if (D > 1) out[1] = __fadd_rn(o1, sm.b4[1]);
}

// Layer 1's A row: (th, tl, th, x0h, x0l, x0h, ..., 1, 1, 0 ...).
template <int D>
SDEMC_DI void inputs_to_tile(unsigned char* A1, float t, const float* x) {
  __nv_bfloat16 a[kK1];
  const __nv_bfloat16 one = __float2bfloat16_rn(1.f), zero = __float2bfloat16_rn(0.f);
#pragma unroll
  for (int i = 0; i <= D; ++i) {
    __nv_bfloat16 h, l;
    split(i == 0 ? t : x[i - 1], h, l);
    a[3 * i] = h;
    a[3 * i + 1] = l;
    a[3 * i + 2] = h;
  }
  a[3 * (D + 1)] = one;
  a[3 * (D + 1) + 1] = one;
#pragma unroll
  for (int k = 3 * (D + 1) + 2; k < kK1; ++k) a[k] = zero;
#pragma unroll
  for (int c = 0; c < kK1 / 8; ++c) {
    uint4 q;
    q.x = pack2b(a[8 * c + 0], a[8 * c + 1]);
    q.y = pack2b(a[8 * c + 2], a[8 * c + 3]);
    q.z = pack2b(a[8 * c + 4], a[8 * c + 5]);
    q.w = pack2b(a[8 * c + 6], a[8 * c + 7]);
    *reinterpret_cast<uint4*>(A1 + core_offset(threadIdx.x, 8 * c, kK1)) = q;
  }
}
template <int D>
SDEMC_DI void inputs_to_A1(TcSmem& sm, float t, const float* x) { inputs_to_tile<D>(sm.A1, t, x); }

// The network on the CTA's 128 rows (this thread: row threadIdx.x with
// inputs t, x); out[D] = f(t, x).  All 128 threads call it together, the same
// number of times.  `fail` carries a gave-up wait from call to call: the
// barriers agree on it (__syncthreads_or), so once any thread's wait gave up
// every thread returns false from then on without touching the tensor cores.
template <int D>
SDEMC_DI bool forward_rows(TcSmem& sm, float t, const float* x, float* out, uint32_t& phase, bool& fail) {
  inputs_to_A1<D>(sm, t, x);
  fence_async_smem();
  fence_before_sync();
  if (__syncthreads_or(fail)) { fail = true; return false; }
  bool ok = product(sm, sm.A1, sm.B1, kK1, phase);
  if (ok) relu_to_A(sm);
  fence_async_smem();
  fence_before_sync();
  if (__syncthreads_or(!ok)) { fail = true; return false; }
  ok = product(sm, sm.A, sm.B2, kKH, phase);
  if (ok) relu_to_A(sm);
  fence_async_smem();
  fence_before_sync();
  if (__syncthreads_or(!ok)) { fail = true; return false; }
  ok = product(sm, sm.A, sm.B3, kKH, phase);
  if (!ok) { fail = true; return false; }
  relu_layer4<D>(sm, out);
  return true;
}

}  // namespace tc
}  // namespace sdemc
