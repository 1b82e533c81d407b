// sdemc_device.cuh — device building blocks shared by every path kernel.
//
//  * Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as
//    easy as 1, 2, 3", SC'11), written from the paper; counter-based, so any
//    path's draws are a pure function of (seed, stream, path index, block).
//    The ten round keys depend on the seed only and are precomputed per
//    launch, so the kernels read them as constants.
//  * Box-Muller normals on MUFU intrinsics (__logf, rsqrtf, __sinf/__cosf).
//  * The reference's jump-adapted Euler loop (sde_mc/solvers.py:164-226) with
//    its exact float32 grid arithmetic, written with _rn intrinsics so that no
//    multiply-add contraction changes a rounding the reference does not make.
//  * Payoffs of sde_mc/options.py:167-321.
#pragma once
#include <stdint.h>
#include <cuda_runtime.h>
#include "../../include/sdemc.h"

namespace sdemc {

#define SDEMC_DI __device__ __forceinline__
#define SDEMC_HDI __host__ __device__ __forceinline__
constexpr unsigned kFull = 0xffffffffu;
constexpr float kTwoPi = 6.283185307179586f;
constexpr float kPi = 3.141592653589793f;

// ---------------------------------------------------------------- Philox ----
struct U4 { uint32_t x, y, z, w; };

// Round r of Philox4x32-10 uses key (k0 + r*0x9E3779B9, k1 + r*0xBB67AE85).
struct RoundKeys { uint32_t k[20]; };

SDEMC_HDI RoundKeys make_round_keys(uint64_t seed) {
  RoundKeys rk;
  uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
  for (int r = 0; r < 10; ++r) {
    rk.k[2 * r] = k0; rk.k[2 * r + 1] = k1;
    k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
  }
  return rk;
}

// Key sources: the round keys as launch constants (single-instance kernels,
// where they become constant-bank operands), or the seed in two registers
// with the key schedule folded into each round (kernels whose instance
// changes per chunk and would otherwise hold twenty keys in registers).
struct SeedKeys {
  uint32_t k0, k1;
  SDEMC_DI uint32_t a(int r) const { return k0 + (uint32_t)r * 0x9E3779B9u; }
  SDEMC_DI uint32_t b(int r) const { return k1 + (uint32_t)r * 0xBB67AE85u; }
  // A copy whose schedule the compiler must derive again at each use, so the
  // 20 round keys are not held live across a whole path loop.
  SDEMC_DI SeedKeys fresh() const {
    SeedKeys c = *this;
    asm volatile("" : "+r"(c.k0), "+r"(c.k1));
    return c;
  }
};
struct ConstKeys {
  const RoundKeys* rk;
  SDEMC_DI uint32_t a(int r) const { return rk->k[2 * r]; }
  SDEMC_DI uint32_t b(int r) const { return rk->k[2 * r + 1]; }
};

template <class KS>
SDEMC_DI const KS& fresh_keys(const KS& ks) { return ks; }
SDEMC_DI SeedKeys fresh_keys(const SeedKeys& ks) { return ks.fresh(); }

template <class KS>
SDEMC_DI U4 philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, const KS& ks_in) {
  const auto ks = fresh_keys(ks_in);
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    const uint32_t lo0 = 0xD2511F53u * c0, hi0 = __umulhi(0xD2511F53u, c0);
    const uint32_t lo1 = 0xCD9E8D57u * c2, hi1 = __umulhi(0xCD9E8D57u, c2);
    const uint32_t n0 = hi1 ^ c1 ^ ks.a(r), n2 = hi0 ^ c3 ^ ks.b(r);
    c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
  }
  return U4{c0, c1, c2, c3};
}

// Uniform on (0,1): (2m+1) 2^-24 from the top 23 bits m of w (exact, never 0/1).
SDEMC_DI float u01(uint32_t w) {
  return __fsub_rn(__uint_as_float(0x3F800000u | (w >> 9)), 0.99999994f);
}

// Box-Muller pair: r = sqrt(-2 ln ua), th = 2 pi ub - pi.
SDEMC_DI float bm_radius(uint32_t wa) {
  const float e = -2.0f * __logf(u01(wa));
  return e * rsqrtf(e);
}
SDEMC_DI float bm_angle(uint32_t wb) { return __fmaf_rn(kTwoPi, u01(wb), -kPi); }

// Stream tags (counter word c2 high half).
constexpr uint32_t kTagDiffusion = 0u;
constexpr uint32_t kTagJumps = 1u;

// Counter words of one path: c1 = path low word, c2 = path high 16 bits |
// tag << 16, c3 = stream id; c0 is the block index.
template <class KS>
struct PathStream {
  KS ks;
  uint32_t c1, c2base, c3;
  SDEMC_DI void init(const KS& keys, uint32_t stream_id, uint64_t gpath) {
    ks = keys;
    c1 = (uint32_t)gpath;
    c2base = (uint32_t)(gpath >> 32) & 0xFFFFu;
    c3 = stream_id;
  }
  SDEMC_DI U4 block(uint32_t tag, uint32_t b) const {
    return philox4x32_10(b, c1, c2base | (tag << 16), c3, ks);
  }
};

// ------------------------------------------------------------- layouts -----
template <int D, int NOISE> struct Layout {
  // normals per step drawn from the diffusion stream
  static constexpr int ZD = NOISE == SDEMC_NOISE_DIAG ? D
                          : NOISE == SDEMC_NOISE_INDEP_SHARED ? D + 1 : 2 * D;
  static constexpr int NB = (ZD + 3) / 4;                        // blocks per step (ZD > 2)
  static constexpr int NW = NOISE == SDEMC_NOISE_DIAG ? 1 : 2;   // noise columns
};

SDEMC_DI float chol_at(const sdemc_inst& I, int i, int j) { return I.chol[i * (i + 1) / 2 + j]; }

// dW = L (z * sq), evaluated as the oracle mirrors it: zs_j = z_j*sq, then a
// multiply-add chain over j = 0..i.  For d == 1 the reference's L = [[1.]].
template <int D>
SDEMC_DI void correlate(const sdemc_inst& I, const float* z, float sq, float* dW) {
  float zs[D];
#pragma unroll
  for (int j = 0; j < D; ++j) zs[j] = __fmul_rn(z[j], sq);
  if constexpr (D == 1) {
    dW[0] = zs[0];
  } else {
#pragma unroll
    for (int i = 0; i < D; ++i) {
      float acc = __fmul_rn(chol_at(I, i, 0), zs[0]);
#pragma unroll
      for (int j = 1; j <= i; ++j) acc = __fmaf_rn(chol_at(I, i, j), zs[j], acc);
      dW[i] = acc;
    }
  }
}

// InverseCdf.__call__ (sde_mc/levy.py:22-30): piecewise inverse of the
// truncated two-sided tempered-stable jump measure.  mark_p = cm, cp, mu,
// alpha, eps, lda, y1, y2, y3, shift, eps^-alpha, -1/alpha.
// Every operation is an explicit _rn intrinsic so that no kernel's inlining
// context can change a rounding (results must not depend on the kernel).
SDEMC_DI float inverse_cdf(const sdemc_inst& I, float y) {
  const float cm = I.mark_p[0], cp = I.mark_p[1], mu = I.mark_p[2], al = I.mark_p[3];
  const float lda = I.mark_p[5], y1 = I.mark_p[6], y2 = I.mark_p[7], y3 = I.mark_p[8];
  const float epa = I.mark_p[10], nia = I.mark_p[11];
  const float ly = __fmul_rn(lda, y);
  const float inv_mu = __fdiv_rn(1.0f, mu);
  if (y <= y1)
    return __fsub_rn(__fdiv_rn(logf(__fdiv_rn(__fmul_rn(mu, ly), cm)), mu), 1.0f);
  if (y < y2)
    return -powf(__fadd_rn(__fmul_rn(al, __fsub_rn(__fdiv_rn(ly, cm), inv_mu)), 1.0f), nia);
  if (y < y3) {
    const float tail = __fmul_rn(cm, __fdiv_rn(__fsub_rn(epa, 1.0f), al));
    const float arg = __fsub_rn(__fsub_rn(ly, __fdiv_rn(cm, mu)), tail);
    return powf(__fadd_rn(__fmul_rn(__fdiv_rn(-al, cp), arg), epa), nia);
  }
  const float q = __fdiv_rn(__fmul_rn(__fmul_rn(mu, lda), __fsub_rn(1.0f, y)), cp);
  return __fsub_rn(1.0f, __fmul_rn(inv_mu, logf(q)));
}

// One jump-stream block: x -> exponential gap, y (,z) -> lognormal mark (Box-
// Muller cosine branch) or the inverse-CDF uniform, w -> asset pick.
struct JumpDraw { float gap, mark; int sel; };

template <int D>
SDEMC_DI JumpDraw jump_from_block(const sdemc_inst& I, U4 w) {
  JumpDraw j;
  j.gap = __fmul_rn(-logf(u01(w.x)), I.inv_rate);
  if (I.mark == SDEMC_MARK_LOGNORMAL) {
    const float zn = __fmul_rn(bm_radius(w.y), __cosf(bm_angle(w.z)));
    j.mark = __fsub_rn(expf(__fmaf_rn(I.mark_p[1], zn, I.mark_p[0])), 1.0f);
  } else if (I.mark == SDEMC_MARK_INVCDF) {
    j.mark = inverse_cdf(I, __fadd_rn(u01(w.y), I.mark_p[9]));
  } else {
    j.mark = 0.f;
  }
  j.sel = 0;
  if (I.jump_target == SDEMC_JUMP_ONE_ASSET) {
    const float us = u01(w.w);
#pragma unroll
    for (int i = 0; i < D - 1; ++i) j.sel += (us >= I.jump_cdf[i]) ? 1 : 0;
  }
  return j;
}

SDEMC_DI float inf_f() { return __int_as_float(0x7f800000); }

// Iteration cap of the adapted loop: nominal steps plus a Poisson tail bound
// on the jump count, plus room for end-of-interval steps.  A path that needs
// more is reported as SDEMC_EOVERFLOW (the reference raises IndexError when
// it runs out of pre-drawn jump times, sde_mc/solvers.py:133, 187).
SDEMC_HDI int max_iterations_hd(const sdemc_inst& I) {
  if (I.grid == SDEMC_GRID_UNIFORM) return I.num_steps;
  const double lam = (double)I.rate * (double)I.T;
  const double tail = lam + 12.0 * sqrt(lam > 1.0 ? lam : 1.0) + 64.0;
  const double cap = (double)I.num_steps + 2.0 * tail + 8.0;
  return cap > 2.0e9 ? 2000000000 : (int)cap;
}

// ------------------------------------------------------------- draws -------
// Native draws: counter-based Philox streams of one path.
//
// Jump stream: every lane holds the next jump (time nj, mark, asset) and one
// reserve jump (gap, mark, asset; gap < 0 when empty).  Firing uses the held
// jump and promotes the reserve — a few instructions in the divergent branch.
// Reserves are refilled by the whole warp at once (after_step): the w-th lane
// that needs a block computes it for the w-th requester and hands it back
// through shuffles, so one pass with all lanes busy serves many lanes.  The
// jump times, marks and picks are those of blocks 0, 1, 2, ... of the path's
// jump stream, whichever lane computes them.
constexpr int kRefillBatch = 8;
constexpr int kRefillEvery = 4;

template <int D, int NOISE, class KS = ConstKeys>
struct NativeDraws {
  using L = Layout<D, NOISE>;
  PathStream<KS> ps;
  float buf[4];          // buffered normals when ZD in {1,2}
  float sq_h, h_nom;     // cached sqrt of the nominal step
  float cur_mark, res_gap, res_mark;
  uint32_t jblk;         // next jump-stream block to draw
  int cur_sel, res_sel;

  SDEMC_DI void init(const sdemc_inst& I, uint64_t gpath, const KS& ks) {
    ps.init(ks, I.stream_id, I.path_offset + gpath);
    h_nom = I.h;
    sq_h = sqrtf(I.h);
  }

  SDEMC_DI void fill4(uint32_t b, float* o) const {
    const U4 w = ps.block(kTagDiffusion, b);
    const float r0 = bm_radius(w.x), a0 = bm_angle(w.y);
    const float r1 = bm_radius(w.z), a1 = bm_angle(w.w);
    o[0] = r0 * __cosf(a0); o[1] = r0 * __sinf(a0);
    o[2] = r1 * __cosf(a1); o[3] = r1 * __sinf(a1);
  }

  // Step k of a dense stream (ZD not a multiple of 4): normals k ZD ..
  // k ZD + ZD - 1 of the path's diffusion stream.  O = (k ZD) mod 4 says how
  // many normals the previous step left in buf (4 - O, or none when O = 0);
  // they come first, then new blocks, and the unused tail of the last new
  // block is carried to the next step.  O is a template argument so every
  // register index is static.
  template <int O>
  SDEMC_DI void dense_step(int k, float* z) {
    constexpr int ZD = L::ZD;
    constexpr int NC = O == 0 ? 0 : 4 - O;
    constexpr int TAKE = NC < ZD ? NC : ZD;
    constexpr int NBLK = (ZD - TAKE + 3) / 4;
    float carry[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) carry[j] = buf[j];
#pragma unroll
    for (int j = 0; j < TAKE; ++j) z[j] = carry[j];
    const uint32_t b0 = (uint32_t)((k * ZD + TAKE) >> 2);
#pragma unroll
    for (int nb = 0; nb < NBLK; ++nb) {
      float o[4];
      fill4(b0 + (uint32_t)nb, o);
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int idx = TAKE + 4 * nb + q;
        if (idx < ZD) z[idx] = o[q];
        else buf[idx - ZD] = o[q];
      }
    }
  }

  // Raw standard normals of step k (k is warp-uniform in lock-step loops).
  // The path's diffusion stream is read densely for ZD in {1, 2, 3, 5, 6}:
  // step k takes its normals k ZD .. k ZD + ZD - 1, four per Philox block, so
  // no normal is discarded; ZD = 4, 8 use whole blocks anyway, and ZD = 7
  // takes the first seven normals of two blocks per step.
  SDEMC_DI void normals(int k, float* z) {
    constexpr int ZD = L::ZD;
    if (ZD == 1 || ZD == 2) {
      const int pos = (k * ZD) & 3;
      if (pos == 0) fill4((uint32_t)((k * ZD) >> 2), buf);
      if (ZD == 1) {
        z[0] = buf[0]; buf[0] = buf[1]; buf[1] = buf[2]; buf[2] = buf[3];
      } else {
        z[0] = buf[0]; z[1] = buf[1]; buf[0] = buf[2]; buf[1] = buf[3];
      }
    } else if (ZD % 4 == 0 || ZD == 7) {
      // whole blocks per step (for ZD = 7 one normal of every second block
      // is left unused: the carried state would cost the served kernels more
      // registers than the eighth of a block it saves)
#pragma unroll
      for (int b = 0; b < L::NB; ++b) {
        float o[4];
        fill4((uint32_t)(k * L::NB + b), o);
#pragma unroll
        for (int q = 0; q < 4; ++q)
          if (4 * b + q < ZD) z[4 * b + q] = o[q];
      }
    } else {
      switch ((k * ZD) & 3) {
        case 0: dense_step<0>(k, z); break;
        case 1: dense_step<1>(k, z); break;
        case 2: dense_step<2>(k, z); break;
        default: dense_step<3>(k, z); break;
      }
    }
  }

  // Step increments for step k of length dt.
  SDEMC_DI void increments(const sdemc_inst& I, int k, float dt, float* dW, float* dW2, float* z) {
    normals(k, z);
    float sq = sq_h;
    if (dt != h_nom) sq = sqrtf(dt);
    correlate<D>(I, z, sq, dW);
    if (NOISE == SDEMC_NOISE_INDEP_SHARED) {
      const float s = __fmul_rn(z[D], sq);
#pragma unroll
      for (int i = 0; i < D; ++i) dW2[i] = s;
    } else if (NOISE == SDEMC_NOISE_INDEP_PAIR) {
      correlate<D>(I, z + D, sq, dW2);
    }
  }

  // First jump time; fills the held and the reserve jump (all lanes together).
  SDEMC_DI float jump_first(const sdemc_inst& I) {
    cur_mark = 0.f; cur_sel = 0; res_gap = -1.f; res_mark = 0.f; res_sel = 0;
    jblk = 0;
    if (I.rate <= 0.f) return inf_f();
    const JumpDraw j0 = jump_from_block<D>(I, ps.block(kTagJumps, 0));
    const JumpDraw j1 = jump_from_block<D>(I, ps.block(kTagJumps, 1));
    cur_mark = j0.mark; cur_sel = j0.sel;
    res_gap = j1.gap; res_mark = j1.mark; res_sel = j1.sel;
    jblk = 2;
    return j0.gap;
  }

  // Divergent: the held jump fires now; returns the next jump time.  The
  // reserve (res_gap >= 0) is promoted; a lane whose reserve is still empty
  // draws its next block itself (rare: only between two batched refills).
  SDEMC_DI float on_fire(const sdemc_inst& I, int /*k*/, float nj, float& J, int& sel) {
    J = cur_mark;
    sel = cur_sel;
    float gap;
    if (res_gap >= 0.f) {
      gap = res_gap;
      cur_mark = res_mark; cur_sel = res_sel;
    } else {
      const JumpDraw j = jump_from_block<D>(I, ps.block(kTagJumps, jblk));
      ++jblk;
      gap = j.gap;
      cur_mark = j.mark; cur_sel = j.sel;
    }
    res_gap = -1.f;
    return __fadd_rn(nj, gap);
  }

  // Warp-synchronous (all 32 lanes), every kRefillEvery-th step: when at
  // least kRefillBatch live lanes have an empty reserve, refill them in one
  // pass: worker w draws the block of the w-th requester and hands it back.
  // `live` = the lane still steps (t < T) and may fire again.
  SDEMC_DI void after_step(const sdemc_inst& I, int k, float& /*nj*/, bool live) {
    if (I.rate <= 0.f || (k & (kRefillEvery - 1)) != kRefillEvery - 1) return;
    const unsigned need = __ballot_sync(kFull, live && res_gap < 0.f);
    const int nreq = __popc(need);
    if (nreq < kRefillBatch) return;
    const int lane = threadIdx.x & 31;
    const int src = lane < nreq ? (int)__fns(need, 0, lane + 1) : lane;
    const uint32_t c1 = __shfl_sync(kFull, ps.c1, src);
    const uint32_t c2 = __shfl_sync(kFull, ps.c2base, src);
    const uint32_t b = __shfl_sync(kFull, jblk, src);
    const JumpDraw j = jump_from_block<D>(I, philox4x32_10(b, c1, c2 | (kTagJumps << 16), ps.c3, ps.ks));
    const int w = __popc(need & ((1u << lane) - 1u));
    const float g = __shfl_sync(kFull, j.gap, w);
    const float m = __shfl_sync(kFull, j.mark, w);
    const int s = __shfl_sync(kFull, j.sel, w);
    if (need & (1u << lane)) {
      ++jblk;
      res_gap = g; res_mark = m; res_sel = s;
    }
  }
};

// Replay draws: increments, marks and jump times recorded from the reference.
template <int D, int NOISE>
struct ReplayDraws {
  using L = Layout<D, NOISE>;
  const float* dw;      // (S, D * NW) row of this path
  const float* marks;   // (S)
  const int32_t* asset; // (S) or null
  const float* jt;      // (MJ)
  int S, MJ, jidx;
  bool overflow;

  SDEMC_DI void increments(const sdemc_inst&, int k, float, float* dW, float* dW2, float*) {
    if (k >= S) {
#pragma unroll
      for (int i = 0; i < D; ++i) { dW[i] = 0.f; dW2[i] = 0.f; }
      overflow = true;
      return;
    }
    const float* r = dw + (size_t)k * D * L::NW;
#pragma unroll
    for (int i = 0; i < D; ++i) {
      if (L::NW == 1) { dW[i] = r[i]; dW2[i] = 0.f; }
      else { dW[i] = r[2 * i]; dW2[i] = r[2 * i + 1]; }
    }
  }
  SDEMC_DI float jump_first(const sdemc_inst& I) {
    jidx = 0;
    if (I.rate <= 0.f || MJ <= 0) return inf_f();
    return jt[0];
  }
  // the reference draws a mark every step (sde_mc/solvers.py:211) and uses
  // the one of the step where the jump fires
  SDEMC_DI float on_fire(const sdemc_inst&, int k, float, float& J, int& sel) {
    J = (k < S) ? marks[k] : 0.f;
    sel = (asset != nullptr && k < S) ? asset[k] : 0;
    ++jidx;
    if (jidx >= MJ) { overflow = true; return inf_f(); }
    return jt[jidx];
  }
  SDEMC_DI void after_step(const sdemc_inst&, int, float&, bool) {}
};

// ------------------------------------------------------------- scheme -----
// HestonScheme.step (sde_mc/schemes.py:16-22) with Heston's coefficients
// (sde_mc/sde.py:269-279) and solve_quadratic (sde_mc/helpers.py:36-48), in
// the reference's float32 operation order in both Euler modes:
//   S' = S + (r S) h + (sqrt(v) S) dW_0
//   a = -1 - kappa h, b = xi dW_1, c = (v + (kappa theta) h) - (0.5 h) xi^2
//   y = max((-b + sqrt(b b - (4 a) c)) / (2 a), (-b - sqrt(..)) / (2 a)),  v' = y y
// Under the Feller condition (asserted by Heston) c > 0 and a < 0, so the
// discriminant is positive.
SDEMC_DI void heston_step(const sdemc_inst& I, float* x, float dt, const float* dW) {
  const float S = x[0], v = x[1];
  const float dr = __fmul_rn(I.drift_b[0], S);
  const float sg = __fmul_rn(__fsqrt_rn(v), S);
  x[0] = __fadd_rn(__fadd_rn(S, __fmul_rn(dr, dt)), __fmul_rn(sg, dW[0]));
  const float a = __fsub_rn(-1.f, __fmul_rn(I.mark_p[0], dt));
  const float b = __fmul_rn(I.mark_p[2], dW[1]);
  const float c = __fsub_rn(__fadd_rn(v, __fmul_rn(I.mark_p[1], dt)), __fmul_rn(__fmul_rn(0.5f, dt), I.mark_p[3]));
  const float sq = __fsqrt_rn(__fsub_rn(__fmul_rn(b, b), __fmul_rn(__fmul_rn(4.f, a), c)));
  const float a2 = __fmul_rn(2.f, a);
  const float r1 = __fdiv_rn(__fadd_rn(-b, sq), a2);
  const float r2 = __fdiv_rn(__fsub_rn(-b, sq), a2);
  const float y = fmaxf(r1, r2);
  x[1] = __fmul_rn(y, y);
}

// EulerScheme.step (sde_mc/schemes.py:7-10) for the affine coefficient form.
// EXACT: the reference's unfused float32 order  x + drift*h + diffusion*dW.
// fast : a fixed chain of fused multiply-adds (mirrored by the oracle).
// MODEL_ASIAN: component 1 is AsianWrapper's running integral
// (sde_mc/sde.py:390-397): y + x_0 h + 0 dW_1, x_0 taken before the step.
template <int D, int NOISE, bool EXACT>
SDEMC_DI void euler(const sdemc_inst& I, float* x, float dt, const float* dW, const float* dW2) {
  if (D == 2 && I.model == SDEMC_MODEL_HESTON) { heston_step(I, x, dt, dW); return; }
  const bool asian = D == 2 && I.model == SDEMC_MODEL_ASIAN;
  const float x0_old = x[0];
#pragma unroll
  for (int i = 0; i < D; ++i) {
    const float xi = x[i];
    if (D == 2 && i == 1 && asian) {
      x[1] = EXACT ? __fadd_rn(xi, __fmul_rn(x0_old, dt)) : __fmaf_rn(x0_old, dt, xi);
      continue;
    }
    if (EXACT) {
      const float dr = __fadd_rn(I.drift_a[i], __fmul_rn(I.drift_b[i], xi));
      const float sg = __fadd_rn(I.diff_s[i], __fmul_rn(I.diff_q[i], xi));
      const float base = __fadd_rn(xi, __fmul_rn(dr, dt));
      if (NOISE == SDEMC_NOISE_DIAG) {
        x[i] = __fadd_rn(base, __fmul_rn(sg, dW[i]));
      } else {
        const float sg2 = __fadd_rn(I.diff2_s[i], __fmul_rn(I.diff2_q[i], xi));
        x[i] = __fadd_rn(base, __fadd_rn(__fmul_rn(sg, dW[i]), __fmul_rn(sg2, dW2[i])));
      }
    } else {
      const float dr = __fmaf_rn(I.drift_b[i], xi, I.drift_a[i]);
      const float sg = __fmaf_rn(I.diff_q[i], xi, I.diff_s[i]);
      float xn = __fmaf_rn(dr, dt, xi);
      xn = __fmaf_rn(sg, dW[i], xn);
      if (NOISE != SDEMC_NOISE_DIAG) {
        const float sg2 = __fmaf_rn(I.diff2_q[i], xi, I.diff2_s[i]);
        xn = __fmaf_rn(sg2, dW2[i], xn);
      }
      x[i] = xn;
    }
  }
}

// add_jumps (sde_mc/solvers.py:140-141, 214-217): x + (g + k*base) * J.
template <int D, bool EXACT>
SDEMC_DI void apply_jump(const sdemc_inst& I, float* x, const float* base, float J, int sel) {
  const bool one = I.jump_target == SDEMC_JUMP_ONE_ASSET;
#pragma unroll
  for (int i = 0; i < D; ++i) {
    if (one && i != sel) continue;
    if (EXACT)
      x[i] = __fadd_rn(x[i], __fmul_rn(__fadd_rn(I.jump_g[i], __fmul_rn(I.jump_k[i], base[i])), J));
    else
      x[i] = __fmaf_rn(__fmaf_rn(I.jump_k[i], base[i], I.jump_g[i]), J, x[i]);
  }
}

// torch.isclose(next_jump_time, t, atol=1e-12) with the default rtol=1e-5,
// in float32 as torch evaluates it: |nj - t| <= 1e-12f + |1e-5f * t|.
SDEMC_DI bool jump_due(float nj, float t) {
  const float err = fabsf(__fsub_rn(nj, t));
  const float tol = __fadd_rn(1e-12f, fabsf(__fmul_rn(1e-5f, t)));
  return (nj == t) || (err <= tol);
}

// ------------------------------------------------------------- payoff -----
// Option.__call__ = payoff(transform(x)) (sde_mc/options.py:167-176).
template <int D>
SDEMC_DI float payoff(const sdemc_inst& I, const float* xin) {
  float s[D];
#pragma unroll
  for (int i = 0; i < D; ++i) {
    const float sp = I.payoff_log ? expf(xin[i]) : xin[i];
    s[i] = __fmul_rn(I.payoff_scale, sp);
  }
  const float K = I.strike;
  switch (I.payoff) {
    case SDEMC_PAYOFF_EUROCALL: return s[0] > K ? __fsub_rn(s[0], K) : 0.f;
    case SDEMC_PAYOFF_EUROPUT: return s[0] < K ? __fsub_rn(K, s[0]) : 0.f;
    case SDEMC_PAYOFF_BINARY_AON: return s[0] >= K ? s[0] : 0.f;
    case SDEMC_PAYOFF_DIGITAL: return s[0] > K ? 1.f : 0.f;
    case SDEMC_PAYOFF_BASKET_ARITH: {
      float acc = s[0];
#pragma unroll
      for (int i = 1; i < D; ++i) acc = __fadd_rn(acc, s[i]);
      const float m = __fdiv_rn(acc, (float)D);
      return m > K ? __fsub_rn(m, K) : 0.f;
    }
    case SDEMC_PAYOFF_BASKET_GEO: {
      float acc = logf(s[0]);
#pragma unroll
      for (int i = 1; i < D; ++i) acc = __fadd_rn(acc, logf(s[i]));
      const float m = expf(__fdiv_rn(acc, (float)D));
      return m > K ? __fsub_rn(m, K) : 0.f;
    }
    case SDEMC_PAYOFF_RAINBOW: {
      float m = s[0];
#pragma unroll
      for (int i = 1; i < D; ++i) m = fmaxf(m, s[i]);
      return m > K ? __fsub_rn(m, K) : 0.f;
    }
    case SDEMC_PAYOFF_BESTOF: {
      float m = s[0];
#pragma unroll
      for (int i = 1; i < D; ++i) m = fmaxf(m, s[i]);
      return fmaxf(m, K);
    }
    case SDEMC_PAYOFF_ASIANCALL: {
      if (D < 2) return 0.f;
      const float a = __fdiv_rn(s[D > 1 ? 1 : 0], I.T);
      const float sp = I.payoff_log ? expf(a) : a;
      return sp > K ? __fsub_rn(sp, K) : 0.f;
    }
    case SDEMC_PAYOFF_HESTON_RAINBOW: {
      float m = s[0];
#pragma unroll
      for (int i = 2; i < D; i += 2) m = fmaxf(m, s[i]);
      return m > K ? __fsub_rn(m, K) : 0.f;
    }
    default: return 0.f;
  }
}

// ------------------------------------------------------------- sinks ------
struct NullSink {
  static constexpr bool kWantsLeft = false;
  template <int D> SDEMC_DI void init(const float*) {}
  template <int D, int NW> SDEMC_DI void step(int, const float*, const float*, float, float, int,
                                              const float*, const float*, const float*, int, const float*, float) {}
  template <int D, int NW> SDEMC_DI void finish(int, const float*, float) {}
};

// AdaptedPathData layout (sde_mc/nets.py:192-207 / solvers.py:150-162):
// paths, left, jumps (S+1, D); time (S+1); normals (S, D*NW); optional raw
// normals z (S, zdim).  One row per path, S = steps cap.
struct StoreSink {
  static constexpr bool kWantsLeft = true;
  float *paths, *left, *time, *jumps, *normals, *z;
  int S, zdim;

  template <int D> SDEMC_DI void init(const float* x) {
    if (paths) for (int i = 0; i < D; ++i) paths[i] = x[i];
    if (left) for (int i = 0; i < D; ++i) left[i] = x[i];
    if (jumps) for (int i = 0; i < D; ++i) jumps[i] = 0.f;
    if (time) time[0] = 0.f;
  }
  template <int D, int NW>
  SDEMC_DI void step(int k, const float* xl, const float* x, float t, float J, int sel,
                     const float* dW, const float* dW2, const float* zr, int jump_one, const float*, float) {
    if (k >= S) return;
    const size_t c = (size_t)(k + 1) * D;
    if (paths) for (int i = 0; i < D; ++i) paths[c + i] = x[i];
    if (left) for (int i = 0; i < D; ++i) left[c + i] = xl[i];
    if (jumps) for (int i = 0; i < D; ++i) jumps[c + i] = (jump_one && i != sel) ? 0.f : J;
    if (time) time[k + 1] = t;
    if (normals) {
      float* n = normals + (size_t)k * D * NW;
      for (int i = 0; i < D; ++i) {
        if (NW == 1) n[i] = dW[i];
        else { n[2 * i] = dW[i]; n[2 * i + 1] = dW2[i]; }
      }
    }
    if (z && zr) for (int j = 0; j < zdim; ++j) z[(size_t)k * zdim + j] = zr[j];
  }
  template <int D, int NW>
  SDEMC_DI void finish(int kend, const float* x, float t) {
    for (int k = kend; k < S; ++k) {
      const size_t c = (size_t)(k + 1) * D;
      if (paths) for (int i = 0; i < D; ++i) paths[c + i] = x[i];
      if (left) for (int i = 0; i < D; ++i) left[c + i] = x[i];
      if (jumps) for (int i = 0; i < D; ++i) jumps[c + i] = 0.f;
      if (time) time[k + 1] = t;
      if (normals) for (int i = 0; i < D * NW; ++i) normals[(size_t)k * D * NW + i] = 0.f;
      if (z) for (int j = 0; j < zdim; ++j) z[(size_t)k * zdim + j] = 0.f;
    }
  }
};


// ------------------------------------------------------------ the loop ----
// Loop variants: kModeExact selects the reference's unfused Euler order;
// kModeNominal keeps the state after num_steps steps for the payoff (what
// mc_simple(payoff_time='terminal') reads from a jump solver's storage,
// sde_mc/mc.py:84-86, 92).
constexpr int kModeExact = 1;
constexpr int kModeNominal = 2;
// All warps of the CTA step together (the loop runs while any lane of the CTA
// is active): for sinks that evaluate something CTA-wide at every step.
constexpr int kModeCtaSync = 4;

// One path per lane; the warp steps in lock-step so that step k of every lane
// draws from block k of its own stream (warp-uniform control, no divergence
// on refills).  A lane whose t reached T is frozen (dt = 0, no jumps), which
// is what the reference's batch-global loop does to finished paths
// (sde_mc/solvers.py:182, 190-191).  Returns the number of active steps.
template <int D, int NOISE, int MODE, class Draws, class Sink>
SDEMC_DI int simulate(const sdemc_inst& I, Draws& dr, Sink& sk, float* x, int max_iters, bool& overflow) {
  using L = Layout<D, NOISE>;
  constexpr bool EXACT = (MODE & kModeExact) != 0;
#pragma unroll
  for (int i = 0; i < D; ++i) x[i] = I.x0[i];
  sk.template init<D>(x);
  float t = 0.f;
  float dW[D], dW2[D], z[L::ZD];
#pragma unroll
  for (int i = 0; i < D; ++i) dW2[i] = 0.f;
  const int jump_one = I.jump_target == SDEMC_JUMP_ONE_ASSET;
  int k = 0;
  if (I.grid == SDEMC_GRID_UNIFORM) {
    // DiffusionSolver.solve: exactly num_steps steps of h, t += h.
    const float h = I.h;
    for (; k < I.num_steps; ++k) {
      dr.increments(I, k, h, dW, dW2, z);
      float old[D];
#pragma unroll
      for (int i = 0; i < D; ++i) old[i] = x[i];
      euler<D, NOISE, EXACT>(I, x, h, dW, dW2);
      const float t0 = t;
      t = __fadd_rn(t, h);
      sk.template step<D, L::NW>(k, x, x, t, 0.f, 0, dW, dW2, z, 0, old, t0);
    }
    sk.template finish<D, L::NW>(k, x, t);
    return k;
  }
  const float T = I.T;
  float h = I.h;
  float nj = dr.jump_first(I);
  int own = 0;
  bool act = t < T;
  float xcap[(MODE & kModeNominal) ? D : 1];
  if (MODE & kModeNominal) {
#pragma unroll
    for (int i = 0; i < D; ++i) xcap[i] = x[i];
  }
  while ((MODE & kModeCtaSync) ? __syncthreads_or(act) : __any_sync(kFull, act)) {
    if (k >= max_iters) { overflow = true; break; }
    // h = min(h, max(T - t, 0)); dt = min(h, next_jump - t)
    h = fminf(h, fmaxf(__fsub_rn(T, t), 0.f));
    float dt = fminf(h, __fsub_rn(nj, t));
    if (!act) dt = 0.f;
    dr.increments(I, k, dt, dW, dW2, z);
    float old[D];
#pragma unroll
    for (int i = 0; i < D; ++i) old[i] = x[i];
    euler<D, NOISE, EXACT>(I, x, dt, dW, dW2);
    const float t0 = t;
    t = __fadd_rn(t, dt);
    float xl[D];
    if (Sink::kWantsLeft) {
#pragma unroll
      for (int i = 0; i < D; ++i) xl[i] = x[i];
    }
    float J = 0.f;
    int sel = 0;
    if (act && jump_due(nj, t)) {
      nj = dr.on_fire(I, k, nj, J, sel);
      apply_jump<D, EXACT>(I, x, I.exact_jumps ? x : old, J, sel);
    }
    sk.template step<D, L::NW>(k, Sink::kWantsLeft ? xl : x, x, t, J, sel, dW, dW2, z, jump_one, old, t0);
    own += act ? 1 : 0;
    if (MODE & kModeNominal) {
      if (act && own == I.num_steps) {
#pragma unroll
        for (int i = 0; i < D; ++i) xcap[i] = x[i];
      }
    }
    ++k;
    act = t < T;
    dr.after_step(I, k, nj, act);
  }
  sk.template finish<D, L::NW>(k, x, t);
  if (MODE & kModeNominal) {
    if (own >= I.num_steps) {
#pragma unroll
      for (int i = 0; i < D; ++i) x[i] = xcap[i];
    }
  }
  return own;
}

// Two paths per lane (paths-per-thread tiling): simulate() with a NullSink for
// paths a and b stepped together.  Each path goes through exactly the
// operations simulate() gives it (a path that has reached T takes dt = 0
// steps, which leave it unchanged, while its partner still runs; the jump
// stream of a path is its blocks 0, 1, 2, ... whoever draws them), so both
// end bit-identical to simulate()'s; the two instruction streams are
// independent and give the scheduler twice the work between waits.
template <int D, int NOISE, int MODE, class Draws>
SDEMC_DI void simulate2(const sdemc_inst& I, Draws& da, Draws& db, float* xa, float* xb, int max_iters,
                        bool& overflow) {
  using L = Layout<D, NOISE>;
  constexpr bool EXACT = (MODE & kModeExact) != 0;
  float dWa[D], dW2a[D], za[L::ZD], dWb[D], dW2b[D], zb[L::ZD];
#pragma unroll
  for (int i = 0; i < D; ++i) {
    xa[i] = I.x0[i]; xb[i] = I.x0[i];
    dW2a[i] = 0.f; dW2b[i] = 0.f;
  }
  if (I.grid == SDEMC_GRID_UNIFORM) {
    const float h = I.h;
    for (int k = 0; k < I.num_steps; ++k) {
      da.increments(I, k, h, dWa, dW2a, za);
      db.increments(I, k, h, dWb, dW2b, zb);
      euler<D, NOISE, EXACT>(I, xa, h, dWa, dW2a);
      euler<D, NOISE, EXACT>(I, xb, h, dWb, dW2b);
    }
    return;
  }
  const float T = I.T;
  float ha = I.h, hb = I.h, ta = 0.f, tb = 0.f;
  float nja = da.jump_first(I), njb = db.jump_first(I);
  int owna = 0, ownb = 0, k = 0;
  bool acta = ta < T, actb = tb < T;
  constexpr int NC = (MODE & kModeNominal) ? D : 1;
  float capa[NC], capb[NC];
  if (MODE & kModeNominal) {
#pragma unroll
    for (int i = 0; i < D; ++i) { capa[i] = xa[i]; capb[i] = xb[i]; }
  }
  while (__any_sync(kFull, acta || actb)) {
    if (k >= max_iters) { overflow = true; break; }
    ha = fminf(ha, fmaxf(__fsub_rn(T, ta), 0.f));
    hb = fminf(hb, fmaxf(__fsub_rn(T, tb), 0.f));
    float dta = fminf(ha, __fsub_rn(nja, ta));
    float dtb = fminf(hb, __fsub_rn(njb, tb));
    if (!acta) dta = 0.f;
    if (!actb) dtb = 0.f;
    da.increments(I, k, dta, dWa, dW2a, za);
    db.increments(I, k, dtb, dWb, dW2b, zb);
    float olda[D], oldb[D];
#pragma unroll
    for (int i = 0; i < D; ++i) { olda[i] = xa[i]; oldb[i] = xb[i]; }
    euler<D, NOISE, EXACT>(I, xa, dta, dWa, dW2a);
    euler<D, NOISE, EXACT>(I, xb, dtb, dWb, dW2b);
    ta = __fadd_rn(ta, dta);
    tb = __fadd_rn(tb, dtb);
    if (acta && jump_due(nja, ta)) {
      float J;
      int sel;
      nja = da.on_fire(I, k, nja, J, sel);
      apply_jump<D, EXACT>(I, xa, I.exact_jumps ? xa : olda, J, sel);
    }
    if (actb && jump_due(njb, tb)) {
      float J;
      int sel;
      njb = db.on_fire(I, k, njb, J, sel);
      apply_jump<D, EXACT>(I, xb, I.exact_jumps ? xb : oldb, J, sel);
    }
    owna += acta ? 1 : 0;
    ownb += actb ? 1 : 0;
    if (MODE & kModeNominal) {
      if (acta && owna == I.num_steps) {
#pragma unroll
        for (int i = 0; i < D; ++i) capa[i] = xa[i];
      }
      if (actb && ownb == I.num_steps) {
#pragma unroll
        for (int i = 0; i < D; ++i) capb[i] = xb[i];
      }
    }
    ++k;
    acta = ta < T;
    actb = tb < T;
    da.after_step(I, k, nja, acta);
    db.after_step(I, k, njb, actb);
  }
  if (MODE & kModeNominal) {
    if (owna >= I.num_steps) {
#pragma unroll
      for (int i = 0; i < D; ++i) xa[i] = capa[i];
    }
    if (ownb >= I.num_steps) {
#pragma unroll
      for (int i = 0; i < D; ++i) xb[i] = capb[i];
    }
  }
}

// Warp sum (fixed xor butterfly: every lane ends with the same bits).
SDEMC_DI float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
  return v;
}

}  // namespace sdemc
