// serve_kernels.cuh — device side of the pricing server (K9).
//
// A server slot is device-resident: the request's descriptor, its RNG path
// counter (`cursor`, the next local path index), the end of its current
// phase and its FP64 running sums.  A tick is a list of entries, one slice of
// one slot each, grouped into classes of equal (kind, noise, loop variant,
// dim) with one persistent kernel per class.  A warp takes the next 32-path
// chunk from the class counter, finds its entry by binary search, stages the
// slot's descriptor in shared memory and runs the per-path code of K1
// (simulate + payoff + warp butterfly) on paths cursor + chunk*32 + lane.
// serve_reduce_kernel then folds each entry's chunk partials, in a fixed
// order, into its slot and advances the slot's cursor; entries that finish a
// phase copy the slot's sums to the tick's completion records.
//
// Kinds:
//   kKindPlain       payoff only: (sum, sum^2, n)
//   kKindLcv         payoff - beta . r with the regressors r of DeltaCvSink
//   kKindPilotStats  payoff and r: sums of P, P^2, n, r_a, r_a r_b, P r_a for
//                    the regression that fits beta on the pilot
#pragma once
#include "sdemc_device.cuh"
#include "sdemc_host.cuh"

namespace sdemc {

constexpr int kServeMaxR = 2 * SDEMC_MAX_DIM + 1;  // control-variate regressors
constexpr int kServeMaxW = 3 + 2 * kServeMaxR + kServeMaxR * (kServeMaxR + 1) / 2;  // 190
constexpr int kServeMaxWarps = 8;  // CTAs of up to 256 threads
enum { kKindPlain = 0, kKindLcv = 1, kKindPilotStats = 2, kNumKinds = 3 };

// Pilot partial layout over the R = 2d + 1 regressors r (see DeltaCvSink):
// P, P^2, n, r[R], r_a r_b (a <= b, row-major), P r[R].
SDEMC_HDI int num_regressors(int d) { return 2 * d + 1; }
SDEMC_HDI int pilot_width(int d) {
  const int R = num_regressors(d);
  return 3 + 2 * R + R * (R + 1) / 2;
}
SDEMC_HDI int kind_width(int kind, int d) { return kind == kKindPilotStats ? pilot_width(d) : 3; }

// Integrand weights of the control variate (sdemc_cv_weights in the header):
// w(t, X) = N(d1) (call-like payoffs) or N(d1) - 1 (puts) of a lognormal
// proxy of the payoff's underlying A = payoff_scale * agg(X) (asset 0, mean
// or max): d1 = (ln(A/K) + drift tau) / (sig sqrt(tau)), tau = T - t; w = 1
// when wkind == 0 — a delta; and g(t, X) = (A/K) phi(d1) / (sig sqrt(tau))
// (g = 1 when wkind == 0) — a gamma scaled by A^2/K.  Any deterministic
// weights keep the control variate unbiased; these make it close to a delta
// hedge plus the second-order jump exposure.  comp[i] is the jump
// compensator rate lambda_i E[J] of asset i and comp_j2 = lambda E[J^2]
// (inv_comp, inv_comp_j2 their reciprocals); jump regressors are on only when
// those rates are known exactly (lognormal marks).
using CvWeights = sdemc_cv_weights;

// The weights the server derives for a descriptor at admission (host).
CvWeights serve_cv_weights(const sdemc_inst& I);

struct ServeState {
  int64_t cursor;              // next local path index (the request's RNG counter)
  int64_t phase_end;           // local path index where the current phase ends
  int32_t phase, width, status, kind;
  float beta[kServeMaxR];      // control-variate coefficients of the main run
  CvWeights cw;
  double acc[kServeMaxW];      // FP64 running sums of the current phase
};

struct ServeSlot {
  sdemc_inst inst;
  ServeState st;
};

struct ServeEntry {
  int32_t slot, width, done, kind;
  int64_t chunk_begin;  // global chunk index of the entry's first chunk in the tick
  int64_t nchunks;
  int64_t part_off;     // offset (doubles) of its chunk partials
  int64_t base, end;    // the slice's first local path and the end of its phase
};

struct ServeDone {
  int32_t slot, status, width, phase;
  int64_t cursor;
  double acc[kServeMaxW];
};

// Host -> device slot writes of one tick: a whole slot (admission) or only
// its state (phase change).
struct ServeInstall {
  int32_t slot, whole;
  int32_t pad[2];
  ServeSlot rec;
};

struct ServeParams {
  ServeSlot* slots;
  const ServeEntry* entries;
  int first, count;
  int64_t chunk_begin, chunk_end;
  unsigned long long* counter;
  double* part;
  // when every entry of the class has the same seed, the Philox round keys as
  // launch constants (the d = 5, 6 control-variate classes use them; the
  // others derive the keys from the seed per chunk: with constant keys the
  // compiler holds them in registers, which spills at d = 7, 8 and d <= 4)
  int32_t uniform_seed;
  RoundKeys rk;
};

template <class KS> SDEMC_DI KS serve_keys(const ServeParams& P, const sdemc_inst& I);
template <> SDEMC_DI SeedKeys serve_keys<SeedKeys>(const ServeParams&, const sdemc_inst& I) {
  return SeedKeys{(uint32_t)I.seed, (uint32_t)(I.seed >> 32)};
}
template <> SDEMC_DI ConstKeys serve_keys<ConstKeys>(const ServeParams& P, const sdemc_inst&) {
  return ConstKeys{&P.rk};
}

// The control variate's regressors, per asset i:
//   r_i     = sum_k w_k X^i_k dW^i_k
//   r_{d+i} = sum_k w_k X^i_k (J^i_{k+1} - comp_i dt_k)
// and one more,
//   r_{2d}  = sum_k g_k (J_{k+1}^2 - comp_j2 dt_k),
// with X_k the state at the start of step k (after the previous step's
// jump), dW_k the step's correlated increment, J_{k+1} the mark of a jump at
// the end of the step (J^i_{k+1} the part applied to asset i; 0 without a
// jump) and (w_k, g_k) the weights at the start of the step's 4-step block
// (evaluated at t_j, X_j, j = 4 floor(k / 4): known at t_k).  All are
// stochastic integrals of predictable integrands against martingales (the
// Brownian increments; the jump measures of J and J^2 minus their
// compensators on the jump-adapted grid), so each has mean exactly zero under
// the Euler scheme whatever the weights.  Frozen lanes (dt = 0, dW = 0, no
// jump) add nothing.  A jump regressor is carried as a with r = -comp a:
// every step adds weight x dt, a jump subtracts weight x J x (1 / comp) (the
// compensator rates are nonzero whenever jumps are on; the reciprocals are
// rounded once, on the host).
constexpr int kWeightEvery = 4;

template <int D>
struct DeltaCvSink {
  static constexpr bool kWantsLeft = false;
  const CvWeights* cw;
  float r[D], a[D];
  float w, g, ag;

  // (w, g) at time ts and state xs
  SDEMC_DI void weights(const float* xs, float ts) {
    if (cw->wkind == 0) { w = 1.f; g = 1.f; return; }
    float m = xs[0];
    if (cw->agg == 1) {
#pragma unroll
      for (int i = 1; i < D; ++i) m = __fadd_rn(m, xs[i]);
      m = __fmul_rn(m, 1.f / (float)D);
    } else if (cw->agg == 2) {
#pragma unroll
      for (int i = 1; i < D; ++i) m = fmaxf(m, xs[i]);
    }
    m = __fmul_rn(m, cw->scale_over_k);
    const float tau = fmaxf(__fsub_rn(cw->T, ts), 1e-6f);
    const float is = __fmul_rn(rsqrtf(tau), cw->inv_sig);
    if (m > 0.f) {
      const float d1 = __fmul_rn(__fmaf_rn(cw->drift, tau, __logf(m)), is);
      const float v = normcdff(d1);
      w = cw->wkind == 2 ? v - 1.f : v;
      g = __fmul_rn(__fmul_rn(m, is), __fmul_rn(0.39894228f, __expf(__fmul_rn(-0.5f, __fmul_rn(d1, d1)))));
    } else {
      w = cw->wkind == 2 ? -1.f : 0.f;
      g = 0.f;
    }
  }

  template <int DD> SDEMC_DI void init(const float* x) {
#pragma unroll
    for (int i = 0; i < D; ++i) { r[i] = 0.f; a[i] = 0.f; }
    ag = 0.f;
    weights(x, 0.f);
  }
  // xp, tp: the state and time at the start of step k (after the previous
  // step's jump); t: the time at its end.
  template <int DD, int NW>
  SDEMC_DI void step(int k, const float*, const float*, float t, float J, int sel, const float* dW, const float*,
                     const float*, int jump_one, const float* xp, float tp) {
    if (k > 0 && (k & (kWeightEvery - 1)) == 0) weights(xp, tp);  // k is warp-uniform
#pragma unroll
    for (int i = 0; i < D; ++i) r[i] = __fmaf_rn(xp[i], __fmul_rn(w, dW[i]), r[i]);
    if (cw->jumps) {
      const float dt = __fsub_rn(t, tp);
      const float wdt = __fmul_rn(w, dt);
#pragma unroll
      for (int i = 0; i < D; ++i) a[i] = __fmaf_rn(xp[i], wdt, a[i]);
      ag = __fmaf_rn(g, dt, ag);
      if (J != 0.f) {
#pragma unroll
        for (int i = 0; i < D; ++i)
          if (!jump_one || i == sel) a[i] = __fmaf_rn(-__fmul_rn(w, xp[i]), __fmul_rn(J, cw->inv_comp[i]), a[i]);
        ag = __fmaf_rn(-g, __fmul_rn(__fmul_rn(J, J), cw->inv_comp_j2), ag);
      }
    }
  }
  template <int DD, int NW> SDEMC_DI void finish(int, const float*, float) {}

  // Regressor q (0 <= q < 2D + 1).
  SDEMC_DI float reg(int q) const {
    if (q < D) return r[q];
    if (q < 2 * D) return -__fmul_rn(cw->comp[q - D], a[q - D]);
    return -__fmul_rn(cw->comp_j2, ag);
  }
};

// Register budget: 80 per thread (24 resident warps per SM) for d <= 4; the
// d >= 5 classes, which spill 76-126 bytes per thread at 80, get 128 (16
// warps), which measured faster on the served stream than 80 for every d or
// 128 from d = 3 on.
template <int D> struct ServeMinBlocks { static constexpr int value = D >= 5 ? 2 : 3; };

template <int D, int NOISE, int MODE, int KIND, class KS>
__global__ void __launch_bounds__(256, ServeMinBlocks<D>::value)
serve_kernel(const __grid_constant__ ServeParams P) {
  __shared__ __align__(16) sdemc_inst s_inst[kServeMaxWarps];  // 16-byte aligned arrays: vector loads
  __shared__ float s_beta[kServeMaxWarps][2 * D + 1];
  __shared__ CvWeights s_cw[kServeMaxWarps];
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int slot = -1;
  int64_t lo = 0, hi = 0, base = 0, end = 0, part_off = 0;
  int max_iters = 0;
  bool ovf = false;
  constexpr int R = 2 * D + 1;
  constexpr int W = KIND == kKindPilotStats ? 3 + 2 * R + R * (R + 1) / 2 : 3;
  for (;;) {
    unsigned long long g = 0;
    if (lane == 0) g = atomicAdd(P.counter, 1ull);
    g = __shfl_sync(kFull, g, 0);
    const int64_t gc = P.chunk_begin + (int64_t)g;
    if (gc >= P.chunk_end) break;
    if (gc < lo || gc >= hi) {
      if (ovf && lane == 0) atomicOr(&P.slots[slot].st.status, SDEMC_EOVERFLOW);
      ovf = false;
      int a = P.first, b = P.first + P.count;  // entries[a].chunk_begin <= gc < entries[b].chunk_begin
      while (b - a > 1) {
        const int m = (a + b) >> 1;
        if (P.entries[m].chunk_begin <= gc) a = m; else b = m;
      }
      const ServeEntry& E = P.entries[a];
      lo = E.chunk_begin;
      hi = lo + E.nchunks;
      part_off = E.part_off;
      slot = E.slot;
      const ServeSlot& S = P.slots[slot];
      // the slice's bounds come with the entry: a class kernel reads only the
      // slot's descriptor and coefficients, which no running tick writes, so
      // it may overlap the previous tick's kernels and reduction
      base = E.base;
      end = E.end;
      __syncwarp();
      const uint32_t* src = reinterpret_cast<const uint32_t*>(&S.inst);
      uint32_t* dst = reinterpret_cast<uint32_t*>(&s_inst[wid]);
      for (int q = lane; q < (int)(sizeof(sdemc_inst) / 4); q += 32) dst[q] = src[q];
      if (KIND == kKindLcv && lane < R) s_beta[wid][lane] = S.st.beta[lane];
      if (KIND != kKindPlain) {
        const uint32_t* cs = reinterpret_cast<const uint32_t*>(&S.st.cw);
        uint32_t* cd = reinterpret_cast<uint32_t*>(&s_cw[wid]);
        for (int q = lane; q < (int)(sizeof(CvWeights) / 4); q += 32) cd[q] = cs[q];
      }
      __syncwarp();
      max_iters = max_iterations_hd(s_inst[wid]);
    }
    const sdemc_inst& I = s_inst[wid];
    const int64_t p = base + (gc - lo) * kChunk + lane;
    const bool valid = p < end;
    NativeDraws<D, NOISE, KS> dr;
    dr.init(I, (uint64_t)p, serve_keys<KS>(P, I));
    float x[D];
    if (KIND == kKindPlain) {
      NullSink sk;
      simulate<D, NOISE, MODE>(I, dr, sk, x, max_iters, ovf);
      double* out = P.part + part_off + (gc - lo) * W;
      const int n = __popc(__ballot_sync(kFull, valid));
      const float v = valid ? __fmul_rn(payoff<D>(I, x), I.discount) : 0.f;
      const float s = warp_sum(v), s2 = warp_sum(__fmul_rn(v, v));
      if (lane == 0) { out[0] = (double)s; out[1] = (double)s2; out[2] = (double)n; }
    } else {
      DeltaCvSink<D> sk;
      sk.cw = &s_cw[wid];
      simulate<D, NOISE, MODE>(I, dr, sk, x, max_iters, ovf);
      double* out = P.part + part_off + (gc - lo) * W;
      const int n = __popc(__ballot_sync(kFull, valid));
      const float pv = valid ? __fmul_rn(payoff<D>(I, x), I.discount) : 0.f;
      float y[R];
#pragma unroll
      for (int i = 0; i < R; ++i) y[i] = valid ? sk.reg(i) : 0.f;
      if (KIND == kKindLcv) {
        float v = pv;
#pragma unroll
        for (int i = 0; i < R; ++i) v = __fmaf_rn(-s_beta[wid][i], y[i], v);
        const float s = warp_sum(v), s2 = warp_sum(__fmul_rn(v, v));
        if (lane == 0) { out[0] = (double)s; out[1] = (double)s2; out[2] = (double)n; }
      } else {
        const float s = warp_sum(pv), s2 = warp_sum(__fmul_rn(pv, pv));
        if (lane == 0) { out[0] = (double)s; out[1] = (double)s2; out[2] = (double)n; }
#pragma unroll
        for (int i = 0; i < R; ++i) {
          const float a = warp_sum(y[i]);
          if (lane == 0) out[3 + i] = (double)a;
        }
        int q = 3 + R;
#pragma unroll
        for (int i = 0; i < R; ++i)
#pragma unroll
          for (int j = i; j < R; ++j) {
            const float a = warp_sum(__fmul_rn(y[i], y[j]));
            if (lane == 0) out[q] = (double)a;
            ++q;
          }
#pragma unroll
        for (int i = 0; i < R; ++i) {
          const float a = warp_sum(__fmul_rn(pv, y[i]));
          if (lane == 0) out[q + i] = (double)a;
        }
      }
    }
  }
  if (ovf && lane == 0 && slot >= 0) atomicOr(&P.slots[slot].st.status, SDEMC_EOVERFLOW);
}

template <int D, int NOISE, int MODE, int KIND>
int launch_serve_t(const ServeParams& P, int threads, int64_t chunks, cudaStream_t s) {
  auto kern = serve_kernel<D, NOISE, MODE, KIND, SeedKeys>;
  if constexpr ((D == 5 || D == 6) && KIND != kKindPlain) {
    if (P.uniform_seed) kern = serve_kernel<D, NOISE, MODE, KIND, ConstKeys>;
  }
  int per_sm = 0;
  int rc = check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, 0), "occupancy query");
  if (rc) return rc;
  if (per_sm < 1) per_sm = 1;
  const int64_t warps = threads / 32;
  int64_t ctas = (chunks + warps - 1) / warps;
  const int64_t resident = (int64_t)num_sms() * per_sm;
  if (ctas > resident) ctas = resident;
  if (ctas < 1) ctas = 1;
  kern<<<(unsigned)ctas, threads, 0, s>>>(P);
  return check_cuda(cudaGetLastError(), "serve_kernel launch");
}

// Defined in k_serve_plain.cu (kKindPlain, every noise layout and loop
// variant) and k_serve_cv.cu (kKindLcv / kKindPilotStats, diagonal noise,
// terminal payoff).
int launch_serve_plain(int dim, int noise, int mode, const ServeParams& P, int threads, int64_t chunks,
                       cudaStream_t s);
int launch_serve_cv(int kind, int dim, const ServeParams& P, int threads, int64_t chunks, cudaStream_t s);
int launch_serve_install(ServeSlot* slots, const ServeInstall* inst, int n, unsigned long long* counters,
                         int ncounters, cudaStream_t s);
int launch_serve_reduce(ServeSlot* slots, const ServeEntry* entries, int n, const double* part, ServeDone* done,
                        cudaStream_t s);

}  // namespace sdemc
