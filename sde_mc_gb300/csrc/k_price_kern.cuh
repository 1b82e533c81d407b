// k_price_kern.cuh — K1's path kernel and its launch, shared by the
// translation units that instantiate it: k_price_diag.cu,
// k_price_indep_shared.cu and k_price_indep_pair.cu each compile the kernels
// of one noise layout (so the three compile in parallel), and k_price.cu
// holds the entry points.
#pragma once
#include "sdemc_device.cuh"
#include "sdemc_host.cuh"

namespace sdemc {

struct PriceParams {
  sdemc_inst I;
  RoundKeys rk;
};

// Payoff of lane path p (terminal state x) and the chunk's FP32 butterfly
// sums, stored as chunk c's FP64 partial.
template <int D>
SDEMC_DI void emit_chunk(const sdemc_inst& I, const float* x, int64_t p, int64_t c, double* part,
                         float* payoffs) {
  const int lane = threadIdx.x & 31;
  const bool valid = p < I.num_paths;
  const float pay = __fmul_rn(payoff<D>(I, x), I.discount);
  const float v = valid ? pay : 0.f;
  if (valid && payoffs) payoffs[p] = pay;
  const float s = warp_sum(v);
  const float s2 = warp_sum(__fmul_rn(v, v));
  const int n = __popc(__ballot_sync(kFull, valid));
  if (lane == 0) {
    part[c * 3 + 0] = (double)s;
    part[c * 3 + 1] = (double)s2;
    part[c * 3 + 2] = (double)n;
  }
}

// PATHS = paths per lane: 1, or 2 (chunks c and c + 1 stepped together by
// simulate2; the same bits per chunk).
template <int D, int NOISE, int MODE, int PATHS>
__global__ void __launch_bounds__(256)
price_kernel(const __grid_constant__ PriceParams P, double* __restrict__ part,
             float* __restrict__ payoffs, int32_t* __restrict__ status, int64_t nchunks,
             int max_iters) {
  const sdemc_inst& I = P.I;
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  bool ovf = false;
  for (int64_t c = warp * PATHS; c < nchunks; c += nwarps * PATHS) {
    const int64_t p = c * kChunk + lane;
    if (PATHS == 1) {
      NativeDraws<D, NOISE> dr;
      dr.init(I, (uint64_t)p, ConstKeys{&P.rk});
      NullSink sk;
      float x[D];
      simulate<D, NOISE, MODE>(I, dr, sk, x, max_iters, ovf);
      emit_chunk<D>(I, x, p, c, part, payoffs);
    } else {
      // the partner chunk c + 1 may lie past the end: its paths run (beyond
      // num_paths, like the tail lanes of a last chunk) and are not stored
      const int64_t pb = p + kChunk;
      NativeDraws<D, NOISE> da, db;
      da.init(I, (uint64_t)p, ConstKeys{&P.rk});
      db.init(I, (uint64_t)pb, ConstKeys{&P.rk});
      float xa[D], xb[D];
      simulate2<D, NOISE, MODE>(I, da, db, xa, xb, max_iters, ovf);
      emit_chunk<D>(I, xa, p, c, part, payoffs);
      if (c + 1 < nchunks) emit_chunk<D>(I, xb, pb, c + 1, part, payoffs);
    }
  }
  if (ovf) atomicOr(status, SDEMC_EOVERFLOW);
}

template <int D, int NOISE, int MODE>
int launch_price_t(const sdemc_inst& I, const sdemc_cfg& cfg, double* part,
                          float* payoffs, int32_t* status, int64_t nchunks, cudaStream_t s) {
  const int paths = cfg.interleave == 2 ? 2 : 1;
  auto kern = paths == 2 ? price_kernel<D, NOISE, MODE, 2> : price_kernel<D, NOISE, MODE, 1>;
  const int threads = cfg.block_threads > 0 ? cfg.block_threads : 128;
  int per_sm = 0;
  int rc = check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, 0),
                      "occupancy query");
  if (rc) return rc;
  if (cfg.ctas_per_sm > 0 && cfg.ctas_per_sm < per_sm) per_sm = cfg.ctas_per_sm;
  if (per_sm < 1) per_sm = 1;
  const int64_t resident = (int64_t)num_sms() * per_sm;
  const int64_t chunks_per_cta = threads / 32 * paths;
  int64_t ctas = (nchunks + chunks_per_cta - 1) / chunks_per_cta;
  if (ctas > resident) ctas = resident;
  if (ctas < 1) ctas = 1;
  PriceParams P;
  P.I = I;
  P.rk = make_round_keys(I.seed);
  kern<<<(unsigned)ctas, threads, 0, s>>>(P, part, payoffs, status, nchunks, max_iterations(&I));
  return check_cuda(cudaGetLastError(), "price_kernel launch");
}

// Every dimension and loop variant of one noise layout (dispatched on
// I.dim and the exact/nominal flags); instantiated once per layout.
template <int NOISE>
int launch_price_noise(const sdemc_inst& I, const sdemc_cfg& cfg, bool exact, bool nominal, double* part,
                       float* payoffs, int32_t* status, int64_t nch, cudaStream_t s) {
  int rc = SDEMC_OK;
#define SDEMC_PRICE_CASE(D_, N_)                                                                          \
  rc = nominal ? (exact ? launch_price_t<D_, N_, kModeExact | kModeNominal>(I, cfg, part, payoffs, status, \
                                                                          nch, s)                         \
                        : launch_price_t<D_, N_, kModeNominal>(I, cfg, part, payoffs, status, nch, s))    \
               : (exact ? launch_price_t<D_, N_, kModeExact>(I, cfg, part, payoffs, status, nch, s)       \
                        : launch_price_t<D_, N_, 0>(I, cfg, part, payoffs, status, nch, s));
  SDEMC_DISPATCH_DIM(NOISE, I.dim, SDEMC_PRICE_CASE)
#undef SDEMC_PRICE_CASE
  return rc;
}

#define SDEMC_PRICE_NOISE_SIG(N_)                                                                   \
  int launch_price_noise<N_>(const sdemc_inst&, const sdemc_cfg&, bool, bool, double*, float*, int32_t*, \
                             int64_t, cudaStream_t)
extern template SDEMC_PRICE_NOISE_SIG(SDEMC_NOISE_DIAG);
extern template SDEMC_PRICE_NOISE_SIG(SDEMC_NOISE_INDEP_SHARED);
extern template SDEMC_PRICE_NOISE_SIG(SDEMC_NOISE_INDEP_PAIR);

}  // namespace sdemc
