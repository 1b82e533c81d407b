// k_price_f64.cu — K11: the FP64 reference run.
//
// Prices a descriptor with every path operation in double precision — the
// grid, the Euler and Heston steps, the jumps, the transforms of the draws
// and the payoff — from the same Philox words K1 uses for the same paths
// (uniforms (2m+1) 2^-24 from the top 23 bits of a word, Box-Muller pairs,
// exponential gaps, lognormal marks, asset picks).  It is the FP64 oracle
// against which the FP32 kernels' prices are stated: on the same paths the
// difference of the two means is the FP32 arithmetic's error alone, and with
// many more paths it is an independent reference value for payoffs without a
// closed form (rainbow, basket).
//
// The jump-adapted grid is the exact one: a step ends at the next jump time
// when that falls inside it (the float32 grid's isclose test is an artefact
// of float32 and not needed here).  Coefficients are the descriptor's float32
// values.  Noise: 'diag'; marks: none or lognormal.  One thread per path; a
// warp's 32 consecutive paths form one chunk of (sum, sum_sq, n) in FP64,
// reduced by K10 in a fixed order, so results do not depend on the launch.
#include "sdemc_device.cuh"
#include "sdemc_host.cuh"

namespace sdemc {

namespace {

constexpr double kTwoPiD = 6.283185307179586476925286766559;
constexpr double kPiD = 3.1415926535897932384626433832795;

__device__ __forceinline__ double u01d(uint32_t w) {
  return ((double)(w >> 9) * 2.0 + 1.0) * 0x1p-24;
}

template <int D>
struct DrawsF64 {
  PathStream<ConstKeys> ps;
  double buf[4];
  uint32_t jblk;

  __device__ void fill4(uint32_t b, double* o) const {
    const U4 w = ps.block(kTagDiffusion, b);
    const double r0 = sqrt(-2.0 * log(u01d(w.x))), a0 = kTwoPiD * u01d(w.y) - kPiD;
    const double r1 = sqrt(-2.0 * log(u01d(w.z))), a1 = kTwoPiD * u01d(w.w) - kPiD;
    double s0, c0, s1, c1;
    sincos(a0, &s0, &c0);
    sincos(a1, &s1, &c1);
    o[0] = r0 * c0; o[1] = r0 * s0; o[2] = r1 * c1; o[3] = r1 * s1;
  }
  // the dense schedule of NativeDraws::dense_step: the previous step's unused
  // normals first, then new blocks, the last block's tail carried
  template <int O>
  __device__ void dense_step(int k, double* z) {
    constexpr int NC = O == 0 ? 0 : 4 - O;
    constexpr int TAKE = NC < D ? NC : D;
    constexpr int NBLK = (D - TAKE + 3) / 4;
    double carry[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) carry[j] = buf[j];
#pragma unroll
    for (int j = 0; j < TAKE; ++j) z[j] = carry[j];
    const uint32_t b0 = (uint32_t)((k * D + TAKE) >> 2);
#pragma unroll
    for (int nb = 0; nb < NBLK; ++nb) {
      double o[4];
      fill4(b0 + (uint32_t)nb, o);
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int idx = TAKE + 4 * nb + q;
        if (idx < D) z[idx] = o[q];
        else buf[idx - D] = o[q];
      }
    }
  }
  // the same block schedule as NativeDraws::normals
  __device__ void normals(int k, double* z) {
    if (D == 1 || D == 2) {
      const int pos = (k * D) & 3;
      if (pos == 0) fill4((uint32_t)((k * D) >> 2), buf);
      z[0] = buf[pos];
      if (D == 2) z[1] = buf[pos + 1];
    } else if (D % 4 == 0 || D == 7) {
      constexpr int NB = (D + 3) / 4;
#pragma unroll
      for (int b = 0; b < NB; ++b) {
        double o[4];
        fill4((uint32_t)(k * NB + b), o);
#pragma unroll
        for (int q = 0; q < 4; ++q)
          if (4 * b + q < D) z[4 * b + q] = o[q];
      }
    } else {
      switch ((k * D) & 3) {
        case 0: dense_step<0>(k, z); break;
        case 1: dense_step<1>(k, z); break;
        case 2: dense_step<2>(k, z); break;
        default: dense_step<3>(k, z); break;
      }
    }
  }
  // the jump stream's block j: gap, mark and asset as jump_from_block
  __device__ double jump(const sdemc_inst& I, double& mark, int& sel) {
    const U4 w = ps.block(kTagJumps, jblk++);
    const double gap = -log(u01d(w.x)) / (double)I.rate;
    mark = 0.0;
    if (I.mark == SDEMC_MARK_LOGNORMAL) {
      const double zn = sqrt(-2.0 * log(u01d(w.y))) * cos(kTwoPiD * u01d(w.z) - kPiD);
      mark = expm1((double)I.mark_p[0] + (double)I.mark_p[1] * zn);
    }
    sel = 0;
    if (I.jump_target == SDEMC_JUMP_ONE_ASSET) {
      const double us = u01d(w.w);
#pragma unroll
      for (int i = 0; i < D - 1; ++i) sel += (us >= (double)I.jump_cdf[i]) ? 1 : 0;
    }
    return gap;
  }
};

template <int D>
__device__ __forceinline__ void step_f64(const sdemc_inst& I, double* x, double dt, const double* dW) {
  if (D == 2 && I.model == SDEMC_MODEL_HESTON) {
    const double S = x[0], v = x[1];
    x[0] = S + (double)I.drift_b[0] * S * dt + sqrt(v) * S * dW[0];
    const double a = -1.0 - (double)I.mark_p[0] * dt;
    const double b = (double)I.mark_p[2] * dW[1];
    const double c = v + (double)I.mark_p[1] * dt - 0.5 * dt * (double)I.mark_p[3];
    const double sq = sqrt(b * b - 4.0 * a * c);
    const double y = fmax((-b + sq) / (2.0 * a), (-b - sq) / (2.0 * a));
    x[1] = y * y;
    return;
  }
  const double x0 = x[0];
#pragma unroll
  for (int i = 0; i < D; ++i) {
    if (D == 2 && i == 1 && I.model == SDEMC_MODEL_ASIAN) { x[1] += x0 * dt; continue; }
    const double xi = x[i];
    x[i] = xi + ((double)I.drift_a[i] + (double)I.drift_b[i] * xi) * dt +
           ((double)I.diff_s[i] + (double)I.diff_q[i] * xi) * dW[i];
  }
}

template <int D>
__device__ double payoff_f64(const sdemc_inst& I, const double* xin) {
  double s[D];
#pragma unroll
  for (int i = 0; i < D; ++i) s[i] = (double)I.payoff_scale * (I.payoff_log ? exp(xin[i]) : xin[i]);
  const double K = (double)I.strike;
  double m = s[0];
  switch (I.payoff) {
    case SDEMC_PAYOFF_EUROCALL: return fmax(s[0] - K, 0.0);
    case SDEMC_PAYOFF_EUROPUT: return fmax(K - s[0], 0.0);
    case SDEMC_PAYOFF_BINARY_AON: return s[0] >= K ? s[0] : 0.0;
    case SDEMC_PAYOFF_DIGITAL: return s[0] > K ? 1.0 : 0.0;
    case SDEMC_PAYOFF_BASKET_ARITH:
#pragma unroll
      for (int i = 1; i < D; ++i) m += s[i];
      return fmax(m / D - K, 0.0);
    case SDEMC_PAYOFF_BASKET_GEO:
      m = log(s[0]);
#pragma unroll
      for (int i = 1; i < D; ++i) m += log(s[i]);
      return fmax(exp(m / D) - K, 0.0);
    case SDEMC_PAYOFF_RAINBOW:
#pragma unroll
      for (int i = 1; i < D; ++i) m = fmax(m, s[i]);
      return fmax(m - K, 0.0);
    case SDEMC_PAYOFF_BESTOF:
#pragma unroll
      for (int i = 1; i < D; ++i) m = fmax(m, s[i]);
      return fmax(m, K);
    case SDEMC_PAYOFF_ASIANCALL: {
      if (D < 2) return 0.0;
      const double a = s[D > 1 ? 1 : 0] / (double)I.T;
      return fmax((I.payoff_log ? exp(a) : a) - K, 0.0);
    }
    case SDEMC_PAYOFF_HESTON_RAINBOW:
#pragma unroll
      for (int i = 2; i < D; i += 2) m = fmax(m, s[i]);
      return fmax(m - K, 0.0);
    default: return 0.0;
  }
}

struct PriceF64Params {
  sdemc_inst I;
  RoundKeys rk;
  double discount;
};

template <int D>
__global__ void __launch_bounds__(128)
price_f64_kernel(const __grid_constant__ PriceF64Params P, double* __restrict__ part,
                 int32_t* __restrict__ status, int64_t nchunks, int max_iters) {
  const sdemc_inst& I = P.I;
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  bool ovf = false;
  for (int64_t c = warp; c < nchunks; c += nwarps) {
    const int64_t p = c * kChunk + lane;
    const bool valid = p < I.num_paths;
    double pay = 0.0;
    if (valid) {
      DrawsF64<D> dr;
      dr.ps.init(ConstKeys{&P.rk}, I.stream_id, I.path_offset + (uint64_t)p);
      dr.jblk = 0;
      double x[D], z[D], zs[D], dW[D];
#pragma unroll
      for (int i = 0; i < D; ++i) x[i] = (double)I.x0[i];
      const double T = (double)I.T;
      double h = T / (double)I.num_steps;
      const bool adapted = I.grid == SDEMC_GRID_ADAPTED;
      double mark = 0.0;
      int sel = 0;
      double nj = (adapted && I.rate > 0.f) ? dr.jump(I, mark, sel) : INFINITY;
      double t = 0.0;
      for (int k = 0; adapted ? t < T : k < I.num_steps; ++k) {
        if (k >= max_iters) { ovf = true; break; }
        bool fire = false;
        double dt = h;
        if (adapted) {
          h = fmin(h, T - t);
          fire = nj - t <= h;
          dt = fire ? nj - t : h;
        }
        dr.normals(k, z);
        const double sq = sqrt(dt);
#pragma unroll
        for (int j = 0; j < D; ++j) zs[j] = z[j] * sq;
#pragma unroll
        for (int i = 0; i < D; ++i) {
          double acc = 0.0;
#pragma unroll
          for (int j = 0; j <= i; ++j) acc += (D == 1 ? 1.0 : (double)chol_at(I, i, j)) * zs[j];
          dW[i] = acc;
        }
        double old[D];
#pragma unroll
        for (int i = 0; i < D; ++i) old[i] = x[i];
        step_f64<D>(I, x, dt, dW);
        t = fire ? nj : t + dt;
        if (fire) {
          const bool one = I.jump_target == SDEMC_JUMP_ONE_ASSET;
#pragma unroll
          for (int i = 0; i < D; ++i) {
            if (one && i != sel) continue;
            const double base = I.exact_jumps ? x[i] : old[i];
            x[i] += ((double)I.jump_g[i] + (double)I.jump_k[i] * base) * mark;
          }
          nj += dr.jump(I, mark, sel);
        }
      }
      pay = payoff_f64<D>(I, x) * P.discount;
    }
    __syncwarp();
    double s = pay, s2 = pay * pay;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      s += __shfl_xor_sync(kFull, s, o);
      s2 += __shfl_xor_sync(kFull, s2, o);
    }
    const int n = __popc(__ballot_sync(kFull, valid));
    if (lane == 0) {
      part[c * 3 + 0] = s;
      part[c * 3 + 1] = s2;
      part[c * 3 + 2] = (double)n;
    }
  }
  if (ovf) atomicOr(status, SDEMC_EOVERFLOW);
}

template <int D>
int launch_f64(const sdemc_inst& I, double* part, int32_t* status, int64_t nchunks, cudaStream_t s) {
  auto kern = price_f64_kernel<D>;
  constexpr int threads = 128;
  int per_sm = 0;
  int rc = check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, 0),
                      "occupancy query");
  if (rc) return rc;
  if (per_sm < 1) per_sm = 1;
  int64_t ctas = (nchunks + threads / 32 - 1) / (threads / 32);
  const int64_t resident = (int64_t)num_sms() * per_sm;
  if (ctas > resident) ctas = resident;
  PriceF64Params P;
  P.I = I;
  P.rk = make_round_keys(I.seed);
  // discounter(T): exp(-r T) in FP64 for a constant short rate, else the
  // descriptor's float32 value
  P.discount = I.disc_rate != 0.f ? exp(-(double)I.disc_rate * (double)I.T) : (double)I.discount;
  kern<<<(unsigned)ctas, threads, 0, s>>>(P, part, status, nchunks, max_iterations(&I));
  return check_cuda(cudaGetLastError(), "price_f64_kernel launch");
}

}  // namespace

}  // namespace sdemc

using namespace sdemc;

extern "C" int sdemc_price_f64(const sdemc_inst* h_inst, void* d_scratch, size_t scratch_bytes, double* d_out,
                               void* stream) {
  int rc = validate_inst(h_inst);
  if (rc) return rc;
  if (!d_scratch || !d_out) return fail(SDEMC_EINVAL, "null scratch or output");
  const size_t need = scratch_bytes_for(num_chunks(h_inst), 3);
  if (scratch_bytes < need) return fail(SDEMC_ENOMEM, "scratch %zu bytes < required %zu", scratch_bytes, need);
  const sdemc_inst& I = *h_inst;
  if (I.noise != SDEMC_NOISE_DIAG) return fail(SDEMC_EUNSUPPORTED, "the FP64 run takes 'diag' noise only");
  if (I.rate > 0.f && I.mark != SDEMC_MARK_LOGNORMAL)
    return fail(SDEMC_EUNSUPPORTED, "the FP64 run takes lognormal marks only");
  if (I.flags & SDEMC_INST_PAYOFF_AT_NOMINAL_STEP)
    return fail(SDEMC_EUNSUPPORTED, "the FP64 run prices the terminal state only");
  cudaStream_t s = (cudaStream_t)stream;
  const int64_t nch = num_chunks(h_inst);
  if (nch > 0) {
    switch (I.dim) {
      case 1: rc = launch_f64<1>(I, scratch_chunks(d_scratch), scratch_status(d_scratch), nch, s); break;
      case 2: rc = launch_f64<2>(I, scratch_chunks(d_scratch), scratch_status(d_scratch), nch, s); break;
      case 3: rc = launch_f64<3>(I, scratch_chunks(d_scratch), scratch_status(d_scratch), nch, s); break;
      case 4: rc = launch_f64<4>(I, scratch_chunks(d_scratch), scratch_status(d_scratch), nch, s); break;
      case 5: rc = launch_f64<5>(I, scratch_chunks(d_scratch), scratch_status(d_scratch), nch, s); break;
      case 6: rc = launch_f64<6>(I, scratch_chunks(d_scratch), scratch_status(d_scratch), nch, s); break;
      case 7: rc = launch_f64<7>(I, scratch_chunks(d_scratch), scratch_status(d_scratch), nch, s); break;
      case 8: rc = launch_f64<8>(I, scratch_chunks(d_scratch), scratch_status(d_scratch), nch, s); break;
      default: return fail(SDEMC_EINVAL, "dim %d out of range", I.dim);
    }
    if (rc) return rc;
  }
  return launch_reduce(d_scratch, nch, 3, d_out, s);
}
