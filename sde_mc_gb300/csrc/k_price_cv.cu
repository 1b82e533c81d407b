// k_price_cv.cu — K7: paths, payoff and the learned control variate in one
// pass.
//
// apply_adapted_control_variates with g = 0 (sde_mc/varred.py:98-131) without
// materialising anything: a CTA of 128 threads simulates 128 paths (one per
// thread, warps in lock-step as in K1, and the four warps stepping together),
// and at every step the 128 rows (t_k, X_k) go through the network on the
// tensor cores (mlp_tc.cuh); each thread adds e^{-r t_k} f(t_k, X_k) . dW_k to
// its path's control variate in 32-step ranges, exactly as K5 on tcgen05 sums
// a materialised path, so Gamma matches that kernel bit for bit.  A 32-path
// chunk stores (sum Gamma, sum Gamma^2, n, sum P, sum P^2) in FP64 — the plain
// estimator stays alongside as the fallback and the yardstick of the control
// variate — and K10 sums the chunks in a fixed order.
#include "mlp_tc.cuh"
#include "sdemc_host.cuh"

namespace sdemc {

struct PriceCvParams {
  sdemc_inst I;
  RoundKeys rk;
  const float* prm;
  float rate;
};

constexpr int kCvRange = 32;  // the tcgen05 forward kernel's step range

template <int D>
struct NetCvSink {
  static constexpr bool kWantsLeft = false;
  tc::TcSmem* sm;
  uint32_t* phase;
  bool* fail;
  float rate;
  float range_acc, total;

  template <int DD> SDEMC_DI void init(const float*) {
    range_acc = 0.f;
    total = 0.f;
  }
  // xp, tp: the state and time at the start of step k
  template <int DD, int NW>
  SDEMC_DI void step(int k, const float*, const float*, float, float, int, const float* dW, const float*,
                     const float*, int, const float* xp, float tp) {
    if (k > 0 && k % kCvRange == 0) {  // k is uniform over the CTA
      total = __fadd_rn(total, range_acc);
      range_acc = 0.f;
    }
    float o[D];
    if (tc::forward_rows<D>(*sm, tp, xp, o, *phase, *fail)) {
      float a = 0.f;
#pragma unroll
      for (int i = 0; i < D; ++i) a = __fmaf_rn(o[i], dW[i], a);
      range_acc = __fadd_rn(range_acc, __fmul_rn(expf(-tp * rate), a));
    }
  }
  template <int DD, int NW> SDEMC_DI void finish(int, const float*, float) {}
  SDEMC_DI float value() const { return __fadd_rn(total, range_acc); }
};

template <int D, int MODE>
__global__ void __launch_bounds__(tc::kRows)
price_cv_kernel(const __grid_constant__ PriceCvParams P, double* __restrict__ part, float* __restrict__ gamma_out,
                int32_t* __restrict__ status, int64_t ngroups, int max_iters) {
  extern __shared__ unsigned char smem_raw[];
  tc::TcSmem& sm = *reinterpret_cast<tc::TcSmem*>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~static_cast<uintptr_t>(1023));
  tc::setup<D>(sm, P.prm);
  const sdemc_inst& I = P.I;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  uint32_t phase = 0;
  bool fail = false, ovf = false;
  for (int64_t g = blockIdx.x; g < ngroups; g += gridDim.x) {  // uniform over the CTA
    const int64_t p = g * tc::kRows + threadIdx.x;
    NativeDraws<D, SDEMC_NOISE_DIAG> dr;
    dr.init(I, (uint64_t)p, ConstKeys{&P.rk});
    NetCvSink<D> sk;
    sk.sm = &sm;
    sk.phase = &phase;
    sk.fail = &fail;
    sk.rate = P.rate;
    float x[D];
    simulate<D, SDEMC_NOISE_DIAG, MODE | kModeCtaSync>(I, dr, sk, x, max_iters, ovf);
    const bool valid = p < I.num_paths;
    const float pay = __fmul_rn(payoff<D>(I, x), I.discount);
    const float gam = __fadd_rn(pay, sk.value());
    if (valid && gamma_out) gamma_out[p] = gam;
    const float v = valid ? gam : 0.f, w = valid ? pay : 0.f;
    const float s = warp_sum(v), s2 = warp_sum(__fmul_rn(v, v));
    const float sp = warp_sum(w), sp2 = warp_sum(__fmul_rn(w, w));
    const int n = __popc(__ballot_sync(kFull, valid));
    if (lane == 0) {
      double* row = part + (g * (tc::kRows / kChunk) + wid) * 5;
      row[0] = (double)s;
      row[1] = (double)s2;
      row[2] = (double)n;
      row[3] = (double)sp;
      row[4] = (double)sp2;
    }
  }
  if (threadIdx.x == 0) {
    if (fail) atomicOr(status, SDEMC_ETIMEOUT);
  }
  if (ovf) atomicOr(status, SDEMC_EOVERFLOW);
  tc::teardown(sm);
}

template <int D, int MODE>
static int launch_price_cv_t(const PriceCvParams& P, double* part, float* gamma, int32_t* status, int64_t ngroups,
                             cudaStream_t s) {
  auto kern = price_cv_kernel<D, MODE>;
  const size_t smem = sizeof(tc::TcSmem) + 1024;
  int rc = check_cuda(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                      "smem attribute");
  if (rc) return rc;
  if ((rc = check_cuda(cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout,
                                            (int)cudaSharedmemCarveoutMaxShared), "carveout attribute")))
    return rc;
  cudaFuncAttributes fa;
  int dev = 0, smem_sm = 0;
  if ((rc = check_cuda(cudaFuncGetAttributes(&fa, kern), "function attributes"))) return rc;
  if ((rc = check_cuda(cudaGetDevice(&dev), "cudaGetDevice"))) return rc;
  if ((rc = check_cuda(cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev),
                       "smem per SM")))
    return rc;
  int per_sm = 65536 / (((fa.numRegs + 7) / 8 * 8) * tc::kRows);
  const int by_smem = smem_sm / (int)(smem + 1024);
  if (per_sm > by_smem) per_sm = by_smem;
  if (per_sm > 512 / tc::kTmemCols) per_sm = 512 / tc::kTmemCols;
  if (per_sm < 1) per_sm = 1;
  int64_t ctas = (int64_t)num_sms() * per_sm;
  if (ctas > ngroups) ctas = ngroups;
  if (ctas < 1) ctas = 1;
  kern<<<(unsigned)ctas, tc::kRows, smem, s>>>(P, part, gamma, status, ngroups, max_iterations(&P.I));
  return check_cuda(cudaGetLastError(), "price_cv_kernel launch");
}

}  // namespace sdemc

using namespace sdemc;

// Chunks of 32 paths, rounded up to whole 128-path CTA groups.
static int64_t cv_chunks(const sdemc_inst* I) {
  const int64_t groups = (I->num_paths + tc::kRows - 1) / tc::kRows;
  return groups * (tc::kRows / kChunk);
}

extern "C" size_t sdemc_price_cv_scratch_bytes(const sdemc_inst* h_inst) {
  if (!h_inst || h_inst->num_paths < 0) return 0;
  return scratch_bytes_for(cv_chunks(h_inst), 5);
}

extern "C" int sdemc_price_cv(const sdemc_inst* h_inst, const float* d_params, float disc_rate, void* d_scratch,
                              size_t scratch_bytes, double* d_out, float* d_gamma, void* stream) {
  if (!h_inst || !d_params || !d_scratch || !d_out) return fail(SDEMC_EINVAL, "null price_cv argument");
  int rc = validate_inst(h_inst);
  if (rc) return rc;
  if (h_inst->noise != SDEMC_NOISE_DIAG || (h_inst->dim != 1 && h_inst->dim != 2))
    return fail(SDEMC_EUNSUPPORTED, "learned control variate in the path loop: diagonal noise, d in {1, 2}");
  const int64_t nch = cv_chunks(h_inst);
  if (scratch_bytes < scratch_bytes_for(nch, 5))
    return fail(SDEMC_ENOMEM, "scratch %zu < %zu", scratch_bytes, scratch_bytes_for(nch, 5));
  if (h_inst->num_paths == 0) return fail(SDEMC_EINVAL, "no paths");
  cudaStream_t s = (cudaStream_t)stream;
  PriceCvParams P;
  P.I = *h_inst;
  P.rk = make_round_keys(h_inst->seed);
  P.prm = d_params;
  P.rate = disc_rate;
  const int64_t ngroups = nch / (tc::kRows / kChunk);
  const bool nominal = (h_inst->flags & SDEMC_INST_PAYOFF_AT_NOMINAL_STEP) != 0;
  double* part = scratch_chunks(d_scratch);
  int32_t* st = scratch_status(d_scratch);
  if (h_inst->dim == 1)
    rc = nominal ? launch_price_cv_t<1, kModeNominal>(P, part, d_gamma, st, ngroups, s)
                 : launch_price_cv_t<1, 0>(P, part, d_gamma, st, ngroups, s);
  else
    rc = nominal ? launch_price_cv_t<2, kModeNominal>(P, part, d_gamma, st, ngroups, s)
                 : launch_price_cv_t<2, 0>(P, part, d_gamma, st, ngroups, s);
  if (rc) return rc;
  return launch_reduce(d_scratch, nch, 5, d_out, s);
}
