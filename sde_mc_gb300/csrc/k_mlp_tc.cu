// k_mlp_tc.cu — K5 on tcgen05: the control-variate forward pass for large
// batches of materialised paths.
//
// A CTA takes 128 paths (one per thread) and a contiguous range of their
// steps; at every step the 128 rows (t_k, X_k) go through the network on the
// 5th-generation tensor cores (mlp_tc.cuh) and each thread adds
// e^{-r t_k} f . m_k to its FP32 partial, m_k being the row's multipliers (the
// Brownian increments for f; marks minus compensator for g).  Ranges of 32
// steps split a path's rows over several CTAs so small batches still fill the
// GPU; cv_gamma_finish_kernel adds a path's partials in range order to its
// payoff, so a path's Gamma does not depend on the grid or on the batch.
#include "mlp_tc.cuh"
#include "sdemc_host.cuh"

namespace sdemc {

template <int D>
__global__ void __launch_bounds__(tc::kRows)
cv_forward_tc_kernel(const float* __restrict__ prm, const float* __restrict__ time, const float* __restrict__ paths,
                     const float* __restrict__ mult, const int64_t* idx, int64_t n, int S, float rate, int nranges,
                     int range_len, float* __restrict__ partial, int32_t* status) {
  extern __shared__ unsigned char smem_raw[];
  tc::TcSmem& sm = *reinterpret_cast<tc::TcSmem*>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~static_cast<uintptr_t>(1023));
  tc::setup<D>(sm, prm);
  uint32_t phase = 0;
  bool fail = false;
  const int64_t groups = (n + tc::kRows - 1) / tc::kRows;
  const int64_t units = groups * nranges;
  for (int64_t u = blockIdx.x; u < units; u += gridDim.x) {  // uniform over the CTA
    const int64_t g = u / nranges;
    const int r = (int)(u % nranges);
    const int64_t q = g * tc::kRows + threadIdx.x;
    const bool has = q < n;
    const int64_t p = has ? (idx ? idx[q] : q) : 0;
    const int k0 = r * range_len;
    const int k1 = min(S, k0 + range_len);
    float acc = 0.f;
    // row k's inputs are loaded while row k-1 is in the network
    float tn = time[p * (S + 1) + k0], xn[D], mn[D];
#pragma unroll
    for (int i = 0; i < D; ++i) {
      xn[i] = paths[(p * (S + 1) + k0) * D + i];
      mn[i] = mult[(p * S + k0) * D + i];
    }
    for (int k = k0; k < k1; ++k) {
      const float tk = tn;
      float x[D], m[D], o[D];
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
      if (tc::forward_rows<D>(sm, tk, x, o, phase, fail)) {
        float a = 0.f;
#pragma unroll
        for (int i = 0; i < D; ++i) a = __fmaf_rn(o[i], m[i], a);
        acc = __fadd_rn(acc, __fmul_rn(expf(-tk * rate), a));
      }
    }
    if (has) partial[q * nranges + r] = fail ? __int_as_float(0x7fc00000) : acc;
  }
  if (fail && threadIdx.x == 0) atomicOr(status, SDEMC_ETIMEOUT);
  tc::teardown(sm);
}

__global__ void cv_gamma_finish_kernel(const float* __restrict__ partial, int nranges,
                                       const float* __restrict__ payoffs, const int64_t* idx, int64_t n,
                                       float* __restrict__ gamma) {
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  float acc = 0.f;
  for (int r = 0; r < nranges; ++r) acc = __fadd_rn(acc, partial[q * nranges + r]);
  const float pay = payoffs ? payoffs[idx ? idx[q] : q] : 0.f;
  gamma[q] = __fadd_rn(pay, acc);
}

// Fixed step ranges of 32 rows: a path's partials (and so its Gamma) do not
// depend on the batch it is in or on the grid; 128-path groups x ranges give
// enough CTAs to fill the GPU even for training minibatches.
constexpr int kRangeLen = 32;
static void tc_ranges(int64_t, int S, int* nranges, int* range_len) {
  *range_len = kRangeLen;
  *nranges = (S + kRangeLen - 1) / kRangeLen;
}

template <int D>
static int launch_tc(const float* prm, const float* time, const float* paths, const float* mult,
                     const float* payoffs, const int64_t* idx, int64_t n, int S, float rate, float* gamma,
                     float* partial, int32_t* status, int nranges, int range_len, cudaStream_t s) {
  auto kern = cv_forward_tc_kernel<D>;
  const size_t smem = sizeof(tc::TcSmem) + 1024;
  int rc = check_cuda(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                      "smem attribute");
  if (rc) return rc;
  // all of the unified L1/shared storage as shared memory, so several CTAs
  // (each with its A tile and weights) share an SM
  if ((rc = check_cuda(cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout,
                                            (int)cudaSharedmemCarveoutMaxShared), "carveout attribute")))
    return rc;
  // resident CTAs per SM from registers, shared memory and tensor memory
  // (kTmemCols of 512 columns each, so that no allocation ever waits)
  cudaFuncAttributes fa;
  int dev = 0, smem_sm = 0;
  if ((rc = check_cuda(cudaFuncGetAttributes(&fa, kern), "function attributes"))) return rc;
  if ((rc = check_cuda(cudaGetDevice(&dev), "cudaGetDevice"))) return rc;
  if ((rc = check_cuda(cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev),
                       "smem per SM")))
    return rc;
  const int regs_cta = ((fa.numRegs + 7) / 8 * 8) * tc::kRows;
  int per_sm = 65536 / (regs_cta > 0 ? regs_cta : 1);
  const int by_smem = smem_sm / (int)(smem + 1024);
  if (per_sm > by_smem) per_sm = by_smem;
  if (per_sm > 512 / tc::kTmemCols) per_sm = 512 / tc::kTmemCols;
  if (per_sm < 1) per_sm = 1;
  const int64_t units = ((n + tc::kRows - 1) / tc::kRows) * nranges;
  int64_t ctas = (int64_t)num_sms() * per_sm;
  if (ctas > units) ctas = units;
  if (ctas < 1) ctas = 1;
  kern<<<(unsigned)ctas, tc::kRows, smem, s>>>(prm, time, paths, mult, idx, n, S, rate, nranges, range_len,
                                                partial, status);
  if ((rc = check_cuda(cudaGetLastError(), "cv_forward_tc_kernel launch"))) return rc;
  cv_gamma_finish_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(partial, nranges, payoffs, idx, n, gamma);
  return check_cuda(cudaGetLastError(), "cv_gamma_finish_kernel launch");
}

}  // namespace sdemc

using namespace sdemc;

// The give-up path of the bounded waits: one warp waits, through the same
// tc::mbar_wait the tensor-core kernels use, on an mbarrier that nothing
// arrives at, and records SDEMC_ETIMEOUT when the wait returns false.
__global__ void wait_probe_kernel(int spins, int32_t* status) {
  __shared__ uint64_t bar;
  const uint32_t a = tc::saddr_of(&bar);
  if (threadIdx.x == 0) {
    tc::mbar_init(a);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  const bool ok = tc::mbar_wait(a, 0u, spins);
  if (!ok && threadIdx.x == 0) atomicOr(status, SDEMC_ETIMEOUT);
}

extern "C" int sdemc_wait_probe(int spins, int32_t* d_status, void* stream) {
  if (spins < 1 || spins > tc::kMaxSpins || !d_status) return fail(SDEMC_EINVAL, "bad wait_probe arguments");
  wait_probe_kernel<<<1, 32, 0, (cudaStream_t)stream>>>(spins, d_status);
  return check_cuda(cudaGetLastError(), "wait_probe launch");
}

extern "C" size_t sdemc_cv_forward_tc_scratch_bytes(int64_t n, int steps) {
  if (n < 1 || steps < 1) return 0;
  int nr = 1, len = 1;
  tc_ranges(n, steps, &nr, &len);
  return (size_t)n * (size_t)nr * sizeof(float);
}

extern "C" int sdemc_cv_forward_tc(int dim, const float* d_params, const float* d_time, const float* d_paths,
                                   const float* d_mult, const float* d_payoffs, const int64_t* d_index, int64_t n,
                                   int steps, float disc_rate, float* d_gamma, void* d_scratch, size_t scratch_bytes,
                                   int32_t* d_status, void* stream) {
  if (n < 0 || steps < 1 || !d_params || !d_time || !d_paths || !d_mult || !d_gamma || !d_status)
    return fail(SDEMC_EINVAL, "bad cv_forward_tc arguments");
  if (n == 0) return SDEMC_OK;
  int nr = 1, len = 1;
  tc_ranges(n, steps, &nr, &len);
  if (!d_scratch || scratch_bytes < (size_t)n * nr * sizeof(float))
    return fail(SDEMC_ENOMEM, "cv_forward_tc scratch %zu < %zu", scratch_bytes, (size_t)n * nr * sizeof(float));
  cudaStream_t s = (cudaStream_t)stream;
  float* partial = static_cast<float*>(d_scratch);
  switch (dim) {
    case 1: return launch_tc<1>(d_params, d_time, d_paths, d_mult, d_payoffs, d_index, n, steps, disc_rate, d_gamma,
                                partial, d_status, nr, len, s);
    case 2: return launch_tc<2>(d_params, d_time, d_paths, d_mult, d_payoffs, d_index, n, steps, disc_rate, d_gamma,
                                partial, d_status, nr, len, s);
    default: return fail(SDEMC_EUNSUPPORTED, "control-variate network for dim %d (supported: 1, 2)", dim);
  }
}
