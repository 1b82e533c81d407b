// api.cu — library-wide C ABI entry points (errors, ABI description, device
// info, raw Philox export) and the deterministic FP64 reduction K10 that
// stands in for mc_estimates (sde_mc/helpers.py:51-68).
#include <math.h>
#include <stddef.h>
#include "sdemc_device.cuh"
#include "sdemc_host.cuh"

namespace sdemc {

static thread_local char g_err[512] = "";

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

int fail(int code, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
  return code;
}

int check_cuda(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return SDEMC_OK;
  return fail(SDEMC_ECUDA, "%s: %s", what, cudaGetErrorString(e));
}

int num_sms() {
  static thread_local int cached_dev = -1, cached_sms = 0;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  if (dev != cached_dev) {
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
    cached_dev = dev;
    cached_sms = sms;
  }
  return cached_sms;
}

int validate_inst(const sdemc_inst* I) {
  if (!I) return fail(SDEMC_EINVAL, "null descriptor");
  if (I->dim < 1 || I->dim > SDEMC_MAX_DIM) return fail(SDEMC_EINVAL, "dim %d out of range 1..%d", I->dim, SDEMC_MAX_DIM);
  if (I->noise < 0 || I->noise > SDEMC_NOISE_INDEP_PAIR) return fail(SDEMC_EINVAL, "noise layout %d unknown", I->noise);
  if (I->grid != SDEMC_GRID_ADAPTED && I->grid != SDEMC_GRID_UNIFORM) return fail(SDEMC_EINVAL, "grid %d unknown", I->grid);
  if (I->num_steps < 1) return fail(SDEMC_EINVAL, "num_steps %d < 1", I->num_steps);
  if (I->num_paths < 0) return fail(SDEMC_EINVAL, "num_paths %lld < 0", (long long)I->num_paths);
  if (!(I->T > 0.f) || !(I->h > 0.f)) return fail(SDEMC_EINVAL, "time interval and step must be positive");
  if (I->mark < SDEMC_MARK_NONE || I->mark > SDEMC_MARK_INVCDF) return fail(SDEMC_EINVAL, "mark law %d unknown", I->mark);
  if (I->rate > 0.f && I->mark == SDEMC_MARK_NONE) return fail(SDEMC_EINVAL, "positive jump rate without a mark law");
  if (I->grid == SDEMC_GRID_UNIFORM && I->rate > 0.f) return fail(SDEMC_EUNSUPPORTED, "uniform grid with jumps");
  if (I->payoff < SDEMC_PAYOFF_EUROCALL || I->payoff > SDEMC_PAYOFF_HESTON_RAINBOW) return fail(SDEMC_EUNSUPPORTED, "payoff %d unknown", I->payoff);
  if (I->noise == SDEMC_NOISE_INDEP_PAIR && I->grid != SDEMC_GRID_UNIFORM) return fail(SDEMC_EUNSUPPORTED, "paired noise only on the uniform grid");
  if (I->model > SDEMC_MODEL_ASIAN) return fail(SDEMC_EINVAL, "model %u unknown", I->model);
  if (I->model != SDEMC_MODEL_AFFINE && (I->dim != 2 || I->noise != SDEMC_NOISE_DIAG))
    return fail(SDEMC_EUNSUPPORTED, "Heston and Asian models are 2-D with 'diag' noise");
  if (I->model == SDEMC_MODEL_HESTON && (I->rate > 0.f || I->grid != SDEMC_GRID_UNIFORM))
    return fail(SDEMC_EUNSUPPORTED, "Heston runs on the uniform grid (HestonSolver), without jumps");
  if (I->model == SDEMC_MODEL_ASIAN && I->jump_target != SDEMC_JUMP_COMMON)
    return fail(SDEMC_EUNSUPPORTED, "the Asian integral takes common jumps only");
  return SDEMC_OK;
}

int max_iterations(const sdemc_inst* I) { return max_iterations_hd(*I); }

// ----------------------------------------------------------------- K10 -----
// Two fixed levels in one launch.  CTA g sums chunks [256g, 256g + 256) with a
// halving tree into group partial g; the CTA that completes last (completion
// counter) has thread i add group partials i, i+256, ... in order and runs the
// same tree, then writes sums, mean, sample variance and the status word and
// resets the counter.  Which CTA finishes last does not change any bit.
constexpr int kRedThreads = kGroup;
constexpr int kRedMaxW = 5;

__global__ void __launch_bounds__(kRedThreads)
reduce_kernel(const double* __restrict__ part, int64_t nchunks, int width, double* groups,
              int64_t ngroups, int32_t* status, unsigned* counter, double* __restrict__ out) {
  __shared__ double sh[kRedMaxW][kRedThreads];
  __shared__ bool last;
  const int t = threadIdx.x;
  const int64_t c = (int64_t)blockIdx.x * kRedThreads + t;
#pragma unroll
  for (int w = 0; w < kRedMaxW; ++w) sh[w][t] = (w < width && c < nchunks) ? part[c * width + w] : 0.0;
  __syncthreads();
  for (int o = kRedThreads / 2; o > 0; o >>= 1) {
    if (t < o)
      for (int w = 0; w < width; ++w) sh[w][t] += sh[w][t + o];
    __syncthreads();
  }
  if (t == 0) {
    for (int w = 0; w < width; ++w) groups[blockIdx.x * width + w] = sh[w][0];
    __threadfence();
    last = atomicAdd(counter, 1u) == (unsigned)(ngroups - 1);
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  double acc[kRedMaxW];
#pragma unroll
  for (int w = 0; w < kRedMaxW; ++w) acc[w] = 0.0;
  for (int64_t q = t; q < ngroups; q += kRedThreads)
    for (int w = 0; w < width; ++w) acc[w] += __ldcg(&groups[q * width + w]);
  __syncthreads();
#pragma unroll
  for (int w = 0; w < kRedMaxW; ++w) sh[w][t] = acc[w];
  __syncthreads();
  for (int o = kRedThreads / 2; o > 0; o >>= 1) {
    if (t < o)
      for (int w = 0; w < width; ++w) sh[w][t] += sh[w][t + o];
    __syncthreads();
  }
  if (t == 0) {
    const double s = sh[0][0], s2 = sh[1][0], n = sh[2][0];
    for (int w = 0; w < width; ++w) out[w] = sh[w][0];
    // mc_estimates: mean = S/n, var = (S2 - S^2/n)/(n-1)
    out[width] = n > 0 ? s / n : 0.0;
    out[width + 1] = n > 1 ? (s2 - s * s / n) / (n - 1.0) : 0.0;
    const int st = *status;
    *status = 0;
    out[width + 2] = (double)st;
    *counter = 0u;
  }
}

int launch_reduce(void* scratch, int64_t nchunks, int width, double* out, cudaStream_t s) {
  if (width < 3 || width > kRedMaxW) return fail(SDEMC_EINVAL, "reduce width %d", width);
  const int64_t ngroups = num_groups_for(nchunks);
  if (ngroups > 0x7fffffff) return fail(SDEMC_EINVAL, "too many chunks");
  double* part = scratch_chunks(scratch);
  double* groups = part + nchunks * width;
  reduce_kernel<<<(unsigned)ngroups, kRedThreads, 0, s>>>(part, nchunks, width, groups, ngroups,
                                                          scratch_status(scratch), scratch_counter(scratch),
                                                          out);
  return check_cuda(cudaGetLastError(), "reduce_kernel launch");
}

__global__ void philox_kernel(uint64_t seed, uint32_t stream_id, uint32_t tag, uint64_t path,
                              uint32_t first, int n, uint32_t* out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const RoundKeys rk = make_round_keys(seed);
  PathStream<ConstKeys> k;
  k.init(ConstKeys{&rk}, stream_id, path);
  const U4 w = k.block(tag, first + (uint32_t)i);
  out[4 * i + 0] = w.x; out[4 * i + 1] = w.y; out[4 * i + 2] = w.z; out[4 * i + 3] = w.w;
}

// FP32 throughput probe: 8 independent FMA chains per thread, full occupancy.
// Used to measure the FP32 roofline denominator on the box itself.
__global__ void __launch_bounds__(256) fp32_probe_kernel(int iters, float b, float c, float never,
                                                         float* out, int out_len) {
  float a0 = threadIdx.x * 1e-7f, a1 = a0 + 1e-7f, a2 = a0 + 2e-7f, a3 = a0 + 3e-7f;
  float a4 = a0 + 4e-7f, a5 = a0 + 5e-7f, a6 = a0 + 6e-7f, a7 = a0 + 7e-7f;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      a0 = __fmaf_rn(a0, b, c); a1 = __fmaf_rn(a1, b, c); a2 = __fmaf_rn(a2, b, c); a3 = __fmaf_rn(a3, b, c);
      a4 = __fmaf_rn(a4, b, c); a5 = __fmaf_rn(a5, b, c); a6 = __fmaf_rn(a6, b, c); a7 = __fmaf_rn(a7, b, c);
    }
  }
  const float s = ((a0 + a1) + (a2 + a3)) + ((a4 + a5) + (a6 + a7));
  // keeps the chains live; `never` is NaN, so the store is never taken, and
  // even then it stays inside the caller's buffer
  if (s == never) out[blockIdx.x % out_len] = s;
}

// MUFU throughput probe: 8 independent reciprocal-square-root chains per
// thread (rsqrt.approx is one special-function-unit operation; the chains
// converge to 1 and stay finite), full occupancy.
__global__ void __launch_bounds__(256) mufu_probe_kernel(int iters, float never, float* out, int out_len) {
  float a[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) a[j] = 1.5f + (threadIdx.x + j) * 1e-3f;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int u = 0; u < 4; ++u) {
#pragma unroll
      for (int j = 0; j < 8; ++j) asm("rsqrt.approx.ftz.f32 %0, %0;" : "+f"(a[j]));
    }
  }
  const float s = ((a[0] + a[1]) + (a[2] + a[3])) + ((a[4] + a[5]) + (a[6] + a[7]));
  if (s == never) out[blockIdx.x % out_len] = s;
}

}  // namespace sdemc

using namespace sdemc;

extern "C" int sdemc_mufu_probe(int iters, float* d_sink, int sink_len, double* h_ops, void* stream) {
  if (iters < 1 || !h_ops || !d_sink || sink_len < 1) return fail(SDEMC_EINVAL, "bad probe args");
  const int sms = num_sms();
  if (sms <= 0) return fail(SDEMC_ECUDA, "no CUDA device");
  const int blocks = sms * 8;
  mufu_probe_kernel<<<blocks, 256, 0, (cudaStream_t)stream>>>(iters, __builtin_nanf(""), d_sink, sink_len);
  *h_ops = (double)blocks * 256.0 * iters * 32.0;
  return check_cuda(cudaGetLastError(), "mufu_probe_kernel launch");
}

extern "C" int sdemc_fp32_probe(int iters, float* d_sink, int sink_len, double* h_flops, void* stream) {
  if (iters < 1 || !h_flops || !d_sink || sink_len < 1) return fail(SDEMC_EINVAL, "bad probe args");
  const int sms = num_sms();
  if (sms <= 0) return fail(SDEMC_ECUDA, "no CUDA device");
  const int blocks = sms * 8;
  fp32_probe_kernel<<<blocks, 256, 0, (cudaStream_t)stream>>>(iters, 0.999999f, 1e-7f, __builtin_nanf(""),
                                                               d_sink, sink_len);
  *h_flops = (double)blocks * 256.0 * iters * 32.0 * 2.0;
  return check_cuda(cudaGetLastError(), "fp32_probe_kernel launch");
}

extern "C" {

int sdemc_abi_version(void) { return SDEMC_ABI_VERSION; }
static_assert(offsetof(sdemc_inst, x0) % 16 == 0 && sizeof(sdemc_inst) % 16 == 0,
              "the descriptor's arrays start on 16-byte boundaries");
size_t sdemc_inst_size(void) { return sizeof(sdemc_inst); }

int sdemc_inst_offsets(size_t* h_offsets, int* n) {
  static const size_t offs[] = {
      offsetof(sdemc_inst, dim), offsetof(sdemc_inst, noise), offsetof(sdemc_inst, grid),
      offsetof(sdemc_inst, num_steps), offsetof(sdemc_inst, mark), offsetof(sdemc_inst, jump_target),
      offsetof(sdemc_inst, exact_jumps), offsetof(sdemc_inst, payoff), offsetof(sdemc_inst, payoff_log),
      offsetof(sdemc_inst, flags), offsetof(sdemc_inst, stream_id), offsetof(sdemc_inst, model),
      offsetof(sdemc_inst, seed), offsetof(sdemc_inst, path_offset), offsetof(sdemc_inst, num_paths),
      offsetof(sdemc_inst, T), offsetof(sdemc_inst, h), offsetof(sdemc_inst, rate),
      offsetof(sdemc_inst, inv_rate), offsetof(sdemc_inst, strike), offsetof(sdemc_inst, payoff_scale),
      offsetof(sdemc_inst, discount), offsetof(sdemc_inst, disc_rate), offsetof(sdemc_inst, reserved0),
      offsetof(sdemc_inst, x0),
      offsetof(sdemc_inst, drift_a), offsetof(sdemc_inst, drift_b), offsetof(sdemc_inst, diff_s),
      offsetof(sdemc_inst, diff_q), offsetof(sdemc_inst, diff2_s), offsetof(sdemc_inst, diff2_q),
      offsetof(sdemc_inst, jump_g), offsetof(sdemc_inst, jump_k), offsetof(sdemc_inst, jump_cdf),
      offsetof(sdemc_inst, chol), offsetof(sdemc_inst, mark_p)};
  const int cnt = (int)(sizeof(offs) / sizeof(offs[0]));
  if (!n) return fail(SDEMC_EINVAL, "null count");
  if (h_offsets) {
    const int m = *n < cnt ? *n : cnt;
    for (int i = 0; i < m; ++i) h_offsets[i] = offs[i];
  }
  *n = cnt;
  return SDEMC_OK;
}

int sdemc_last_error(char* h_buf, size_t len) {
  if (!h_buf || len == 0) return SDEMC_EINVAL;
  strncpy(h_buf, g_err, len - 1);
  h_buf[len - 1] = '\0';
  return SDEMC_OK;
}

int sdemc_device_sms(int* h_sms) {
  if (!h_sms) return fail(SDEMC_EINVAL, "null out");
  const int s = num_sms();
  if (s <= 0) return fail(SDEMC_ECUDA, "no CUDA device");
  *h_sms = s;
  return SDEMC_OK;
}

int sdemc_philox(uint64_t seed, uint32_t stream_id, uint32_t tag, uint64_t path,
                 uint32_t first_block, int nblocks, uint32_t* d_out, void* stream) {
  if (nblocks < 0 || (nblocks > 0 && !d_out)) return fail(SDEMC_EINVAL, "bad philox export args");
  if (nblocks == 0) return SDEMC_OK;
  philox_kernel<<<(nblocks + 255) / 256, 256, 0, (cudaStream_t)stream>>>(seed, stream_id, tag, path,
                                                                      first_block, nblocks, d_out);
  return check_cuda(cudaGetLastError(), "philox_kernel launch");
}

}  // extern "C"
