// k_serve_cv.cu — K9 class kernels of the linear control variate (pilot
// statistics and main run; diagonal noise, terminal payoff), the slot
// install kernel, the per-slot reduction, and the per-path view of the
// control variate (sdemc_serve_cv_paths) that exports what the class kernels
// compute path by path.
#include "serve_kernels.cuh"

namespace sdemc {

int launch_serve_cv(int kind, int dim, const ServeParams& P, int threads, int64_t chunks, cudaStream_t s) {
  int rc = SDEMC_OK;
#define SDEMC_SERVE_CASE(D_, N_)                                                                    \
  rc = kind == kKindLcv ? launch_serve_t<D_, N_, 0, kKindLcv>(P, threads, chunks, s)                 \
                        : launch_serve_t<D_, N_, 0, kKindPilotStats>(P, threads, chunks, s);
  SDEMC_DISPATCH_DIM(SDEMC_NOISE_DIAG, dim, SDEMC_SERVE_CASE)
#undef SDEMC_SERVE_CASE
  return rc;
}

// Writes the tick's staged slot records and clears the class counters.
__global__ void serve_install_kernel(ServeSlot* slots, const ServeInstall* inst, int n,
                                     unsigned long long* counters, int ncounters) {
  if (blockIdx.x == 0)
    for (int c = threadIdx.x; c < ncounters; c += blockDim.x) counters[c] = 0ull;
  for (int i = blockIdx.x; i < n; i += gridDim.x) {
    const ServeInstall& I = inst[i];
    const uint32_t* src;
    uint32_t* dst;
    int words;
    if (I.whole) {
      src = reinterpret_cast<const uint32_t*>(&I.rec);
      dst = reinterpret_cast<uint32_t*>(&slots[I.slot]);
      words = (int)(sizeof(ServeSlot) / 4);
    } else {
      src = reinterpret_cast<const uint32_t*>(&I.rec.st);
      dst = reinterpret_cast<uint32_t*>(&slots[I.slot].st);
      words = (int)(sizeof(ServeState) / 4);
    }
    for (int q = threadIdx.x; q < words; q += blockDim.x) dst[q] = src[q];
  }
}

int launch_serve_install(ServeSlot* slots, const ServeInstall* inst, int n, unsigned long long* counters,
                         int ncounters, cudaStream_t s) {
  const int blocks = n > 0 ? (n < 1024 ? n : 1024) : 1;
  serve_install_kernel<<<blocks, 128, 0, s>>>(slots, inst, n, counters, ncounters);
  return check_cuda(cudaGetLastError(), "serve_install_kernel launch");
}

// One CTA per entry: the entry's chunk partials, thread t summing chunks
// t, t+256, ... in order and a fixed tree across threads, are added to the
// slot's running sums; the cursor moves past the slice.
constexpr int kRedCols = 8;
__global__ void __launch_bounds__(256)
serve_reduce_kernel(ServeSlot* slots, const ServeEntry* entries, const double* part, ServeDone* done) {
  __shared__ double sh[kRedCols][256];
  __shared__ double tot[kServeMaxW];
  const ServeEntry E = entries[blockIdx.x];
  const int t = threadIdx.x;
  const int W = E.width;
  for (int w0 = 0; w0 < W; w0 += kRedCols) {
    double a[kRedCols];
#pragma unroll
    for (int j = 0; j < kRedCols; ++j) a[j] = 0.0;
    for (int64_t c = t; c < E.nchunks; c += 256) {
      const double* row = part + E.part_off + c * W;
#pragma unroll
      for (int j = 0; j < kRedCols; ++j)
        if (w0 + j < W) a[j] += row[w0 + j];
    }
#pragma unroll
    for (int j = 0; j < kRedCols; ++j) sh[j][t] = a[j];
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
      if (t < o)
#pragma unroll
        for (int j = 0; j < kRedCols; ++j) sh[j][t] += sh[j][t + o];
      __syncthreads();
    }
    if (t == 0)
      for (int j = 0; j < kRedCols && w0 + j < W; ++j) tot[w0 + j] = sh[j][0];
    __syncthreads();
  }
  if (t == 0) {
    ServeState& S = slots[E.slot].st;
    for (int w = 0; w < W; ++w) S.acc[w] += tot[w];
    const int64_t c = S.cursor + E.nchunks * kChunk;
    S.cursor = c < S.phase_end ? c : S.phase_end;
    if (E.done >= 0) {
      ServeDone& R = done[E.done];
      R.slot = E.slot;
      R.status = S.status;
      R.width = W;
      R.phase = S.phase;
      R.cursor = S.cursor;
      for (int w = 0; w < W; ++w) R.acc[w] = S.acc[w];
    }
  }
}

int launch_serve_reduce(ServeSlot* slots, const ServeEntry* entries, int n, const double* part, ServeDone* done,
                        cudaStream_t s) {
  if (n <= 0) return SDEMC_OK;
  serve_reduce_kernel<<<n, 256, 0, s>>>(slots, entries, part, done);
  return check_cuda(cudaGetLastError(), "serve_reduce_kernel launch");
}

// The per-path view: DeltaCvSink exactly as the class kernels run it, plus
// exports of the raw normals of the path's own steps and of the weights
// (w, g) evaluated at the start of each of its 4-step blocks.  A lane whose
// path has reached T (frozen by the warp's lock-step) records nothing.
template <int D>
struct CvTraceSink {
  static constexpr bool kWantsLeft = false;
  DeltaCvSink<D> cv;
  float* z;     // (S, D) of this path, or null
  float* wg;    // (wcap, 2) of this path, or null
  int S, wcap;
  float T;
  bool trunc;

  SDEMC_DI void record(int b) {
    if (!wg) return;
    if (b < wcap) {
      wg[2 * b] = cv.w;
      wg[2 * b + 1] = cv.g;
    } else {
      trunc = true;
    }
  }
  template <int DD> SDEMC_DI void init(const float* x) {
    cv.template init<DD>(x);
    record(0);
  }
  template <int DD, int NW>
  SDEMC_DI void step(int k, const float* xl, const float* x, float t, float J, int sel, const float* dW,
                     const float* dW2, const float* zr, int jump_one, const float* xp, float tp) {
    const bool live = tp < T;  // the step started before T
    cv.template step<DD, NW>(k, xl, x, t, J, sel, dW, dW2, zr, jump_one, xp, tp);
    if (!live) return;
    if (k > 0 && (k & (kWeightEvery - 1)) == 0) record(k / kWeightEvery);
    if (z) {
      if (k < S) {
#pragma unroll
        for (int j = 0; j < D; ++j) z[(size_t)k * D + j] = zr[j];
      } else {
        trunc = true;
      }
    }
  }
  template <int DD, int NW> SDEMC_DI void finish(int, const float*, float) {}
};

template <int D>
__global__ void __launch_bounds__(128)
serve_cv_paths_kernel(const __grid_constant__ sdemc_inst I, const __grid_constant__ CvWeights cw, int S,
                      float* d_pay, float* d_reg, float* zout, float* jt, float* jm, int32_t* jsel, int jcap,
                      float* wg, int wcap, int32_t* status, int max_iters) {
  constexpr int R = 2 * D + 1;
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const bool valid = p < I.num_paths;
  NativeDraws<D, SDEMC_NOISE_DIAG, SeedKeys> dr;
  dr.init(I, (uint64_t)p, SeedKeys{(uint32_t)I.seed, (uint32_t)(I.seed >> 32)});
  CvTraceSink<D> sk;
  sk.cv.cw = &cw;
  sk.z = (valid && zout) ? zout + (size_t)p * S * D : nullptr;
  sk.wg = (valid && wg) ? wg + (size_t)p * wcap * 2 : nullptr;
  sk.S = S;
  sk.wcap = wcap;
  sk.T = I.T;
  sk.trunc = false;
  bool ovf = false;
  float x[D];
  simulate<D, SDEMC_NOISE_DIAG, 0>(I, dr, sk, x, max_iters, ovf);
  if (!valid) return;
  d_pay[p] = __fmul_rn(payoff<D>(I, x), I.discount);
#pragma unroll
  for (int q = 0; q < R; ++q) d_reg[(size_t)p * R + q] = sk.cv.reg(q);
  if (ovf || sk.trunc) atomicOr(status, SDEMC_EOVERFLOW);
  // the path's jump stream (blocks 0, 1, 2, ...), times accumulated as the loop does
  if (jcap > 0 && (jt || jm || jsel)) {
    float nj = inf_f();
    for (int j = 0; j < jcap; ++j) {
      JumpDraw d{0.f, 0.f, 0};
      if (I.rate > 0.f) {
        d = jump_from_block<D>(I, dr.ps.block(kTagJumps, (uint32_t)j));
        nj = j == 0 ? d.gap : __fadd_rn(nj, d.gap);
      }
      if (jt) jt[(size_t)p * jcap + j] = nj;
      if (jm) jm[(size_t)p * jcap + j] = d.mark;
      if (jsel) jsel[(size_t)p * jcap + j] = d.sel;
    }
  }
}

}  // namespace sdemc

using namespace sdemc;

extern "C" int sdemc_serve_cv_weights(const sdemc_inst* h_inst, sdemc_cv_weights* h_out) {
  int rc = validate_inst(h_inst);
  if (rc) return rc;
  if (!h_out) return fail(SDEMC_EINVAL, "null weights output");
  *h_out = serve_cv_weights(*h_inst);
  return SDEMC_OK;
}

extern "C" int sdemc_serve_cv_paths(const sdemc_inst* h_inst, int steps_cap, float* d_payoff, float* d_reg,
                                    float* d_z, float* d_jt, float* d_jm, int32_t* d_jsel, int jcap, float* d_wg,
                                    int wcap, int32_t* d_status, void* stream) {
  int rc = validate_inst(h_inst);
  if (rc) return rc;
  const sdemc_inst& I = *h_inst;
  if (I.noise != SDEMC_NOISE_DIAG || (I.flags & SDEMC_INST_PAYOFF_AT_NOMINAL_STEP))
    return fail(SDEMC_EUNSUPPORTED, "the served control variate needs diagonal noise and the terminal payoff");
  if (!d_payoff || !d_reg || !d_status) return fail(SDEMC_EINVAL, "null payoff, regressor or status buffer");
  if (d_z && steps_cap < 1) return fail(SDEMC_EINVAL, "steps_cap %d < 1 with normals exported", steps_cap);
  if (d_wg && wcap < 1) return fail(SDEMC_EINVAL, "wcap %d < 1 with weights exported", wcap);
  if ((d_jt || d_jm || d_jsel) && jcap < 1) return fail(SDEMC_EINVAL, "jcap %d < 1 with jumps exported", jcap);
  if (I.num_paths == 0) return SDEMC_OK;
  const CvWeights cw = serve_cv_weights(I);
  const unsigned blocks = (unsigned)((I.num_paths + 127) / 128);
  cudaStream_t s = (cudaStream_t)stream;
  const int mi = max_iterations(&I);
#define SDEMC_CVP_CASE(D_, N_)                                                                              \
  serve_cv_paths_kernel<D_><<<blocks, 128, 0, s>>>(I, cw, steps_cap, d_payoff, d_reg, d_z, d_jt, d_jm, d_jsel, \
                                                   jcap, d_wg, wcap, d_status, mi);
  SDEMC_DISPATCH_DIM(SDEMC_NOISE_DIAG, I.dim, SDEMC_CVP_CASE)
#undef SDEMC_CVP_CASE
  return check_cuda(cudaGetLastError(), "serve_cv_paths_kernel launch");
}
