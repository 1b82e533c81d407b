// k_price.cu — K1: fused path simulation + payoff + reduction.
//
// Stands in for mc_simple (sde_mc/mc.py:53-123) driving JumpDiffusionSolver
// .solve (sde_mc/solvers.py:164-226) or DiffusionSolver.solve (:68-88) and
// Option.__call__ (sde_mc/options.py:175-176).  Nothing path-shaped touches
// HBM: each lane keeps its path in registers and draws its increments from its
// own Philox stream.  A chunk of SDEMC_CHUNK_PATHS = 32 consecutive paths (one
// warp round) is reduced by a fixed xor butterfly in FP32 and stored as
// (sum, sum_sq, n) in FP64 at its own slot, so the bits never depend on the
// grid shape; K10 then sums the slots in a fixed order.
#include <mutex>

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
static int launch_price_t(const sdemc_inst& I, const sdemc_cfg& cfg, double* part,
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

}  // namespace sdemc

using namespace sdemc;

extern "C" size_t sdemc_price_scratch_bytes(const sdemc_inst* h_inst) {
  if (!h_inst) return 0;
  return scratch_bytes_for(num_chunks(h_inst), 3);
}

extern "C" int sdemc_price_chunks(const sdemc_inst* h_inst, const sdemc_cfg* h_cfg, void* d_scratch,
                                  size_t scratch_bytes, float* d_payoffs, void* stream) {
  int rc = validate_inst(h_inst);
  if (rc) return rc;
  if (!d_scratch) return fail(SDEMC_EINVAL, "null scratch");
  if (scratch_bytes < sdemc_price_scratch_bytes(h_inst))
    return fail(SDEMC_ENOMEM, "scratch %zu bytes < required %zu", scratch_bytes,
                sdemc_price_scratch_bytes(h_inst));
  if (h_cfg && (h_cfg->block_threads % 32 != 0 || h_cfg->block_threads > 256 || h_cfg->block_threads < 0))
    return fail(SDEMC_EINVAL, "block_threads %d: need a multiple of 32 in [32, 256]", h_cfg->block_threads);
  if (h_cfg && (h_cfg->interleave < 0 || h_cfg->interleave > 2))
    return fail(SDEMC_EINVAL, "interleave %d: paths per lane are 1 or 2 (0 = 1)", h_cfg->interleave);
  sdemc_cfg cfg{};
  if (h_cfg) cfg = *h_cfg;
  const sdemc_inst& I = *h_inst;
  cudaStream_t s = (cudaStream_t)stream;
  int32_t* status = scratch_status(d_scratch);
  double* part = scratch_chunks(d_scratch);
  const int64_t nch = num_chunks(h_inst);
  if (nch == 0) return SDEMC_OK;
  const bool exact = (cfg.flags & SDEMC_CFG_EXACT_EULER) != 0;
  const bool nominal = (I.flags & SDEMC_INST_PAYOFF_AT_NOMINAL_STEP) != 0;
#define SDEMC_PRICE_CASE(D_, N_)                                                                   \
  rc = nominal ? (exact ? launch_price_t<D_, N_, kModeExact | kModeNominal>(I, cfg, part, d_payoffs, \
                                                                          status, nch, s)          \
                        : launch_price_t<D_, N_, kModeNominal>(I, cfg, part, d_payoffs, status,   \
                                                               nch, s))                           \
               : (exact ? launch_price_t<D_, N_, kModeExact>(I, cfg, part, d_payoffs, status, nch, s) \
                        : launch_price_t<D_, N_, 0>(I, cfg, part, d_payoffs, status, nch, s));
  SDEMC_DISPATCH(I.dim, I.noise, SDEMC_PRICE_CASE)
#undef SDEMC_PRICE_CASE
  return rc;
}

extern "C" int sdemc_reduce_chunks(void* d_scratch, int64_t nchunks, int width, double* d_out,
                                   void* stream) {
  if (!d_scratch || !d_out || nchunks < 0) return fail(SDEMC_EINVAL, "bad reduce args");
  return launch_reduce(d_scratch, nchunks, width, d_out, (cudaStream_t)stream);
}

extern "C" int sdemc_price(const sdemc_inst* h_inst, const sdemc_cfg* h_cfg, void* d_scratch,
                           size_t scratch_bytes, double* d_out, float* d_payoffs, void* stream) {
  if (!d_out) return fail(SDEMC_EINVAL, "null output");
  int rc = sdemc_price_chunks(h_inst, h_cfg, d_scratch, scratch_bytes, d_payoffs, stream);
  if (rc) return rc;
  return sdemc_reduce_chunks(d_scratch, num_chunks(h_inst), 3, d_out, stream);
}

// ---------------------------------------------------------------------------
// Pricing without any allocation, for callers that cannot call cudaMalloc.
//
// Some hosts of this library own the GPU's memory themselves: a process that
// hands out all device memory through its own pool (so a stray cudaMalloc
// would fail or fragment it), code running inside a CUDA graph it is building,
// or a plugin whose host forbids allocations from third-party code.  Those
// callers still pass their inputs and outputs, but cannot provide scratch.
// sdemc_price_noalloc keeps the per-chunk partials, the status word and the
// reduction's completion counter in the array below, which lives in this
// library's module: every GPU that loads the library holds
// kNoallocScratchBytes (about 6.3 MB) of it until the process exits.  The
// limit is SDEMC_NOALLOC_MAX_PATHS paths per call.
// ---------------------------------------------------------------------------
static constexpr int64_t kNoallocMaxChunks =
    ((int64_t)SDEMC_NOALLOC_MAX_PATHS + kChunk - 1) / kChunk;
static constexpr size_t kNoallocScratchBytes = scratch_bytes_for(kNoallocMaxChunks, 3);

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocScratchBytes];

// Device address of g_noalloc_scratch, looked up once per device.  In host code
// the symbol is only a host-side stand-in, so the address must come from
// cudaGetSymbolAddress with that device current.
static constexpr int kNoallocMaxDevices = 64;
static void* g_noalloc_addr[kNoallocMaxDevices] = {};
static std::mutex g_noalloc_mutex;

static int noalloc_scratch_address(void** out) {
  int dev = 0;
  int rc = check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
  if (rc) return rc;
  if (dev < 0 || dev >= kNoallocMaxDevices) return fail(SDEMC_EINVAL, "device %d out of range", dev);
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (!g_noalloc_addr[dev]) {
    void* p = nullptr;
    rc = check_cuda(cudaGetSymbolAddress(&p, g_noalloc_scratch), "cudaGetSymbolAddress(no-alloc scratch)");
    if (rc) return rc;
    g_noalloc_addr[dev] = p;
  }
  *out = g_noalloc_addr[dev];
  return SDEMC_OK;
}

extern "C" size_t sdemc_price_noalloc_scratch_bytes(void) { return kNoallocScratchBytes; }

extern "C" int sdemc_price_noalloc(const sdemc_inst* h_inst, const sdemc_cfg* h_cfg, double* d_out,
                                   float* d_payoffs, void* stream) {
  int rc = validate_inst(h_inst);
  if (rc) return rc;
  if (!d_out) return fail(SDEMC_EINVAL, "null output");
  if (h_inst->num_paths > (int64_t)SDEMC_NOALLOC_MAX_PATHS)
    return fail(SDEMC_ENOMEM, "num_paths %lld exceeds the no-allocation limit of %d paths per call",
                (long long)h_inst->num_paths, SDEMC_NOALLOC_MAX_PATHS);
  void* scratch = nullptr;
  if ((rc = noalloc_scratch_address(&scratch))) return rc;
  // The array keeps the previous call's contents: the status word and the
  // completion counter must start at zero (the partials are all rewritten).
  if ((rc = check_cuda(cudaMemsetAsync(scratch, 0, 2 * sizeof(int32_t), (cudaStream_t)stream),
                       "clear no-alloc status")))
    return rc;
  return sdemc_price(h_inst, h_cfg, scratch, kNoallocScratchBytes, d_out, d_payoffs, stream);
}
