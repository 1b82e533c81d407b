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
#include <cuda.h>  // CUcontext / CUresult types only: the library does not link libcuda
#include <mutex>

#include "k_price_kern.cuh"

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
  switch (I.noise) {
    case SDEMC_NOISE_DIAG:
      rc = launch_price_noise<SDEMC_NOISE_DIAG>(I, cfg, exact, nominal, part, d_payoffs, status, nch, s);
      break;
    case SDEMC_NOISE_INDEP_SHARED:
      rc = launch_price_noise<SDEMC_NOISE_INDEP_SHARED>(I, cfg, exact, nominal, part, d_payoffs, status, nch, s);
      break;
    case SDEMC_NOISE_INDEP_PAIR:
      rc = launch_price_noise<SDEMC_NOISE_INDEP_PAIR>(I, cfg, exact, nominal, part, d_payoffs, status, nch, s);
      break;
    default: return fail(SDEMC_EINVAL, "noise layout %d unknown", I.noise);
  }
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

// Device address of g_noalloc_scratch, looked up once per CUDA context.  In
// host code the symbol is only a host-side stand-in, so the address must come
// from cudaGetSymbolAddress with the device current.  The module (and so the
// array) is loaded per context: after cudaDeviceReset, or under another
// context made current on the same device, it lives at a new address.  The
// cache therefore keeps, per device, the unique id of the context the address
// belongs to (cuCtxGetId, reached through cudaGetDriverEntryPointByVersion so
// that the library needs no link to libcuda) and looks the address up again
// when the current context differs.
static constexpr int kNoallocMaxDevices = 64;
struct NoallocAddr {
  unsigned long long ctx_id;  // 0: nothing cached
  void* addr;
};
static NoallocAddr g_noalloc_addr[kNoallocMaxDevices] = {};
static std::mutex g_noalloc_mutex;

typedef CUresult (*CtxGetCurrentFn)(CUcontext*);
typedef CUresult (*CtxGetIdFn)(CUcontext, unsigned long long*);

// Unique id of the calling thread's current context, 0 when none is current
// (the runtime has not set one up yet) or the driver cannot tell.
static unsigned long long current_context_id() {
  static CtxGetCurrentFn get_current = nullptr;
  static CtxGetIdFn get_id = nullptr;
  static bool resolved = false;
  if (!resolved) {  // called with g_noalloc_mutex held
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_current = (CtxGetCurrentFn)f;
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = (CtxGetIdFn)f;
    resolved = true;
  }
  if (!get_current || !get_id) return 0;
  CUcontext ctx = nullptr;
  if (get_current(&ctx) != CUDA_SUCCESS || !ctx) return 0;
  unsigned long long id = 0;
  if (get_id(ctx, &id) != CUDA_SUCCESS) return 0;
  return id;
}

static int noalloc_scratch_address(void** out) {
  int dev = 0;
  int rc = check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
  if (rc) return rc;
  if (dev < 0 || dev >= kNoallocMaxDevices) return fail(SDEMC_EINVAL, "device %d out of range", dev);
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  const unsigned long long ctx = current_context_id();
  NoallocAddr& c = g_noalloc_addr[dev];
  if (ctx != 0 && c.ctx_id == ctx && c.addr) {
    *out = c.addr;
    return SDEMC_OK;
  }
  void* p = nullptr;
  rc = check_cuda(cudaGetSymbolAddress(&p, g_noalloc_scratch), "cudaGetSymbolAddress(no-alloc scratch)");
  if (rc) return rc;
  // the lookup makes the runtime's context current if none was: key by it
  c.ctx_id = ctx != 0 ? ctx : current_context_id();
  c.addr = p;
  *out = p;
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
