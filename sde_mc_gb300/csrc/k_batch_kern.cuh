// k_batch_kern.cuh — K8's class kernel and its launch, shared by the
// translation units that instantiate it: k_batch_diag.cu,
// k_batch_indep_shared.cu and k_batch_indep_pair.cu each compile the class
// kernels of one noise layout (so the three compile in parallel), and
// k_batch.cu holds the planner, the reduction and the entry points.
#pragma once
#include "sdemc_device.cuh"
#include "sdemc_host.cuh"

namespace sdemc {

constexpr int kBatchMaxWarps = 8;  // CTAs of up to 256 threads

struct BatchParams {
  const sdemc_inst* insts;       // plan order
  const int64_t* chunk_prefix;   // plan order, global chunk offsets
  int first, count;
  int64_t chunk_begin, chunk_end;
  unsigned long long* counter;   // this class's chunk counter
  int32_t* status;               // per instance (plan order)
  double* part;                  // chunk partials, 3 doubles per global chunk
  // when every instance of the class has the same seed, the Philox round keys
  // are launch constants (as in K1); otherwise each warp derives them
  int32_t uniform_seed;
  RoundKeys rk;
};

template <class KS> SDEMC_DI KS batch_keys(const BatchParams& B, const sdemc_inst& I);
template <> SDEMC_DI SeedKeys batch_keys<SeedKeys>(const BatchParams&, const sdemc_inst& I) {
  return SeedKeys{(uint32_t)I.seed, (uint32_t)(I.seed >> 32)};
}
template <> SDEMC_DI ConstKeys batch_keys<ConstKeys>(const BatchParams& B, const sdemc_inst&) {
  return ConstKeys{&B.rk};
}

// Find the instance of global chunk gc (binary search on the chunk prefix),
// stage its descriptor in shared memory and flush the previous instance's
// overflow flag.  Warp-uniform.
SDEMC_DI void stage_instance(const BatchParams& B, int64_t gc, sdemc_inst* slot, int& cur, int64_t& lo,
                             int64_t& hi, int& max_iters, bool& ovf) {
  const int lane = threadIdx.x & 31;
  if (ovf && lane == 0 && cur >= 0) atomicOr(&B.status[cur], SDEMC_EOVERFLOW);
  ovf = false;
  int a = B.first, b = B.first + B.count;  // chunk_prefix[a] <= gc < chunk_prefix[b]
  while (b - a > 1) {
    const int m = (a + b) >> 1;
    if (B.chunk_prefix[m] <= gc) a = m; else b = m;
  }
  cur = a;
  lo = B.chunk_prefix[a];
  hi = B.chunk_prefix[a + 1];
  __syncwarp();
  const uint32_t* src = reinterpret_cast<const uint32_t*>(&B.insts[cur]);
  uint32_t* dst = reinterpret_cast<uint32_t*>(slot);
  for (int q = lane; q < (int)(sizeof(sdemc_inst) / 4); q += 32) dst[q] = src[q];
  __syncwarp();
  max_iters = max_iterations_hd(*slot);
}

// Payoff and butterfly sums of one chunk into its FP64 partial.
template <int D>
SDEMC_DI void batch_emit(const BatchParams& B, const sdemc_inst& I, const float* x, int64_t p, int64_t gc) {
  const int lane = threadIdx.x & 31;
  const bool valid = p < I.num_paths;
  const float v = valid ? __fmul_rn(payoff<D>(I, x), I.discount) : 0.f;
  const float s = warp_sum(v);
  const float s2 = warp_sum(__fmul_rn(v, v));
  const int n = __popc(__ballot_sync(kFull, valid));
  if (lane == 0) {
    B.part[gc * 3 + 0] = (double)s;
    B.part[gc * 3 + 1] = (double)s2;
    B.part[gc * 3 + 2] = (double)n;
  }
}

// PATHS = paths per lane (1 or 2).  With 2, a warp takes two consecutive
// chunks; when both belong to one instance they step together (simulate2),
// otherwise one after the other.  Either way every chunk's bits are those of
// the one-path loop.
template <int D, int NOISE, int MODE, int PATHS, class KS>
__global__ void __launch_bounds__(256)
batch_kernel(const __grid_constant__ BatchParams B) {
  __shared__ __align__(16) sdemc_inst s_inst[kBatchMaxWarps];  // 16-byte aligned arrays: vector loads
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int cur = -1;
  int64_t lo = 0, hi = 0;
  int max_iters = 0;
  bool ovf = false;
  for (;;) {
    unsigned long long g = 0;
    if (lane == 0) g = atomicAdd(B.counter, (unsigned long long)PATHS);
    g = __shfl_sync(kFull, g, 0);
    const int64_t gc = B.chunk_begin + (int64_t)g;
    if (gc >= B.chunk_end) break;
    if (gc < lo || gc >= hi) stage_instance(B, gc, &s_inst[wid], cur, lo, hi, max_iters, ovf);
    const sdemc_inst& I = s_inst[wid];
    const KS keys = batch_keys<KS>(B, I);
    const int64_t p = (gc - lo) * kChunk + lane;
    if (PATHS == 2 && gc + 1 < hi) {
      NativeDraws<D, NOISE, KS> da, db;
      da.init(I, (uint64_t)p, keys);
      db.init(I, (uint64_t)(p + kChunk), keys);
      float xa[D], xb[D];
      simulate2<D, NOISE, MODE>(I, da, db, xa, xb, max_iters, ovf);
      batch_emit<D>(B, I, xa, p, gc);
      batch_emit<D>(B, I, xb, p + kChunk, gc + 1);
      continue;
    }
    {
      NativeDraws<D, NOISE, KS> dr;
      dr.init(I, (uint64_t)p, keys);
      NullSink sk;
      float x[D];
      simulate<D, NOISE, MODE>(I, dr, sk, x, max_iters, ovf);
      batch_emit<D>(B, I, x, p, gc);
    }
    if (PATHS == 2 && gc + 1 < B.chunk_end) {  // the partner chunk starts the next instance
      const int64_t gc1 = gc + 1;
      stage_instance(B, gc1, &s_inst[wid], cur, lo, hi, max_iters, ovf);
      const sdemc_inst& J = s_inst[wid];
      const int64_t p1 = (gc1 - lo) * kChunk + lane;
      NativeDraws<D, NOISE, KS> dr;
      dr.init(J, (uint64_t)p1, batch_keys<KS>(B, J));
      NullSink sk;
      float x[D];
      simulate<D, NOISE, MODE>(J, dr, sk, x, max_iters, ovf);
      batch_emit<D>(B, J, x, p1, gc1);
    }
  }
  if (ovf && lane == 0 && cur >= 0) atomicOr(&B.status[cur], SDEMC_EOVERFLOW);
}

template <int D, int NOISE, int MODE>
int launch_batch_t(const BatchParams& B, const sdemc_cfg* cfg, int64_t chunks, cudaStream_t s) {
  const int paths = cfg && cfg->interleave == 2 ? 2 : 1;
  auto kern = B.uniform_seed ? (paths == 2 ? batch_kernel<D, NOISE, MODE, 2, ConstKeys> : batch_kernel<D, NOISE, MODE, 1, ConstKeys>)
                             : (paths == 2 ? batch_kernel<D, NOISE, MODE, 2, SeedKeys> : batch_kernel<D, NOISE, MODE, 1, SeedKeys>);
  int threads = cfg && cfg->block_threads > 0 ? cfg->block_threads : 128;
  int per_sm = 0;
  int rc = check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, 0), "occupancy query");
  if (rc) return rc;
  if (cfg && cfg->ctas_per_sm > 0 && cfg->ctas_per_sm < per_sm) per_sm = cfg->ctas_per_sm;
  if (per_sm < 1) per_sm = 1;
  const int64_t per_cta = threads / 32 * paths;
  int64_t ctas = (chunks + per_cta - 1) / per_cta;
  const int64_t resident = (int64_t)num_sms() * per_sm;
  if (ctas > resident) ctas = resident;
  if (ctas < 1) ctas = 1;
  kern<<<(unsigned)ctas, threads, 0, s>>>(B);
  return check_cuda(cudaGetLastError(), "batch_kernel launch");
}

// Every dimension and loop variant of one noise layout; instantiated once
// per layout.
template <int NOISE>
int launch_batch_noise(int dim, int mode, const BatchParams& B, const sdemc_cfg* cfg, int64_t chunks,
                       cudaStream_t s) {
  int rc = SDEMC_OK;
#define SDEMC_BATCH_CASE(D_, N_)                                                      \
  rc = mode == kModeNominal ? launch_batch_t<D_, N_, kModeNominal>(B, cfg, chunks, s) \
                            : launch_batch_t<D_, N_, 0>(B, cfg, chunks, s);
  SDEMC_DISPATCH_DIM(NOISE, dim, SDEMC_BATCH_CASE)
#undef SDEMC_BATCH_CASE
  return rc;
}

#define SDEMC_BATCH_NOISE_SIG(N_) \
  int launch_batch_noise<N_>(int, int, const BatchParams&, const sdemc_cfg*, int64_t, cudaStream_t)
extern template SDEMC_BATCH_NOISE_SIG(SDEMC_NOISE_DIAG);
extern template SDEMC_BATCH_NOISE_SIG(SDEMC_NOISE_INDEP_SHARED);
extern template SDEMC_BATCH_NOISE_SIG(SDEMC_NOISE_INDEP_PAIR);

}  // namespace sdemc
