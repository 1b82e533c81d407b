// k_serve_cv.cu — K9 class kernels of the linear control variate (pilot
// statistics and main run; diagonal noise, terminal payoff), the slot
// install kernel and the per-slot reduction.
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

}  // namespace sdemc
