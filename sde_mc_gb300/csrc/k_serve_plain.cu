// k_serve_plain.cu — K9 class kernels of the plain estimator (every noise
// layout, both loop variants) for the pricing server.
#include "serve_kernels.cuh"

namespace sdemc {

int launch_serve_plain(int dim, int noise, int mode, const ServeParams& P, int threads, int64_t chunks,
                       cudaStream_t s) {
  int rc = SDEMC_OK;
#define SDEMC_SERVE_CASE(D_, N_)                                                                  \
  rc = mode == kModeNominal ? launch_serve_t<D_, N_, kModeNominal, kKindPlain>(P, threads, chunks, s) \
                            : launch_serve_t<D_, N_, 0, kKindPlain>(P, threads, chunks, s);
  SDEMC_DISPATCH(dim, noise, SDEMC_SERVE_CASE)
#undef SDEMC_SERVE_CASE
  return rc;
}

}  // namespace sdemc
