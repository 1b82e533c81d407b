// k_price_diag.cu — K1 kernels of the diag noise layout (every dimension and
// loop variant), compiled apart from the other layouts so they build in parallel.
#include "k_price_kern.cuh"

namespace sdemc {
template SDEMC_PRICE_NOISE_SIG(SDEMC_NOISE_DIAG);
}  // namespace sdemc
