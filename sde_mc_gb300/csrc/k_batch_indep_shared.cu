// k_batch_indep_shared.cu — K8 class kernels of the indep shared noise layout (every dimension
// and loop variant), compiled apart from the other layouts so they build in parallel.
#include "k_batch_kern.cuh"

namespace sdemc {
template SDEMC_BATCH_NOISE_SIG(SDEMC_NOISE_INDEP_SHARED);
}  // namespace sdemc
