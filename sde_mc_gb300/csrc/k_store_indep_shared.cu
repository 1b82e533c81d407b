// k_store_indep_shared.cu — K4 and K3 kernels of the indep shared noise layout (every
// dimension and loop variant), compiled apart from the other layouts so they
// build in parallel.
#include "k_store_kern.cuh"

namespace sdemc {
template SDEMC_MATERIALISE_NOISE_SIG(SDEMC_NOISE_INDEP_SHARED);
template SDEMC_REPLAY_NOISE_SIG(SDEMC_NOISE_INDEP_SHARED);
}  // namespace sdemc
