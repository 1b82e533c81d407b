// sdemc_host.cuh — host-side glue shared by the translation units: error
// reporting, descriptor validation, grid sizing and the (D, noise) dispatch.
#pragma once
#include <stdarg.h>
#include <stdio.h>
#include <string.h>
#include <cuda_runtime.h>
#include "../../include/sdemc.h"

namespace sdemc {

void set_error(const char* fmt, ...);
int fail(int code, const char* fmt, ...);
int check_cuda(cudaError_t e, const char* what);
int num_sms();

// Validate the parts of a descriptor every kernel relies on.
int validate_inst(const sdemc_inst* I);

// Iteration cap of the adapted loop (max_iterations_hd in sdemc_device.cuh).
int max_iterations(const sdemc_inst* I);

constexpr int kChunk = SDEMC_CHUNK_PATHS;
constexpr int kGroup = 256;              // chunks per first-level reduction group
constexpr size_t kScratchHeader = 256;   // status word, completion counter, padding

inline int64_t num_chunks(const sdemc_inst* I) {
  return (I->num_paths + kChunk - 1) / kChunk;
}

// Scratch layout: [header][nchunks x width doubles][ngroups x width doubles].
constexpr int64_t num_groups_for(int64_t nchunks) {
  return nchunks > 0 ? (nchunks + kGroup - 1) / kGroup : 1;
}
constexpr size_t scratch_bytes_for(int64_t nchunks, int width) {
  return kScratchHeader + (size_t)(nchunks + num_groups_for(nchunks)) * width * sizeof(double);
}
inline int32_t* scratch_status(void* s) { return (int32_t*)s; }
inline unsigned* scratch_counter(void* s) { return (unsigned*)((char*)s + 4); }
inline double* scratch_chunks(void* s) { return (double*)((char*)s + kScratchHeader); }

// Launch the deterministic FP64 chunk reduction (K10) over the chunk partials
// in `scratch`; writes sums, mean, var and the status word to out.
int launch_reduce(void* scratch, int64_t nchunks, int width, double* out, cudaStream_t s);

}  // namespace sdemc

// Expand F(D, NOISE) for the runtime (dim, noise) pair.
#define SDEMC_DISPATCH_DIM(NOISE_, dim_, F)                         \
  switch (dim_) {                                                   \
    case 1: { F(1, NOISE_); } break;                                \
    case 2: { F(2, NOISE_); } break;                                \
    case 3: { F(3, NOISE_); } break;                                \
    case 4: { F(4, NOISE_); } break;                                \
    case 5: { F(5, NOISE_); } break;                                \
    case 6: { F(6, NOISE_); } break;                                \
    case 7: { F(7, NOISE_); } break;                                \
    case 8: { F(8, NOISE_); } break;                                \
    default: return sdemc::fail(SDEMC_EINVAL, "dim %d out of range", dim_); \
  }

#define SDEMC_DISPATCH(dim_, noise_, F)                                         \
  switch (noise_) {                                                             \
    case SDEMC_NOISE_DIAG: SDEMC_DISPATCH_DIM(SDEMC_NOISE_DIAG, dim_, F) break; \
    case SDEMC_NOISE_INDEP_SHARED:                                              \
      SDEMC_DISPATCH_DIM(SDEMC_NOISE_INDEP_SHARED, dim_, F) break;              \
    case SDEMC_NOISE_INDEP_PAIR:                                                \
      SDEMC_DISPATCH_DIM(SDEMC_NOISE_INDEP_PAIR, dim_, F) break;                \
    default: return sdemc::fail(SDEMC_EINVAL, "noise layout %d unknown", noise_); \
  }
