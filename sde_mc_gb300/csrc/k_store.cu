// k_store.cu — K4 (materialised paths) and K3 (replay of recorded draws).
//
// K4 is JumpDiffusionSolver.solve / DiffusionSolver.solve with full storage
// (sde_mc/solvers.py:150-162, 205-222): it writes the AdaptedPathData layout
// (sde_mc/nets.py:192-207) and, for the oracle, the raw draws it used.
// K3 runs the same loop on increments, marks and jump times recorded from the
// reference, which pins the step and grid arithmetic to the reference's.
// Both share simulate() with K1, so K1 inherits what K3 and K4 prove.
#include "k_store_kern.cuh"

using namespace sdemc;

extern "C" int sdemc_materialise(const sdemc_inst* h_inst, int steps_cap, float* d_paths,
                                 float* d_left, float* d_time, float* d_jumps, float* d_normals,
                                 float* d_payoffs, int32_t* d_steps, float* d_z, int zdim,
                                 float* d_jt, float* d_jm, int32_t* d_jsel, int jcap,
                                 int32_t* d_status, void* stream) {
  int rc = validate_inst(h_inst);
  if (rc) return rc;
  if (steps_cap < 1) return fail(SDEMC_EINVAL, "steps_cap %d < 1", steps_cap);
  if (!d_status) return fail(SDEMC_EINVAL, "null status");
  const sdemc_inst& I = *h_inst;
  if (I.grid == SDEMC_GRID_UNIFORM && steps_cap < I.num_steps)
    return fail(SDEMC_EINVAL, "steps_cap %d < num_steps %d", steps_cap, I.num_steps);
  if (I.num_paths == 0) return SDEMC_OK;
  const unsigned blocks = (unsigned)((I.num_paths + kStoreThreads - 1) / kStoreThreads);
  cudaStream_t s = (cudaStream_t)stream;
  const int mi = max_iterations(&I);
  StoreParams P;
  P.I = I;
  P.rk = make_round_keys(I.seed);
  const bool nominal = (I.flags & SDEMC_INST_PAYOFF_AT_NOMINAL_STEP) != 0;
  const int zd = I.noise == SDEMC_NOISE_DIAG ? I.dim : I.noise == SDEMC_NOISE_INDEP_SHARED ? I.dim + 1 : 2 * I.dim;
  if (d_z && zdim != zd) return fail(SDEMC_EINVAL, "zdim %d != %d for this layout", zdim, zd);
  switch (I.noise) {
#define SDEMC_MAT_NOISE(N_)                                                                                     \
  case N_:                                                                                                      \
    return launch_materialise_noise<N_>(P, nominal, blocks, steps_cap, d_paths, d_left, d_time, d_jumps,        \
                                        d_normals, d_payoffs, d_steps, d_z, d_jt, d_jm, d_jsel, jcap, d_status, \
                                        mi, s);
    SDEMC_MAT_NOISE(SDEMC_NOISE_DIAG)
    SDEMC_MAT_NOISE(SDEMC_NOISE_INDEP_SHARED)
    SDEMC_MAT_NOISE(SDEMC_NOISE_INDEP_PAIR)
#undef SDEMC_MAT_NOISE
    default: return fail(SDEMC_EINVAL, "noise layout %d unknown", I.noise);
  }
}

extern "C" int sdemc_replay(const sdemc_inst* h_inst, int bs, int steps_cap, int max_jumps,
                            const float* d_jump_times, const float* d_dw, const float* d_marks,
                            const int32_t* d_asset, float* d_paths, float* d_left, float* d_time,
                            float* d_jumps, float* d_payoffs, int32_t* d_steps, int32_t* d_status,
                            void* stream) {
  int rc = validate_inst(h_inst);
  if (rc) return rc;
  if (bs < 0 || steps_cap < 1) return fail(SDEMC_EINVAL, "bad replay shape bs=%d S=%d", bs, steps_cap);
  if (!d_dw || !d_paths || !d_status) return fail(SDEMC_EINVAL, "null replay buffer");
  const sdemc_inst& I = *h_inst;
  if (I.rate > 0.f && (!d_jump_times || !d_marks || max_jumps < 1))
    return fail(SDEMC_EINVAL, "jump replay needs jump times and marks");
  if (bs == 0) return SDEMC_OK;
  cudaStream_t s = (cudaStream_t)stream;
  const unsigned blocks = (unsigned)((bs + 127) / 128);
  switch (I.noise) {
#define SDEMC_REPLAY_NOISE(N_)                                                                           \
  case N_:                                                                                               \
    return launch_replay_noise<N_>(I, blocks, bs, steps_cap, max_jumps, d_jump_times, d_dw, d_marks,     \
                                   d_asset, d_paths, d_left, d_time, d_jumps, d_payoffs, d_steps, d_status, \
                                   s);
    SDEMC_REPLAY_NOISE(SDEMC_NOISE_DIAG)
    SDEMC_REPLAY_NOISE(SDEMC_NOISE_INDEP_SHARED)
    SDEMC_REPLAY_NOISE(SDEMC_NOISE_INDEP_PAIR)
#undef SDEMC_REPLAY_NOISE
    default: return fail(SDEMC_EINVAL, "noise layout %d unknown", I.noise);
  }
}
