// k_store.cu — K4 (materialised paths) and K3 (replay of recorded draws).
//
// K4 is JumpDiffusionSolver.solve / DiffusionSolver.solve with full storage
// (sde_mc/solvers.py:150-162, 205-222): it writes the AdaptedPathData layout
// (sde_mc/nets.py:192-207) and, for the oracle, the raw draws it used.
// K3 runs the same loop on increments, marks and jump times recorded from the
// reference, which pins the step and grid arithmetic to the reference's.
// Both share simulate() with K1, so K1 inherits what K3 and K4 prove.
#include "sdemc_device.cuh"
#include "sdemc_host.cuh"

namespace sdemc {

struct StoreParams {
  sdemc_inst I;
  RoundKeys rk;
};

template <int D, int NOISE, int MODE>
__global__ void __launch_bounds__(128)
materialise_kernel(const __grid_constant__ StoreParams P, int S, float* paths, float* left,
                   float* time, float* jumps, float* normals, float* payoffs, int32_t* steps,
                   float* zout, int zdim, float* jt, float* jm, int32_t* jsel, int jcap,
                   int32_t* status, int max_iters) {
  using L = Layout<D, NOISE>;
  const sdemc_inst& I = P.I;
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const bool valid = p < I.num_paths;
  StoreSink sk{};
  sk.S = S;
  sk.zdim = zdim;
  if (valid) {
    const size_t row = (size_t)p * (S + 1);
    sk.paths = paths ? paths + row * D : nullptr;
    sk.left = left ? left + row * D : nullptr;
    sk.time = time ? time + row : nullptr;
    sk.jumps = jumps ? jumps + row * D : nullptr;
    sk.normals = normals ? normals + (size_t)p * S * D * L::NW : nullptr;
    sk.z = zout ? zout + (size_t)p * S * zdim : nullptr;
  }
  NativeDraws<D, NOISE> dr;
  dr.init(I, (uint64_t)p, ConstKeys{&P.rk});
  bool ovf = false;
  float x[D];
  const int it = max_iters < S ? max_iters : S;
  const int own = simulate<D, NOISE, MODE>(I, dr, sk, x, it, ovf);
  if (!valid) return;
  if (payoffs) payoffs[p] = __fmul_rn(payoff<D>(I, x), I.discount);
  if (steps) steps[p] = own;
  if (ovf) atomicOr(status, SDEMC_EOVERFLOW);
  // Export the jump stream (times, marks, picks) for the oracle: blocks 0, 1,
  // 2, ... of the path's jump stream, times accumulated as the loop does.
  if (jcap > 0 && (jt || jm || jsel)) {
    float nj = inf_f();
    for (int j = 0; j < jcap; ++j) {
      JumpDraw d{0.f, 0.f, 0};
      if (I.rate > 0.f) {
        d = jump_from_block<D>(I, dr.ps.block(kTagJumps, (uint32_t)j));
        nj = j == 0 ? d.gap : __fadd_rn(nj, d.gap);
      }
      if (jt) jt[(size_t)p * jcap + j] = nj;
      if (jm) jm[(size_t)p * jcap + j] = d.mark;
      if (jsel) jsel[(size_t)p * jcap + j] = d.sel;
    }
  }
}

template <int D, int NOISE>
__global__ void __launch_bounds__(128)
replay_kernel(const __grid_constant__ sdemc_inst I, int bs, int S, int MJ, const float* jt,
              const float* dw, const float* marks, const int32_t* asset, float* paths,
              float* left, float* time, float* jumps, float* payoffs, int32_t* steps,
              int32_t* status) {
  using L = Layout<D, NOISE>;
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  const bool valid = p < bs;
  StoreSink sk{};
  sk.S = S;
  sk.zdim = 0;
  ReplayDraws<D, NOISE> dr{};
  dr.S = 0;
  dr.MJ = 0;
  if (valid) {
    const size_t row = (size_t)p * (S + 1);
    sk.paths = paths + row * D;
    sk.left = left ? left + row * D : nullptr;
    sk.time = time ? time + row : nullptr;
    sk.jumps = jumps ? jumps + row * D : nullptr;
    dr.dw = dw + (size_t)p * S * D * L::NW;
    dr.marks = marks ? marks + (size_t)p * S : nullptr;
    dr.asset = asset ? asset + (size_t)p * S : nullptr;
    dr.jt = jt ? jt + (size_t)p * MJ : nullptr;
    dr.S = S;
    dr.MJ = jt ? MJ : 0;
  }
  dr.overflow = false;
  bool ovf = false;
  float x[D];
  const int own = simulate<D, NOISE, kModeExact>(I, dr, sk, x, S, ovf);
  if (!valid) return;
  if (payoffs) payoffs[p] = __fmul_rn(payoff<D>(I, x), I.discount);
  if (steps) steps[p] = own;
  if (ovf || dr.overflow) atomicOr(status, SDEMC_EOVERFLOW);
}

}  // namespace sdemc

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
  const unsigned blocks = (unsigned)((I.num_paths + 127) / 128);
  cudaStream_t s = (cudaStream_t)stream;
  const int mi = max_iterations(&I);
  StoreParams P;
  P.I = I;
  P.rk = make_round_keys(I.seed);
  const bool nominal = (I.flags & SDEMC_INST_PAYOFF_AT_NOMINAL_STEP) != 0;
#define SDEMC_MAT_CASE(D_, N_)                                                                   \
  {                                                                                              \
    constexpr int ZD = Layout<D_, N_>::ZD;                                                       \
    if (d_z && zdim != ZD) return fail(SDEMC_EINVAL, "zdim %d != %d for this layout", zdim, ZD); \
    auto kern = nominal ? materialise_kernel<D_, N_, kModeNominal> : materialise_kernel<D_, N_, 0>; \
    kern<<<blocks, 128, 0, s>>>(P, steps_cap, d_paths, d_left, d_time, d_jumps, d_normals,      \
                                d_payoffs, d_steps, d_z, ZD, d_jt, d_jm, d_jsel, jcap, d_status, mi); \
  }
  SDEMC_DISPATCH(I.dim, I.noise, SDEMC_MAT_CASE)
#undef SDEMC_MAT_CASE
  return check_cuda(cudaGetLastError(), "materialise_kernel launch");
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
#define SDEMC_REPLAY_CASE(D_, N_)                                                        \
  replay_kernel<D_, N_><<<blocks, 128, 0, s>>>(I, bs, steps_cap, max_jumps, d_jump_times, \
                                               d_dw, d_marks, d_asset, d_paths, d_left,   \
                                               d_time, d_jumps, d_payoffs, d_steps, d_status);
  SDEMC_DISPATCH(I.dim, I.noise, SDEMC_REPLAY_CASE)
#undef SDEMC_REPLAY_CASE
  return check_cuda(cudaGetLastError(), "replay_kernel launch");
}
