// k_mlmc.cu — K2: one multilevel Monte Carlo level in one launch.
//
// JumpDiffusionSolver.multilevel_solve (sde_mc/solvers.py:228-307) couples a
// fine path (h_f) and a coarse path (h_c = factor * h_f) through one jump
// clock: each coarse step is `factor` fine sub-steps whose increments it sums,
// both levels get the same mark, and after a jump the remaining fine sub-steps
// have dt = 0.  Here the fine and coarse states of a path live in the same
// thread, the sub-step increments are drawn once, and the level's
// sum/sum-of-squares of Y = disc*(P_f - P_c) (sde_mc/mlmc.py:59-69) are reduced
// as in K1.  The replay twin runs the same loop on recorded draws.
#include "sdemc_device.cuh"
#include "sdemc_host.cuh"

namespace sdemc {

// What the coupled loop records besides the terminal states.  NullPairSink:
// nothing (the estimators).  ColumnPairSink: every column multilevel_solve
// returns — on the jump-adapted grid the fine and coarse states after each
// coarse step (sde_mc/solvers.py:298-305), frozen after the path ends as the
// reference's batch loop leaves them; on the uniform grid every fine state,
// every coarse state and the fine increments (sde_mc/solvers.py:104-119).
struct NullPairSink {
  SDEMC_DI void init(const float*) {}
  SDEMC_DI void fine(int, const float*, const float*, const float*) {}
  SDEMC_DI void coarse(int, const float*, const float*) {}
  SDEMC_DI void finish(int, const float*, const float*) {}
};

template <int D, int NW>
struct ColumnPairSink {
  float* pf;   // (capf, D) fine columns of this path
  float* pc;   // (capc, D) coarse columns
  float* nz;   // uniform grid: (fine steps, D * NW) increments, or null
  int capf, capc, nfine;
  bool uniform, over;

  SDEMC_DI void put(float* base, int cap, int col, const float* x) {
    if (col >= cap) { over = true; return; }
#pragma unroll
    for (int i = 0; i < D; ++i) base[(size_t)col * D + i] = x[i];
  }
  SDEMC_DI void init(const float* x0) {
    put(pf, capf, 0, x0);
    put(pc, capc, 0, x0);
  }
  SDEMC_DI void fine(int kf, const float* xf, const float* dW, const float* dW2) {
    put(pf, capf, kf + 1, xf);
    if (nz && kf < nfine) {
#pragma unroll
      for (int i = 0; i < D; ++i) {
        if (NW == 1) {
          nz[(size_t)kf * D + i] = dW[i];
        } else {
          nz[(size_t)kf * D * 2 + 2 * i] = dW[i];
          nz[(size_t)kf * D * 2 + 2 * i + 1] = dW2[i];
        }
      }
    }
  }
  SDEMC_DI void coarse(int kc, const float* xf, const float* xc) {
    if (!uniform) put(pf, capf, kc + 1, xf);
    put(pc, capc, kc + 1, xc);
  }
  // jump-adapted grid: columns after the warp's last step hold the final states
  SDEMC_DI void finish(int kc, const float* xf, const float* xc) {
    if (uniform) return;
    for (int c = kc + 1; c < capc; ++c) put(pc, capc, c, xc);
    for (int c = kc + 1; c < capf; ++c) put(pf, capf, c, xf);
  }
};

// Returns the path's own coarse steps (those that started before T).
template <int D, int NOISE, bool EXACT, class Draws, class Sink>
SDEMC_DI int simulate_pair(const sdemc_inst& I, Draws& dr, int factor, float hf0, float hc0,
                           float* xf, float* xc, int max_iters, bool& overflow, Sink& sk) {
  using L = Layout<D, NOISE>;
#pragma unroll
  for (int i = 0; i < D; ++i) { xf[i] = I.x0[i]; xc[i] = I.x0[i]; }
  const float T = I.T;
  float tf = 0.f, tc = 0.f, hf = hf0, hc = hc0;
  float dW[D], dW2[D], z[L::ZD], sW[D], sW2[D], oldf[D], oldc[D];
#pragma unroll
  for (int i = 0; i < D; ++i) { dW2[i] = 0.f; oldf[i] = xf[i]; }
  sk.init(xf);
  int kf = 0, kc = 0, own = 0;
  if (I.grid == SDEMC_GRID_UNIFORM) {
    // DiffusionSolver.multilevel_solve (sde_mc/solvers.py:90-119): `coarse`
    // blocks of `factor` fine steps of h_f, then one coarse step of h_c driven
    // by the summed increments; no time checks.
    const int coarse = I.num_steps;
    for (kc = 0; kc < coarse; ++kc) {
#pragma unroll
      for (int i = 0; i < D; ++i) { sW[i] = 0.f; sW2[i] = 0.f; }
      for (int sub = 0; sub < factor; ++sub) {
        dr.increments(I, kf, hf, dW, dW2, z);
        euler<D, NOISE, EXACT>(I, xf, hf, dW, dW2);
#pragma unroll
        for (int i = 0; i < D; ++i) { sW[i] = __fadd_rn(sW[i], dW[i]); sW2[i] = __fadd_rn(sW2[i], dW2[i]); }
        sk.fine(kf, xf, dW, dW2);
        ++kf;
      }
      euler<D, NOISE, EXACT>(I, xc, hc, sW, sW2);
      sk.coarse(kc, xf, xc);
    }
    return coarse;
  }
  float nj = dr.jump_first(I);
  bool act = tf < T;
  while (__any_sync(kFull, act)) {
    if (kc >= max_iters) { overflow = true; break; }
#pragma unroll
    for (int i = 0; i < D; ++i) { sW[i] = 0.f; sW2[i] = 0.f; }
    for (int sub = 0; sub < factor; ++sub) {
      hf = fminf(hf, fmaxf(__fsub_rn(T, tf), 0.f));
      float dtf = fminf(hf, __fsub_rn(nj, tf));
      if (!act) dtf = 0.f;
      dr.increments(I, kf, dtf, dW, dW2, z);
#pragma unroll
      for (int i = 0; i < D; ++i) oldf[i] = xf[i];
      euler<D, NOISE, EXACT>(I, xf, dtf, dW, dW2);
      tf = __fadd_rn(tf, dtf);
#pragma unroll
      for (int i = 0; i < D; ++i) { sW[i] = __fadd_rn(sW[i], dW[i]); sW2[i] = __fadd_rn(sW2[i], dW2[i]); }
      ++kf;
    }
    hc = fminf(hc, fmaxf(__fsub_rn(T, tc), 0.f));
    float dtc = fminf(hc, __fsub_rn(nj, tc));
    if (!act) dtc = 0.f;
#pragma unroll
    for (int i = 0; i < D; ++i) oldc[i] = xc[i];
    euler<D, NOISE, EXACT>(I, xc, dtc, sW, sW2);
    tc = __fadd_rn(tc, dtc);
    if (act && jump_due(nj, tf)) {
      float J;
      int sel;
      nj = dr.on_fire(I, kc, nj, J, sel);
      apply_jump<D, EXACT>(I, xf, I.exact_jumps ? xf : oldf, J, sel);
      apply_jump<D, EXACT>(I, xc, I.exact_jumps ? xc : oldc, J, sel);
    }
    sk.coarse(kc, xf, xc);
    own += act ? 1 : 0;
    ++kc;
    act = tf < T;
    dr.after_step(I, kc, nj, act);
  }
  sk.finish(kc - 1, xf, xc);
  return own;
}

// Optional column outputs of a coupled run (all null: terminal states only).
struct PairCols {
  float *pf, *pc, *nz;
  int32_t* steps;
  int capf, capc, nfine;
};

template <int D, int NOISE>
SDEMC_DI ColumnPairSink<D, Layout<D, NOISE>::NW> column_sink(const PairCols& C, int64_t p, bool valid, bool uniform) {
  ColumnPairSink<D, Layout<D, NOISE>::NW> sk;
  sk.pf = valid ? C.pf + (size_t)p * C.capf * D : nullptr;
  sk.pc = valid ? C.pc + (size_t)p * C.capc * D : nullptr;
  sk.nz = (valid && C.nz) ? C.nz + (size_t)p * C.nfine * D * Layout<D, NOISE>::NW : nullptr;
  sk.capf = valid ? C.capf : 0;  // an invalid lane stores nothing (every put is out of its range)
  sk.capc = valid ? C.capc : 0;
  sk.nfine = C.nfine;
  sk.uniform = uniform;
  sk.over = false;
  return sk;
}

struct LevelParams {
  sdemc_inst I;
  RoundKeys rk;
};

template <int D, int NOISE>
__global__ void __launch_bounds__(128)
mlmc_kernel(const __grid_constant__ LevelParams P, int factor, float hf, float hc,
            double* __restrict__ part, float* __restrict__ yout, int32_t* __restrict__ status,
            int64_t nchunks, int max_iters) {
  const sdemc_inst& I = P.I;
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  bool ovf = false;
  for (int64_t c = warp; c < nchunks; c += nwarps) {
    const int64_t p = c * kChunk + lane;
    NativeDraws<D, NOISE> dr;
    dr.init(I, (uint64_t)p, ConstKeys{&P.rk});
    float xf[D], xc[D];
    NullPairSink sk;
    simulate_pair<D, NOISE, false>(I, dr, factor, hf, hc, xf, xc, max_iters, ovf, sk);
    const bool valid = p < I.num_paths;
    const float pf = payoff<D>(I, xf), pc = payoff<D>(I, xc);
    const float Y = valid ? __fmul_rn(I.discount, __fsub_rn(pf, pc)) : 0.f;
    const float F = valid ? __fmul_rn(pf, I.discount) : 0.f;
    if (valid && yout) yout[p] = Y;
    const float s = warp_sum(Y), s2 = warp_sum(__fmul_rn(Y, Y));
    const float f = warp_sum(F), f2 = warp_sum(__fmul_rn(F, F));
    const int n = __popc(__ballot_sync(kFull, valid));
    if (lane == 0) {
      double* o = part + c * 5;
      o[0] = (double)s; o[1] = (double)s2; o[2] = (double)n; o[3] = (double)f; o[4] = (double)f2;
    }
  }
  if (ovf) atomicOr(status, SDEMC_EOVERFLOW);
}

template <int D, int NOISE, bool COLS>
__global__ void __launch_bounds__(128)
mlmc_replay_kernel(const __grid_constant__ sdemc_inst I, int factor, float hf, float hc, int bs,
                   int Sf, int Sc, int MJ, const float* jt, const float* dw, const float* marks,
                   const int32_t* asset, float* xf_out, float* xc_out, int32_t* status, PairCols C) {
  using L = Layout<D, NOISE>;
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  const bool valid = p < bs;
  ReplayDraws<D, NOISE> dr{};
  if (valid) {
    dr.dw = dw + (size_t)p * Sf * D * L::NW;
    dr.marks = marks ? marks + (size_t)p * Sc : nullptr;
    dr.asset = asset ? asset + (size_t)p * Sc : nullptr;
    dr.jt = jt ? jt + (size_t)p * MJ : nullptr;
    dr.S = Sf;
    dr.MJ = jt ? MJ : 0;
  }
  bool ovf = false;
  float xf[D], xc[D];
  int own;
  bool over = false;
  if (COLS) {
    auto sk = column_sink<D, NOISE>(C, p, valid, I.grid == SDEMC_GRID_UNIFORM);
    own = simulate_pair<D, NOISE, true>(I, dr, factor, hf, hc, xf, xc, Sc, ovf, sk);
    over = sk.over;
  } else {
    NullPairSink sk;
    own = simulate_pair<D, NOISE, true>(I, dr, factor, hf, hc, xf, xc, Sc, ovf, sk);
  }
  if (!valid) return;
#pragma unroll
  for (int i = 0; i < D; ++i) { xf_out[(size_t)p * D + i] = xf[i]; xc_out[(size_t)p * D + i] = xc[i]; }
  if (COLS && C.steps) C.steps[p] = own;
  if (ovf || dr.overflow || over) atomicOr(status, SDEMC_EOVERFLOW);
}

template <int D, int NOISE, bool COLS>
__global__ void __launch_bounds__(128)
mlmc_terminals_kernel(const __grid_constant__ LevelParams P, int factor, float hf, float hc,
                      float* xf_out, float* xc_out, int32_t* status, int max_iters, PairCols C) {
  const sdemc_inst& I = P.I;
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const bool valid = p < I.num_paths;
  NativeDraws<D, NOISE> dr;
  dr.init(I, (uint64_t)p, ConstKeys{&P.rk});
  bool ovf = false, over = false;
  float xf[D], xc[D];
  int own;
  if (COLS) {
    auto sk = column_sink<D, NOISE>(C, p, valid, I.grid == SDEMC_GRID_UNIFORM);
    own = simulate_pair<D, NOISE, false>(I, dr, factor, hf, hc, xf, xc, max_iters, ovf, sk);
    over = sk.over;
  } else {
    NullPairSink sk;
    own = simulate_pair<D, NOISE, false>(I, dr, factor, hf, hc, xf, xc, max_iters, ovf, sk);
  }
  if (!valid) return;
  if (xf_out) {
#pragma unroll
    for (int i = 0; i < D; ++i) { xf_out[p * D + i] = xf[i]; xc_out[p * D + i] = xc[i]; }
  }
  if (COLS && C.steps) C.steps[p] = own;
  if (ovf || over) atomicOr(status, SDEMC_EOVERFLOW);
}

static int check_levels(const sdemc_inst* I, int fine, int coarse, float hf, float hc) {
  if (fine < 1 || coarse < 1 || fine % coarse != 0)
    return fail(SDEMC_EINVAL, "levels (%d, %d): fine must be a multiple of coarse", fine, coarse);
  if (!(hf > 0.f) || !(hc > 0.f)) return fail(SDEMC_EINVAL, "non-positive level steps");
  if (I->grid == SDEMC_GRID_ADAPTED && I->noise == SDEMC_NOISE_INDEP_PAIR)
    return fail(SDEMC_EUNSUPPORTED, "paired noise on the adapted grid");
  return SDEMC_OK;
}

}  // namespace sdemc

using namespace sdemc;

extern "C" size_t sdemc_mlmc_scratch_bytes(const sdemc_inst* h_inst) {
  if (!h_inst) return 0;
  return scratch_bytes_for(num_chunks(h_inst), 5);
}

extern "C" int sdemc_mlmc_level(const sdemc_inst* h_inst, int fine, int coarse, float h_fine,
                                float h_coarse, const sdemc_cfg* h_cfg, void* d_scratch,
                                size_t scratch_bytes, double* d_out, float* d_y, void* stream) {
  int rc = validate_inst(h_inst);
  if (rc) return rc;
  if ((rc = check_levels(h_inst, fine, coarse, h_fine, h_coarse))) return rc;
  if (!d_scratch || !d_out) return fail(SDEMC_EINVAL, "null scratch or output");
  if (scratch_bytes < sdemc_mlmc_scratch_bytes(h_inst))
    return fail(SDEMC_ENOMEM, "scratch %zu bytes < required %zu", scratch_bytes,
                sdemc_mlmc_scratch_bytes(h_inst));
  sdemc_cfg cfg{};
  if (h_cfg) cfg = *h_cfg;
  sdemc_inst I = *h_inst;
  I.num_steps = coarse;  // iteration cap counts coarse steps
  cudaStream_t s = (cudaStream_t)stream;
  int32_t* status = scratch_status(d_scratch);
  double* part = scratch_chunks(d_scratch);
  const int64_t nch = num_chunks(h_inst);
  const int factor = fine / coarse;
  const int mi = max_iterations(&I);
  LevelParams P;
  P.I = I;
  P.rk = make_round_keys(I.seed);
  if (nch > 0) {
    const int threads = cfg.block_threads > 0 ? cfg.block_threads : 128;
#define SDEMC_MLMC_CASE(D_, N_)                                                                  \
  {                                                                                              \
    auto kern = mlmc_kernel<D_, N_>;                                                             \
    int per_sm = 0;                                                                              \
    if ((rc = check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, 0), \
                         "occupancy query")))                                                    \
      return rc;                                                                                 \
    if (cfg.ctas_per_sm > 0 && cfg.ctas_per_sm < per_sm) per_sm = cfg.ctas_per_sm;               \
    if (per_sm < 1) per_sm = 1;                                                                  \
    int64_t ctas = (nch + threads / 32 - 1) / (threads / 32);                                    \
    const int64_t resident = (int64_t)num_sms() * per_sm;                                        \
    if (ctas > resident) ctas = resident;                                                        \
    kern<<<(unsigned)ctas, threads, 0, s>>>(P, factor, h_fine, h_coarse, part, d_y, status, nch, mi); \
  }
    SDEMC_DISPATCH(I.dim, I.noise, SDEMC_MLMC_CASE)
#undef SDEMC_MLMC_CASE
    if ((rc = check_cuda(cudaGetLastError(), "mlmc_kernel launch"))) return rc;
  }
  return launch_reduce(d_scratch, nch, 5, d_out, s);
}

extern "C" int sdemc_mlmc_replay(const sdemc_inst* h_inst, int fine, int coarse, float h_fine,
                                 float h_coarse, int bs, int fine_cap, int coarse_cap,
                                 int max_jumps, const float* d_jump_times, const float* d_dw,
                                 const float* d_marks, const int32_t* d_asset, float* d_xf,
                                 float* d_xc, int32_t* d_status, void* stream) {
  int rc = validate_inst(h_inst);
  if (rc) return rc;
  if ((rc = check_levels(h_inst, fine, coarse, h_fine, h_coarse))) return rc;
  if (bs < 0 || fine_cap < 1 || coarse_cap < 1) return fail(SDEMC_EINVAL, "bad replay shape");
  if (!d_dw || !d_xf || !d_xc || !d_status) return fail(SDEMC_EINVAL, "null replay buffer");
  if (h_inst->rate > 0.f && (!d_jump_times || !d_marks || max_jumps < 1))
    return fail(SDEMC_EINVAL, "jump replay needs jump times and marks");
  if (bs == 0) return SDEMC_OK;
  sdemc_inst I = *h_inst;
  I.num_steps = coarse;
  cudaStream_t s = (cudaStream_t)stream;
  const unsigned blocks = (unsigned)((bs + 127) / 128);
  const int factor = fine / coarse;
  const PairCols C{};
#define SDEMC_MLMC_REPLAY_CASE(D_, N_)                                                               \
  mlmc_replay_kernel<D_, N_, false><<<blocks, 128, 0, s>>>(I, factor, h_fine, h_coarse, bs, fine_cap, \
                                                           coarse_cap, max_jumps, d_jump_times, d_dw, \
                                                           d_marks, d_asset, d_xf, d_xc, d_status, C);
  SDEMC_DISPATCH(I.dim, I.noise, SDEMC_MLMC_REPLAY_CASE)
#undef SDEMC_MLMC_REPLAY_CASE
  return check_cuda(cudaGetLastError(), "mlmc_replay_kernel launch");
}

extern "C" int sdemc_mlmc_terminals(const sdemc_inst* h_inst, int fine, int coarse, float h_fine,
                                    float h_coarse, float* d_xf, float* d_xc, int32_t* d_status,
                                    void* stream) {
  int rc = validate_inst(h_inst);
  if (rc) return rc;
  if ((rc = check_levels(h_inst, fine, coarse, h_fine, h_coarse))) return rc;
  if (!d_xf || !d_xc || !d_status) return fail(SDEMC_EINVAL, "null output");
  if (h_inst->num_paths == 0) return SDEMC_OK;
  sdemc_inst I = *h_inst;
  I.num_steps = coarse;
  cudaStream_t s = (cudaStream_t)stream;
  const unsigned blocks = (unsigned)((I.num_paths + 127) / 128);
  const int factor = fine / coarse;
  const int mi = max_iterations(&I);
  LevelParams P;
  P.I = I;
  P.rk = make_round_keys(I.seed);
  const PairCols C{};
#define SDEMC_MLMC_TERM_CASE(D_, N_)                                                      \
  mlmc_terminals_kernel<D_, N_, false><<<blocks, 128, 0, s>>>(P, factor, h_fine, h_coarse, \
                                                              d_xf, d_xc, d_status, mi, C);
  SDEMC_DISPATCH(I.dim, I.noise, SDEMC_MLMC_TERM_CASE)
#undef SDEMC_MLMC_TERM_CASE
  return check_cuda(cudaGetLastError(), "mlmc_terminals_kernel launch");
}

// Column shapes of multilevel_solve: on the jump-adapted grid both levels
// hold cols columns (coarse steps + 1); on the uniform grid fine + 1 and
// coarse + 1.
static int check_cols(const sdemc_inst& I, int fine, int coarse, int cols_fine, int cols_coarse) {
  if (I.grid == SDEMC_GRID_UNIFORM) {
    if (cols_fine < fine + 1 || cols_coarse < coarse + 1)
      return fail(SDEMC_EINVAL, "uniform grid: %d/%d columns, need %d/%d", cols_fine, cols_coarse, fine + 1,
                  coarse + 1);
  } else if (cols_fine < 2 || cols_fine != cols_coarse) {
    return fail(SDEMC_EINVAL, "jump-adapted grid: fine and coarse column counts %d/%d must be equal and >= 2",
                cols_fine, cols_coarse);
  }
  return SDEMC_OK;
}

extern "C" int sdemc_mlmc_paths(const sdemc_inst* h_inst, int fine, int coarse, float h_fine, float h_coarse,
                                int cols_fine, int cols_coarse, float* d_paths_fine, float* d_paths_coarse,
                                float* d_normals, int32_t* d_steps, int32_t* d_status, void* stream) {
  int rc = validate_inst(h_inst);
  if (rc) return rc;
  if ((rc = check_levels(h_inst, fine, coarse, h_fine, h_coarse))) return rc;
  if (!d_paths_fine || !d_paths_coarse || !d_status) return fail(SDEMC_EINVAL, "null column output");
  if ((rc = check_cols(*h_inst, fine, coarse, cols_fine, cols_coarse))) return rc;
  if (h_inst->num_paths == 0) return SDEMC_OK;
  sdemc_inst I = *h_inst;
  I.num_steps = coarse;
  cudaStream_t s = (cudaStream_t)stream;
  const unsigned blocks = (unsigned)((I.num_paths + 127) / 128);
  const int factor = fine / coarse;
  const int mi = max_iterations(&I);
  LevelParams P;
  P.I = I;
  P.rk = make_round_keys(I.seed);
  const PairCols C{d_paths_fine, d_paths_coarse, I.grid == SDEMC_GRID_UNIFORM ? d_normals : nullptr, d_steps,
                   cols_fine, cols_coarse, fine};
#define SDEMC_MLMC_PATHS_CASE(D_, N_)                                                   \
  mlmc_terminals_kernel<D_, N_, true><<<blocks, 128, 0, s>>>(P, factor, h_fine, h_coarse, \
                                                             nullptr, nullptr, d_status, mi, C);
  SDEMC_DISPATCH(I.dim, I.noise, SDEMC_MLMC_PATHS_CASE)
#undef SDEMC_MLMC_PATHS_CASE
  return check_cuda(cudaGetLastError(), "mlmc_terminals_kernel launch");
}

extern "C" int sdemc_mlmc_replay_paths(const sdemc_inst* h_inst, int fine, int coarse, float h_fine,
                                       float h_coarse, int bs, int fine_cap, int coarse_cap, int max_jumps,
                                       const float* d_jump_times, const float* d_dw, const float* d_marks,
                                       const int32_t* d_asset, int cols_fine, int cols_coarse,
                                       float* d_paths_fine, float* d_paths_coarse, float* d_xf, float* d_xc,
                                       int32_t* d_steps, int32_t* d_status, void* stream) {
  int rc = validate_inst(h_inst);
  if (rc) return rc;
  if ((rc = check_levels(h_inst, fine, coarse, h_fine, h_coarse))) return rc;
  if (bs < 0 || fine_cap < 1 || coarse_cap < 1) return fail(SDEMC_EINVAL, "bad replay shape");
  if (!d_dw || !d_xf || !d_xc || !d_status || !d_paths_fine || !d_paths_coarse)
    return fail(SDEMC_EINVAL, "null replay buffer");
  if ((rc = check_cols(*h_inst, fine, coarse, cols_fine, cols_coarse))) return rc;
  if (h_inst->rate > 0.f && (!d_jump_times || !d_marks || max_jumps < 1))
    return fail(SDEMC_EINVAL, "jump replay needs jump times and marks");
  if (bs == 0) return SDEMC_OK;
  sdemc_inst I = *h_inst;
  I.num_steps = coarse;
  cudaStream_t s = (cudaStream_t)stream;
  const unsigned blocks = (unsigned)((bs + 127) / 128);
  const int factor = fine / coarse;
  const PairCols C{d_paths_fine, d_paths_coarse, nullptr, d_steps, cols_fine, cols_coarse, fine};
#define SDEMC_MLMC_REPLAY_PATHS_CASE(D_, N_)                                                        \
  mlmc_replay_kernel<D_, N_, true><<<blocks, 128, 0, s>>>(I, factor, h_fine, h_coarse, bs, fine_cap, \
                                                          coarse_cap, max_jumps, d_jump_times, d_dw, \
                                                          d_marks, d_asset, d_xf, d_xc, d_status, C);
  SDEMC_DISPATCH(I.dim, I.noise, SDEMC_MLMC_REPLAY_PATHS_CASE)
#undef SDEMC_MLMC_REPLAY_PATHS_CASE
  return check_cuda(cudaGetLastError(), "mlmc_replay_kernel launch");
}
