/*
 * sdemc.h — C ABI of the GB300 (sm_103a) Monte Carlo path-integration library.
 *
 * Everything here is plain C: POD descriptors, raw pointers, sizes and a
 * cudaStream_t passed as void*.  No torch types cross this boundary.  All
 * array arguments named d_* are caller-owned DEVICE memory; h_* are host
 * memory.  The library never allocates per call.  Every entry point returns an
 * int status (SDEMC_OK == 0); sdemc_last_error() gives the message of the last
 * failure on the calling thread.
 *
 * The reference (piers-hinds/sde_mc, pure Python on PyTorch) has no native
 * code; each entry point below replaces a torch op chain of the reference and
 * cites the Python it stands in for (path:line inside the sde_mc project).
 */
#ifndef SDEMC_H
#define SDEMC_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SDEMC_ABI_VERSION 1
#define SDEMC_MAX_DIM 8
#define SDEMC_CHOL_LEN 36       /* packed lower triangle of an 8x8 matrix */
#define SDEMC_MARK_PARAMS 12
#define SDEMC_CHUNK_PATHS 32    /* paths per reduction slot: one warp round */

/* ---- status codes ---------------------------------------------------- */
enum {
  SDEMC_OK = 0,
  SDEMC_EINVAL = 1,        /* bad argument (shape, size, null pointer)          */
  SDEMC_EUNSUPPORTED = 2,  /* model/payoff/dim combination not implemented      */
  SDEMC_ENOMEM = 3,        /* caller buffer too small / admission over budget   */
  SDEMC_ETIMEOUT = 4,      /* a bounded device wait gave up (tensor-core
                              kernels): the kernel stopped and freed its tensor
                              memory while its last product may still have been
                              writing it, so every output of that launch, and of
                              any other tensor-core launch that ran on the device
                              at the same time, is void and must be discarded  */
  SDEMC_ECUDA = 5,         /* CUDA runtime error                                */
  SDEMC_EOVERFLOW = 6      /* a path needed more steps/jumps than storage holds */
};

/* ---- descriptor enums ------------------------------------------------- */
/* noise layout (Sde.diffusion_struct, sde_mc/sde.py:20-32)                  */
enum {
  SDEMC_NOISE_DIAG = 0,          /* dW = L z sqrt(dt)                          */
  SDEMC_NOISE_INDEP_SHARED = 1,  /* jump solver 'indep': [L z, z'] with one
                                    shared uncorrelated scalar z'
                                    (sde_mc/solvers.py:197-201)               */
  SDEMC_NOISE_INDEP_PAIR = 2     /* diffusion solver 'indep': two correlated
                                    BMs L z1, L z2 (sde_mc/solvers.py:79-81)  */
};
/* time grid (which solver family)                                          */
enum {
  SDEMC_GRID_ADAPTED = 0,  /* JumpDiffusionSolver.solve, sde_mc/solvers.py:164-226 */
  SDEMC_GRID_UNIFORM = 1   /* DiffusionSolver.solve,     sde_mc/solvers.py:68-88   */
};
/* jump mark law                                                            */
enum {
  SDEMC_MARK_NONE = 0,
  SDEMC_MARK_LOGNORMAL = 1,  /* exp(N(alpha, gamma)) - 1, sde_mc/sde.py:325-326 */
  SDEMC_MARK_INVCDF = 2      /* InverseCdf of a truncated Levy measure,
                                sde_mc/levy.py:10-30, 85-87                    */
};
/* which components a jump event moves                                      */
enum {
  SDEMC_JUMP_COMMON = 0,     /* one scalar mark repeated over all dims
                                (sde_mc/solvers.py:146-148)                   */
  SDEMC_JUMP_ONE_ASSET = 1   /* superposition of independent per-asset
                                compound Poisson processes: each event picks
                                asset k with probability rate_k / sum(rate)   */
};
/* payoffs (sde_mc/options.py:179-321)                                      */
enum {
  SDEMC_PAYOFF_EUROCALL = 0,
  SDEMC_PAYOFF_EUROPUT = 1,
  SDEMC_PAYOFF_BINARY_AON = 2,
  SDEMC_PAYOFF_BASKET_ARITH = 3,
  SDEMC_PAYOFF_BASKET_GEO = 4,
  SDEMC_PAYOFF_RAINBOW = 5,
  SDEMC_PAYOFF_DIGITAL = 6,
  SDEMC_PAYOFF_BESTOF = 7,
  SDEMC_PAYOFF_ASIANCALL = 8,
  SDEMC_PAYOFF_HESTON_RAINBOW = 9
};

/*
 * One pricing instance: an affine-in-state SDE, its jump law, its time grid,
 * the payoff and the RNG stream.  Component i of the state moves by
 *
 *   dx_i = (a_i + b_i x_i) dt + (s_i + q_i x_i) dW_i
 *          [+ (s2_i + q2_i x_i) dW2_i]           (INDEP layouts)
 *          + (g_i + k_i x_i^-) J                  (at a jump)
 *
 * which covers Gbm, LogGbm, DoubleGbm, Merton (sde_mc/sde.py:179-375) and the
 * LevySde adapters (sde_mc/levy.py:65-192).  Scalars are float32 exactly as
 * the reference evaluates them (the host lowering computes them with the
 * reference's own float32 expressions).
 */
typedef struct sdemc_inst {
  int32_t dim;          /* 1..SDEMC_MAX_DIM                                 */
  int32_t noise;        /* SDEMC_NOISE_*                                    */
  int32_t grid;         /* SDEMC_GRID_*                                     */
  int32_t num_steps;    /* nominal steps; h = fl32(T / num_steps)           */
  int32_t mark;         /* SDEMC_MARK_*                                     */
  int32_t jump_target;  /* SDEMC_JUMP_*                                     */
  int32_t exact_jumps;  /* 0: jump scaled by the pre-step state (reference
                           default), 1: by the post-diffusion state         */
  int32_t payoff;       /* SDEMC_PAYOFF_*                                   */
  int32_t payoff_log;   /* Option.log: exp() the state before the payoff    */
  int32_t flags;        /* SDEMC_INST_* bits                                */
  uint32_t stream_id;   /* RNG substream (MLMC level, request id ...)       */
  uint32_t model;       /* SDEMC_MODEL_*                                    */
  uint64_t seed;        /* RNG key                                          */
  uint64_t path_offset; /* global index of this instance's first path      */
  int64_t num_paths;
  float T;              /* time_interval, float32                           */
  float h;              /* fl32(T / num_steps)                              */
  float rate;           /* total jump intensity sum(jump_rate()), 0 = none  */
  float inv_rate;       /* fl32(1 / rate)                                   */
  float strike;
  float payoff_scale;   /* Option.discount                                  */
  float discount;       /* discounter(T) as float32                         */
  float disc_rate;      /* ConstantShortRate.r (for per-step discounting)   */
  int32_t reserved0[2]; /* zero; the arrays below start on 16-byte boundaries,
                           so kernels that stage the descriptor in shared
                           memory read them with vector loads             */
  float x0[SDEMC_MAX_DIM];
  float drift_a[SDEMC_MAX_DIM], drift_b[SDEMC_MAX_DIM];
  float diff_s[SDEMC_MAX_DIM], diff_q[SDEMC_MAX_DIM];
  float diff2_s[SDEMC_MAX_DIM], diff2_q[SDEMC_MAX_DIM];
  float jump_g[SDEMC_MAX_DIM], jump_k[SDEMC_MAX_DIM];
  float jump_cdf[SDEMC_MAX_DIM];  /* ONE_ASSET: cumulative pick probabilities */
  float chol[SDEMC_CHOL_LEN];     /* Cholesky factor of corr, packed rows     */
  float mark_p[SDEMC_MARK_PARAMS];/* LOGNORMAL: alpha, gamma.
                                     INVCDF: cm, cp, mu, alpha, eps, lda,
                                     y1, y2, y3, uniform_shift.
                                     MODEL_HESTON (no marks): kappa,
                                     kappa*theta, xi, xi^2                  */
} sdemc_inst;

/* sdemc_inst.model: how the Euler step reads the coefficients.
   AFFINE: x_i += (a_i + b_i x_i) dt + (s_i + q_i x_i) dW_i (+ second
           Brownian for the 'indep' pairs), every Sde class of sde_mc/sde.py
           except the two below.
   HESTON: dim 2 (price, variance), HestonScheme.step (sde_mc/schemes.py:16-22,
           sde_mc/sde.py:258-279): the price takes an Euler step with drift
           r S (r = drift_b[0]) and diffusion sqrt(v) S; sqrt of the new
           variance is the larger root of a v'^2 + b v' + c = 0 with
           a = -1 - kappa h, b = xi dW_1, c = v + kappa theta h - h xi^2 / 2.
   ASIAN:  dim 2, AsianWrapper (sde_mc/sde.py:378-406) around a 1-D affine
           model in component 0; component 1 integrates it: y += x_0 dt. */
enum {
  SDEMC_MODEL_AFFINE = 0,
  SDEMC_MODEL_HESTON = 1,
  SDEMC_MODEL_ASIAN = 2
};

/* Launch tuning; all-zero means "choose for me". */
typedef struct sdemc_cfg {
  int32_t block_threads;   /* threads per CTA (multiple of 32), 0 = auto    */
  int32_t ctas_per_sm;     /* persistent grid = SMs x this, 0 = auto        */
  int32_t interleave;      /* paths a lane steps together: 1 or 2 (0 = 1)   */
  int32_t flags;           /* SDEMC_CFG_*                                   */
  int64_t timeout_ns;      /* bound for device-side waits, 0 = default      */
} sdemc_cfg;

enum { SDEMC_CFG_EXACT_EULER = 1 }; /* use the reference's unfused op order */

/* sdemc_inst.flags */
enum {
  /* Evaluate the payoff on the state after num_steps steps instead of the
     terminal state: what mc_simple(payoff_time='terminal') reads from a jump
     solver's storage (paths[:, num_steps], sde_mc/mc.py:84-86, 92).        */
  SDEMC_INST_PAYOFF_AT_NOMINAL_STEP = 1
};

/* ---- library / device info ------------------------------------------ */
int sdemc_abi_version(void);
size_t sdemc_inst_size(void);
/* offsetof() of every sdemc_inst field in declaration order (count in *n). */
int sdemc_inst_offsets(size_t* h_offsets, int* n);
int sdemc_last_error(char* h_buf, size_t len);
int sdemc_device_sms(int* h_sms);
/* FP32 FMA throughput probe (no reference counterpart): launches 8 CTAs of
 * 256 threads per SM running 8 independent FMA chains for `iters` x 4 steps;
 * *h_flops receives the flops of the launch (time it with events on the
 * stream).  d_sink (sink_len floats) only keeps the chains live.           */
int sdemc_fp32_probe(int iters, float* d_sink, int sink_len, double* h_flops,
                     void* stream);
/* Special-function-unit (MUFU) throughput probe, same launch shape: 8
 * independent rsqrt.approx chains per thread; *h_ops receives the MUFU
 * operations of the launch.                                                */
int sdemc_mufu_probe(int iters, float* d_sink, int sink_len, double* h_ops,
                     void* stream);
/* The give-up path of the tensor-core kernels' bounded mbarrier waits: one
 * warp waits, through the same wait, on a barrier that nothing arrives at and
 * gives up after `spins` polls (1 .. 2^22), OR-ing SDEMC_ETIMEOUT into
 * *d_status; the context stays usable.  For tests of the failure path.     */
int sdemc_wait_probe(int spins, int32_t* d_status, void* stream);

/* ---- K1: fused pricing ------------------------------------------------
 * Replaces mc_simple (sde_mc/mc.py:53-123) over JumpDiffusionSolver.solve
 * (sde_mc/solvers.py:164-226) / DiffusionSolver.solve (:68-88), payoff
 * (sde_mc/options.py:175-176) and mc_estimates (sde_mc/helpers.py:51-68).
 * Every path lives in registers; per-chunk (sum, sum_sq, n) go to d_scratch;
 * d_out receives (sum, sum_sq, n, mean, var, status) in FP64, status being a
 * SDEMC_* code raised on the device (e.g. SDEMC_EOVERFLOW).  d_payoffs
 * (nullable) receives each path's discounted payoff.  d_scratch must be
 * zeroed before its first use; every call leaves its status word at zero.   */
size_t sdemc_price_scratch_bytes(const sdemc_inst* h_inst);
int sdemc_price(const sdemc_inst* h_inst, const sdemc_cfg* h_cfg,
                void* d_scratch, size_t scratch_bytes, double* d_out,
                float* d_payoffs, void* stream);
/* The two halves of sdemc_price: the path kernel writing the chunk partials
 * into d_scratch, and the FP64 reduction K10 of `nchunks` partials of `width`
 * doubles (3 for prices, 5 for MLMC levels) into d_out (sums, mean, var,
 * status).  nchunks = ceil(num_paths / SDEMC_CHUNK_PATHS).                 */
int sdemc_price_chunks(const sdemc_inst* h_inst, const sdemc_cfg* h_cfg,
                       void* d_scratch, size_t scratch_bytes, float* d_payoffs,
                       void* stream);
int sdemc_reduce_chunks(void* d_scratch, int64_t nchunks, int width,
                        double* d_out, void* stream);

/* K11: the FP64 reference run.  Prices *h_inst with every path operation in
   double precision (grid, steps, jumps, transforms of the draws, payoff) from
   the same Philox words sdemc_price uses for the same paths, so the two means
   differ by the FP32 arithmetic's error alone; with more paths it is the
   FP64 oracle for payoffs without a closed form.  'diag' noise, no marks or
   lognormal marks, terminal payoff.  Scratch as sdemc_price_scratch_bytes;
   d_out receives (sum, sum_sq, n, mean, var, status).  Stands in for no
   reference function: the reference's own numbers are float32. */
int sdemc_price_f64(const sdemc_inst* h_inst, void* d_scratch, size_t scratch_bytes,
                    double* d_out, void* stream);

/* ---- pricing without allocation ----------------------------------------
 * No counterpart in the reference (which has no native code): sdemc_price for
 * callers that cannot allocate device memory — a host that owns all GPU
 * memory through its own pool, or code that must not call cudaMalloc while
 * it builds a CUDA graph.  The caller passes only d_out (6 doubles, as
 * sdemc_price) and the optional d_payoffs; the scratch is a fixed array of
 * sdemc_price_noalloc_scratch_bytes() (~6.3 MB) inside the library, held on
 * every GPU that loads the library until the process exits.  Calls with more
 * than SDEMC_NOALLOC_MAX_PATHS paths fail with SDEMC_ENOMEM.  The first call
 * on each device looks up the array's device address (cudaGetSymbolAddress)
 * with that device current, so make that first call before any stream
 * capture; the address is kept per CUDA context, and the first call after the
 * context changes (cudaDeviceReset, or another context made current on that
 * device) looks it up again, so it too belongs outside a capture.  All calls
 * share the one array: calls that overlap on the GPU
 * (different streams, or different host threads, on one device) race and
 * must be serialised by the caller.  Nothing here calls cudaMalloc/cudaFree. */
#define SDEMC_NOALLOC_MAX_PATHS (1 << 23)
size_t sdemc_price_noalloc_scratch_bytes(void);
int sdemc_price_noalloc(const sdemc_inst* h_inst, const sdemc_cfg* h_cfg,
                        double* d_out, float* d_payoffs, void* stream);

/* ---- K8: batched heterogeneous pricing --------------------------------
 * No single reference counterpart: it prices many instances (different dim,
 * steps, paths, payoffs) in one pass, each exactly as sdemc_price would
 * alone (bit-identical results), i.e. a loop of mc_simple calls
 * (sde_mc/mc.py:53-123) over run_mc requests (sde_mc/mc.py:437-440).
 *
 * sdemc_batch_plan (host only) groups the instances into classes of equal
 * (dim, noise layout, loop variant), orders each class by descending cost and
 * writes a self-contained plan blob of sdemc_batch_plan_bytes(n) bytes into
 * h_blob.  The caller copies the blob to device memory (d_blob) and calls
 * sdemc_price_batch, which launches one persistent kernel per class (warps
 * take 32-path chunks from a per-class counter) and one FP64 reduction for
 * all instances.  d_out receives n rows of (sum, sum_sq, n, mean, var,
 * status) in the caller's instance order.  d_scratch (size
 * sdemc_batch_scratch_bytes(h_blob)) must be zeroed before its first use.
 * h_cfgs (nullable) holds one launch configuration per class in class order;
 * side_streams (nullable, n_side entries) lets class kernels overlap; the
 * calls on them are joined back into `stream` before the reduction.  A class
 * whose instances share one seed gets its Philox round keys from h_blob at
 * launch as kernel arguments (a captured launch keeps them): edit path
 * offsets in place between replays, but plan again to change seeds.         */
typedef struct sdemc_batch_class {
  int32_t dim, noise, mode, count;  /* mode: bit 0 exact Euler, bit 1 nominal */
  int32_t first;                    /* first instance (plan order)            */
  int32_t reserved;
  int64_t chunk_begin, chunk_end;   /* global chunk range of the class        */
} sdemc_batch_class;

typedef struct sdemc_batch_header {
  int32_t n_inst, n_class;
  int64_t total_chunks, total_groups;
  int64_t off_classes, off_insts, off_order, off_chunk_prefix, off_group_prefix;
} sdemc_batch_header;

size_t sdemc_batch_plan_bytes(int n);
int sdemc_batch_plan(const sdemc_inst* h_insts, int n, void* h_blob, size_t blob_bytes);
size_t sdemc_batch_scratch_bytes(const void* h_blob);
int sdemc_price_batch(const void* h_blob, const void* d_blob, void* d_scratch,
                      size_t scratch_bytes, double* d_out, const sdemc_cfg* h_cfgs,
                      void* const* side_streams, int n_side, void* stream);

/* The project's launch-shape autotuner for a planned batch (the plan blob
 * already on the device): times sdemc_price_batch with CUDA events on
 * `stream` for every candidate (h_block_threads[c], h_side_counts[c] side
 * streams out of the max_side given), then tries two paths per lane class by
 * class, keeping it when the whole batch gets >1% faster.  Writes one
 * sdemc_cfg per class to h_cfgs (n_class entries), the chosen side-stream
 * count to *h_n_side, the best time (ms) to *h_ms and, when h_cand_ms is
 * not null, each candidate's time.  Synchronises the stream; d_out holds the
 * results of the last timed launch.  No reference counterpart (the
 * reference prices one problem per call).                                  */
int sdemc_batch_autotune(const void* h_blob, const void* d_blob, void* d_scratch,
                         size_t scratch_bytes, double* d_out,
                         const int32_t* h_block_threads, const int32_t* h_side_counts,
                         int n_cand, void* const* side_streams, int max_side,
                         int repeats, sdemc_cfg* h_cfgs, int* h_n_side, float* h_ms,
                         float* h_cand_ms, void* stream);

/* ---- K3: replay of recorded draws --------------------------------------
 * Runs the reference's jump-adapted loop (sde_mc/solvers.py:164-226, or its
 * uniform-grid twin :68-88) on draws exported from the reference: d_jump_times
 * (bs, max_jumps) cumulative jump times, d_dw (bs, S, dim[, 2]) the per-step
 * noise exactly as the reference fed it to the scheme, d_marks (bs, S) the
 * per-step mark, d_asset (bs, S, nullable) the picked asset for ONE_ASSET.
 * Writes the AdaptedPathData layout (sde_mc/nets.py:192-207) at S+1 columns:
 * d_paths/d_left/d_jumps (bs, S+1, dim), d_time (bs, S+1), and d_payoffs (bs).
 * d_steps (bs) receives each path's own step count.                         */
int sdemc_replay(const sdemc_inst* h_inst, int bs, int steps_cap,
                 int max_jumps, const float* d_jump_times, const float* d_dw,
                 const float* d_marks, const int32_t* d_asset, float* d_paths,
                 float* d_left, float* d_time, float* d_jumps,
                 float* d_payoffs, int32_t* d_steps, int32_t* d_status,
                 void* stream);

/* ---- K4: materialised paths -------------------------------------------
 * JumpDiffusionSolver.solve / DiffusionSolver.solve with full storage
 * (sde_mc/solvers.py:150-162, 205-222): paths/left/jumps (N, S+1, dim), time
 * (N, S+1), normals (N, S, dim[, 2]), payoffs (N), per-path step counts.
 * Optional export of the raw draws for the oracle: d_z (N, S, zdim) standard
 * normals before scaling, d_jt (N, jcap) jump times, d_jm (N, jcap) marks.
 * Every pointer may be NULL (d_jsel holds the ONE_ASSET picks).  S =
 * steps_cap; paths needing more steps set *d_status = SDEMC_EOVERFLOW.
 * Columns after a path's last step hold its frozen state (dt = 0).          */
int sdemc_materialise(const sdemc_inst* h_inst, int steps_cap, float* d_paths,
                      float* d_left, float* d_time, float* d_jumps,
                      float* d_normals, float* d_payoffs, int32_t* d_steps,
                      float* d_z, int zdim, float* d_jt, float* d_jm,
                      int32_t* d_jsel, int jcap, int32_t* d_status,
                      void* stream);

/* ---- K2: MLMC level ----------------------------------------------------
 * One level of mc_multilevel (sde_mc/mlmc.py:57-69) over the coupled
 * JumpDiffusionSolver.multilevel_solve (sde_mc/solvers.py:228-307): fine and
 * coarse paths run in the same thread from the same increments and marks.
 * d_out receives (sum Y, sum Y^2, n, sum Pf, sum Pf^2, mean, var, status)
 * with Y = disc*(payoff(fine) - payoff(coarse)) and Pf = disc*payoff(fine).
 * The uniform grid couples DiffusionSolver.multilevel_solve (:90-119).      */
size_t sdemc_mlmc_scratch_bytes(const sdemc_inst* h_inst);
int sdemc_mlmc_level(const sdemc_inst* h_inst, int fine, int coarse,
                     float h_fine, float h_coarse, const sdemc_cfg* h_cfg,
                     void* d_scratch, size_t scratch_bytes, double* d_out,
                     float* d_y, void* stream);

/* Terminal fine/coarse states of num_paths coupled paths (d_xf, d_xc:
 * (num_paths, dim)), i.e. multilevel_solve's last columns.                  */
int sdemc_mlmc_terminals(const sdemc_inst* h_inst, int fine, int coarse,
                         float h_fine, float h_coarse, float* d_xf, float* d_xc,
                         int32_t* d_status, void* stream);

/* MLMC replay on recorded draws: d_dw (bs, Sf, dim) per fine step, d_marks
 * (bs, Sc) per coarse step.  Writes terminal fine/coarse states (bs, dim).  */
int sdemc_mlmc_replay(const sdemc_inst* h_inst, int fine, int coarse,
                      float h_fine, float h_coarse, int bs, int fine_cap,
                      int coarse_cap, int max_jumps, const float* d_jump_times,
                      const float* d_dw, const float* d_marks,
                      const int32_t* d_asset, float* d_xf, float* d_xc,
                      int32_t* d_status, void* stream);

/* Every column multilevel_solve returns, for num_paths coupled paths with the
 * Philox draws of sdemc_mlmc_level.  Jump-adapted grid
 * (JumpDiffusionSolver.multilevel_solve, sde_mc/solvers.py:228-307): d_paths_fine
 * and d_paths_coarse (n, cols, dim) hold the initial state and the fine and
 * coarse states after each coarse step (cols_fine == cols_coarse = the
 * reference's storage, coarse + max_jumps + 1); a path keeps its final state in
 * the columns after its own last step, as the reference's batch loop leaves
 * it, and d_steps (n, nullable) receives its own coarse steps, so the
 * reference's total_steps_coarse is their maximum.  Uniform grid
 * (DiffusionSolver.multilevel_solve, :90-119): d_paths_fine (n, fine + 1, dim),
 * d_paths_coarse (n, coarse + 1, dim) and, nullable, the fine increments
 * d_normals (n, fine, dim[, 2]).  A path needing more columns sets
 * SDEMC_EOVERFLOW in *d_status (the reference raises IndexError).           */
int sdemc_mlmc_paths(const sdemc_inst* h_inst, int fine, int coarse, float h_fine, float h_coarse,
                     int cols_fine, int cols_coarse, float* d_paths_fine, float* d_paths_coarse,
                     float* d_normals, int32_t* d_steps, int32_t* d_status, void* stream);

/* sdemc_mlmc_replay with the columns of sdemc_mlmc_paths as well.         */
int sdemc_mlmc_replay_paths(const sdemc_inst* h_inst, int fine, int coarse, float h_fine,
                            float h_coarse, int bs, int fine_cap, int coarse_cap, int max_jumps,
                            const float* d_jump_times, const float* d_dw, const float* d_marks,
                            const int32_t* d_asset, int cols_fine, int cols_coarse,
                            float* d_paths_fine, float* d_paths_coarse, float* d_xf, float* d_xc,
                            int32_t* d_steps, int32_t* d_status, void* stream);

/* ---- K5/K6: learned control variate -------------------------------------
 * The integrand network of the adapted control variate, the reference's
 * Mlp(1+d, [64, 64, 64], d) with ReLU and no batch norm (sde_mc/nets.py:39-93),
 * for d in {1, 2}.  Parameters: one FP32 vector of sdemc_cv_nparams(d) values
 * in torch's order (W1 (64, 1+d), b1, W2, b2, W3, b3, W4 (d, 64), b4).
 * Data: the AdaptedPathData tensors of a materialised run (d_time (N, S+1),
 * d_paths (N, S+1, d), d_normals (N, S, d), discounted d_payoffs (N)); the
 * last column is dropped as sde_mc/nets.py:194-199 does.  d_index (nullable,
 * n entries) selects and orders the paths (a shuffled minibatch).
 *
 * sdemc_cv_forward: d_gamma[q] = payoff + sum_k e^{-r t_k} f(t_k, X_k) . dW_k
 * for path index[q] (apply_adapted_control_variates with g = 0,
 * sde_mc/varred.py:98-131, integrate_cv :202-214); d_fout (nullable, (N, S, d))
 * receives f.  Hidden 64x64 layers on BF16 tensor cores, FP32 accumulation.
 * sdemc_cv_backward: gradient of Var(Gamma) over the n selected paths
 * (sde_mc/varred.py:160-180) into d_grad, using d_gamma from a forward call on
 * the same selection; d_partials holds nparts x nparams floats.
 * sdemc_adam_step: one torch.optim.Adam step (no weight decay).
 * sdemc_adam_bias: its bias corrections for step t >= 1, h_bc[0] = 1 - b1^t,
 * h_bc[1] = sqrt(1 - b2^t) (host only, the arithmetic sdemc_adam_step uses).
 * sdemc_adam_step_dev: the same step with the corrections read from device
 * memory d_bc (2 floats), for CUDA graphs of many steps whose corrections
 * the host refills between replays.                                       */
int sdemc_cv_nparams(int dim);
int sdemc_cv_forward(int dim, const float* d_params, const float* d_time,
                     const float* d_paths, const float* d_normals,
                     const float* d_payoffs, const int64_t* d_index, int64_t n,
                     int steps, float disc_rate, float* d_gamma, float* d_fout,
                     void* stream);
int sdemc_cv_backward(int dim, const float* d_params, const float* d_time,
                      const float* d_paths, const float* d_normals,
                      const int64_t* d_index, int64_t n, int steps,
                      float disc_rate, const float* d_gamma, float* d_partials,
                      int nparts, float* d_grad, void* stream);
int sdemc_adam_step(float* d_params, const float* d_grad, float* d_m, float* d_v,
                    int nparam, int step, float lr, float beta1, float beta2,
                    float eps, void* stream);
int sdemc_adam_bias(int step, float beta1, float beta2, float* h_bc);
int sdemc_adam_step_dev(float* d_params, const float* d_grad, float* d_m,
                        float* d_v, int nparam, const float* d_bc, float lr,
                        float beta1, float beta2, float eps, void* stream);

/* K6 on the 5th-generation tensor cores: the gradient of sdemc_cv_backward
 * (same arguments and partial layout, d_mult as in sdemc_cv_forward_tc),
 * every product a tcgen05.mma (forward recompute, the two dgrad products,
 * the weight gradients accumulated in tensor memory over the CTA's rows).
 * Uses at most nparts CTAs; a bounded wait that gives up sets SDEMC_ETIMEOUT
 * in *d_status and NaN in the gradient.  Replaces loss.backward() inside
 * train_adapted_control_variates (sde_mc/varred.py:160-180).               */
int sdemc_cv_backward_tc(int dim, const float* d_params, const float* d_time,
                         const float* d_paths, const float* d_mult,
                         const int64_t* d_index, int64_t n, int steps,
                         float disc_rate, const float* d_gamma,
                         float* d_partials, int nparts, float* d_grad,
                         int32_t* d_status, void* stream);

/* K5 on the 5th-generation tensor cores (tcgen05.mma, accumulators in tensor
 * memory) for large batches: d_gamma[q] = payoff[index[q]] + sum_k
 * e^{-r t_k} f(t_k, X_k) . d_mult[k] over the selected paths, where d_mult
 * (N, S, d) holds each row's multipliers (the Brownian increments for the
 * integrand f; marks minus compensator for the jump integrand g) and
 * d_payoffs may be null (no payoff term).  d_scratch holds
 * sdemc_cv_forward_tc_scratch_bytes(n, steps) bytes of per-range partial
 * sums; a bounded wait that gives up sets SDEMC_ETIMEOUT in *d_status.    */
size_t sdemc_cv_forward_tc_scratch_bytes(int64_t n, int steps);

/* K7: paths, payoff and the learned control variate (integrand f, g = 0) in
 * one pass, no materialised paths (apply_adapted_control_variates,
 * sde_mc/varred.py:98-131).  The network runs on the tensor cores at every
 * step of 128 paths per CTA.  d_out receives 8 doubles: sum Gamma,
 * sum Gamma^2, n, sum payoff, sum payoff^2, mean Gamma, var Gamma, status;
 * d_gamma (nullable) the per-path Gamma.  Diagonal noise, d in {1, 2}.    */
size_t sdemc_price_cv_scratch_bytes(const sdemc_inst* h_inst);
int sdemc_price_cv(const sdemc_inst* h_inst, const float* d_params, float disc_rate,
                   void* d_scratch, size_t scratch_bytes, double* d_out,
                   float* d_gamma, void* stream);
int sdemc_cv_forward_tc(int dim, const float* d_params, const float* d_time,
                        const float* d_paths, const float* d_mult,
                        const float* d_payoffs, const int64_t* d_index, int64_t n,
                        int steps, float disc_rate, float* d_gamma, void* d_scratch,
                        size_t scratch_bytes, int32_t* d_status, void* stream);

/* ---- K9: pricing server (continuous batching) ---------------------------
 * A request is one run_mc (sde_mc/mc.py:418-440): a pilot of inst.num_paths
 * paths sizes the main run for a 95% half-width of rel_target * |price|
 * (find_num_trials, :418-427), then the main run prices fresh paths.  The
 * server owns one host thread, one CUDA stream (plus side streams) and its
 * device memory.  Each request lives in a device-resident slot holding its
 * descriptor, its RNG path counter and its FP64 running sums; every tick the
 * thread packs a slice of every scheduled slot into per-dimension persistent
 * kernels (same per-path code as K1), reduces each slot's chunk sums in a
 * fixed order into its slot, and reads back only the slots that finished a
 * phase.  Requests are admitted while slots and the device-memory budget
 * allow; later arrivals join between ticks while others are running.
 * A slot's slices depend only on its own request, so a result is the same
 * bits whether the request ran alone or in any mix.
 *
 * Estimators: SDEMC_EST_PLAIN is the reference's plain estimator.
 * SDEMC_EST_LINEAR_CV adds 2d + 1 control variates, per asset i
 *   sum_k w_k X^i_k dW^i_k  and  sum_k w_k X^i_k (J^i_{k+1} - lambda_i E[J] dt_k),
 * and sum_k g_k (J_{k+1}^2 - lambda E[J^2] dt_k): stochastic integrals against
 * the Brownian increments and the compensated jump measures of the
 * jump-adapted grid (mean exactly zero under the Euler scheme), with w_k a
 * Black-Scholes delta and g_k a scaled gamma of the payoff's underlying; their
 * coefficients are fitted by regression on the pilot and the main run prices
 * payoff - beta . r on fresh paths, so it stays unbiased.  Jump terms are on
 * for lognormal marks (E[J] known exactly).  When the pilot shows no variance
 * reduction the server falls back to the plain estimator; descriptors with
 * non-diagonal noise or the payoff at the nominal step use the plain one. */
enum { SDEMC_EST_PLAIN = 0, SDEMC_EST_LINEAR_CV = 1 };
enum { SDEMC_SERVE_FIFO = 0, SDEMC_SERVE_SRPT = 1 };  /* tick fill order */

typedef struct sdemc_server sdemc_server;

typedef struct {
  int32_t device;           /* CUDA device ordinal                              */
  int32_t max_slots;        /* requests resident at once (1..65536)             */
  int64_t mem_budget;       /* device bytes for slots and tick partials        */
  int64_t tick_work;        /* path-step x dim units per tick (0: 2^33)         */
  int64_t slice_work;       /* path-step x dim units per slot slice (0: 2^27)   */
  int32_t block_threads;    /* class-kernel CTA size, multiple of 32 (0: 256)   */
  int32_t side_streams;     /* class kernels spread over this many streams      */
  int32_t policy;           /* SDEMC_SERVE_FIFO or SDEMC_SERVE_SRPT             */
  int32_t reserved;
} sdemc_server_cfg;

typedef struct {
  sdemc_inst inst;          /* num_paths = pilot paths; path_offset = first path */
  double rel_target;        /* target 95% half-width / |price|                  */
  int64_t max_paths;        /* cap on main-run paths (0: 2^36)                  */
  uint64_t tag;             /* caller's id, returned with the result            */
  int32_t estimator;        /* SDEMC_EST_*                                      */
  int32_t reserved;
} sdemc_request;

typedef struct {
  uint64_t tag;
  int32_t status;           /* SDEMC_OK or an error code                        */
  int32_t estimator;        /* estimator of the main run                        */
  double mean, se;          /* main-run price and its standard error            */
  double pilot_mean, pilot_se;
  double vrf;               /* pilot variance / control-variate residual var.   */
  int64_t pilot_paths, main_paths;
  int64_t t_arrive_ns, t_admit_ns, t_done_ns;  /* CLOCK_MONOTONIC               */
  float beta[2 * SDEMC_MAX_DIM + 1];  /* control-variate coefficients     */
  float reserved1;
} sdemc_result;

typedef struct {
  int64_t submitted, admitted, completed, pending, active;
  int64_t ticks, mem_in_use, mem_peak;
  int64_t path_steps;       /* expected path-steps of all slices (nominal steps
                               plus expected jumps per path)                   */
  int64_t launches;         /* kernels launched (install, class, reduce)        */
  int64_t h2d_bytes, d2h_bytes;  /* plan/slot uploads and phase-record readbacks */
  double busy_s;            /* sum of tick durations on the device              */
  /* tick durations on the device: bucket 0 below 0.125 ms, bucket b in
     [0.125 * 2^(b-1), 0.125 * 2^b) ms, bucket 15 from 2048 ms up            */
  int64_t tick_hist[16];
} sdemc_server_stats;

/* Integrand-weight parameters of SDEMC_EST_LINEAR_CV for one descriptor, as
 * the server derives them at admission.  w(t, X) = N(d1) (call-like) or
 * N(d1) - 1 (puts) with d1 = (ln A + drift tau) inv_sig / sqrt(tau), A =
 * scale_over_k * agg(X) (agg 0: asset 0, 1: mean, 2: max), tau = T - t, and
 * g(t, X) = A inv_sig phi(d1) / sqrt(tau); wkind 0 means w = g = 1.  comp[i]
 * is the jump compensator rate lambda_i E[J] of asset i, comp_j2 = lambda
 * E[J^2]; inv_comp / inv_comp_j2 are their float reciprocals (0 for a zero
 * rate); jumps = 1 when the jump regressors are on (lognormal marks).     */
typedef struct sdemc_cv_weights {
  float comp[SDEMC_MAX_DIM];
  float inv_comp[SDEMC_MAX_DIM];
  float scale_over_k, inv_sig, drift, T, comp_j2, inv_comp_j2;
  int32_t agg, wkind, jumps;
  int32_t reserved;
} sdemc_cv_weights;

/* Host only: the weight parameters the server uses for *h_inst.           */
int sdemc_serve_cv_weights(const sdemc_inst* h_inst, sdemc_cv_weights* h_out);

/* The served control variate path by path, for checking it against an
 * independent restatement: runs the server kernels' per-path code (the same
 * loop, draws and regressor accumulation) on paths [0, num_paths) of *h_inst
 * (diagonal noise, terminal payoff) and writes each path's discounted payoff
 * d_payoff (n) and its 2d + 1 regressors d_reg (n, 2d + 1).  Optional
 * exports (nullable): the raw draws as sdemc_materialise exports them (d_z
 * (n, steps_cap, dim) standard normals, d_jt / d_jm / d_jsel (n, jcap) the
 * jump stream) and the integrand weights evaluated at the start of every
 * 4-step block, d_wg (n, wcap, 2) as (w, g).  Steps past steps_cap or blocks
 * past wcap are not exported and set SDEMC_EOVERFLOW in *d_status.  No
 * reference function computes these regressors; their estimator stands in
 * for run_mc's plain estimate (sde_mc/mc.py:418-440), with the pilot's
 * variance sizing the main run as find_num_trials does (:418-427).        */
int sdemc_serve_cv_paths(const sdemc_inst* h_inst, int steps_cap, float* d_payoff, float* d_reg,
                         float* d_z, float* d_jt, float* d_jm, int32_t* d_jsel, int jcap,
                         float* d_wg, int wcap, int32_t* d_status, void* stream);

int sdemc_server_create(const sdemc_server_cfg* cfg, sdemc_server** out);
/* Enqueue one request (thread-safe; arrival time = now).  Rejects invalid
 * descriptors and requests that could never fit the budget.               */
int sdemc_server_admit(sdemc_server* srv, const sdemc_request* req);
/* Move up to max finished results into out; waits up to wait_ns for one.  */
int sdemc_server_poll(sdemc_server* srv, sdemc_result* out, int max, int* n_out,
                      int64_t wait_ns);
int sdemc_server_stats_get(sdemc_server* srv, sdemc_server_stats* out);
int sdemc_server_destroy(sdemc_server* srv);
/* sizeof of sdemc_server_cfg, sdemc_request, sdemc_result and
 * sdemc_server_stats (n >= 4), for bindings that mirror the structs.      */
int sdemc_serve_sizes(size_t* out, int n);

/* ---- RNG export (for the oracle and for users who want the raw draws) --
 * Philox4x32-10 blocks for counter (c0 = first_block + i, c1 = path lo,
 * c2 = path hi | tag << 16, c3 = stream_id), key = seed.                   */
int sdemc_philox(uint64_t seed, uint32_t stream_id, uint32_t tag,
                 uint64_t path, uint32_t first_block, int nblocks,
                 uint32_t* d_out, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* SDEMC_H */
