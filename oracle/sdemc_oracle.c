/*
 * sdemc_oracle.c — CPU oracle for the sde_mc path-integration hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline leg of bench.py may load this library, and only to check the
 * kernels' results or as the timed CPU baseline — never as part of the
 * product path.
 *
 * A plain-C restatement of the reference's algorithm (piers-hinds/sde_mc):
 *   - the jump-adapted Euler loop of JumpDiffusionSolver.solve
 *     (sde_mc/solvers.py:164-226): h = min(h, max(T - t, 0)),
 *     dt = min(h, next_jump - t), x += drift*dt + diffusion*dW, t += dt, and a
 *     jump when torch.isclose(next_jump, t, atol=1e-12) (rtol 1e-5), applied
 *     with the pre-step state unless exact_jumps (:212-217);
 *   - the uniform grid of DiffusionSolver.solve (sde_mc/solvers.py:68-88);
 *   - the coupled fine/coarse loop of multilevel_solve (:228-307);
 *   - EulerScheme.step (sde_mc/schemes.py:6-13), the Merton/Gbm/Levy affine
 *     coefficients (sde_mc/sde.py:203-219, 368-375; sde_mc/levy.py:74-83);
 *   - Option payoffs (sde_mc/options.py:167-321) and mc_estimates
 *     (sde_mc/helpers.py:51-68).
 * Draw sources: (1) arrays recorded from the reference (replay), (2) the raw
 * draws a GPU run exported (so the GPU is checked step by step), (3) its own
 * Philox4x32-10 streams with libm transforms (the CPU baseline).  Float
 * arithmetic is written op by op (compile with -ffp-contract=off) so modes
 * (1)/(2) reproduce the GPU's rounding exactly.
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include "../include/sdemc.h"

#define MAXD SDEMC_MAX_DIM

/* ------------------------------------------------------------- Philox --- */
static void philox(uint32_t c[4], uint32_t k0, uint32_t k1) {
  for (int r = 0; r < 10; ++r) {
    if (r) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
    uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
    uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
    uint32_t n0 = (uint32_t)(p1 >> 32) ^ c[1] ^ k0;
    uint32_t n2 = (uint32_t)(p0 >> 32) ^ c[3] ^ k1;
    c[0] = n0; c[1] = (uint32_t)p1; c[2] = n2; c[3] = (uint32_t)p0;
  }
}

typedef struct { uint32_t k0, k1, c1, c2base, c3; } skey_t;

static void skey_init(skey_t* k, uint64_t seed, uint32_t stream, uint64_t gpath) {
  k->k0 = (uint32_t)seed; k->k1 = (uint32_t)(seed >> 32);
  k->c1 = (uint32_t)gpath; k->c2base = (uint32_t)(gpath >> 32) & 0xFFFFu; k->c3 = stream;
}

static void skey_block(const skey_t* k, uint32_t tag, uint32_t b, uint32_t out[4]) {
  out[0] = b; out[1] = k->c1; out[2] = k->c2base | (tag << 16); out[3] = k->c3;
  philox(out, k->k0, k->k1);
}

static float u01(uint32_t w) {
  union { uint32_t u; float f; } v;
  v.u = 0x3F800000u | (w >> 9);
  return v.f - 0.99999994f;
}

static const float kTwoPi = 6.283185307179586f, kPi = 3.141592653589793f;

static float bm_radius(uint32_t w) { return sqrtf(-2.0f * logf(u01(w))); }
static float bm_angle(uint32_t w) { return fmaf(kTwoPi, u01(w), -kPi); }

/* ------------------------------------------------------------- layout --- */
static int zdim_of(int D, int noise) {
  return noise == SDEMC_NOISE_DIAG ? D : noise == SDEMC_NOISE_INDEP_SHARED ? D + 1 : 2 * D;
}
static int nw_of(int noise) { return noise == SDEMC_NOISE_DIAG ? 1 : 2; }

static float chol_at(const sdemc_inst* I, int i, int j) { return I->chol[i * (i + 1) / 2 + j]; }

static void correlate(const sdemc_inst* I, int D, const float* z, float sq, float* dW) {
  float zs[MAXD];
  for (int j = 0; j < D; ++j) zs[j] = z[j] * sq;
  if (D == 1) { dW[0] = zs[0]; return; }
  for (int i = 0; i < D; ++i) {
    float acc = chol_at(I, i, 0) * zs[0];
    for (int j = 1; j <= i; ++j) acc = fmaf(chol_at(I, i, j), zs[j], acc);
    dW[i] = acc;
  }
}

/* ------------------------------------------------------------- draws ---- */
enum { DRAW_NATIVE = 0, DRAW_REPLAY = 1, DRAW_EXPORT = 2 };

typedef struct {
  int mode;
  /* replay */
  const float* dw; const float* marks; const int32_t* asset; const float* jt; int S; int MJ;
  /* export */
  const float* z; int zdim; const float* xjt; const float* xjm; const int32_t* xjsel; int jcap;
  /* native */
  skey_t key; float buf[4]; uint32_t jblock; float jmark; int jsel;
  /* state */
  int jidx; int overflow; float sq_h, h_nom;
} draws_t;

static float inverse_cdf(const sdemc_inst* I, float y) {
  const float cm = I->mark_p[0], cp = I->mark_p[1], mu = I->mark_p[2], al = I->mark_p[3];
  const float lda = I->mark_p[5], y1 = I->mark_p[6], y2 = I->mark_p[7], y3 = I->mark_p[8];
  const float epa = I->mark_p[10], nia = I->mark_p[11];
  const float ly = lda * y, inv_mu = 1.0f / mu;
  if (y <= y1) return logf((mu * ly) / cm) / mu - 1.0f;
  if (y < y2) return -powf(al * (ly / cm - inv_mu) + 1.0f, nia);
  if (y < y3) {
    const float tail = cm * ((epa - 1.0f) / al);
    return powf((-al / cp) * ((ly - cm / mu) - tail) + epa, nia);
  }
  return 1.0f - inv_mu * logf(((mu * lda) * (1.0f - y)) / cp);
}

static float native_load_jump(const sdemc_inst* I, int D, draws_t* d, uint32_t j) {
  uint32_t w[4];
  skey_block(&d->key, 1u, j, w);
  float gap = -logf(u01(w[0])) * I->inv_rate;
  if (I->mark == SDEMC_MARK_LOGNORMAL) {
    float zn = bm_radius(w[1]) * cosf(bm_angle(w[2]));
    d->jmark = expf(I->mark_p[1] * zn + I->mark_p[0]) - 1.0f;
  } else if (I->mark == SDEMC_MARK_INVCDF) {
    d->jmark = inverse_cdf(I, u01(w[1]) + I->mark_p[9]);
  } else {
    d->jmark = 0.f;
  }
  d->jsel = 0;
  if (I->jump_target == SDEMC_JUMP_ONE_ASSET) {
    float us = u01(w[3]);
    for (int i = 0; i < D - 1; ++i) d->jsel += (us >= I->jump_cdf[i]) ? 1 : 0;
  }
  return gap;
}

static void native_fill4(const draws_t* d, uint32_t b, float* o) {
  uint32_t w[4];
  skey_block(&d->key, 0u, b, w);
  float r0 = bm_radius(w[0]), a0 = bm_angle(w[1]), r1 = bm_radius(w[2]), a1 = bm_angle(w[3]);
  o[0] = r0 * cosf(a0); o[1] = r0 * sinf(a0); o[2] = r1 * cosf(a1); o[3] = r1 * sinf(a1);
}

/* Normals of step k (called for k = 0, 1, 2, ... in turn), as the kernels
 * draw them: for ZD in {1, 2, 3, 5, 6} the path's diffusion stream read
 * densely, step k taking normals k ZD .. k ZD + ZD - 1, four per Philox block
 * (the unused tail of a step's last block kept in d->buf for the next step);
 * for ZD = 4, 7, 8 whole blocks per step, the first ZD normals used. */
static void native_normals(draws_t* d, int ZD, int k, float* z) {
  if (ZD == 1 || ZD == 2) {
    int pos = (k * ZD) & 3;
    if (pos == 0) native_fill4(d, (uint32_t)((k * ZD) >> 2), d->buf);
    for (int i = 0; i < ZD; ++i) z[i] = d->buf[pos + i];
  } else if (ZD % 4 == 0 || ZD == 7) {
    int nb = (ZD + 3) / 4;
    for (int b = 0; b < nb; ++b) {
      float o[4];
      native_fill4(d, (uint32_t)(k * nb + b), o);
      for (int q = 0; q < 4; ++q) if (4 * b + q < ZD) z[4 * b + q] = o[q];
    }
  } else {
    const int off = (k * ZD) & 3, nc = off ? 4 - off : 0, take = nc < ZD ? nc : ZD;
    float carry[4];
    memcpy(carry, d->buf, sizeof(carry));
    for (int j = 0; j < take; ++j) z[j] = carry[j];
    const uint32_t b0 = (uint32_t)((k * ZD + take) >> 2);
    const int nblk = (ZD - take + 3) / 4;
    for (int nb = 0; nb < nblk; ++nb) {
      float o[4];
      native_fill4(d, b0 + (uint32_t)nb, o);
      for (int q = 0; q < 4; ++q) {
        const int idx = take + 4 * nb + q;
        if (idx < ZD) z[idx] = o[q];
        else d->buf[idx - ZD] = o[q];
      }
    }
  }
}

static void draws_increments(const sdemc_inst* I, int D, draws_t* d, int k, float dt,
                             float* dW, float* dW2) {
  const int noise = I->noise, ZD = zdim_of(D, noise), NW = nw_of(noise);
  for (int i = 0; i < D; ++i) dW2[i] = 0.f;
  if (d->mode == DRAW_REPLAY) {
    if (k >= d->S) { for (int i = 0; i < D; ++i) dW[i] = 0.f; d->overflow = 1; return; }
    const float* r = d->dw + (size_t)k * D * NW;
    for (int i = 0; i < D; ++i) {
      if (NW == 1) dW[i] = r[i];
      else { dW[i] = r[2 * i]; dW2[i] = r[2 * i + 1]; }
    }
    return;
  }
  float z[2 * MAXD];
  if (d->mode == DRAW_EXPORT) {
    if (k >= d->S) { for (int j = 0; j < ZD; ++j) z[j] = 0.f; d->overflow = 1; }
    else memcpy(z, d->z + (size_t)k * d->zdim, sizeof(float) * ZD);
  } else {
    native_normals(d, ZD, k, z);
  }
  const float sq = (dt == d->h_nom) ? d->sq_h : sqrtf(dt);
  correlate(I, D, z, sq, dW);
  if (noise == SDEMC_NOISE_INDEP_SHARED) {
    float s = z[D] * sq;
    for (int i = 0; i < D; ++i) dW2[i] = s;
  } else if (noise == SDEMC_NOISE_INDEP_PAIR) {
    correlate(I, D, z + D, sq, dW2);
  }
}

static const float kInf = INFINITY;

static float draws_jump_first(const sdemc_inst* I, int D, draws_t* d) {
  d->jidx = 0;
  if (I->rate <= 0.f) return kInf;
  if (d->mode == DRAW_REPLAY) return d->MJ > 0 ? d->jt[0] : kInf;
  if (d->mode == DRAW_EXPORT) return d->jcap > 0 ? d->xjt[0] : kInf;
  d->jblock = 0;
  return native_load_jump(I, D, d, 0);
}

static void draws_jump_mark(const draws_t* d, int k, float* J, int* sel) {
  if (d->mode == DRAW_REPLAY) {
    *J = k < d->S ? d->marks[k] : 0.f;
    *sel = (d->asset && k < d->S) ? d->asset[k] : 0;
  } else if (d->mode == DRAW_EXPORT) {
    *J = d->jidx < d->jcap ? d->xjm[d->jidx] : 0.f;
    *sel = (d->xjsel && d->jidx < d->jcap) ? d->xjsel[d->jidx] : 0;
  } else {
    *J = d->jmark; *sel = d->jsel;
  }
}

static float draws_jump_next(const sdemc_inst* I, int D, draws_t* d, float nj) {
  d->jidx++;
  if (d->mode == DRAW_REPLAY) {
    if (d->jidx >= d->MJ) { d->overflow = 1; return kInf; }
    return d->jt[d->jidx];
  }
  if (d->mode == DRAW_EXPORT) {
    if (d->jidx >= d->jcap) { d->overflow = 1; return kInf; }
    return d->xjt[d->jidx];
  }
  d->jblock++;
  return nj + native_load_jump(I, D, d, d->jblock);
}

/* ------------------------------------------------------------- scheme --- */
/* HestonScheme.step (sde_mc/schemes.py:16-22): Euler price step, then the
   larger root of Heston.quadratic_parameters (sde_mc/sde.py:275-279) by
   solve_quadratic (sde_mc/helpers.py:36-48) squared.  Same float32 order in
   both Euler modes. */
static void heston_step(const sdemc_inst* I, float* x, float dt, const float* dW) {
  float S = x[0], v = x[1];
  float dr = I->drift_b[0] * S;
  float sg = sqrtf(v) * S;
  float base = S + dr * dt;
  x[0] = base + sg * dW[0];
  float a = -1.0f - I->mark_p[0] * dt;
  float b = I->mark_p[2] * dW[1];
  float c0 = v + I->mark_p[1] * dt;
  float c = c0 - (0.5f * dt) * I->mark_p[3];
  float bb = b * b;
  float a4 = 4.0f * a;
  float sq = sqrtf(bb - a4 * c);
  float a2 = 2.0f * a;
  float r1 = (-b + sq) / a2;
  float r2 = (-b - sq) / a2;
  float y = fmaxf(r1, r2);
  x[1] = y * y;
}

static void euler(const sdemc_inst* I, int D, int exact, float* x, float dt, const float* dW,
                  const float* dW2) {
  if (D == 2 && I->model == SDEMC_MODEL_HESTON) { heston_step(I, x, dt, dW); return; }
  int asian = D == 2 && I->model == SDEMC_MODEL_ASIAN;
  float x0_old = x[0];
  for (int i = 0; i < D; ++i) {
    float xi = x[i];
    if (asian && i == 1) {
      /* AsianWrapper's integral component (sde_mc/sde.py:390-397) */
      x[1] = exact ? xi + x0_old * dt : fmaf(x0_old, dt, xi);
      continue;
    }
    if (exact) {
      float dr = I->drift_a[i] + I->drift_b[i] * xi;
      float sg = I->diff_s[i] + I->diff_q[i] * xi;
      float base = xi + dr * dt;
      if (I->noise == SDEMC_NOISE_DIAG) x[i] = base + sg * dW[i];
      else {
        float sg2 = I->diff2_s[i] + I->diff2_q[i] * xi;
        x[i] = base + (sg * dW[i] + sg2 * dW2[i]);
      }
    } else {
      float dr = fmaf(I->drift_b[i], xi, I->drift_a[i]);
      float sg = fmaf(I->diff_q[i], xi, I->diff_s[i]);
      float xn = fmaf(dr, dt, xi);
      xn = fmaf(sg, dW[i], xn);
      if (I->noise != SDEMC_NOISE_DIAG) {
        float sg2 = fmaf(I->diff2_q[i], xi, I->diff2_s[i]);
        xn = fmaf(sg2, dW2[i], xn);
      }
      x[i] = xn;
    }
  }
}

static void apply_jump(const sdemc_inst* I, int D, int exact, float* x, const float* base, float J,
                       int sel) {
  int one = I->jump_target == SDEMC_JUMP_ONE_ASSET;
  for (int i = 0; i < D; ++i) {
    if (one && i != sel) continue;
    if (exact) x[i] = x[i] + (I->jump_g[i] + I->jump_k[i] * base[i]) * J;
    else x[i] = fmaf(fmaf(I->jump_k[i], base[i], I->jump_g[i]), J, x[i]);
  }
}

static int jump_due(float nj, float t) {
  float err = fabsf(nj - t);
  float tol = 1e-12f + fabsf(1e-5f * t);
  return (nj == t) || (err <= tol);
}

float oracle_payoff(const sdemc_inst* I, const float* xin) {
  const int D = I->dim;
  float s[MAXD];
  for (int i = 0; i < D; ++i) {
    float sp = I->payoff_log ? expf(xin[i]) : xin[i];
    s[i] = I->payoff_scale * sp;
  }
  const float K = I->strike;
  float m;
  switch (I->payoff) {
    case SDEMC_PAYOFF_EUROCALL: return s[0] > K ? s[0] - K : 0.f;
    case SDEMC_PAYOFF_EUROPUT: return s[0] < K ? K - s[0] : 0.f;
    case SDEMC_PAYOFF_BINARY_AON: return s[0] >= K ? s[0] : 0.f;
    case SDEMC_PAYOFF_DIGITAL: return s[0] > K ? 1.f : 0.f;
    case SDEMC_PAYOFF_BASKET_ARITH:
      m = s[0];
      for (int i = 1; i < D; ++i) m = m + s[i];
      m = m / (float)D;
      return m > K ? m - K : 0.f;
    case SDEMC_PAYOFF_BASKET_GEO:
      m = logf(s[0]);
      for (int i = 1; i < D; ++i) m = m + logf(s[i]);
      m = expf(m / (float)D);
      return m > K ? m - K : 0.f;
    case SDEMC_PAYOFF_RAINBOW:
      m = s[0];
      for (int i = 1; i < D; ++i) m = fmaxf(m, s[i]);
      return m > K ? m - K : 0.f;
    case SDEMC_PAYOFF_BESTOF:
      m = s[0];
      for (int i = 1; i < D; ++i) m = fmaxf(m, s[i]);
      return fmaxf(m, K);
    case SDEMC_PAYOFF_ASIANCALL: {
      if (D < 2) return 0.f;
      float a = s[1] / I->T;
      float sp = I->payoff_log ? expf(a) : a;
      return sp > K ? sp - K : 0.f;
    }
    case SDEMC_PAYOFF_HESTON_RAINBOW:
      m = s[0];
      for (int i = 2; i < D; i += 2) m = fmaxf(m, s[i]);
      return m > K ? m - K : 0.f;
    default: return 0.f;
  }
}

/* ------------------------------------------- served control variate --- */
/* The pricing server's linear control variate, restated per path: with X_k
 * the state at the start of step k, dW_k its correlated increment and J the
 * mark of a jump at the end of the step,
 *   r_i     = sum_k w_k X^i_k dW^i_k
 *   r_{d+i} = -comp_i a_i,  a_i = sum_k w_k X^i_k (dt_k - J^i / comp_i)
 *   r_{2d}  = -comp_j2 ag,  ag  = sum_k g_k (dt_k - J^2 / comp_j2)
 * i.e. sum_k w_k X^i_k (J^i - comp_i dt_k) and sum_k g_k (J^2 - comp_j2 dt_k):
 * stochastic integrals of predictable integrands against the Brownian
 * increments and the compensated jump measures, each with mean zero.  The
 * weights (w, g) are evaluated at the start of every 4-step block of the
 * path's own steps.  Operation order as the kernel's, every multiply-add an
 * fmaf, the reciprocals of the compensator rates taken from the weights.
 * No reference function computes these; the estimator P - beta . r they
 * feed replaces run_mc's plain estimate (sde_mc/mc.py:418-440). */
typedef struct {
  const sdemc_cv_weights* cw;
  const float* wg;   /* recorded (w, g) per block, or NULL: evaluate here */
  int wcap, D, bad;
  float xp[MAXD], r[MAXD], a[MAXD], tp, w, g, ag;
  double wstat[3];   /* worst |dw| / bound, worst |dg| / bound, blocks checked */
} cvacc_t;

/* Normal cdf and density of the weights, from libm's erfcf and expf. */
static float cv_ncdf(float d1) { return 0.5f * erfcf(-d1 * 0.70710678f); }

/* Evaluate (w, g) at the accumulator's block-start state (xp, tp); d1_out,
 * is_out and lm_out receive the intermediates (for the error bound). */
static void cv_eval(const cvacc_t* c, float* w, float* g, float* d1_out, float* is_out, float* lm_out, float* v_out) {
  const sdemc_cv_weights* cw = c->cw;
  *d1_out = 0.f; *is_out = 0.f; *lm_out = 0.f; *v_out = 0.f;
  if (cw->wkind == 0) { *w = 1.f; *g = 1.f; return; }
  float m = c->xp[0];
  if (cw->agg == 1) {
    for (int i = 1; i < c->D; ++i) m = m + c->xp[i];
    m = m * (1.f / (float)c->D);
  } else if (cw->agg == 2) {
    for (int i = 1; i < c->D; ++i) m = fmaxf(m, c->xp[i]);
  }
  m = m * cw->scale_over_k;
  const float tau = fmaxf(cw->T - c->tp, 1e-6f);
  const float is = (1.f / sqrtf(tau)) * cw->inv_sig;
  if (m > 0.f) {
    const float lm = logf(m);
    const float d1 = fmaf(cw->drift, tau, lm) * is;
    const float v = cv_ncdf(d1);
    *w = cw->wkind == 2 ? v - 1.f : v;
    *g = (m * is) * (0.39894228f * expf(-0.5f * (d1 * d1)));
    *d1_out = d1; *is_out = is; *lm_out = lm; *v_out = v;
  } else {
    *w = cw->wkind == 2 ? -1.f : 0.f;
    *g = 0.f;
  }
}

/* Weights of block b: the recorded ones (each checked against this file's
 * own evaluation within an error bound) or this file's own. */
static void cv_weights_block(cvacc_t* c, int b) {
  float w, g, d1, is, lm, v;
  cv_eval(c, &w, &g, &d1, &is, &lm, &v);
  if (!c->wg) { c->w = w; c->g = g; return; }
  if (b >= c->wcap) { c->bad = 1; c->w = w; c->g = g; return; }
  const float rw = c->wg[2 * b], rg = c->wg[2 * b + 1];
  /* The kernel evaluates ln, 1/sqrt, the normal cdf and exp with CUDA's
   * intrinsics (absolute error of __logf <= 2^-21.41 near 1, otherwise 3 ulp;
   * rsqrtf 2 ulp; normcdff 5 ulp; __expf 2 + 1.173|x| ulp); propagate those
   * through d1 = (ln m + drift tau) is, w = N(d1) (or N(d1) - 1), g = m is
   * phi(d1), with a factor 2 to spare. */
  const double ulp = 1.0 / 8388608.0;
  const double dd1 = fabs((double)is) * (4.0e-7 + 8.0 * ulp * fabs((double)lm)) + fabs((double)d1) * 8.0 * ulp;
  const double phi = 0.3989422804014327 * exp(-0.5 * (double)d1 * d1);
  /* a put's weight N(d1) - 1 rounds once more on each side: half an ulp of |w| each */
  const double bw = 2.0 * (phi * dd1 + 8.0 * ulp * fabs((double)v) + ulp * fabs((double)w)) + 1e-12;
  const double x = 0.5 * (double)d1 * d1;
  const double bg = 2.0 * fabs((double)g) * (8.0 * ulp + fabs((double)d1) * dd1 + (8.0 + 1.2 * x) * ulp) + 1e-12;
  const double ew = fabs((double)rw - (double)w) / bw, eg = fabs((double)rg - (double)g) / bg;
  if (ew > c->wstat[0]) c->wstat[0] = ew;
  if (eg > c->wstat[1]) c->wstat[1] = eg;
  c->wstat[2] += 1.0;
  c->w = rw; c->g = rg;
}

static void cv_init(cvacc_t* c, const float* x) {
  for (int i = 0; i < c->D; ++i) { c->xp[i] = x[i]; c->r[i] = 0.f; c->a[i] = 0.f; }
  c->tp = 0.f; c->ag = 0.f;
  cv_weights_block(c, 0);
}

static void cv_step(cvacc_t* c, int k, const float* x, float t, float J, int sel, const float* dW, int jump_one) {
  const sdemc_cv_weights* cw = c->cw;
  if (k > 0 && (k & 3) == 0) cv_weights_block(c, k >> 2);
  for (int i = 0; i < c->D; ++i) c->r[i] = fmaf(c->xp[i], c->w * dW[i], c->r[i]);
  if (cw->jumps) {
    const float dt = t - c->tp;
    const float wdt = c->w * dt;
    for (int i = 0; i < c->D; ++i) c->a[i] = fmaf(c->xp[i], wdt, c->a[i]);
    c->ag = fmaf(c->g, dt, c->ag);
    if (J != 0.f) {
      for (int i = 0; i < c->D; ++i)
        if (!jump_one || i == sel) c->a[i] = fmaf(-(c->w * c->xp[i]), J * cw->inv_comp[i], c->a[i]);
      c->ag = fmaf(-c->g, (J * J) * cw->inv_comp_j2, c->ag);
    }
  }
  for (int i = 0; i < c->D; ++i) c->xp[i] = x[i];
  c->tp = t;
}

static float cv_reg(const cvacc_t* c, int q) {
  const int D = c->D;
  if (q < D) return c->r[q];
  if (q < 2 * D) return -(c->cw->comp[q - D] * c->a[q - D]);
  return -(c->cw->comp_j2 * c->ag);
}

/* One path of the reference loop.  Storage pointers may be NULL; when given
 * they follow the AdaptedPathData layout with S = cap columns (+1). Returns
 * the path's active step count (or -1 on overflow). A path runs alone here,
 * so "frozen" steps of the batch-global loop are simply not taken; storage
 * columns after the last step hold the frozen values. */
static int run_path(const sdemc_inst* I, draws_t* d, int exact, int cap, float* paths, float* left,
                    float* time, float* jumps, float* normals, float* x, cvacc_t* cv) {
  const int D = I->dim, NW = nw_of(I->noise);
  int jump_one = I->jump_target == SDEMC_JUMP_ONE_ASSET;
  for (int i = 0; i < D; ++i) x[i] = I->x0[i];
  if (paths) for (int i = 0; i < D; ++i) paths[i] = x[i];
  if (left) for (int i = 0; i < D; ++i) left[i] = x[i];
  if (jumps) for (int i = 0; i < D; ++i) jumps[i] = 0.f;
  if (time) time[0] = 0.f;
  if (cv) cv_init(cv, x);
  float t = 0.f, dW[MAXD], dW2[MAXD], old[MAXD], xl[MAXD];
  int k = 0;
  if (I->grid == SDEMC_GRID_UNIFORM) {
    for (; k < I->num_steps; ++k) {
      draws_increments(I, D, d, k, I->h, dW, dW2);
      euler(I, D, exact, x, I->h, dW, dW2);
      t = t + I->h;
      if (cv) cv_step(cv, k, x, t, 0.f, 0, dW, 0);
      if (k < cap) {
        size_t c = (size_t)(k + 1) * D;
        if (paths) for (int i = 0; i < D; ++i) paths[c + i] = x[i];
        if (left) for (int i = 0; i < D; ++i) left[c + i] = x[i];
        if (jumps) for (int i = 0; i < D; ++i) jumps[c + i] = 0.f;
        if (time) time[k + 1] = t;
        if (normals) for (int i = 0; i < D; ++i) {
          if (NW == 1) normals[(size_t)k * D + i] = dW[i];
          else { normals[(size_t)k * D * 2 + 2 * i] = dW[i]; normals[(size_t)k * D * 2 + 2 * i + 1] = dW2[i]; }
        }
      }
    }
  } else {
    const float T = I->T;
    float h = I->h;
    float nj = draws_jump_first(I, D, d);
    int maxit = cap;
    while (t < T) {
      if (k >= maxit) return -1;
      h = fminf(h, fmaxf(T - t, 0.f));
      float dt = fminf(h, nj - t);
      draws_increments(I, D, d, k, dt, dW, dW2);
      memcpy(old, x, sizeof(float) * D);
      euler(I, D, exact, x, dt, dW, dW2);
      t = t + dt;
      memcpy(xl, x, sizeof(float) * D);
      float J = 0.f;
      int sel = 0;
      if (jump_due(nj, t)) {
        draws_jump_mark(d, k, &J, &sel);
        apply_jump(I, D, exact, x, I->exact_jumps ? x : old, J, sel);
        nj = draws_jump_next(I, D, d, nj);
      }
      if (cv) cv_step(cv, k, x, t, J, sel, dW, jump_one);
      size_t c = (size_t)(k + 1) * D;
      if (paths) for (int i = 0; i < D; ++i) paths[c + i] = x[i];
      if (left) for (int i = 0; i < D; ++i) left[c + i] = xl[i];
      if (jumps) for (int i = 0; i < D; ++i) jumps[c + i] = (jump_one && i != sel) ? 0.f : J;
      if (time) time[k + 1] = t;
      if (normals) for (int i = 0; i < D; ++i) {
        if (NW == 1) normals[(size_t)k * D + i] = dW[i];
        else { normals[(size_t)k * D * 2 + 2 * i] = dW[i]; normals[(size_t)k * D * 2 + 2 * i + 1] = dW2[i]; }
      }
      ++k;
    }
  }
  for (int kk = k; kk < cap; ++kk) {
    size_t c = (size_t)(kk + 1) * D;
    if (paths) for (int i = 0; i < D; ++i) paths[c + i] = x[i];
    if (left) for (int i = 0; i < D; ++i) left[c + i] = x[i];
    if (jumps) for (int i = 0; i < D; ++i) jumps[c + i] = 0.f;
    if (time) time[kk + 1] = t;
    if (normals) for (int i = 0; i < D * NW; ++i) normals[(size_t)kk * D * NW + i] = 0.f;
  }
  return d->overflow ? -1 : k;
}

static void draws_native_init(const sdemc_inst* I, draws_t* d, int64_t p) {
  memset(d, 0, sizeof(*d));
  d->mode = DRAW_NATIVE;
  skey_init(&d->key, I->seed, I->stream_id, I->path_offset + (uint64_t)p);
  d->h_nom = I->h;
  d->sq_h = sqrtf(I->h);
}

/* ------------------------------------------------------------- exports -- */

void oracle_philox(uint64_t seed, uint32_t stream, uint32_t tag, uint64_t path, uint32_t first,
                   int n, uint32_t* out) {
  skey_t k;
  skey_init(&k, seed, stream, path);
  for (int i = 0; i < n; ++i) skey_block(&k, tag, first + (uint32_t)i, out + 4 * i);
}

/* Native standard normals of steps [0, nsteps) of one path: (nsteps, zdim). */
void oracle_native_normals(const sdemc_inst* I, int64_t p, int nsteps, float* out) {
  draws_t d;
  draws_native_init(I, &d, p);
  const int ZD = zdim_of(I->dim, I->noise);
  for (int k = 0; k < nsteps; ++k) native_normals(&d, ZD, k, out + (size_t)k * ZD);
}

/* Native jump stream of one path: first n jump times, marks and picks. */
void oracle_native_jumps(const sdemc_inst* I, int64_t p, int n, float* jt, float* jm, int32_t* js) {
  draws_t d;
  draws_native_init(I, &d, p);
  float nj = draws_jump_first(I, I->dim, &d);
  for (int j = 0; j < n; ++j) {
    jt[j] = nj; jm[j] = d.jmark; js[j] = d.jsel;
    if (I->rate > 0.f) nj = draws_jump_next(I, I->dim, &d, nj);
  }
}

/* Replay recorded reference draws for bs paths (layouts as sdemc_replay). */
int oracle_replay(const sdemc_inst* I, int bs, int S, int MJ, const float* jt, const float* dw,
                  const float* marks, const int32_t* asset, float* paths, float* left, float* time,
                  float* jumps, float* payoffs, int32_t* steps) {
  const int D = I->dim, NW = nw_of(I->noise);
  int bad = 0;
  for (int p = 0; p < bs; ++p) {
    draws_t d;
    memset(&d, 0, sizeof(d));
    d.mode = DRAW_REPLAY;
    d.dw = dw + (size_t)p * S * D * NW;
    d.marks = marks ? marks + (size_t)p * S : NULL;
    d.asset = asset ? asset + (size_t)p * S : NULL;
    d.jt = jt ? jt + (size_t)p * MJ : NULL;
    d.S = S; d.MJ = jt ? MJ : 0;
    float x[MAXD];
    size_t row = (size_t)p * (S + 1);
    int k = run_path(I, &d, 1, S, paths ? paths + row * D : NULL, left ? left + row * D : NULL,
                     time ? time + row : NULL, jumps ? jumps + row * D : NULL, NULL, x, NULL);
    if (k < 0) bad = 1;
    if (steps) steps[p] = k;
    if (payoffs) payoffs[p] = oracle_payoff(I, x) * I->discount;
  }
  return bad ? SDEMC_EOVERFLOW : SDEMC_OK;
}

/* Re-run paths [0, n) from the raw draws a GPU run exported: z (n, S, zdim),
 * jump times/marks/picks (n, jcap).  exact selects the Euler op order. */
int oracle_from_export(const sdemc_inst* I, int64_t n, int S, const float* z, int zdim,
                       const float* jt, const float* jm, const int32_t* js, int jcap, int exact,
                       float* paths, float* left, float* time, float* jumps, float* normals,
                       float* payoffs, int32_t* steps) {
  const int D = I->dim, NW = nw_of(I->noise);
  int bad = 0;
  for (int64_t p = 0; p < n; ++p) {
    draws_t d;
    memset(&d, 0, sizeof(d));
    d.mode = DRAW_EXPORT;
    d.z = z + (size_t)p * S * zdim; d.zdim = zdim; d.S = S;
    d.xjt = jt ? jt + (size_t)p * jcap : NULL;
    d.xjm = jm ? jm + (size_t)p * jcap : NULL;
    d.xjsel = js ? js + (size_t)p * jcap : NULL;
    d.jcap = jt ? jcap : 0;
    d.h_nom = I->h; d.sq_h = sqrtf(I->h);
    float x[MAXD];
    size_t row = (size_t)p * (S + 1);
    int k = run_path(I, &d, exact, S, paths ? paths + row * D : NULL, left ? left + row * D : NULL,
                     time ? time + row : NULL, jumps ? jumps + row * D : NULL,
                     normals ? normals + (size_t)p * S * D * NW : NULL, x, NULL);
    if (k < 0) bad = 1;
    if (steps) steps[p] = k;
    if (payoffs) payoffs[p] = oracle_payoff(I, x) * I->discount;
  }
  return bad ? SDEMC_EOVERFLOW : SDEMC_OK;
}

/* ------------------------------------------- served control variate --- */
/* The weight parameters the server derives for a descriptor: the jump
 * compensator rates lambda_i E[J] (E[J] = exp(alpha + gamma^2/2) - 1 for
 * lognormal marks; per asset, lambda times the asset's pick probability) and
 * lambda E[J^2]; the delta kind and aggregate of the payoff; and a lognormal
 * proxy volatility of the payoff's underlying (the correlated mean's or the
 * assets' mean variance, plus the jump variance).  All in double, rounded to
 * float at the end, in the server's operation order. */
int oracle_serve_cv_weights(const sdemc_inst* I, sdemc_cv_weights* cw) {
  memset(cw, 0, sizeof(*cw));
  const int d = I->dim;
  double jump_var = 0.0;
  const double a = I->mark_p[0], g = I->mark_p[1];
  const double kappa = exp(a + 0.5 * g * g) - 1.0;
  if (I->rate > 0.f && I->mark == SDEMC_MARK_LOGNORMAL && fabs(kappa) > 1e-9) {
    for (int i = 0; i < d; ++i) {
      double p = 1.0;
      if (I->jump_target == SDEMC_JUMP_ONE_ASSET) {
        const double lo = i > 0 ? I->jump_cdf[i - 1] : 0.0, hi = i < d - 1 ? I->jump_cdf[i] : 1.0;
        p = hi - lo;
      }
      cw->comp[i] = (float)((double)I->rate * p * kappa);
    }
    cw->jumps = 1;
    cw->comp_j2 = (float)((double)I->rate * (exp(2.0 * a + 2.0 * g * g) - 2.0 * exp(a + 0.5 * g * g) + 1.0));
    jump_var = (double)I->rate * (a * a + g * g) / (I->jump_target == SDEMC_JUMP_ONE_ASSET ? d : 1);
  }
  switch (I->payoff) {
    case SDEMC_PAYOFF_EUROCALL: cw->wkind = 1; cw->agg = 0; break;
    case SDEMC_PAYOFF_EUROPUT: cw->wkind = 2; cw->agg = 0; break;
    case SDEMC_PAYOFF_BASKET_ARITH:
    case SDEMC_PAYOFF_BASKET_GEO: cw->wkind = 1; cw->agg = 1; break;
    case SDEMC_PAYOFF_RAINBOW:
    case SDEMC_PAYOFF_BESTOF: cw->wkind = 1; cw->agg = 2; break;
    default: cw->wkind = 0; break;
  }
  if (I->payoff_log || !(I->strike > 0.f)) cw->wkind = 0;
  double L[MAXD][MAXD];
  memset(L, 0, sizeof(L));
  for (int i = 0, q = 0; i < d; ++i)
    for (int j = 0; j <= i; ++j) L[i][j] = I->chol[q++];
  double sig[MAXD];
  for (int i = 0; i < d; ++i) sig[i] = fabs((double)I->diff_q[i]);
  if (I->model == SDEMC_MODEL_HESTON) sig[0] = sqrt((double)I->x0[1] > 0.0 ? (double)I->x0[1] : 0.0);
  double var = 0.0;
  if (cw->agg == 0) {
    var = sig[0] * sig[0];
  } else if (cw->agg == 1) {
    for (int i = 0; i < d; ++i)
      for (int j = 0; j < d; ++j) {
        double c = 0.0;
        for (int k = 0; k < d; ++k) c += L[i][k] * L[j][k];
        var += sig[i] * sig[j] * c;
      }
    var /= (double)d * d;
  } else {
    for (int i = 0; i < d; ++i) var += sig[i] * sig[i];
    var /= d;
  }
  var = var + jump_var > 1e-8 ? var + jump_var : 1e-8;
  cw->inv_sig = (float)(1.0 / sqrt(var));
  cw->drift = (float)((double)I->disc_rate + 0.5 * var);
  cw->T = I->T;
  cw->scale_over_k = cw->wkind ? (float)((double)I->payoff_scale / (double)I->strike) : 1.f;
  for (int i = 0; i < MAXD; ++i) cw->inv_comp[i] = cw->comp[i] != 0.f ? (float)(1.0 / (double)cw->comp[i]) : 0.f;
  cw->inv_comp_j2 = cw->comp_j2 != 0.f ? (float)(1.0 / (double)cw->comp_j2) : 0.f;
  return SDEMC_OK;
}

/* Re-run paths [0, n) from the raw draws a GPU run exported (z (n, S, dim),
 * jump stream (n, jcap)) with the control variate accumulated: payoffs (n)
 * and regressors reg (n, 2 dim + 1).  wg (n, wcap, 2), when given, holds the
 * weights the GPU evaluated per block: they are used for the accumulation
 * (so the accumulation is compared bit for bit) and each is checked against
 * this file's own evaluation; wstat = (worst |dw| / bound, worst |dg| /
 * bound, blocks checked).  Without wg the weights are this file's own. */
int oracle_serve_cv_from_export(const sdemc_inst* I, const sdemc_cv_weights* cw, int64_t n, int S, const float* z,
                                const float* jt, const float* jm, const int32_t* js, int jcap, const float* wg,
                                int wcap, float* payoffs, float* reg, double* wstat) {
  const int D = I->dim, R = 2 * D + 1;
  int bad = 0;
  if (wstat) { wstat[0] = 0.0; wstat[1] = 0.0; wstat[2] = 0.0; }
  for (int64_t p = 0; p < n; ++p) {
    draws_t d;
    memset(&d, 0, sizeof(d));
    d.mode = DRAW_EXPORT;
    d.z = z + (size_t)p * S * D; d.zdim = D; d.S = S;
    d.xjt = jt ? jt + (size_t)p * jcap : NULL;
    d.xjm = jm ? jm + (size_t)p * jcap : NULL;
    d.xjsel = js ? js + (size_t)p * jcap : NULL;
    d.jcap = jt ? jcap : 0;
    d.h_nom = I->h; d.sq_h = sqrtf(I->h);
    cvacc_t c;
    memset(&c, 0, sizeof(c));
    c.cw = cw; c.D = D; c.wcap = wcap;
    c.wg = wg ? wg + (size_t)p * wcap * 2 : NULL;
    float x[MAXD];
    int k = run_path(I, &d, 0, S, NULL, NULL, NULL, NULL, NULL, x, &c);
    if (k < 0 || c.bad) bad = 1;
    payoffs[p] = oracle_payoff(I, x) * I->discount;
    for (int q = 0; q < R; ++q) reg[(size_t)p * R + q] = cv_reg(&c, q);
    if (wstat) {
      if (c.wstat[0] > wstat[0]) wstat[0] = c.wstat[0];
      if (c.wstat[1] > wstat[1]) wstat[1] = c.wstat[1];
      wstat[2] += c.wstat[2];
    }
  }
  return bad ? SDEMC_EOVERFLOW : SDEMC_OK;
}

/* FP32 xor butterfly over one chunk's 32 lane values (as the kernel's warp sum). */
static float butterfly(float* v) {
  float t[32];
  for (int o = 16; o > 0; o >>= 1) {
    for (int l = 0; l < 32; ++l) t[l] = v[l] + v[l ^ o];
    memcpy(v, t, sizeof(t));
  }
  return v[0];
}

/* The server kernels' per-chunk rows over per-path payoffs pv (n) and
 * regressors y (n, R).  beta == NULL: the pilot-statistics kind, W = 3 + 2R
 * + R(R+1)/2 columns (sum P, sum P^2, n, sum r_a, sum r_a r_b for a <= b,
 * sum P r_a); otherwise the control-variate kind, W = 3 over v = P - beta . r
 * (one fmaf per regressor).  Lanes past n contribute 0. */
void oracle_serve_rows(int R, int64_t n, const float* pv, const float* y, const float* beta, double* rows) {
  const int64_t nch = (n + 31) / 32;
  const int W = beta ? 3 : 3 + 2 * R + R * (R + 1) / 2;
  float lp[32], ly[32][2 * MAXD + 1], v[32];
  for (int64_t c = 0; c < nch; ++c) {
    double* out = rows + (size_t)c * W;
    int cnt = 0;
    for (int l = 0; l < 32; ++l) {
      const int64_t p = c * 32 + l;
      const int ok = p < n;
      cnt += ok;
      lp[l] = ok ? pv[p] : 0.f;
      for (int i = 0; i < R; ++i) ly[l][i] = ok ? y[(size_t)p * R + i] : 0.f;
    }
    if (beta) {
      for (int l = 0; l < 32; ++l) {
        float a = lp[l];
        for (int i = 0; i < R; ++i) a = fmaf(-beta[i], ly[l][i], a);
        v[l] = a;
      }
      float sq[32];
      for (int l = 0; l < 32; ++l) sq[l] = v[l] * v[l];
      out[0] = (double)butterfly(v); out[1] = (double)butterfly(sq); out[2] = (double)cnt;
      continue;
    }
    for (int l = 0; l < 32; ++l) { v[l] = lp[l]; }
    out[0] = (double)butterfly(v);
    for (int l = 0; l < 32; ++l) v[l] = lp[l] * lp[l];
    out[1] = (double)butterfly(v);
    out[2] = (double)cnt;
    for (int i = 0; i < R; ++i) {
      for (int l = 0; l < 32; ++l) v[l] = ly[l][i];
      out[3 + i] = (double)butterfly(v);
    }
    int q = 3 + R;
    for (int i = 0; i < R; ++i)
      for (int j = i; j < R; ++j) {
        for (int l = 0; l < 32; ++l) v[l] = ly[l][i] * ly[l][j];
        out[q++] = (double)butterfly(v);
      }
    for (int i = 0; i < R; ++i) {
      for (int l = 0; l < 32; ++l) v[l] = lp[l] * ly[l][i];
      out[q + i] = (double)butterfly(v);
    }
  }
}

/* The server's accumulation of one phase: slices of slice_chunks chunks (the
 * last one shorter), each reduced as its reduction CTA does it — thread t of
 * 256 sums chunks t, t + 256, ... in order, then a halving tree — and added
 * to the phase's running sums (starting at 0) slice after slice. */
void oracle_serve_slices(const double* rows, int64_t nchunks, int W, int64_t slice_chunks, double* acc) {
  static double sh[256];
  for (int w = 0; w < W; ++w) acc[w] = 0.0;
  for (int64_t s0 = 0; s0 < nchunks; s0 += slice_chunks) {
    const int64_t cnt = nchunks - s0 < slice_chunks ? nchunks - s0 : slice_chunks;
    for (int w = 0; w < W; ++w) {
      for (int t = 0; t < 256; ++t) {
        double a = 0.0;
        for (int64_t c = t; c < cnt; c += 256) a += rows[(size_t)(s0 + c) * W + w];
        sh[t] = a;
      }
      for (int o = 128; o > 0; o >>= 1)
        for (int t = 0; t < o; ++t) sh[t] += sh[t + o];
      acc[w] += sh[0];
    }
  }
}

/* ------------------------------------------------------------- MLMC ----- */
static int run_pair(const sdemc_inst* I, draws_t* d, int exact, int factor, float hf0, float hc0,
                    int cap, float* xf, float* xc) {
  const int D = I->dim;
  for (int i = 0; i < D; ++i) { xf[i] = I->x0[i]; xc[i] = I->x0[i]; }
  const float T = I->T;
  float tf = 0.f, tc = 0.f, hf = hf0, hc = hc0;
  float dW[MAXD], dW2[MAXD], sW[MAXD], sW2[MAXD], oldf[MAXD], oldc[MAXD];
  int kf = 0, kc = 0;
  if (I->grid == SDEMC_GRID_UNIFORM) {
    /* DiffusionSolver.multilevel_solve (sde_mc/solvers.py:90-119) */
    for (kc = 0; kc < I->num_steps; ++kc) {
      for (int i = 0; i < D; ++i) { sW[i] = 0.f; sW2[i] = 0.f; }
      for (int sub = 0; sub < factor; ++sub) {
        draws_increments(I, D, d, kf, hf, dW, dW2);
        euler(I, D, exact, xf, hf, dW, dW2);
        for (int i = 0; i < D; ++i) { sW[i] = sW[i] + dW[i]; sW2[i] = sW2[i] + dW2[i]; }
        ++kf;
      }
      euler(I, D, exact, xc, hc, sW, sW2);
    }
    return kc;
  }
  float nj = draws_jump_first(I, D, d);
  while (tf < T) {
    if (kc >= cap) return -1;
    for (int i = 0; i < D; ++i) { sW[i] = 0.f; sW2[i] = 0.f; }
    for (int sub = 0; sub < factor; ++sub) {
      hf = fminf(hf, fmaxf(T - tf, 0.f));
      float dtf = fminf(hf, nj - tf);
      draws_increments(I, D, d, kf, dtf, dW, dW2);
      memcpy(oldf, xf, sizeof(float) * D);
      euler(I, D, exact, xf, dtf, dW, dW2);
      tf = tf + dtf;
      for (int i = 0; i < D; ++i) { sW[i] = sW[i] + dW[i]; sW2[i] = sW2[i] + dW2[i]; }
      ++kf;
    }
    hc = fminf(hc, fmaxf(T - tc, 0.f));
    float dtc = fminf(hc, nj - tc);
    memcpy(oldc, xc, sizeof(float) * D);
    euler(I, D, exact, xc, dtc, sW, sW2);
    tc = tc + dtc;
    if (jump_due(nj, tf)) {
      float J; int sel;
      draws_jump_mark(d, kc, &J, &sel);
      apply_jump(I, D, exact, xf, I->exact_jumps ? xf : oldf, J, sel);
      apply_jump(I, D, exact, xc, I->exact_jumps ? xc : oldc, J, sel);
      nj = draws_jump_next(I, D, d, nj);
    }
    ++kc;
  }
  return d->overflow ? -1 : kc;
}

int oracle_mlmc_replay(const sdemc_inst* I, int factor, float hf, float hc, int bs, int Sf, int Sc,
                       int MJ, const float* jt, const float* dw, const float* marks,
                       const int32_t* asset, float* xf, float* xc) {
  const int D = I->dim, NW = nw_of(I->noise);
  int bad = 0;
  for (int p = 0; p < bs; ++p) {
    draws_t d;
    memset(&d, 0, sizeof(d));
    d.mode = DRAW_REPLAY;
    d.dw = dw + (size_t)p * Sf * D * NW;
    d.marks = marks ? marks + (size_t)p * Sc : NULL;
    d.asset = asset ? asset + (size_t)p * Sc : NULL;
    d.jt = jt ? jt + (size_t)p * MJ : NULL;
    d.S = Sf; d.MJ = jt ? MJ : 0;
    if (run_pair(I, &d, 1, factor, hf, hc, Sc, xf + (size_t)p * D, xc + (size_t)p * D) < 0) bad = 1;
  }
  return bad ? SDEMC_EOVERFLOW : SDEMC_OK;
}

/* ------------------------------------------------- native (baseline) ---- */
typedef struct {
  const sdemc_inst* I; int64_t p0, p1; int cap; int exact; int mode_mlmc; int factor;
  float hf, hc; double s, s2, f, f2; int64_t n; int bad; float* payoffs;
} job_t;

static void* job_run(void* arg) {
  job_t* j = (job_t*)arg;
  const sdemc_inst* I = j->I;
  float x[MAXD], xc[MAXD];
  for (int64_t p = j->p0; p < j->p1; ++p) {
    draws_t d;
    draws_native_init(I, &d, p);
    if (j->mode_mlmc) {
      if (run_pair(I, &d, j->exact, j->factor, j->hf, j->hc, j->cap, x, xc) < 0) j->bad = 1;
      float pf = oracle_payoff(I, x), pc = oracle_payoff(I, xc);
      float y = I->discount * (pf - pc), f = pf * I->discount;
      j->s += y; j->s2 += (double)y * y; j->f += f; j->f2 += (double)f * f;
      if (j->payoffs) j->payoffs[p] = y;
    } else {
      if (run_path(I, &d, j->exact, j->cap, NULL, NULL, NULL, NULL, NULL, x, NULL) < 0) j->bad = 1;
      float P = oracle_payoff(I, x) * I->discount;
      j->s += P; j->s2 += (double)P * P;
      if (j->payoffs) j->payoffs[p] = P;
    }
    j->n++;
  }
  return NULL;
}

static int run_jobs(const sdemc_inst* I, int nthreads, int mlmc, int factor, float hf, float hc,
                    float* payoffs, double* out) {
  if (nthreads < 1) nthreads = 1;
  if (nthreads > 256) nthreads = 256;
  job_t jobs[256];
  pthread_t th[256];
  const int64_t N = I->num_paths;
  const double lam = (double)I->rate * I->T;
  const int cap = I->num_steps + (int)(2.0 * (lam + 12.0 * sqrt(lam > 1 ? lam : 1) + 64.0)) + 8;
  for (int t = 0; t < nthreads; ++t) {
    memset(&jobs[t], 0, sizeof(job_t));
    jobs[t].I = I; jobs[t].p0 = N * t / nthreads; jobs[t].p1 = N * (t + 1) / nthreads;
    jobs[t].cap = cap; jobs[t].exact = 0; jobs[t].mode_mlmc = mlmc; jobs[t].factor = factor;
    jobs[t].hf = hf; jobs[t].hc = hc; jobs[t].payoffs = payoffs;
    pthread_create(&th[t], NULL, job_run, &jobs[t]);
  }
  double s = 0, s2 = 0, f = 0, f2 = 0;
  int64_t n = 0;
  int bad = 0;
  for (int t = 0; t < nthreads; ++t) {
    pthread_join(th[t], NULL);
    s += jobs[t].s; s2 += jobs[t].s2; f += jobs[t].f; f2 += jobs[t].f2; n += jobs[t].n; bad |= jobs[t].bad;
  }
  out[0] = s; out[1] = s2; out[2] = (double)n;
  out[3] = n > 0 ? s / n : 0.0;
  out[4] = n > 1 ? (s2 - s * s / n) / (n - 1.0) : 0.0;
  out[5] = f; out[6] = f2;
  return bad ? SDEMC_EOVERFLOW : SDEMC_OK;
}

/* Price num_paths paths natively: out = (sum, sum_sq, n, mean, var, -, -). */
int oracle_price(const sdemc_inst* I, int nthreads, float* payoffs, double* out) {
  return run_jobs(I, nthreads, 0, 1, 0.f, 0.f, payoffs, out);
}

/* One MLMC level natively: out = (sumY, sumY2, n, mean, var, sumPf, sumPf2). */
int oracle_mlmc_level(const sdemc_inst* I, int factor, float hf, float hc, int nthreads, float* ys,
                      double* out) {
  return run_jobs(I, nthreads, 1, factor, hf, hc, ys, out);
}

/* The GPU's reduction order, restated: per chunk of 32 paths (one warp
 * round) an FP32 xor butterfly of the lane values (0 for paths past n) and of
 * their squares; FP64 chunk rows; groups of 256 chunks summed by a halving
 * tree; then 256 strided FP64 accumulators over the group sums and the same
 * tree.  width 3 (price) or 5 (MLMC: vals2 is the second series).
 * out = sums..., mean, var. */
static void chunk_row(const float* vals, const float* vals2, int64_t n, int64_t c, double* row) {
  float a[32], b[32], e[32], g[32], ta[32], tb[32], te[32], tg[32];
  int cnt = 0;
  for (int l = 0; l < 32; ++l) {
    int64_t p = c * 32 + l;
    float v = p < n ? vals[p] : 0.f;
    float w = (p < n && vals2) ? vals2[p] : 0.f;
    a[l] = v; b[l] = v * v; e[l] = w; g[l] = w * w;
    cnt += p < n;
  }
  for (int o = 16; o > 0; o >>= 1) {
    for (int l = 0; l < 32; ++l) {
      ta[l] = a[l] + a[l ^ o]; tb[l] = b[l] + b[l ^ o]; te[l] = e[l] + e[l ^ o]; tg[l] = g[l] + g[l ^ o];
    }
    memcpy(a, ta, sizeof(a)); memcpy(b, tb, sizeof(b)); memcpy(e, te, sizeof(e)); memcpy(g, tg, sizeof(g));
  }
  row[0] = (double)a[0]; row[1] = (double)b[0]; row[2] = (double)cnt; row[3] = (double)e[0]; row[4] = (double)g[0];
}

void oracle_chunk_reduce(const float* vals, const float* vals2, int64_t n, double* out) {
  const int64_t nch = (n + SDEMC_CHUNK_PATHS - 1) / SDEMC_CHUNK_PATHS;
  const int width = vals2 ? 5 : 3;
  const int64_t ngroups = nch > 0 ? (nch + 255) / 256 : 1;
  double* groups = (double*)calloc((size_t)ngroups * 5, sizeof(double));
  static double sh[256][5];
  for (int64_t gi = 0; gi < ngroups; ++gi) {
    for (int t = 0; t < 256; ++t) {
      int64_t c = gi * 256 + t;
      double row[5] = {0, 0, 0, 0, 0};
      if (c < nch) chunk_row(vals, vals2, n, c, row);
      for (int w = 0; w < 5; ++w) sh[t][w] = w < width ? row[w] : 0.0;
    }
    for (int o = 128; o > 0; o >>= 1)
      for (int i = 0; i < o; ++i)
        for (int w = 0; w < width; ++w) sh[i][w] += sh[i + o][w];
    for (int w = 0; w < width; ++w) groups[gi * 5 + w] = sh[0][w];
  }
  for (int t = 0; t < 256; ++t)
    for (int w = 0; w < 5; ++w) {
      double acc = 0.0;
      if (w < width)
        for (int64_t q = t; q < ngroups; q += 256) acc += groups[q * 5 + w];
      sh[t][w] = acc;
    }
  for (int o = 128; o > 0; o >>= 1)
    for (int i = 0; i < o; ++i)
      for (int w = 0; w < width; ++w) sh[i][w] += sh[i + o][w];
  free(groups);
  for (int w = 0; w < width; ++w) out[w] = sh[0][w];
  double s = sh[0][0], s2 = sh[0][1], m = sh[0][2];
  out[width] = m > 0 ? s / m : 0.0;
  out[width + 1] = m > 1 ? (s2 - s * s / m) / (m - 1.0) : 0.0;
}
