/* A C99 host of the library, as a non-Python caller of the path would be:
   it fills a descriptor by hand (a 1-D Merton call on the jump-adapted grid),
   sizes the scratch, plans a batch and checks that malformed calls are refused
   with the documented status before any device work.  Needs no GPU.
   Exit status 0 = every check passed. */
#include <stdio.h>
#include <string.h>
#include "sdemc.h"

static int fails = 0;
#define CHECK(c) do { if (!(c)) { printf("FAIL %s:%d %s\n", __FILE__, __LINE__, #c); ++fails; } } while (0)

int main(void) {
  CHECK(sdemc_abi_version() == SDEMC_ABI_VERSION);
  CHECK(sdemc_inst_size() == sizeof(sdemc_inst));

  sdemc_inst I;
  memset(&I, 0, sizeof I);
  I.dim = 1; I.noise = SDEMC_NOISE_DIAG; I.grid = SDEMC_GRID_ADAPTED; I.num_steps = 100;
  I.mark = SDEMC_MARK_LOGNORMAL; I.jump_target = SDEMC_JUMP_COMMON; I.payoff = SDEMC_PAYOFF_EUROCALL;
  I.model = SDEMC_MODEL_AFFINE; I.seed = 1; I.num_paths = 1000;
  I.T = 1.0f; I.h = 0.01f; I.rate = 2.0f; I.inv_rate = 0.5f; I.strike = 1.0f; I.payoff_scale = 1.0f;
  I.discount = 0.98019867f; I.disc_rate = 0.02f;
  I.x0[0] = 1.0f; I.drift_b[0] = 0.04f; I.diff_q[0] = 0.2f; I.jump_k[0] = 1.0f; I.chol[0] = 1.0f;
  I.mark_p[0] = -0.1f; I.mark_p[1] = 0.2f;

  /* chunk partials: (1000 + 31) / 32 = 32 chunks, 1 group, 3 doubles each */
  CHECK(sdemc_price_scratch_bytes(&I) == 256 + (32 + 1) * 3 * 8);

  /* refused before any device work: the pointers are never dereferenced */
  void* fake = (void*)(uintptr_t)256;
  sdemc_cfg cfg;
  memset(&cfg, 0, sizeof cfg);
  cfg.interleave = 3;
  CHECK(sdemc_price_chunks(&I, &cfg, fake, (size_t)1 << 30, NULL, NULL) == SDEMC_EINVAL);
  sdemc_inst bad = I;
  bad.model = SDEMC_MODEL_HESTON;  /* Heston: 2-D, uniform grid */
  CHECK(sdemc_price_chunks(&bad, NULL, fake, (size_t)1 << 30, NULL, NULL) == SDEMC_EUNSUPPORTED);
  bad = I;
  bad.dim = 9;
  CHECK(sdemc_price_chunks(&bad, NULL, fake, (size_t)1 << 30, NULL, NULL) == SDEMC_EINVAL);
  CHECK(sdemc_price_chunks(&I, NULL, fake, 16, NULL, NULL) == SDEMC_ENOMEM);
  char msg[256];
  CHECK(sdemc_last_error(msg, sizeof msg) == SDEMC_OK && strlen(msg) > 0);

  /* a batch plan is host work: two instances of one class */
  sdemc_inst two[2] = {I, I};
  two[1].num_paths = 70;
  size_t nb = sdemc_batch_plan_bytes(2);
  static unsigned char blob[1 << 16];
  CHECK(nb > 0 && nb <= sizeof blob);
  CHECK(sdemc_batch_plan(two, 2, blob, sizeof blob) == SDEMC_OK);
  const sdemc_batch_header* H = (const sdemc_batch_header*)blob;
  CHECK(H->n_inst == 2 && H->n_class == 1 && H->total_chunks == 32 + 3);
  CHECK(sdemc_batch_scratch_bytes(blob) > 0);

  if (fails == 0) printf("c abi client ok\n");
  return fails == 0 ? 0 : 1;
}
