/* Compiled as C99 against include/lbm_gb300.h and linked with liblbm_gb300.so
 * by tests/test_c_abi_cpu.py: the header is plain C, the structs have the
 * sizes the bindings assume, and calls with bad arguments fail with
 * LBM_ERR_ARG and a message before any device work (no GPU needed). */
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include "lbm_gb300.h"

#define CHECK(cond)                                         \
  do {                                                      \
    if (!(cond)) {                                          \
      fprintf(stderr, "failed: %s (line %d)\n", #cond, __LINE__); \
      return 1;                                             \
    }                                                       \
  } while (0)

int main(void) {
  CHECK(sizeof(LbmConfig) == 120);
  CHECK(sizeof(LbmNodeLinks) == 240);
  CHECK(sizeof(LbmForceLink) == 32);
  CHECK(sizeof(LbmMovingObstacle) == 144);
  CHECK(sizeof(LbmPopView) == 56);

  LbmConfig cfg;
  memset(&cfg, 0, sizeof cfg);   /* layout LBM_POP_AB, FP64, BGK */
  cfg.nx = 8;
  cfg.ny = 6;
  cfg.omega = 2.5;               /* outside (0, 2) */
  cfg.inv_cs_2 = 3.0;
  cfg.inv_cs_4 = 9.0;
  uint8_t solid[48];
  memset(solid, 0, sizeof solid);
  LbmHandle* h = NULL;
  CHECK(lbm_create(&cfg, solid, NULL, 0, &h) == LBM_ERR_ARG);
  CHECK(h == NULL);
  CHECK(strstr(lbm_last_error(), "omega") != NULL);

  cfg.omega = 1.2;
  cfg.layout = 7;
  CHECK(lbm_create(&cfg, solid, NULL, 0, &h) == LBM_ERR_ARG);
  CHECK(strstr(lbm_last_error(), "layout") != NULL);

  cfg.layout = LBM_POP_AA;       /* no link records: the edge nodes would read outside */
  CHECK(lbm_create(&cfg, solid, NULL, 0, &h) == LBM_ERR_ARG);
  CHECK(strstr(lbm_last_error(), "no link record") != NULL);

  CHECK(lbm_step(NULL, 1) == LBM_ERR_ARG);
  CHECK(lbm_destroy(NULL) == LBM_ERR_ARG);
  float fr[48], fu[96];
  CHECK(lbm_init_fields_f32(NULL, fr, fu, LBM_LAYOUT_INNER) == LBM_ERR_ARG);
  CHECK(strstr(lbm_last_error(), "lbm_init_fields_f32") != NULL);
  CHECK(lbm_get_moments_f32(NULL, fr, fu, LBM_LAYOUT_INNER) == LBM_ERR_ARG);
  CHECK(strstr(lbm_last_error(), "lbm_get_moments_f32") != NULL);
  double out[3];
  CHECK(lbm_residual(NULL, out) == LBM_ERR_ARG);
  CHECK(lbm_residual_at(NULL, 1, out) == LBM_ERR_ARG);
  CHECK(lbm_conservation_noalloc(NULL, NULL, NULL) == LBM_ERR_ARG);
  int64_t nbytes = 0;
  CHECK(lbm_state_size(NULL, &nbytes) == LBM_ERR_ARG);
  CHECK(lbm_save_state(NULL, NULL) == LBM_ERR_ARG);
  CHECK(lbm_load_state(NULL, NULL) == LBM_ERR_ARG);
  printf("ok\n");
  return 0;
}
