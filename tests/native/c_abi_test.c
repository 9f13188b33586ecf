/* The public headers as plain C (C99): every header compiles without C++,
 * and the host-only entry points link and behave (no GPU needed). */
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include "gbr.h"
#include "gbr_hbao.h"
#include "gbr_noise.h"
#include "gbr_replay.h"

static int failures = 0;
#define CHECK(c)                                                             \
  do {                                                                       \
    if (!(c)) {                                                              \
      fprintf(stderr, "%s:%d: check failed: %s\n", __FILE__, __LINE__, #c); \
      ++failures;                                                            \
    }                                                                        \
  } while (0)

int main(void) {
  gbr_config cfg;
  gbr_config_init(&cfg);
  CHECK(cfg.tile_count[0] >= 1 && cfg.tile_count[1] >= 1);

  gbr_replay_config rc;
  gbr_replay_config_init(&rc);
  CHECK(rc.num_environments >= 1);

  int32_t grid[2] = {0, 0};
  CHECK(gbr_replay_environment_grid_size(10, grid) == GBR_OK);
  CHECK(grid[0] == 4 && grid[1] == 3); /* {ceil(sqrt 10), ceil(10 / 4)} */
  CHECK(gbr_replay_environment_grid_size(0, grid) != GBR_OK);
  CHECK(strlen(gbr_last_error()) > 0);

  gbr_hbao_config hc;
  gbr_hbao_config_init(&hc);
  CHECK(hc.radius > 0.0f);
  float jitter[64];
  CHECK(gbr_hbao_jitter_table(jitter) == GBR_OK);

  static float table[GBR_NORMAL_TABLE_SIZE];
  CHECK(gbr_normal_quantile_table(table, GBR_NORMAL_TABLE_SIZE) == GBR_OK);
  CHECK(table[0] < 0.0f && table[GBR_NORMAL_TABLE_SIZE - 1] > 0.0f);
  CHECK(table[GBR_NORMAL_TABLE_SIZE / 2] > -1e-6f && table[GBR_NORMAL_TABLE_SIZE / 2] < 1e-6f);
  CHECK(gbr_normal_quantile_table(table, 7) != GBR_OK);

  if (failures) {
    fprintf(stderr, "%d failures\n", failures);
    return 1;
  }
  puts("c abi ok");
  return 0;
}
