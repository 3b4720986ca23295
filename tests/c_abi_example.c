/* A plain C99 caller of the C ABI, driving the library the way the reference's
 * main loop drives DiskGalaxySimulator (src/nbody.cpp:31-36, 83-123): parse the same
 * positional arguments, build the reference's disk, step, read the state back.
 * Built and run by tests/test_c_abi_cpu.py and tests/test_c_abi_gpu.py. */
#include <stdio.h>
#include <stdlib.h>

#include "nbody_gb300.h"

int main(int argc, char** argv) {
  nb_params p;
  nb_params_default(&p);
  if (nb_params_parse_args(&p, argc, (const char* const*)argv) != NB_OK) {
    fprintf(stderr, "args: %s\n", nb_last_error());
    return 2;
  }
  nb_sim* sim = NULL;
  int st = nb_sim_create_disk_galaxy(&p, &sim);
  if (st == NB_ERR_NO_DEVICE) {
    printf("no device: %s\n", nb_last_error());
    return 0;
  }
  if (st != NB_OK) {
    fprintf(stderr, "create: %s: %s\n", nb_status_string(st), nb_last_error());
    return 1;
  }
  size_t n = (size_t)p.num_particles;
  float* buf = (float*)malloc(6 * n * sizeof(float));
  float ms = 0.f;
  for (int frame = 0; frame < 3; ++frame) {
    if (nb_sim_step(sim) != NB_OK || nb_sim_last_step_ms(sim, &ms) != NB_OK ||
        nb_sim_get_state(sim, buf, buf + n, buf + 2 * n, buf + 3 * n, buf + 4 * n,
                         buf + 5 * n) != NB_OK) {
      fprintf(stderr, "step: %s\n", nb_last_error());
      return 1;
    }
  }
  char name[256];
  nb_device_name(name, sizeof(name));
  printf("ok %s n=%zu last_ms=%.4f x0=%.6f\n", name, n, ms, buf[0]);
  free(buf);
  nb_sim_destroy(sim);
  return 0;
}
