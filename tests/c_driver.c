/*
 * c_driver.c -- the drop-in boundary used from C, the way IMD's shim uses it:
 * plain C types, the header include/imdgpu.h and libimdgpu.so, no Python.
 *
 * Builds an fcc Cu crystal of n^3 cubic cells (a0 3.615 A) with every atom
 * displaced by a fixed pattern, reads IMD eam2 tables (pair, rho, embed),
 * runs calc_forces and `steps` main_loop NVE steps (calc_forces,
 * move_atoms_nve, check_nblist) and prints
 *   epot0 virial0 f0x f0y f0z epot_last ekin_last nbl_count
 * usage: c_driver pair.pt rho.rho embed.emb n steps
 */
#include <stdio.h>
#include <stdlib.h>

#include "imdgpu.h"

#define CHECK(call)                                                    \
  do {                                                                 \
    int rc_ = (call);                                                  \
    if (rc_ < 0) {                                                     \
      fprintf(stderr, "%s failed: %s\n", #call, imdgpu_last_error()); \
      return 1;                                                        \
    }                                                                  \
  } while (0)

int main(int argc, char **argv) {
  if (argc < 6) {
    fprintf(stderr, "usage: %s pair rho embed n steps\n", argv[0]);
    return 2;
  }
  const int nc = atoi(argv[4]), steps = atoi(argv[5]);
  const double a0 = 3.615;
  const int n = 4 * nc * nc * nc;
  const double basis[4][3] = {{0, 0, 0}, {0.5, 0.5, 0}, {0.5, 0, 0.5}, {0, 0.5, 0.5}};
  int *number = malloc(sizeof(int) * n), *type = calloc(n, sizeof(int));
  double *mass = malloc(sizeof(double) * n), *x = malloc(sizeof(double) * 3 * n);
  double *f = malloc(sizeof(double) * 3 * n);
  int k = 0;
  for (int i = 0; i < nc; i++)
    for (int j = 0; j < nc; j++)
      for (int l = 0; l < nc; l++)
        for (int b = 0; b < 4; b++, k++) {
          number[k] = k;
          mass[k] = 63.546;
          x[3 * k] = (i + basis[b][0] + 0.25) * a0 + 0.03 * ((k * 7) % 11 - 5) / 5.0;
          x[3 * k + 1] = (j + basis[b][1] + 0.25) * a0 + 0.03 * ((k * 5) % 13 - 6) / 6.0;
          x[3 * k + 2] = (l + basis[b][2] + 0.25) * a0 + 0.03 * ((k * 3) % 7 - 3) / 3.0;
        }
  const double box[9] = {nc * a0, 0, 0, 0, nc * a0, 0, 0, 0, nc * a0};
  const int pbc[3] = {1, 1, 1};
  imdgpu_sys *s = NULL;
  CHECK(imdgpu_create(&s, 1, IMDGPU_EAM2, IMDGPU_FP64));
  CHECK(imdgpu_read_table(s, IMDGPU_TAB_PAIR, argv[1], 1, 2));
  CHECK(imdgpu_read_table(s, IMDGPU_TAB_RHO, argv[2], 1, 2));
  CHECK(imdgpu_read_table(s, IMDGPU_TAB_EMBED, argv[3], 0, 2));
  CHECK(imdgpu_set_box(s, box, pbc, 0.4, 0.0));
  CHECK(imdgpu_set_atoms(s, n, number, type, mass, x, NULL));
  CHECK(imdgpu_calc_forces(s, 0));
  imdgpu_scalars sc;
  CHECK(imdgpu_get_scalars(s, &sc));
  CHECK(imdgpu_get_atoms(s, NULL, NULL, f, NULL, NULL, NULL));
  const double e0 = sc.tot_pot_energy, v0 = sc.virial;
  for (int st = 0; st < steps; st++) {
    CHECK(imdgpu_calc_forces(s, st));
    CHECK(imdgpu_move_atoms_nve(s, 0.0982266));
    CHECK(imdgpu_check_nblist(s));
  }
  CHECK(imdgpu_get_scalars(s, &sc));
  printf("%.17e %.17e %.17e %.17e %.17e %.17e %.17e %ld\n", e0, v0, f[0], f[1], f[2],
         sc.tot_pot_energy, sc.tot_kin_energy, sc.nbl_count);
  CHECK(imdgpu_destroy(s));
  free(number); free(type); free(mass); free(x); free(f);
  return 0;
}
