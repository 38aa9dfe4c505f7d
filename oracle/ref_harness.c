/*
 * ref_harness.c -- driver linked against objects of the UNMODIFIED reference
 * (itapmd/imd), compiled from its own sources by oracle/Makefile into
 * oracle/_ref/.  Used only in the build container to write the golden
 * vectors under tests/golden/ (tests/golden/make_golden.py) and to time the
 * reference CPU build.  Never shipped, never linked into the product.
 *
 * It replaces IMD's main() (src/imd.c:31; compiled with -Dmain=imd_main so
 * its globals stay defined there) with the same set-up sequence:
 *   read_command_line / read_parameters (src/imd_param.c:3829, :3880)
 *   setup_potentials (src/imd_potential.c:43)
 *   generate_atoms / read_atoms (src/imd_generate.c:50, src/imd_io_3d.c:44)
 *   maxwell (src/imd_main_3d.c:89)
 * and then one of
 *   forces  : calc_forces(0) and dump atoms, totals and the neighbour pairs
 *   snap K E: K main_loop steps from step 0; every E steps the state before
 *             the step and after its calc_forces
 *   nve K   : K main_loop steps calc_forces / move_atoms / check_nblist
 *             (move_atoms of the parameter file's ensemble: nve, nvt, mik)
 *   glok K  : K main_loop steps of the glok ensemble (update_glok before
 *             move_atoms) from steps_min
 *   npt K   : K main_loop steps of ensemble npt_iso or npt_axial from
 *             steps_min
 *   cg K F  : reset_cg, then cg_step until max per-atom |F| <= F
 *   time K  : K NVE steps, print cpu seconds
 */
#include "imd.h"

#include <time.h>

extern int *tl, *tb, *cl_off, *cl_num;

static void dump_state(const char *fname) {
  FILE *out = fopen(fname, "w");
  int k, i;
  fprintf(out, "# number type mass x y z px py pz fx fy fz epot rho dF\n");
  for (k = 0; k < NCELLS; k++) {
    cell *p = CELLPTR(k);
    for (i = 0; i < p->n; i++) {
      double rho = 0.0, df = 0.0;
#ifdef EAM2
      rho = EAM_RHO(p, i);
      df = EAM_DF(p, i);
#endif
      fprintf(out,
              "%ld %d %.17e %.17e %.17e %.17e %.17e %.17e %.17e %.17e %.17e "
              "%.17e %.17e %.17e %.17e\n",
              (long)NUMMER(p, i), (int)SORTE(p, i), MASSE(p, i), ORT(p, i, X),
              ORT(p, i, Y), ORT(p, i, Z), IMPULS(p, i, X), IMPULS(p, i, Y),
              IMPULS(p, i, Z), KRAFT(p, i, X), KRAFT(p, i, Y), KRAFT(p, i, Z),
              POTENG(p, i), rho, df);
    }
  }
  fclose(out);
}

static void dump_box(const char *fname) {
  FILE *out = fopen(fname, "w");
  fprintf(out, "%.17e %.17e %.17e\n%.17e %.17e %.17e\n%.17e %.17e %.17e\n",
          box_x.x, box_x.y, box_x.z, box_y.x, box_y.y, box_y.z, box_z.x,
          box_z.y, box_z.z);
  fprintf(out, "%d %d %d\n", global_cell_dim.x, global_cell_dim.y,
          global_cell_dim.z);
  fprintf(out, "%.17e\n", cellsz);
  fclose(out);
}

/* neighbour pairs: owner numbers and image shift of j (ghost cells map back
 * to the real cell they copy, same in-cell index; src/imd_comm_force_3d.c
 * copy_cell keeps the order) */
static void dump_pairs(const char *fname) {
  FILE *out = fopen(fname, "w");
  int c, i, n = 0;
  int cdx = cell_dim.x, cdy = cell_dim.y, cdz = cell_dim.z;
  for (c = 0; c < ncells; c++) {
    cell *p = cell_array + cnbrs[c].np;
    for (i = 0; i < p->n; i++) {
      int m;
      for (m = tl[n]; m < tl[n + 1]; m++) {
        int cc = cl_num[tb[m]];
        int j = tb[m] - cl_off[cc];
        cell *q = cell_array + cc;
        int bx = cc / (cdy * cdz), by = (cc / cdz) % cdy, bz = cc % cdz;
        int sx = (bx == cdx - 1) ? 1 : (bx == 0 ? -1 : 0);
        int sy = (by == cdy - 1) ? 1 : (by == 0 ? -1 : 0);
        int sz = (bz == cdz - 1) ? 1 : (bz == 0 ? -1 : 0);
        int rx = bx - sx * global_cell_dim.x, ry = by - sy * global_cell_dim.y,
            rz = bz - sz * global_cell_dim.z;
        cell *r = cell_array + (rx * cdy * cdz + ry * cdz + rz);
        vektor d;
        d.x = ORT(q, j, X) - ORT(p, i, X);
        d.y = ORT(q, j, Y) - ORT(p, i, Y);
        d.z = ORT(q, j, Z) - ORT(p, i, Z);
        fprintf(out, "%ld %ld %d %d %d %.17e\n", (long)NUMMER(p, i),
                (long)NUMMER(r, j), sx, sy, sz, SPROD(d, d));
      }
      n++;
    }
  }
  fclose(out);
}

#ifdef STRESS_TENS
/* per-atom PRESSTENS (xx yy zz yz zx xy) and calc_tot_presstens */
static void dump_stress(const char *pre) {
  char fname[600];
  int k, i;
  sprintf(fname, "%s.stress", pre);
  FILE *out = fopen(fname, "w");
  for (k = 0; k < NCELLS; k++) {
    cell *p = CELLPTR(k);
    for (i = 0; i < p->n; i++)
      fprintf(out, "%ld %.17e %.17e %.17e %.17e %.17e %.17e\n", (long)NUMMER(p, i),
              PRESSTENS(p, i, xx), PRESSTENS(p, i, yy), PRESSTENS(p, i, zz),
              PRESSTENS(p, i, yz), PRESSTENS(p, i, zx), PRESSTENS(p, i, xy));
  }
  fclose(out);
  calc_tot_presstens();
  sprintf(fname, "%s.totstress", pre);
  out = fopen(fname, "w");
  fprintf(out, "%.17e %.17e %.17e %.17e %.17e %.17e\n", tot_presstens.xx, tot_presstens.yy,
          tot_presstens.zz, tot_presstens.yz, tot_presstens.zx, tot_presstens.xy);
  fclose(out);
}
#endif

static double max_atom_force(void) {
  int k, i;
  double m = 0.0;
  for (k = 0; k < NCELLS; k++) {
    cell *p = CELLPTR(k);
    for (i = 0; i < p->n; i++) {
      double v = SQR(KRAFT(p, i, X)) + SQR(KRAFT(p, i, Y)) + SQR(KRAFT(p, i, Z));
      if (v > m) m = v;
    }
  }
  return sqrt(m);
}

int main(int argc, char **argv) {
  char fname[600];
  if (argc < 4) {
    fprintf(stderr, "usage: %s param mode outprefix [steps] [fmax]\n", argv[0]);
    return 2;
  }
  const char *mode = argv[2], *pre = argv[3];
  int nsteps = (argc > 4) ? atoi(argv[4]) : 0;
  char *cl[3] = {argv[0], "-p", argv[1]};
  read_command_line(3, cl);
  read_parameters(paramfilename, 1);
  setup_potentials();
  if ('_' == infilename[0]) generate_atoms(infilename);
  else read_atoms(infilename);
  if (0 == imdrestart) {
    if (do_maxwell) maxwell(temperature);
    do_maxwell = 0;
  }
  sprintf(fname, "%s.box", pre);
  dump_box(fname);
  sprintf(fname, "%s.state0", pre);
  dump_state(fname);

  if (0 == strcmp(mode, "forces")) {
#ifdef STRESS_TENS
    do_press_calc = 1;  /* main_loop sets it on output steps (src/imd_main_3d.c:184) */
#endif
    calc_forces(0);
#ifdef STRESS_TENS
    dump_stress(pre);
#endif
    sprintf(fname, "%s.forces", pre);
    dump_state(fname);
    sprintf(fname, "%s.pairs", pre);
    dump_pairs(fname);
    sprintf(fname, "%s.totals", pre);
    FILE *out = fopen(fname, "w");
    fprintf(out, "%.17e %.17e %ld\n", tot_pot_energy, virial, (long)natoms);
    fclose(out);
  } else if (0 == strcmp(mode, "snap")) {
    /* K main_loop steps; every `every` steps (step 0 included) the state
     * before the step, and the forces and energy of its calc_forces */
    int every = (argc > 5) ? atoi(argv[5]) : 100;
    sprintf(fname, "%s.steps", pre);
    FILE *out = fopen(fname, "w");
    for (steps = 0; steps <= nsteps; steps++) {
      if (steps % every == 0) {
        sprintf(fname, "%s.pre%05d", pre, steps);
        dump_state(fname);
      }
      calc_forces(steps);
      if (steps % every == 0) {
        sprintf(fname, "%s.snap%05d", pre, steps);
        dump_state(fname);
      }
      double ep = tot_pot_energy;
      if (steps == nsteps) {
        fprintf(out, "%d %.17e 0 %ld\n", steps, ep, (long)nbl_count);
        break;
      }
      move_atoms();
      fprintf(out, "%d %.17e %.17e %ld\n", steps, ep, tot_kin_energy, (long)nbl_count);
      check_nblist();
    }
    fclose(out);
  } else if (0 == strcmp(mode, "nve") || 0 == strcmp(mode, "time")) {
    sprintf(fname, "%s.steps", pre);
    FILE *out = fopen(fname, "w");
    clock_t t0 = clock();
    for (steps = 1; steps <= nsteps; steps++) {
      calc_forces(steps);
      double ep = tot_pot_energy;
      move_atoms();
      fprintf(out, "%d %.17e %.17e %ld", steps, ep, tot_kin_energy, (long)nbl_count);
#ifdef NVT
      fprintf(out, " %.17e", eta);  /* Nose-Hoover variable after the step */
#endif
#ifdef FNORM
      fprintf(out, " %.17e %.17e", fnorm, f_max2);
#endif
      fprintf(out, "\n");
      check_nblist();
    }
    clock_t t1 = clock();
    fclose(out);
    if (0 == strcmp(mode, "time"))
      printf("cpu_seconds %.6f atom_steps %ld\n", (double)(t1 - t0) / CLOCKS_PER_SEC,
             (long)natoms * nsteps);
    sprintf(fname, "%s.final", pre);
    dump_state(fname);
  }
#ifdef GLOK
  else if (0 == strcmp(mode, "glok")) {
    /* K main_loop steps of the glok ensemble from steps_min, in main_loop's
     * order: calc_forces, update_glok, move_atoms, check_nblist
     * (src/imd_main_3d.c:66-67, :401, :497-501, :559, :769) */
    if (glok_start <= steps_min) glok_start = steps_min;
    sprintf(fname, "%s.steps", pre);
    FILE *out = fopen(fname, "w");
    for (steps = steps_min; steps < steps_min + nsteps; steps++) {
      calc_forces(steps);
      double ep = tot_pot_energy;
      update_glok();
      move_atoms();
      double mx = 0.0, npxf = 0.0;
#ifdef MIX
      mx = mix;
#endif
#ifdef ADAPTGLOK
      npxf = nPxF;
#endif
      fprintf(out, "%d %.17e %.17e %ld %.17e %.17e %.17e %.17e %.17e %d %.0f\n", steps, ep,
              tot_kin_energy, (long)nbl_count, fnorm, f_max2, timestep, mx, PxF, glok_start,
              npxf);
      check_nblist();
    }
    fclose(out);
    sprintf(fname, "%s.final", pre);
    dump_state(fname);
  }
#endif
#ifdef NPT
  else if (0 == strcmp(mode, "npt")) {
    /* K main_loop steps of ensemble npt_iso / npt_axial from steps_min: calc_forces,
     * move_atoms (box scaled inside), check_nblist */
    sprintf(fname, "%s.steps", pre);
    FILE *out = fopen(fname, "w");
    for (steps = steps_min; steps < steps_min + nsteps; steps++) {
      calc_forces(steps);
      double ep = tot_pot_energy;
      move_atoms();
#ifdef NPT_axial
      fprintf(out, "%d %.17e %.17e %ld %.17e %.17e %.17e %.17e %.17e %.17e %.17e %.17e %.17e %.17e\n",
              steps, ep, tot_kin_energy, (long)nbl_count, xi.x, xi.y, xi.z, eta, stress_x,
              stress_y, stress_z, box_x.x, box_y.y, box_z.z);
#else
      fprintf(out, "%d %.17e %.17e %ld %.17e %.17e %.17e %.17e %.17e %.17e\n", steps, ep,
              tot_kin_energy, (long)nbl_count, xi.x, eta, pressure, volume, box_x.x,
              pressure_ext.x);
#endif
      check_nblist();
    }
    fclose(out);
    sprintf(fname, "%s.final", pre);
    dump_state(fname);
    sprintf(fname, "%s.finalbox", pre);
    dump_box(fname);
  }
#endif
#ifdef CG
  else if (0 == strcmp(mode, "cg")) {
    double ftol = (argc > 5) ? atof(argv[5]) : 1e-4;
    clock_t t0 = clock();
    reset_cg();
    double fm = max_atom_force();
    int st = 0;
    while (fm > ftol && st < nsteps) {
      st++;
      steps = st;
      cg_step(st);
      fm = max_atom_force();
      check_nblist();
    }
    clock_t t1 = clock();
    sprintf(fname, "%s.cg", pre);
    FILE *out = fopen(fname, "w");
    fprintf(out, "%d %ld %.17e %.17e %.6f\n", st, (long)nfc, tot_pot_energy, fm,
            (double)(t1 - t0) / CLOCKS_PER_SEC);
    fclose(out);
    sprintf(fname, "%s.final", pre);
    dump_state(fname);
  }
#endif
  return 0;
}
