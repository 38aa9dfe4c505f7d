/******************************************************************************
*
* imd_forces_cuda.c -- IMD's force, neighbour-list, integrator and CG entry
* points on libimdgpu, the GB300 implementation of that path (IMD make
* target `cuda`).
*
* This file takes the place of src/imd_forces_nbl.c in the link of IMD's
* serial NBL build.  It defines the symbols that file exports
*   calc_forces           src/imd_forces_nbl.c:281
*   make_nblist           :136
*   check_nblist          :2007
*   deallocate_nblist     :56
*   estimate_nblist_size  :74
* and the integrators that main_loop calls through the move_atoms pointer
* (src/imd_param.c:382-390): move_atoms_nve (src/imd_integrate.c:32),
* move_atoms_mik (:675) and move_atoms_nvt (:891).  The cuda target
* compiles imd_integrate.c with -Dmove_atoms_nve=move_atoms_nve_host (and
* likewise for _mik and _nvt), so IMD's own integrators keep existing under
* other names and every other IMD source compiles unchanged.  In the CG
* build (option cg) the target links this file in place of src/imd_cg.c as
* well: reset_cg and cg_step (src/imd_cg.c:30, :46) run IMD's CG on the
* device (linmin, mnbrak, brent, cg_calcgamma, set_hg).
*
* Who owns the atoms.  From the first calc_forces of a phase on, the library
* holds positions, momenta and forces on the device; the step runs there
* (calc_forces or cg_step, move_atoms_*, check_nblist), and IMD's cell
* arrays are stale.  They are brought up to date on the steps where main_loop
* reads them (src/imd_main_3d.c:690-694, :760, :792-797, :814): checkpoint,
* distribution and picture steps, the steps where it looks for a write or
* stop file, every step when a wall-time limit is set, the step where
* check_relaxed will find a MIK or CG relaxation done (it writes the relaxed
* configuration), and the last step of the phase.  After
* the last step the cell arrays are the authority again: the next phase
* uploads them (with its box and restrictions) at its first calc_forces.
*
* Atoms are matched by NUMMER: IMD's fix_cells (which main_loop still calls
* every step, on the stale host positions, or on the fresh ones after a
* copy back) may move atoms between cells and slots, so no (cell, slot)
* mapping is kept.
*
* Errors: a fatal library status becomes IMD's error() with the library's
* message; IMDGPU_WARN_SHORT is IMD's "Short distance" warning.
*
******************************************************************************/

#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "imd.h"
#include "imdgpu.h"

#if !defined(NBL)
#error "imd_forces_cuda.c serves the NBL build (make target with nbl and cuda)"
#endif
#if defined(MPI) || defined(OMP)
#error "imd_forces_cuda.c serves the serial build: one process, one GPU"
#endif

static imdgpu_sys *G = NULL;
static int host_owns_atoms = 1;   /* the cell arrays are newer than the device */
static long n_up = 0;             /* atoms of the last upload */
static int *num_caller = NULL;    /* (NUMMER, caller index) pairs, sorted by NUMMER */

static void lib_check(int rc, const char *what)
{
  char msg[640];
  if (rc >= 0) return;
  snprintf(msg, sizeof msg, "%s: %s", what, imdgpu_last_error());
  error(msg);
}

static int cmp_pair(const void *a, const void *b)
{
  const int *x = (const int *)a, *y = (const int *)b;
  return (x[0] > y[0]) - (x[0] < y[0]);
}

/* caller index of the atom with this NUMMER (binary search) */
static long caller_of(int number)
{
  long lo = 0, hi = n_up - 1;
  while (lo <= hi) {
    long mid = (lo + hi) / 2;
    int v = num_caller[2 * mid];
    if (v == number) return num_caller[2 * mid + 1];
    if (v < number) lo = mid + 1; else hi = mid - 1;
  }
  error("imd_forces_cuda: an atom number unknown to the device");
  return -1;
}

static void upload_table(int which, pot_table_t *pt)
{
  lib_check(imdgpu_set_table(G, which, pt->ncols, pt->maxsteps, pt->begin, pt->end,
                             pt->step, pt->invstep, pt->len, pt->table), "imdgpu_set_table");
#ifdef SPLINE
  lib_check(imdgpu_set_table2(G, which, pt->ncols, pt->maxsteps, pt->table2),
            "imdgpu_set_table2");
#endif
}

static void create_system(void)
{
#ifdef EAM2
  const int interaction = IMDGPU_EAM2;
#else
  const int interaction = IMDGPU_PAIR;
#endif
  lib_check(imdgpu_create(&G, ntypes, interaction, IMDGPU_FP64), "imdgpu_create");
#if defined(SPLINE)
  lib_check(imdgpu_set_interpolation(G, IMDGPU_INTERP_SPLINE), "imdgpu_set_interpolation");
#elif defined(FOURPOINT)
  lib_check(imdgpu_set_interpolation(G, IMDGPU_INTERP_FOURPOINT), "imdgpu_set_interpolation");
#endif
  upload_table(IMDGPU_TAB_PAIR, &pair_pot);
#ifdef EAM2
  upload_table(IMDGPU_TAB_RHO, &rho_h_tab);
  upload_table(IMDGPU_TAB_EMBED, &embed_pot);
#endif
}

/* box, restrictions and the atoms of IMD's cell arrays, gathered in cell
 * order (which becomes the library's caller order) */
static void upload_state(void)
{
  double box[9] = {box_x.x, box_x.y, box_x.z, box_y.x, box_y.y, box_y.z,
                   box_z.x, box_z.y, box_z.z};
  int pbc[3] = {pbc_dirs.x, pbc_dirs.y, pbc_dirs.z};
  double *restr = (double *)malloc(3 * ntypes * sizeof(double));
  long n = 0, a;
  int k, i, t;
  int *num, *typ;
  double *m, *x, *p;

  /* cellsz is IMD's list radius^2, margin included (init_cells,
   * src/imd_geom_3d.c:122-126): the library uses the same radius */
  lib_check(imdgpu_set_box(G, box, pbc, nbl_margin, cellsz), "imdgpu_set_box");
  for (t = 0; t < vtypes; t++) {
    vektor r = restrictions[t], q = restrictions[t % ntypes];
    if (r.x != q.x || r.y != q.y || r.z != q.z)
      error("imd_forces_cuda: restrictions must be the same for the virtual types of one "
            "real type");
  }
  for (t = 0; t < ntypes; t++) {
    restr[3 * t] = restrictions[t].x;
    restr[3 * t + 1] = restrictions[t].y;
    restr[3 * t + 2] = restrictions[t].z;
  }
  lib_check(imdgpu_set_restrictions(G, restr), "imdgpu_set_restrictions");
  free(restr);

  for (k = 0; k < NCELLS; k++) n += CELLPTR(k)->n;
  num = (int *)malloc(n * sizeof(int));
  typ = (int *)malloc(n * sizeof(int));
  m = (double *)malloc(n * sizeof(double));
  x = (double *)malloc(3 * n * sizeof(double));
  p = (double *)malloc(3 * n * sizeof(double));
  num_caller = (int *)realloc(num_caller, 2 * n * sizeof(int));
  if (!num || !typ || !m || !x || !p || !num_caller) error("imd_forces_cuda: out of memory");
  a = 0;
  for (k = 0; k < NCELLS; k++) {
    cell *c = CELLPTR(k);
    for (i = 0; i < c->n; i++, a++) {
      num[a] = NUMMER(c, i);
      typ[a] = SORTE(c, i);
      m[a] = MASSE(c, i);
      x[3 * a] = ORT(c, i, X);
      x[3 * a + 1] = ORT(c, i, Y);
      x[3 * a + 2] = ORT(c, i, Z);
      p[3 * a] = IMPULS(c, i, X);
      p[3 * a + 1] = IMPULS(c, i, Y);
      p[3 * a + 2] = IMPULS(c, i, Z);
      num_caller[2 * a] = num[a];
      num_caller[2 * a + 1] = (int)a;
    }
  }
  lib_check(imdgpu_set_atoms(G, (int)n, num, typ, m, x, p), "imdgpu_set_atoms");
  n_up = n;
  qsort(num_caller, n, 2 * sizeof(int), cmp_pair);
  for (a = 1; a < n; a++)
    if (num_caller[2 * a] == num_caller[2 * a - 2])
      error("imd_forces_cuda: atom numbers must be unique");
  free(num); free(typ); free(m); free(x); free(p);
  host_owns_atoms = 0;
}

/* copy the device state into IMD's cell arrays, wherever fix_cells has put
 * each atom */
static void copy_back_to_cells(void)
{
  long n = n_up, a;
  int k, i;
  double *x = (double *)malloc(3 * n * sizeof(double));
  double *p = (double *)malloc(3 * n * sizeof(double));
  double *f = (double *)malloc(3 * n * sizeof(double));
  double *e = (double *)malloc(n * sizeof(double));
#ifdef EAM2
  double *rho = (double *)malloc(n * sizeof(double));
  double *df = (double *)malloc(n * sizeof(double));
#else
  double *rho = NULL, *df = NULL;
#endif
  if (!x || !p || !f || !e) error("imd_forces_cuda: out of memory");
  lib_check(imdgpu_get_atoms(G, x, p, f, e, rho, df), "imdgpu_get_atoms");
  for (k = 0; k < NCELLS; k++) {
    cell *c = CELLPTR(k);
    for (i = 0; i < c->n; i++) {
      a = caller_of(NUMMER(c, i));
      ORT(c, i, X) = x[3 * a];
      ORT(c, i, Y) = x[3 * a + 1];
      ORT(c, i, Z) = x[3 * a + 2];
      IMPULS(c, i, X) = p[3 * a];
      IMPULS(c, i, Y) = p[3 * a + 1];
      IMPULS(c, i, Z) = p[3 * a + 2];
      KRAFT(c, i, X) = f[3 * a];
      KRAFT(c, i, Y) = f[3 * a + 1];
      KRAFT(c, i, Z) = f[3 * a + 2];
      POTENG(c, i) = e[a];
#ifdef EAM2
      EAM_RHO(c, i) = rho[a];
      EAM_DF(c, i) = df[a];
#endif
    }
  }
  free(x); free(p); free(f); free(e); free(rho); free(df);
}

#ifdef RELAX
/* check_relaxed (src/imd_main_3d.c:1741-1770) after this step will find the
 * system relaxed and write it out: the same test on the same globals, made
 * before check_relaxed updates old_epot */
static int will_be_relaxed(void)
{
  real fnorm2 = SQRT(fnorm / nactive);
  real ekin = 2 * tot_kin_energy / nactive;
  real epot = tot_pot_energy / natoms;
  real delta_epot = old_epot - epot;
  if (delta_epot < 0) delta_epot = -delta_epot;
  return (ekin < ekin_threshold) || (fnorm2 < fnorm_threshold) ||
         (delta_epot < delta_epot_threshold);
}
#endif

/* main_loop reads the cell arrays after the move of this step */
static int cells_read_after(int st)
{
  if (st >= steps_max) return 1;   /* end of the phase: final output, next phase */
  if (checkpt_int > 0 && 0 == st % checkpt_int) return 1;
  if (dist_int > 0 && 0 == st % dist_int) return 1;
  if (pic_int > 0 && 0 == st % pic_int) return 1;
  if (watch_int > 0 && 0 == st % watch_int) return 1;   /* check_write */
  if (stop_int > 0 && 0 == st % stop_int) return 1;     /* check_stop */
  if (maxwalltime > 0) return 1;                         /* check_walltime */
#ifdef RELAX
  if ((ensemble == ENS_MIK || ensemble == ENS_CG) && will_be_relaxed()) return 1;
#endif
  return 0;
}

static void after_step(int st)
{
  if (cells_read_after(st)) {
    copy_back_to_cells();
    if (st >= steps_max) host_owns_atoms = 1;
  }
}

static void read_scalars(imdgpu_scalars *sc)
{
  lib_check(imdgpu_get_scalars(G, sc), "imdgpu_get_scalars");
  nfc = (int)sc->nfc;
  nbl_count = (int)sc->nbl_count;
  have_valid_nbl = sc->have_valid_nbl;
  last_nbl_len = (int)sc->nb_entries;
}

/******************************************************************************
*  calc_forces (src/imd_forces_nbl.c:281-1999): list rebuild when needed,
*  pair and EAM2 forces, energies and virial, on the device
******************************************************************************/

void calc_forces(int steps)
{
  imdgpu_scalars sc;
  int rc;
  if (!G) create_system();
  if (host_owns_atoms) upload_state();
  rc = imdgpu_calc_forces(G, steps);
  lib_check(rc, "calc_forces");
  if (rc == IMDGPU_WARN_SHORT) fprintf(stderr, "\n Short distance, step %d!\n", steps);
  read_scalars(&sc);
  tot_pot_energy = sc.tot_pot_energy;
  virial = sc.virial;
  vir_xx = vir_yy = vir_zz = 0.0;
  vir_yz = vir_zx = vir_xy = 0.0;
}

void make_nblist(void)
{
  imdgpu_scalars sc;
  if (!G) create_system();
  if (host_owns_atoms) upload_state();
  lib_check(imdgpu_make_nblist(G), "make_nblist");
  read_scalars(&sc);
}

void check_nblist(void)
{
  imdgpu_scalars sc;
  if (!G || host_owns_atoms) return;   /* nothing on the device to check */
  lib_check(imdgpu_check_nblist(G), "check_nblist");
  read_scalars(&sc);
}

void deallocate_nblist(void)
{
  if (G) lib_check(imdgpu_deallocate_nblist(G), "deallocate_nblist");
  have_valid_nbl = 0;
}

int estimate_nblist_size(void)
{
  long entries = 0;
  if (!G) create_system();
  if (host_owns_atoms) upload_state();
  lib_check(imdgpu_estimate_nblist_size(G, &entries), "estimate_nblist_size");
  return (int)entries;
}

/******************************************************************************
*  move_atoms_nve (src/imd_integrate.c:32-497), ensemble nve
******************************************************************************/

static void read_move_scalars(void)
{
  imdgpu_scalars sc;
  read_scalars(&sc);
  tot_kin_energy = sc.tot_kin_energy;
  fnorm = sc.fnorm;
#ifdef FNORM
  f_max2 = sc.f_max2;
#endif
}

void move_atoms_nve(void)
{
  lib_check(imdgpu_move_atoms_nve(G, timestep), "move_atoms_nve");
  read_move_scalars();
  after_step(steps);
}

/******************************************************************************
*  move_atoms_mik (src/imd_integrate.c:675-873): NVE with microconvergence
******************************************************************************/

void move_atoms_mik(void)
{
#ifdef MIK
  lib_check(imdgpu_move_atoms_mik(G, timestep), "move_atoms_mik");
  read_move_scalars();
  after_step(steps);
#else
  error("the chosen ensemble MIK is not supported by this binary");
#endif
}

/******************************************************************************
*  move_atoms_nvt (src/imd_integrate.c:891-1150): Nose-Hoover NVT; eta moves
*  between IMD's global and the library every step
******************************************************************************/

void move_atoms_nvt(void)
{
#ifdef NVT
  double e = eta;
  lib_check(imdgpu_set_nvt(G, temperature, isq_tau_eta, eta, nactive), "imdgpu_set_nvt");
  lib_check(imdgpu_move_atoms_nvt(G, timestep), "move_atoms_nvt");
  lib_check(imdgpu_get_nvt(G, &e), "imdgpu_get_nvt");
  eta = e;
  read_move_scalars();
  after_step(steps);
#else
  error("the chosen ensemble NVT is not supported by this binary");
#endif
}

/******************************************************************************
*  write_atoms_config (src/imd_io_3d.c:696-948): the atom lines of every
*  configuration IMD writes in text (checkpoints, relaxed configurations),
*  formatted on the device, byte for byte what IMD's sprintf calls print, in
*  IMD's cell order.  The cuda target compiles imd_io_3d.c with
*  -Dwrite_atoms_config=write_atoms_config_host, which keeps IMD's own for
*  binary output, for virtual types, and for builds that write more fields
*  than the device formats.
******************************************************************************/

#if !defined(CNA) && !defined(UNIAX) && !defined(VARCHG) && !defined(EWALD) && \
    !defined(USEFCS) && !defined(NNBR) && !defined(REFPOS) && !defined(DISLOC) && \
    !defined(EEAM) && !defined(NORHOH) && !defined(DIPOLE) && !defined(KERMODE) && \
    !defined(DAMP) && !defined(ADA) && !defined(NYETENSOR) && !defined(LOADBALANCE) && \
    !defined(VISCOUS) && !defined(TWOD)
#define DEVICE_FORMATS_CONFIG 1
#endif

void write_atoms_config_host(FILE *out);

void write_atoms_config(FILE *out)
{
#ifdef DEVICE_FORMATS_CONFIG
  if (G && !host_owns_atoms && !binary_output && vtypes == ntypes) {
    long n = 0, a = 0, len = 0;
    int k, i, flags = 0;
    int *order;
    char *text;
    for (k = 0; k < NCELLS; k++) n += CELLPTR(k)->n;
    order = (int *)malloc((n > 0 ? n : 1) * sizeof(int));
    if (!order) error("imd_forces_cuda: out of memory");
    for (k = 0; k < NCELLS; k++) {
      cell *c = CELLPTR(k);
      for (i = 0; i < c->n; i++) order[a++] = (int)caller_of(NUMMER(c, i));
    }
    if (ensemble != ENS_CG) flags |= IMDGPU_FMT_VELOCITY;
#ifdef HPO
    flags |= IMDGPU_FMT_HPO;
#endif
#ifdef EAM2
    flags |= IMDGPU_FMT_EAM_RHO;
#endif
    lib_check(imdgpu_format_atoms(G, flags, order, (int)n, NULL, 0, &len), "imdgpu_format_atoms");
    text = (char *)malloc(len > 0 ? len : 1);
    if (!text) error("imd_forces_cuda: out of memory");
    lib_check(imdgpu_format_atoms(G, flags, order, (int)n, text, len, &len),
              "imdgpu_format_atoms");
    if (len > 0 && fwrite(text, 1, (size_t)len, out) != (size_t)len)
      error("imd_forces_cuda: writing a configuration failed");
    free(text);
    free(order);
    return;
  }
#endif
  write_atoms_config_host(out);
}

#ifdef CG
/******************************************************************************
*  reset_cg, cg_step (src/imd_cg.c:30-66): IMD's CG with its parameters
*  (linmin_*, cg_glimit, cg_zeps, cg_fr, cg_reset_int; src/globals.h:711-719)
******************************************************************************/

static void read_cg_scalars(void)
{
  imdgpu_scalars sc;
  read_scalars(&sc);
  tot_pot_energy = sc.tot_pot_energy;
  virial = sc.virial;
  fnorm = sc.fnorm;
  f_max2 = sc.f_max2;
}

void reset_cg(void)
{
  if (!G) create_system();
  if (host_owns_atoms) upload_state();
  lib_check(imdgpu_set_cg_params(G, linmin_maxsteps, linmin_tol, linmin_dmax, linmin_dmin,
                                 cg_glimit, cg_zeps, cg_fr, cg_reset_int),
            "imdgpu_set_cg_params");
  lib_check(imdgpu_reset_cg(G), "reset_cg");
  read_cg_scalars();
}

void cg_step(int st)
{
  if (host_owns_atoms) reset_cg();
  lib_check(imdgpu_cg_step(G, st), "cg_step");
  read_cg_scalars();
  after_step(st);
}
#endif
