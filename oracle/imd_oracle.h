/*
 * imd_oracle.h -- CPU restatement of IMD's force / neighbour-list / NVE / CG
 * hot path, used ONLY as the oracle of the tests and as the timed CPU baseline.
 *
 * This is test infrastructure.  Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / reference arm of bench.py may load it.  The GPU library in
 * imd_gb300/ never calls into it.
 *
 * Every routine restates the reference algorithm (itapmd/imd, plain C, FP64)
 * and cites the file:line it follows.  Arithmetic order is kept where it
 * decides bits (r^2, table index, cell index, wrap), and the file is built
 * with -ffp-contract=off so that no multiply-add is fused.
 *
 * Parity pin: tests/golden/ holds outputs of the reference itself, built here
 * from its own sources by oracle/Makefile (target `ref`) and driven by
 * oracle/ref_harness.c; tests/test_oracle_golden.py checks this restatement
 * against them.
 */
#ifndef IMD_ORACLE_H
#define IMD_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Function table, layout as pot_table_t (src/types.h:416-428):
 * value of column `col` at row k is table[k*ncols + col]; two extra rows
 * after maxsteps hold the extrapolation written by init_threepoint. */
typedef struct {
  int     ncols;
  int     maxsteps;
  double *begin, *end, *step, *invstep;
  int    *len;
  double *table;      /* (maxsteps + 2) * ncols */
  double *table2;     /* spline second derivatives (ORC_SPLINE only) */
  int     mode;       /* ORC_QUADRATIC, ORC_FOURPOINT, ORC_SPLINE */
} orc_table_t;

/* interpolation of the tables: the default 3-point quadratic
 * (src/potaccess.h:323-354), 4-point cubic (`4point` targets, :365-410) and
 * cubic spline (`spline` targets, :421-457) */
enum { ORC_QUADRATIC = 0, ORC_FOURPOINT = 1, ORC_SPLINE = 2 };
/* set before reading tables: how read_pot_table initialises them */
void orc_set_interpolation(int mode);

/* read_pot_table (src/imd_potential.c:161-282), formats 1 and 2
 * (:297-376, :394-462) and init_threepoint (:1256-1272).
 * `cellsz` is raised to the largest `end` of radial tables (:367, :406).
 * Returns 0 on success, nonzero with a message in err on failure. */
int  orc_read_table(orc_table_t *pt, const char *fname, int ncols, int radial,
                    int default_format, double *cellsz, char *err, int errlen);
/* Build a table from memory (format-2 semantics: begin/end/step per column,
 * len[col] values each), including the radial shift and threepoint rows. */
int  orc_make_table(orc_table_t *pt, int ncols, const double *begin,
                    const double *end, const double *step, const double *vals,
                    const int *len, int radial, double *cellsz);
void orc_free_table(orc_table_t *pt);

/* PAIR_INT2 / VAL_FUNC2 / DERIV_FUNC2 (src/potaccess.h:323-354, :465-495,
 * :591-621). */
void   orc_pair_int2(const orc_table_t *pt, int col, int inc, double r2,
                     double *pot, double *grad, int *is_short);
double orc_val_func2(const orc_table_t *pt, int col, int inc, double r2,
                     int *is_short);
double orc_deriv_func2(const orc_table_t *pt, int col, int inc, double r2,
                       int *is_short);
/* batch helpers for tests */
void orc_pair_int2_batch(const orc_table_t *pt, int col, int inc, int n,
                         const double *r2, double *pot, double *grad);

enum { ORC_PAIR = 0, ORC_EAM2 = 1 };

typedef struct {
  /* ---- parameters (set by the caller before orc_init) ---- */
  int    ntypes;
  int    interaction;         /* ORC_PAIR or ORC_EAM2 */
  double box[3][3];           /* box_x, box_y, box_z as rows */
  int    pbc[3];
  double nbl_margin;
  double timestep;
  double *restrictions;       /* 3*ntypes, 1.0 = free (NULL = all free) */
  /* CG parameters (src/globals.h:711-719 defaults set by orc_init) */
  int    linmin_maxsteps;
  double linmin_tol, linmin_dmax, linmin_dmin, cg_glimit, cg_zeps;
  int    cg_fr, cg_reset_int;
  int    cg_brent_full;       /* 1: brent over the whole bracket [a, c] (Numerical
                                 Recipes); 0: IMD's [a, b] (src/cg_utils.h:45-46) */

  orc_table_t pair, rho, embed;
  double cellsz;              /* neighbour-list radius^2 after init */

  /* ---- atoms ---- */
  int     n;
  int    *number, *type;
  double *mass;               /* n */
  double *x, *p, *f;          /* 3n, atom-major */
  double *epot, *eam_rho, *eam_df;  /* n */
  double *nbl_pos;            /* 3n */

  /* ---- derived geometry (make_box / init_cells) ---- */
  double tbox[3][3], volume, height[3];
  int    gdim[3], cdim[3];
  int    nallcells, nreal_cells;
  int   *real_cells;          /* buffered linear index, x-major */
  int   *cnbrs;               /* 14 per real cell (-1 = none) */

  /* ---- per-rebuild cell contents (ext numbering: real 0..n-1, ghosts) ---- */
  int    *cell_start, *cell_cnt, *cell_atoms;   /* CSR over nallcells */
  int     next, next_cap;
  double *ex;                 /* 3*next positions (ghosts copied) */
  int    *etype, *esrc, *eowner;  /* ghost source ext index / owning real atom */
  double *eshift;             /* 3*next copy vector for ghosts */
  double *ef, *eepot, *erho, *edf;  /* 3*next, next, next, next */
  int    *order;              /* real atoms in list order (cell order) */

  /* ---- neighbour list (make_nblist, CSR over `order`) ---- */
  int    *tl;                 /* n+1 */
  int    *tb;                 /* ext indices */
  long    nb_cap, nb_len;
  int     have_valid_nbl;
  long    nbl_count, nfc;
  int     is_short;

  /* ---- results ---- */
  double tot_pot_energy, virial, tot_kin_energy, fnorm, f_max2;

  /* ---- CG state (src/imd_cg.c) ---- */
  double *old_x, *cg_g, *cg_h;
  double cg_gamma, cg_poteng, old_cg_poteng, old_alphamin;
  long   nactive;

  /* ---- STRESS_TENS (src/imd_forces_nbl.c:548-581, :1275-1318) ---- */
  int     do_stress;          /* do_press_calc for the next calc_forces */
  double *estress;            /* 6*next: PRESSTENS xx yy zz yz zx xy */
  double *stress;             /* 6n, after the ghost fold */
  double  tot_stress[6];      /* calc_tot_presstens (src/imd_main_3d.c:2069) */

  /* ---- NVT thermostat (globals eta, isq_tau_eta, temperature) ---- */
  double  eta, isq_tau_eta, temperature;

  /* ---- P_AXIAL (src/imd_forces_nbl.c:548-553, :1275-1278): vir_xx, vir_yy,
   * vir_zz of the last calc_forces, summed beside the virial ---- */
  double  vir_axial[3];
  /* tot_pot_energy and virial of the last calc_forces by compensated
   * summation (accurate to a few ulps, unlike IMD's running sums) */
  double  tot_pot_energy_c, virial_c;
} orc_sys_t;

/* set defaults; allocate per-atom arrays for n atoms */
int  orc_init(orc_sys_t *s, int n);
void orc_free(orc_sys_t *s);
/* make_box + init_cells + make_cell_lists (src/imd_geom_3d.c:52-426,
 * :823-1044).  Call after box, tables (cellsz) and nbl_margin are set. */
int  orc_setup_geometry(orc_sys_t *s);
/* fix_cells + make_nblist (src/imd_fix_cells_3d.c:36, src/imd_forces_nbl.c:136) */
int  orc_rebuild(orc_sys_t *s);
/* calc_forces (src/imd_forces_nbl.c:281-1999), PAIR and EAM2 branches */
int  orc_calc_forces(orc_sys_t *s);
/* move_atoms_nve (src/imd_integrate.c:32-497) */
void orc_move_atoms_nve(orc_sys_t *s);
/* check_nblist (src/imd_forces_nbl.c:2007-2037) */
void orc_check_nblist(orc_sys_t *s);
/* one main_loop NVE step: calc_forces, move_atoms_nve, check_nblist */
int  orc_nve_steps(orc_sys_t *s, int nsteps, double *epot_out, double *ekin_out);
/* move_atoms_nvt (src/imd_integrate.c:891-1150, no UNIAX) and move_atoms_mik
 * (src/imd_integrate.c:675-873) */
void orc_move_atoms_nvt(orc_sys_t *s);
void orc_move_atoms_mik(orc_sys_t *s);
/* GLOK relaxer, IMD's FIRE (the `glok`, `mix` and `fire` build options):
 * update_glok (src/imd_main_3d.c:972-1055) before move_atoms_nve with its
 * GLOK / MIX branches (src/imd_integrate.c:297-316, :485-486).  Parameters
 * and state are IMD's globals (src/globals.h:425-437, :580-600). */
typedef struct {
  int    mix_on, adapt;            /* MIX, ADAPTGLOK (ADAPTGLOK needs MIX) */
  double glok_ekin_threshold, glok_fmaxcrit;
  double glok_mix, glok_mixdec;
  double glok_incfac, glok_decfac, glok_maxtimestep;
  int    glok_minsteps, min_nPxF;
  int    steps_min;
  long   nactive;                  /* <= 0: three per atom */
  int    glok_start, glok_int, nPxF;
  double mix, mixforcescalefac, PxF, pnorm;
} orc_glok_t;
/* IMD's INIT values of the parameters and the state */
void orc_glok_defaults(orc_glok_t *g);
/* update_glok for main_loop step `steps` (s->timestep may change) */
void orc_update_glok(orc_sys_t *s, orc_glok_t *g, int steps);
/* move_atoms_nve of the glok ensemble */
void orc_move_atoms_glok(orc_sys_t *s, orc_glok_t *g);
/* main_loop steps step0 .. step0+nsteps-1: calc_forces, update_glok,
 * move_atoms, check_nblist.  Per step 8 values: tot_pot_energy,
 * tot_kin_energy, fnorm, f_max2, timestep, mix, PxF, glok_start */
int  orc_glok_steps(orc_sys_t *s, orc_glok_t *g, int step0, int nsteps, double *out);
/* NPT with isotropic box scaling, move_atoms_npt_iso (src/imd_integrate.c:
 * 1475-1728, the `npt_iso` build: Nose-Hoover eta plus the barostat xi.x).
 * State and parameters are IMD's globals (src/globals.h:405-407, :566-574). */
typedef struct {
  double temperature, isq_tau_eta, eta;
  double isq_tau_xi, xi, xi_old;
  double pressure_ext, pressure_end, pressure, d_pressure;
  double Ekin_old;
  double volume_init;              /* "system seems to explode!" above 8x */
  double cell_size_tolerance;
  double min_height[3], max_height[3];
  int    use_curr_pressure, steps_min, steps_max;
  long   nactive;                  /* <= 0: three per atom */
} orc_npt_t;
void orc_npt_defaults(orc_npt_t *np);
/* init_cells again with the NPT tolerance (src/imd_geom_3d.c:128-133), as
 * IMD sets the grid up for an npt ensemble; the list is rebuilt next */
int  orc_npt_begin(orc_sys_t *s, orc_npt_t *np);
/* move_atoms_npt_iso for main_loop step `steps`, then make_box on the
 * scaled box (a new cell grid when a height leaves its bounds) */
int  orc_move_atoms_npt_iso(orc_sys_t *s, orc_npt_t *np, int steps);
/* main_loop steps step0 .. step0+nsteps-1: calc_forces, move_atoms_npt_iso,
 * check_nblist.  Per step 8 values: tot_pot_energy, tot_kin_energy, xi,
 * eta, pressure, volume, box_x.x, pressure_ext */
int  orc_npt_steps(orc_sys_t *s, orc_npt_t *np, int step0, int nsteps, double *out);
/* NPT with the box scaled per axis, move_atoms_npt_axial
 * (src/imd_integrate.c:1747-1960, the `npt_axial` build, which defines
 * P_AXIAL): per-axis barostats xi driven by the axial stresses
 * (dyn_stress + vir_xx ...) / volume, momenta restricted per type. */
typedef struct {
  double temperature, isq_tau_eta, eta;
  double isq_tau_xi;
  double xi[3], xi_old[3];
  double pressure_ext[3], pressure_end[3], d_pressure[3];
  double stress[3], dyn_stress[3];
  double Ekin_old, volume_init, cell_size_tolerance;
  double min_height[3], max_height[3];
  int    relax_dirs[3];
  int    use_curr_pressure, steps_min, steps_max;
  long   nactive;                  /* <= 0: three per atom */
} orc_npt_axial_t;
void orc_npt_axial_defaults(orc_npt_axial_t *np);
int  orc_npt_axial_begin(orc_sys_t *s, orc_npt_axial_t *np);
int  orc_move_atoms_npt_axial(orc_sys_t *s, orc_npt_axial_t *np, int steps);
/* main_loop steps: per step 12 values: tot_pot_energy, tot_kin_energy,
 * xi (3), eta, stress (3), box_x.x, box_y.y, box_z.z */
int  orc_npt_axial_steps(orc_sys_t *s, orc_npt_axial_t *np, int step0, int nsteps, double *out);
/* main_loop steps with move_atoms of `ensemble` (0 nve, 1 nvt, 2 mik);
 * per step tot_pot_energy, tot_kin_energy and (nvt) eta / (mik) fnorm */
int  orc_md_steps(orc_sys_t *s, int nsteps, int ensemble, double *epot_out,
                  double *ekin_out, double *extra_out);
/* CG: reset_cg, cg_step (src/imd_cg.c:30-66) */
int  orc_reset_cg(orc_sys_t *s);
int  orc_cg_step(orc_sys_t *s, int steps);
/* relax with CG until max per-atom |F| <= fmax (or maxsteps).
 * Returns number of cg steps (>=0) or negative on error. */
int  orc_cg_relax(orc_sys_t *s, double fmax, int maxsteps, double *fmax_out);
double orc_max_atom_force(const orc_sys_t *s);

/* neighbour pair set of the current list: per entry (number_i, number_j,
 * image shift of j relative to i as 3 ints, r2).  Returns count; fills at
 * most cap entries. */
long orc_pairs(const orc_sys_t *s, long cap, int *ni, int *nj, int *shift,
               double *r2);

#ifdef __cplusplus
}
#endif
#endif
