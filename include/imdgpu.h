/*
 * imdgpu.h -- C-ABI of the GB300 replacement for IMD's force, neighbour-list,
 * NVE and CG hot path (itapmd/imd).
 *
 * Plain C types only: opaque handles, pointers and sizes.  Every function
 * returns an int status (IMDGPU_OK = 0, > 0 recoverable, < 0 fatal; the
 * message is in imdgpu_last_error()).  Kernels never trap; device-side
 * problems (list or cell overflow, short distances, CG failures) are
 * reported through status words that these calls read back.
 *
 * Data ownership follows the reference's calc_forces contract
 * (src/imd_forces_nbl.c:281): the caller owns the atoms; the library keeps a
 * device-resident, cell-sorted mirror, and copies in/out only on request.
 * Atom arrays exchanged through this interface are in the caller's order
 * (the order of imdgpu_set_atoms), atom-major (x[3*i+c]).
 */
#ifndef IMDGPU_H
#define IMDGPU_H

#ifdef __cplusplus
extern "C" {
#endif

#define IMDGPU_OK 0
#define IMDGPU_WARN_SHORT 1       /* a pair closer than a table's begin (IMD: "Short distance") */
#define IMDGPU_ERR_ARG (-1)
#define IMDGPU_ERR_CUDA (-2)
#define IMDGPU_ERR_NOMEM (-3)
#define IMDGPU_ERR_GEOM (-4)      /* box too small for one cell of list radius */
#define IMDGPU_ERR_TABLE (-5)
#define IMDGPU_ERR_BRENT (-6)     /* "Too many iterations in brent" */
#define IMDGPU_ERR_CELL (-7)      /* more atoms in one cell than supported */
#define IMDGPU_ERR_STATE (-8)     /* call order (e.g. forces before atoms) */

#define IMDGPU_PAIR 0             /* pair potential only (target imd_*_nbl) */
#define IMDGPU_EAM2 1             /* pair + EAM2 (target imd_*_nbl_eam) */

#define IMDGPU_FP64 0             /* all arithmetic in FP64 */
#define IMDGPU_MIXED 1            /* pair/EAM arithmetic in FP32 on cell-relative
                                     coordinates, FP64 positions/accumulation */

#define IMDGPU_TAB_PAIR 0
#define IMDGPU_TAB_RHO 1
#define IMDGPU_TAB_EMBED 2

typedef struct imdgpu_sys imdgpu_sys;

/* Global results of the last calls; same meaning as IMD's globals
 * (src/globals.h:405-412, :1444 onwards). */
typedef struct {
  double tot_pot_energy;   /* calc_forces */
  double virial;           /* calc_forces */
  double tot_kin_energy;   /* move_atoms_nve (half-step average) */
  double fnorm;            /* sum |F|^2 (move_atoms_nve / calc_fnorm) */
  double f_max2;           /* max squared force component */
  double max_atom_force;   /* max per-atom |F| (CG stopping rule) */
  long nfc;                /* force calls */
  long nbl_count;          /* neighbour-list builds */
  long nb_entries;         /* entries of the current list */
  int have_valid_nbl;
  int gdim[3];             /* global_cell_dim */
  int nghost;              /* buffer-cell (ghost) atoms of the last build */
  int max_cell_atoms;
  int short_distance;      /* nonzero if a pair was below a table begin */
} imdgpu_scalars;

const char *imdgpu_last_error(void);
const char *imdgpu_version(void);
int imdgpu_device_count(int *count);
/* select the CUDA device for systems created afterwards by this thread */
int imdgpu_set_device(int device);

/* Replaces IMD's implicit single global system (src/globals.h). */
int imdgpu_create(imdgpu_sys **sys, int ntypes, int interaction, int precision);
int imdgpu_destroy(imdgpu_sys *sys);
/* 1: evaluate tables with IMD's own unfused formulas (bitwise table values,
 * parity mode); 0 (default): coefficient form with FMA, same results to
 * ~1e-16 relative */
int imdgpu_set_exact(imdgpu_sys *sys, int on);
/* precision may be switched between calls (the list is kept) */
int imdgpu_set_precision(imdgpu_sys *sys, int precision);
/* Deterministic reduction mode for parity runs (no counterpart in IMD,
 * whose serial loops sum in a fixed order, src/imd_forces_nbl.c:907-918).
 * 1: the FP64 density and force passes run on the full neighbour list, each
 * atom's sums formed by one quad of lanes in list order and a fixed shuffle
 * tree, with no atomics, so repeated runs are bitwise equal; about twice the
 * pair arithmetic of the default half-list passes, whose FP64 atomics make
 * the last bits vary from run to run.  One system, FP64; imdgpu_calc_stress,
 * npt_axial and imdgpu_get_pairs need the half list and refuse this mode. */
int imdgpu_set_deterministic(imdgpu_sys *sys, int on);

/* Upload one pot_table_t (src/types.h:416-428) exactly as IMD holds it
 * after read_pot_table + init_threepoint (src/imd_potential.c:161-282,
 * :1256-1272): value of column col at row k is table[k*ncols + col], with
 * (maxsteps + 2) rows.  `which` is IMDGPU_TAB_*. */
int imdgpu_set_table(imdgpu_sys *sys, int which, int ncols, int maxsteps,
                     const double *begin, const double *end, const double *step,
                     const double *invstep, const int *len, const double *table);
/* Interpolation of tables uploaded from now on, as IMD's make targets
 * select it: 0 = 3-point quadratic (default, src/potaccess.h:323),
 * 1 = 4-point cubic (`4point`, :365), 2 = cubic spline (`spline`, :421). */
#define IMDGPU_INTERP_QUADRATIC 0
#define IMDGPU_INTERP_FOURPOINT 1
#define IMDGPU_INTERP_SPLINE 2
int imdgpu_set_interpolation(imdgpu_sys *sys, int mode);
/* spline builds: pot_table_t.table2 of the next imdgpu_set_table(which) */
int imdgpu_set_table2(imdgpu_sys *sys, int which, int ncols, int maxsteps,
                      const double *table2);
/* Read an IMD potential file (formats 1 and 2, src/imd_potential.c:161-462)
 * on the host and upload it.  radial as in read_pot_table. */
int imdgpu_read_table(imdgpu_sys *sys, int which, const char *fname, int radial,
                      int default_format);

/* Box rows box_x, box_y, box_z (box[3*a+c]), periodicity, list margin
 * (nbl_margin, src/globals.h:419).  list_r2 > 0 overrides the neighbour
 * list radius^2 (IMD's cellsz after init_cells); 0 derives it as
 * (sqrt(max radial table end) + nbl_margin)^2 like init_cells
 * (src/imd_geom_3d.c:122-126). */
int imdgpu_set_box(imdgpu_sys *sys, const double *box, const int *pbc, double nbl_margin,
                   double list_r2);
/* per-type restriction vectors (src/globals.h:206), 3*ntypes, 1 = free */
int imdgpu_set_restrictions(imdgpu_sys *sys, const double *restr);

/* Atoms: NUMMER, SORTE, MASSE, ORT (3n), IMPULS (3n, may be NULL).
 * IMDGPU_ERR_ARG for a non-finite position or momentum or a mass <= 0. */
int imdgpu_set_atoms(imdgpu_sys *sys, int n, const int *number, const int *type,
                     const double *mass, const double *x, const double *p);
/* Replace positions and momenta (caller order, 3n each; p may be NULL)
 * without touching the neighbour list: the state IMD's cell arrays hand
 * back to calc_forces each step when they live on the host.  A non-finite
 * value is IMDGPU_ERR_ARG (checked on the device after the copy) and leaves
 * the device state as it was. */
int imdgpu_put_state(imdgpu_sys *sys, const double *x, const double *p);
/* Copy state back (any pointer may be NULL): x, p, f (3n), epot (n),
 * eam_rho, eam_df (n). */
int imdgpu_get_atoms(imdgpu_sys *sys, double *x, double *p, double *f, double *epot,
                     double *eam_rho, double *eam_df);
int imdgpu_get_scalars(imdgpu_sys *sys, imdgpu_scalars *out);
/* One NVE step of main_loop for a caller whose state lives on the host:
 * x and p (caller order, 3n each) up, calc_forces, move_atoms_nve with
 * check_nblist's displacement test, the new x and p down to x_out / p_out
 * (either may be NULL; they may be x and p themselves) and the scalars to
 * *out (may be NULL), with one synchronisation.  A non-finite input is
 * IMDGPU_ERR_ARG and moves no atom. */
int imdgpu_nve_step_host(imdgpu_sys *sys, const double *x, const double *p, double timestep,
                         double *x_out, double *p_out, imdgpu_scalars *out);

/* calc_forces (src/imd_forces_nbl.c:281-1999): fix_cells + make_nblist when
 * the list is invalid, then pair / EAM2 forces, energies and virial. */
int imdgpu_calc_forces(imdgpu_sys *sys, int steps);
/* calc_forces of a step with do_press_calc set, in the `stress` build
 * (STRESS_TENS, src/Makefile:1587-1588): forces as imdgpu_calc_forces, and
 * every atom's PRESSTENS (src/imd_forces_nbl.c:558-580, :1284-1318; ghost
 * parts folded into their owners as src/imd_comm_force_3d.c:916) into
 * presstens (6 per atom, caller order: xx yy zz yz zx xy; may be NULL), and
 * their sum, calc_tot_presstens (src/imd_main_3d.c:2069), into tot (6, may
 * be NULL).  FP64 precision only. */
int imdgpu_calc_stress(imdgpu_sys *sys, double *presstens, double *tot);
/* make_nblist (src/imd_forces_nbl.c:136-273): wrap, bin and rebuild now */
int imdgpu_make_nblist(imdgpu_sys *sys);
/* check_nblist (src/imd_forces_nbl.c:2007-2037) */
int imdgpu_check_nblist(imdgpu_sys *sys);
/* deallocate_nblist (src/imd_forces_nbl.c:56-64): drop the list */
int imdgpu_deallocate_nblist(imdgpu_sys *sys);
/* estimate_nblist_size (src/imd_forces_nbl.c:74-128): entries of a fresh list */
int imdgpu_estimate_nblist_size(imdgpu_sys *sys, long *entries);
/* move_atoms_nve (src/imd_integrate.c:32-497) */
int imdgpu_move_atoms_nve(imdgpu_sys *sys, double timestep);
/* move_atoms_mik (src/imd_integrate.c:675-873): NVE with microconvergence
 * (a momentum against the force is set to zero) */
int imdgpu_move_atoms_mik(imdgpu_sys *sys, double timestep);
/* move_atoms_nvt (src/imd_integrate.c:891-1150): Nose-Hoover NVT.  Its state
 * is IMD's globals temperature (kT), isq_tau_eta (1/tau_eta^2), eta and
 * nactive (degrees of freedom; <= 0 means 3 per atom), set once with
 * imdgpu_set_nvt; each call advances eta as IMD does, imdgpu_get_nvt reads
 * it. */
int imdgpu_set_nvt(imdgpu_sys *sys, double temperature, double isq_tau_eta, double eta,
                   long nactive);
int imdgpu_get_nvt(imdgpu_sys *sys, double *eta);
int imdgpu_move_atoms_nvt(imdgpu_sys *sys, double timestep);
/* The glok ensemble, IMD's FIRE relaxer (build options `glok`, `mix`,
 * `fire`; src/Makefile:1529-1548).  Parameters as IMD parses them
 * (src/imd_param.c:1569-1650), defaults from imdgpu_glok_defaults (IMD's
 * INIT values, src/globals.h:580-600). */
typedef struct {
  int mix;                     /* MIX: momenta turned towards the forces */
  int adapt;                   /* ADAPTGLOK: adaptive time step (needs mix) */
  double glok_ekin_threshold, glok_fmaxcrit;
  double glok_mix, glok_mixdec;
  double glok_incfac, glok_decfac, glok_maxtimestep;
  int glok_minsteps, min_nPxF;
  int steps_min;               /* first main_loop step of the phase */
  long nactive;                /* degrees of freedom; <= 0: 3 per atom */
} imdgpu_glok_params;
/* IMD's globals of the glok state after the last call */
typedef struct {
  double timestep;             /* the adaptive time step */
  double mix, mixforcescalefac;
  double PxF;                  /* P.F / (|F| |P/m|) of the last move */
  double pnorm;                /* sum |P/m|^2 of the last move */
  int glok_start, glok_int, nPxF;
} imdgpu_glok_state;
int imdgpu_glok_defaults(imdgpu_glok_params *prm);
/* start a glok phase: parameters, the start time step (IMD's
 * starttimestep), the state of IMD's globals before the first step */
int imdgpu_set_glok(imdgpu_sys *sys, const imdgpu_glok_params *prm, double timestep);
/* update_glok (src/imd_main_3d.c:972-1055) for main_loop step `steps`,
 * then move_atoms_nve with the GLOK and MIX branches
 * (src/imd_integrate.c:297-316, :485-486): what main_loop runs between
 * calc_forces and check_nblist for `ensemble glok` */
int imdgpu_move_atoms_glok(imdgpu_sys *sys, int steps);
int imdgpu_get_glok(imdgpu_sys *sys, imdgpu_glok_state *st);
/* NPT with isotropic box scaling, move_atoms_npt_iso
 * (src/imd_integrate.c:1475-1728, build option `npt_iso`): the Nose-Hoover
 * eta of NVT plus the barostat xi; the box is scaled after every step, and
 * the cell grid is set up again when a box height leaves its bounds
 * (make_box, src/imd_geom_3d.c:82-86).  Parameters as IMD parses them
 * (src/imd_param.c:2562-2599; defaults src/globals.h:566-574).  FP64,
 * one system. */
typedef struct {
  double temperature, isq_tau_eta, eta;  /* as for imdgpu_set_nvt */
  double isq_tau_xi, xi;
  double pressure_ext, pressure_end;     /* pressure_start, pressure_end */
  int use_curr_pressure;                 /* use_current_pressure */
  int steps_min, steps_max;              /* the ramp of pressure_ext */
  long nactive;                          /* <= 0: 3 per atom */
  double cell_size_tolerance;            /* cell_size_tol */
} imdgpu_npt_params;
typedef struct {
  double xi, eta, pressure, pressure_ext, volume;
  double box[9];                         /* rows box_x, box_y, box_z */
} imdgpu_npt_state;
int imdgpu_npt_defaults(imdgpu_npt_params *prm);
/* start an npt_iso phase; the cell grid is set up with IMD's NPT
 * tolerance at the next calc_forces */
int imdgpu_set_npt(imdgpu_sys *sys, const imdgpu_npt_params *prm);
/* move_atoms_npt_iso for main_loop step `steps` */
int imdgpu_move_atoms_npt_iso(imdgpu_sys *sys, int steps, double timestep);
int imdgpu_get_npt(imdgpu_sys *sys, imdgpu_npt_state *st);
/* NPT with a barostat per axis, move_atoms_npt_axial
 * (src/imd_integrate.c:1747-1960, build option npt_axial, which adds
 * P_AXIAL): each axis a has its own xi[a], driven by its axial stress
 * (dyn_stress_a + vir_aa) / volume against pressure_ext[a]; relax_dirs[a] = 0
 * holds an axis; the momenta are masked by the restrictions after the
 * update; box row a is scaled by its own factor, with make_box and a new
 * cell grid as in npt_iso.  While a phase is set, calc_forces also sums
 * IMD's P_AXIAL virial components vir_xx, vir_yy, vir_zz
 * (src/imd_forces_nbl.c:548-553, :1275-1278).  Parameters as IMD parses
 * them (src/imd_param.c:2562-2640).  FP64, one system. */
typedef struct {
  double temperature, isq_tau_eta, eta;  /* as for imdgpu_set_nvt */
  double isq_tau_xi;
  double xi[3];
  double pressure_ext[3], pressure_end[3];  /* pressure_start, pressure_end per axis */
  int relax_dirs[3];                        /* 1: the axis is coupled, 0: held */
  int use_curr_pressure;
  int steps_min, steps_max;
  long nactive;                             /* <= 0: 3 per atom */
  double cell_size_tolerance;
} imdgpu_npt_axial_params;
typedef struct {
  double xi[3], eta;
  double stress[3];                      /* IMD's stress_x, stress_y, stress_z */
  double pressure_ext[3];
  double vir_axial[3];                   /* vir_xx, vir_yy, vir_zz of the last calc_forces */
  double volume;
  double box[9];
} imdgpu_npt_axial_state;
int imdgpu_npt_axial_defaults(imdgpu_npt_axial_params *prm);
int imdgpu_set_npt_axial(imdgpu_sys *sys, const imdgpu_npt_axial_params *prm);
/* move_atoms_npt_axial for main_loop step `steps` */
int imdgpu_move_atoms_npt_axial(imdgpu_sys *sys, int steps, double timestep);
int imdgpu_get_npt_axial(imdgpu_sys *sys, imdgpu_npt_axial_state *st);
/* nsteps of main_loop (src/imd_main_3d.c:155-870) for ensemble nve:
 * calc_forces, move_atoms_nve, check_nblist, fully on the device.
 * epot/ekin (may be NULL) receive tot_pot_energy and tot_kin_energy of every
 * step. */
int imdgpu_nve_run(imdgpu_sys *sys, int nsteps, double timestep, double *epot,
                   double *ekin);

/* CG (src/imd_cg.c): reset_cg (:30-38), cg_step (:46-66, linmin/mnbrak/brent
 * of src/cg_utils.h:34-194), and a driver that stops on the max per-atom
 * force (the threshold IMD parses as f_max_threshold, src/imd_param.c:850). */
int imdgpu_set_cg_params(imdgpu_sys *sys, int linmin_maxsteps, double linmin_tol,
                         double linmin_dmax, double linmin_dmin, double cg_glimit,
                         double cg_zeps, int cg_fr, int cg_reset_int);
int imdgpu_reset_cg(imdgpu_sys *sys);
int imdgpu_cg_step(imdgpu_sys *sys, int steps);
int imdgpu_cg_relax(imdgpu_sys *sys, double fmax, int maxsteps, int *steps_done,
                    double *fmax_out);

/* Batched CG: many independent periodic cells in one handle (create it with
 * imdgpu_create, upload tables, then call imdgpu_batch_set_cells instead of
 * imdgpu_set_box / imdgpu_set_atoms).  natoms[ncells]; boxes 9 per cell
 * (rows box_x, box_y, box_z); atom arrays grouped by cell, caller order.
 * Every cell runs IMD's CG (reset_cg, then cg_step = linmin/mnbrak/brent,
 * cg_calcgamma, set_hg; src/imd_cg.c, src/cg_utils.h) until its max
 * per-atom |F| <= fmax; one device thread per cell keeps the line-search
 * state, all cells' force evaluations run together.  New: IMD relaxes one
 * cell per process. */
int imdgpu_batch_set_cells(imdgpu_sys *sys, int ncells, const int *natoms,
                           const double *boxes, const int *number, const int *type,
                           const double *mass, const double *x);
int imdgpu_batch_set_margin(imdgpu_sys *sys, double nbl_margin);
int imdgpu_batch_relax(imdgpu_sys *sys, double fmax, int maxsteps, int max_rounds,
                       int *rounds_done);
/* the same in two parts: set up (reset_cg state of every cell), then run up
 * to max_rounds more rounds; *ndone = cells finished so far */
int imdgpu_batch_begin(imdgpu_sys *sys, double fmax, int maxsteps);
int imdgpu_batch_advance(imdgpu_sys *sys, int max_rounds, int *ndone, int *rounds);
/* Compaction: once the unfinished cells hold at most pct % of the atoms on
 * the device, the finished cells leave the device batch (their results and
 * final positions stay with the handle), so that later rounds cost what the
 * unfinished cells cost.  Default 50; 0 turns it off.  Calls that need every
 * cell (imdgpu_batch_begin, imdgpu_get_atoms, imdgpu_calc_forces, the ml_
 * calls) bring all cells back first.  New: IMD has no batches. */
int imdgpu_batch_set_compaction(imdgpu_sys *sys, int pct);
/* positions of every atom of imdgpu_batch_set_cells (3 per atom, in that
 * order), whether or not its cell is still on the device */
int imdgpu_batch_positions(imdgpu_sys *sys, double *x);
/* neighbour-list rebuilds since imdgpu_batch_begin */
int imdgpu_batch_rebuilds(imdgpu_sys *sys, long *n);
/* cells finished since imdgpu_batch_begin and the atoms of the unfinished
 * ones (either pointer may be NULL) */
int imdgpu_batch_progress(imdgpu_sys *sys, int *ndone, long *active_atoms);
/* per cell: final energy, max |F|, CG steps, force calls (nfc), status
 * (0 converged, 1 not converged within maxsteps or the rounds, 2 "Too many
 * iterations in brent", 3 line-search control failure, 4 five line
 * searches in a row ended, without lowering the energy, on a point with a
 * pair closer than a table's first point (IMD's "Short distance"), where the
 * tables clamp and energy and forces no longer match, so CG cannot leave
 * it: the cell is stopped) */
int imdgpu_batch_results(imdgpu_sys *sys, double *epot, double *fmax, int *steps, int *nfc,
                         int *status);

/* Learned starting guess for CG (no counterpart in IMD).  Per directed pair
 * (i, j) with r_ij < 5.5 A: x_ij = [16 Gaussian RBF(r_ij), rho_i/100] ->
 * 64 -> 64 -> 1 (SiLU, BF16 weights, FP32 accumulation) = w_ij; predicted
 * displacement dx_i = sum_j w_ij (r_j - r_i)/r_ij.  Weights: a flat FP32
 * array of imdgpu_ml_nparam() values (W1[64][32] with inputs >= 17 zero,
 * b1[64], W2[64][64], b2[64], W3[64], b3). */
int imdgpu_ml_nparam(void);
/* The forward pass on the fifth-generation tensor cores (tcgen05.mma into
 * tensor memory, 128 pairs per CTA) instead of mma.sync (default 0).  The
 * backward pass stays on mma.sync.  Not yet run on a GPU: off by default. */
int imdgpu_ml_set_tensor_cores(imdgpu_sys *sys, int on);
int imdgpu_ml_set_weights(imdgpu_sys *sys, const float *w, int n);
int imdgpu_ml_get_weights(imdgpu_sys *sys, float *w, int n);
/* Adam first and second moments (imdgpu_ml_nparam() floats each) and step
 * count; with the weights they carry one model's training state from one
 * handle to another (imdgpu_ml_set_weights clears them). */
int imdgpu_ml_get_adam(imdgpu_sys *sys, float *m, float *v, int *step);
int imdgpu_ml_set_adam(imdgpu_sys *sys, const float *m, const float *v, int step);
/* dx (3n, caller order) at the current positions */
int imdgpu_ml_predict(imdgpu_sys *sys, double *dx);
/* loss = sum_i w_i |dx_i - target_i|^2 / n and its gradient (grad may be
 * NULL), w_i = 1 unless imdgpu_ml_set_loss_weights set them;
 * lr > 0: one Adam step (beta 0.9 / 0.999) on the weights */
int imdgpu_ml_train_step(imdgpu_sys *sys, const double *target, double lr, double *loss,
                         float *grad);
/* per-atom weights w_i >= 0 of that loss (n, caller order; NULL: all 1) */
int imdgpu_ml_set_loss_weights(imdgpu_sys *sys, const double *w);
/* Learned start of a batch (after imdgpu_batch_set_cells and
 * imdgpu_ml_set_weights, before imdgpu_batch_begin): per cell the energy
 * at the current positions (e_start), the energy after adding the predicted
 * displacements (e_pred), and used[c] = (e_pred < e_start).  Cells with
 * used[c] == 1 keep the displaced positions, the others go back to theirs;
 * CG then relaxes every cell from its chosen start.  Two force calls.  Any
 * output pointer may be NULL. */
int imdgpu_batch_ml_start(imdgpu_sys *sys, int *used, double *e_start, double *e_pred);

/* IMD's checkpoint text formatted on the device: the atom lines of
 * write_atoms_config (src/imd_io_3d.c:696-948, text branch), byte for byte
 * what its sprintf calls print, so that writing a checkpoint of a large
 * system needs neither the state on the host nor 10 printf conversions per
 * atom there.  Per atom: "%d %d" NUMMER and type, RESOL1 mass, RESOL3
 * position, RESOL3 velocity (momentum / mass; with IMDGPU_FMT_VELOCITY, as
 * every ensemble but CG writes it), RESOL1 POTENG of the last calc_forces,
 * RESOL1 EAM_RHO (with IMDGPU_FMT_EAM_RHO, the EAM2 builds), "\n"; RESOL1
 * is " %12.16f" with IMDGPU_FMT_HPO (IMD's hpo option) and " %f" without
 * (:704-711).  order: n caller indices, the order of the lines (IMD writes
 * cell by cell), or NULL for all atoms in caller order.  *len receives the
 * size of the text; buf (host) receives it when cap >= *len, so a first call
 * with cap = 0 sizes it.  A value of magnitude 2^63 or more is
 * IMDGPU_ERR_ARG. */
#define IMDGPU_FMT_HPO 1
#define IMDGPU_FMT_VELOCITY 2
#define IMDGPU_FMT_EAM_RHO 4
int imdgpu_format_atoms(imdgpu_sys *sys, int flags, const int *order, int n, char *buf,
                        long cap, long *len);
/* The formatter alone: n doubles (host), each as printf("%*.*f\n", width,
 * prec, x) (prec 0..17, width 0..64), into buf as imdgpu_format_atoms. */
int imdgpu_format_fixed(const double *x, int n, int prec, int width, char *buf, long cap,
                        long *len);

/* Neighbour pairs of the current list: NUMMER of both atoms, image shift of
 * the second (3 ints, in box vectors) and r^2 as used for the list test.
 * With cap == 0 only *count is set. */
int imdgpu_get_pairs(imdgpu_sys *sys, long cap, int *ni, int *nj, int *shift,
                     double *r2, long *count);

/* Autotuner (no counterpart in IMD): the density pass, then the force
 * pass, run with blocks of 32, 64, 96 and 128 threads on the current list,
 * timed with CUDA events; the fastest of each is kept for this system until
 * its size, precision or number of cells changes.  The chosen blocks go to
 * *block_density and *block_force (either may be NULL).
 * imdgpu_batch_begin tunes every new batch shape first unless
 * imdgpu_batch_set_autotune(sys, 0); imdgpu_set_blocks fixes them by hand
 * (multiples of 32, at most 128). */
int imdgpu_autotune(imdgpu_sys *sys, int *block_density, int *block_force);
int imdgpu_set_blocks(imdgpu_sys *sys, int block_density, int block_force);
/* The tile the autotuner chose besides the blocks: lanes per atom (1, 2 or
 * 4) of the FP64 pair passes with the pair cache and of the mixed density
 * pass of one species. */
int imdgpu_get_tile(imdgpu_sys *sys, int *lanes_per_atom);
int imdgpu_batch_set_autotune(imdgpu_sys *sys, int on);
/* A batch round's CG work (the sums of the last evaluation, the control of
 * every cell, the move and set_hg of its atoms, the list displacement test)
 * runs in one persistent kernel whose resident blocks take cells largest
 * first (default 1); 0 runs it as four kernels, with the same arithmetic. */
int imdgpu_batch_set_engine(imdgpu_sys *sys, int on);
/* Per-system rebuilds (default 0): every cell of the batch gets a fixed
 * ghost range with head-room, and a round rebuilds the lists of the cells
 * that moved past skin/2 only, instead of the whole batch. */
int imdgpu_batch_set_partial_rebuild(imdgpu_sys *sys, int on);
/* List capacity of a batch at imdgpu_batch_begin and after a compaction:
 * factor x the most entries an atom has (default 1.3, within [1, 4]).  A
 * chunk of rounds that overflows the list or the ghosts is replayed from
 * its start with grown buffers; imdgpu_batch_replays counts those replays
 * since imdgpu_batch_begin. */
int imdgpu_batch_set_list_headroom(imdgpu_sys *sys, double factor);
int imdgpu_batch_replays(imdgpu_sys *sys, long *n);
/* Test hook for the replay path, no counterpart in the reference: after
 * every `every` completed chunks of imdgpu_batch_advance, the next chunk is
 * replayed from its snapshot as if it had overflowed (without growing a
 * buffer), `count` times in all; call after imdgpu_batch_begin.  The
 * replays are counted by imdgpu_batch_replays. */
int imdgpu_batch_inject_replays(imdgpu_sys *sys, int every, int count);

/* Timing of the dominant kernels of the last nve_run (device ms, CUDA
 * events on the system's stream). */
typedef struct {
  double ms_total;
  double ms_density;
  double ms_force;
  double ms_integrate;
  double ms_rebuild;
  int steps;
  int rebuilds;
  long kernel_launches;
} imdgpu_timing;
int imdgpu_get_timing(imdgpu_sys *sys, imdgpu_timing *out);
/* enable per-kernel event timing in nve_run (adds event records) */
int imdgpu_set_profiling(imdgpu_sys *sys, int on);
/* Between the steps of nve_run write `bytes` of scratch so that each timed
 * step starts with a cold L2 (benchmarking); the write is outside the timed
 * windows.  0 disables. */
int imdgpu_set_l2_flush(imdgpu_sys *sys, long bytes);
/* nve_run replays each full chunk of 25 steps from a captured CUDA graph
 * (default 1); 0 issues every launch from the host. */
int imdgpu_set_graphs(imdgpu_sys *sys, int on);
/* Mixed precision, one species, pair and density tables quadratic on one
 * grid: the force pass reads fused rows (pair value and gradient, density
 * gradient; 32 bytes a row) and, with staging on (default 1) and rows that
 * fit two blocks per SM, copies them into shared memory once per resident
 * block (bulk asynchronous copies completing on an mbarrier).  0 reads them
 * from global memory, with the same arithmetic. */
int imdgpu_set_table_staging(imdgpu_sys *sys, int on);
/* FP64, one species, EAM2 with pair and density tables on one grid: the
 * density pass, which finds r^2 and the table index of every pair anyway,
 * stores the pair's table terms per list entry (32 bytes) and the force pass
 * reads them instead of computing them again (default 1; trades FP64
 * arithmetic, the bound of these passes, for memory traffic).  The forces
 * have the same per-pair terms either way. */
int imdgpu_set_pair_cache(imdgpu_sys *sys, int on);
/* Measured FP64 FMA throughput of this device (TFLOP/s): a roofline
 * denominator for the FP64 force kernels. */
int imdgpu_probe_fp64_peak(double *tflops);

/* Bounds-checked build (compiled with -DIMDGPU_CHECK; `python -m
 * imd_gb300.build --check` writes imd_gb300/libimdgpu_check.so).  No
 * counterpart in the reference.  The kernels check the indices they take
 * from device data before using them; imdgpu_check_sites returns the checks
 * that failed since the system was created, as a mask: 1 a list partner
 * outside the real and ghost slots, 2 a ghost's owner outside the real
 * atoms, 4 a table row or column outside its table, 8 an atom's bin outside
 * the cell grid, 16 a permutation slot or caller index outside the atoms.
 * A failed check also sets flag 32 of the status word, and the access is
 * skipped or its index clamped.  *checked is 0 (and *sites 0) in the
 * default build, which has no checks. */
int imdgpu_check_sites(imdgpu_sys *sys, int *checked, int *sites);

/* move_atoms_nve for callers that cannot allocate device memory.  No
 * counterpart in the reference: IMD allocates everything itself.  Meant for
 * host programs whose device memory all comes from their own pool or arena,
 * or that must not meet the device synchronisation cudaMalloc/cudaFree can
 * cause inside a time step: this call allocates nothing.  The caller passes
 * its own device arrays, atom-major (x, p, f: 3n doubles; mass: n doubles;
 * type: n ints; x_ref: 3n doubles or NULL, the positions of the last list
 * build), host `restr` (3*ntypes, NULL = all free) and host `out` (4
 * doubles: tot_kin_energy, fnorm, f_max2, max |x - x_ref|^2); stream may be
 * NULL (default stream).  The types are read on the device: atoms whose type
 * lies outside 0..ntypes-1 are left unmoved, the others move, and the call
 * returns IMDGPU_ERR_ARG naming the lowest such atom.  The kinetic-energy
 * and norm partial sums go to a fixed file-scope device array of 2.5 MiB
 * per device, so n is limited to 16,777,216 atoms (IMDGPU_ERR_ARG beyond).
 * The first call on each device looks up that array's device address (with
 * the device current).  All calls on a device share the array and leave
 * their partial sums in it; each call overwrites every slot it reads, so
 * nothing needs clearing, but calls that overlap on the GPU (two streams at
 * once) race on it.  Every call copies its results to the host `out` and
 * waits on `stream` until they are there, so no call can be captured into a
 * CUDA graph. */
int imdgpu_move_atoms_nve_noalloc(int n, int ntypes, double *x, double *p, double *f,
                                  const double *mass, const int *type, const double *restr,
                                  double timestep, const double *x_ref, double *out,
                                  void *stream);

#ifdef __cplusplus
}
#endif
#endif
