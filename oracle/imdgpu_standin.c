/*
 * imdgpu_standin.c -- TEST INFRASTRUCTURE: the part of libimdgpu's C-ABI
 * (include/imdgpu.h) that IMD's `cuda` shim calls, implemented on the CPU by
 * the oracle (imd_oracle.c).
 *
 * Only the shim test links it.  IMD's own main program, linked with the shim
 * (integration/imd_forces_cuda.c) and this stand-in instead of libimdgpu,
 * runs on a machine without a GPU, so the shim's data movement (cell arrays
 * to the library's caller order and back by NUMMER, the globals it sets, the
 * steps where it copies the state back, the phases) can be compared with
 * IMD's own serial NBL run of the same parameter file.  The device library
 * itself is compared with the oracle through the same entry points by the
 * GPU tests.  Nothing of the product links this file.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../include/imdgpu.h"
#include "imd_oracle.h"

struct imdgpu_sys {
  orc_sys_t s;
  int ntypes, interaction, interp;
  int have_atoms;
  double box[9];
  int pbc[3];
  double margin, list_r2;
  double *restr;
  orc_table_t tab[3];
  int have_tab[3];
};

static char last_err[256] = "";

static int fail(int code, const char *msg) {
  snprintf(last_err, sizeof last_err, "%s", msg);
  return code;
}

const char *imdgpu_last_error(void) { return last_err; }

int imdgpu_create(imdgpu_sys **sys, int ntypes, int interaction, int precision) {
  if (!sys || ntypes < 1 || precision != IMDGPU_FP64) return fail(IMDGPU_ERR_ARG, "create");
  imdgpu_sys *g = (imdgpu_sys *)calloc(1, sizeof(imdgpu_sys));
  if (!g) return fail(IMDGPU_ERR_NOMEM, "create");
  g->ntypes = ntypes;
  g->interaction = interaction;
  *sys = g;
  return IMDGPU_OK;
}

int imdgpu_set_interpolation(imdgpu_sys *g, int mode) {
  g->interp = mode;
  return IMDGPU_OK;
}

/* the table as IMD holds it after read_pot_table and its init_* step */
int imdgpu_set_table(imdgpu_sys *g, int which, int ncols, int maxsteps, const double *begin,
                     const double *end, const double *step, const double *invstep,
                     const int *len, const double *table) {
  if (which < 0 || which > 2) return fail(IMDGPU_ERR_ARG, "table kind");
  orc_table_t *t = &g->tab[which];
  memset(t, 0, sizeof *t);
  t->ncols = ncols;
  t->maxsteps = maxsteps;
  t->begin = (double *)malloc(ncols * sizeof(double));
  t->end = (double *)malloc(ncols * sizeof(double));
  t->step = (double *)malloc(ncols * sizeof(double));
  t->invstep = (double *)malloc(ncols * sizeof(double));
  t->len = (int *)malloc(ncols * sizeof(int));
  memcpy(t->begin, begin, ncols * sizeof(double));
  memcpy(t->end, end, ncols * sizeof(double));
  memcpy(t->step, step, ncols * sizeof(double));
  memcpy(t->invstep, invstep, ncols * sizeof(double));
  memcpy(t->len, len, ncols * sizeof(int));
  size_t nv = (size_t)ncols * (maxsteps + 2);
  t->table = (double *)malloc(nv * sizeof(double));
  memcpy(t->table, table, nv * sizeof(double));
  t->mode = g->interp;
  g->have_tab[which] = 1;
  return IMDGPU_OK;
}

int imdgpu_set_table2(imdgpu_sys *g, int which, int ncols, int maxsteps, const double *table2) {
  orc_table_t *t = &g->tab[which];
  size_t nv = (size_t)ncols * (maxsteps + 2);
  t->table2 = (double *)malloc(nv * sizeof(double));
  memcpy(t->table2, table2, nv * sizeof(double));
  return IMDGPU_OK;
}

int imdgpu_set_box(imdgpu_sys *g, const double *box, const int *pbc, double margin,
                   double list_r2) {
  memcpy(g->box, box, sizeof g->box);
  memcpy(g->pbc, pbc, sizeof g->pbc);
  g->margin = margin;
  g->list_r2 = list_r2;
  return IMDGPU_OK;
}

int imdgpu_set_restrictions(imdgpu_sys *g, const double *restr) {
  free(g->restr);
  g->restr = (double *)malloc(3 * g->ntypes * sizeof(double));
  memcpy(g->restr, restr, 3 * g->ntypes * sizeof(double));
  return IMDGPU_OK;
}

int imdgpu_set_atoms(imdgpu_sys *g, int n, const int *number, const int *type,
                     const double *mass, const double *x, const double *p) {
  orc_sys_t *s = &g->s;
  if (g->have_atoms) {
    /* keep the tables: orc_free releases them with the system */
    memset(&s->pair, 0, sizeof s->pair);
    memset(&s->rho, 0, sizeof s->rho);
    memset(&s->embed, 0, sizeof s->embed);
    orc_free(s);
  }
  memset(s, 0, sizeof *s);
  s->ntypes = g->ntypes;
  s->interaction = g->interaction == IMDGPU_EAM2 ? ORC_EAM2 : ORC_PAIR;
  for (int a = 0; a < 3; a++) {
    for (int c = 0; c < 3; c++) s->box[a][c] = g->box[3 * a + c];
    s->pbc[a] = g->pbc[a];
  }
  s->nbl_margin = g->margin;
  s->restrictions = g->restr;
  s->pair = g->tab[IMDGPU_TAB_PAIR];
  if (s->interaction == ORC_EAM2) {
    s->rho = g->tab[IMDGPU_TAB_RHO];
    s->embed = g->tab[IMDGPU_TAB_EMBED];
  }
  if (orc_init(s, n)) return fail(IMDGPU_ERR_NOMEM, "oracle init");
  /* IMD's cellsz: the largest end of the radial tables (read_pot_table),
   * the margin added by init_cells */
  double cz = 0.0;
  for (int c = 0; c < s->pair.ncols; c++) cz = cz > s->pair.end[c] ? cz : s->pair.end[c];
  if (s->interaction == ORC_EAM2)
    for (int c = 0; c < s->rho.ncols; c++) cz = cz > s->rho.end[c] ? cz : s->rho.end[c];
  s->cellsz = cz;
  memcpy(s->number, number, n * sizeof(int));
  memcpy(s->type, type, n * sizeof(int));
  memcpy(s->mass, mass, n * sizeof(double));
  memcpy(s->x, x, 3 * (size_t)n * sizeof(double));
  if (p) memcpy(s->p, p, 3 * (size_t)n * sizeof(double));
  if (orc_setup_geometry(s)) return fail(IMDGPU_ERR_GEOM, "oracle geometry");
  if (g->list_r2 > 0.0 && g->list_r2 != s->cellsz)
    return fail(IMDGPU_ERR_ARG, "list radius differs from the tables' end plus the margin");
  g->have_atoms = 1;
  return IMDGPU_OK;
}

int imdgpu_get_atoms(imdgpu_sys *g, double *x, double *p, double *f, double *epot,
                     double *eam_rho, double *eam_df) {
  orc_sys_t *s = &g->s;
  size_t n = (size_t)s->n;
  if (x) memcpy(x, s->x, 3 * n * sizeof(double));
  if (p) memcpy(p, s->p, 3 * n * sizeof(double));
  if (f) memcpy(f, s->f, 3 * n * sizeof(double));
  if (epot) memcpy(epot, s->epot, n * sizeof(double));
  if (eam_rho) memcpy(eam_rho, s->eam_rho, n * sizeof(double));
  if (eam_df) memcpy(eam_df, s->eam_df, n * sizeof(double));
  return IMDGPU_OK;
}

int imdgpu_get_scalars(imdgpu_sys *g, imdgpu_scalars *o) {
  orc_sys_t *s = &g->s;
  memset(o, 0, sizeof *o);
  o->tot_pot_energy = s->tot_pot_energy;
  o->virial = s->virial;
  o->tot_kin_energy = s->tot_kin_energy;
  o->fnorm = s->fnorm;
  o->f_max2 = s->f_max2;
  o->nfc = s->nfc;
  o->nbl_count = s->nbl_count;
  o->nb_entries = s->nb_len;
  o->have_valid_nbl = s->have_valid_nbl;
  for (int a = 0; a < 3; a++) o->gdim[a] = s->gdim[a];
  o->short_distance = s->is_short;
  return IMDGPU_OK;
}

int imdgpu_calc_forces(imdgpu_sys *g, int steps) {
  (void)steps;
  if (!g->have_atoms) return fail(IMDGPU_ERR_STATE, "no atoms");
  if (orc_calc_forces(&g->s)) return fail(IMDGPU_ERR_CELL, "oracle calc_forces");
  return g->s.is_short ? IMDGPU_WARN_SHORT : IMDGPU_OK;
}

int imdgpu_make_nblist(imdgpu_sys *g) {
  return orc_rebuild(&g->s) ? fail(IMDGPU_ERR_CELL, "oracle rebuild") : IMDGPU_OK;
}

int imdgpu_check_nblist(imdgpu_sys *g) {
  orc_check_nblist(&g->s);
  return IMDGPU_OK;
}

int imdgpu_deallocate_nblist(imdgpu_sys *g) {
  g->s.have_valid_nbl = 0;
  return IMDGPU_OK;
}

int imdgpu_estimate_nblist_size(imdgpu_sys *g, long *entries) {
  *entries = g->s.nb_len;
  return IMDGPU_OK;
}

int imdgpu_move_atoms_nve(imdgpu_sys *g, double timestep) {
  g->s.timestep = timestep;
  orc_move_atoms_nve(&g->s);
  return IMDGPU_OK;
}

int imdgpu_move_atoms_mik(imdgpu_sys *g, double timestep) {
  g->s.timestep = timestep;
  orc_move_atoms_mik(&g->s);
  return IMDGPU_OK;
}

int imdgpu_set_nvt(imdgpu_sys *g, double temperature, double isq_tau_eta, double eta,
                   long nactive) {
  g->s.temperature = temperature;
  g->s.isq_tau_eta = isq_tau_eta;
  g->s.eta = eta;
  g->s.nactive = nactive > 0 ? nactive : 3L * g->s.n;
  return IMDGPU_OK;
}

int imdgpu_get_nvt(imdgpu_sys *g, double *eta) {
  *eta = g->s.eta;
  return IMDGPU_OK;
}

int imdgpu_move_atoms_nvt(imdgpu_sys *g, double timestep) {
  g->s.timestep = timestep;
  orc_move_atoms_nvt(&g->s);
  return IMDGPU_OK;
}

int imdgpu_set_cg_params(imdgpu_sys *g, int linmin_maxsteps, double linmin_tol,
                         double linmin_dmax, double linmin_dmin, double cg_glimit,
                         double cg_zeps, int cg_fr, int cg_reset_int) {
  orc_sys_t *s = &g->s;
  s->linmin_maxsteps = linmin_maxsteps;
  s->linmin_tol = linmin_tol;
  s->linmin_dmax = linmin_dmax;
  s->linmin_dmin = linmin_dmin;
  s->cg_glimit = cg_glimit;
  s->cg_zeps = cg_zeps;
  s->cg_fr = cg_fr;
  s->cg_reset_int = cg_reset_int;
  return IMDGPU_OK;
}

int imdgpu_reset_cg(imdgpu_sys *g) {
  return orc_reset_cg(&g->s) < 0 ? fail(IMDGPU_ERR_STATE, "oracle reset_cg") : IMDGPU_OK;
}

int imdgpu_cg_step(imdgpu_sys *g, int steps) {
  return orc_cg_step(&g->s, steps) < 0 ? fail(IMDGPU_ERR_BRENT, "Too many iterations in brent")
                                       : IMDGPU_OK;
}

/* write_atoms_config's text lines (the device formats them in the library),
 * here by snprintf: the format the library must reproduce */
int imdgpu_format_atoms(imdgpu_sys *g, int flags, const int *order, int n, char *buf,
                        long cap, long *len) {
  orc_sys_t *s = &g->s;
  const char *f = (flags & IMDGPU_FMT_HPO) ? " %12.16f" : " %f";
  char line[512];
  long total = 0;
  if (!order) n = s->n;
  for (int a = 0; a < n; a++) {
    const int i = order ? order[a] : a;
    int l = snprintf(line, sizeof line, "%d %d", s->number[i], s->type[i]);
    double vals[9];
    int nv = 0;
    vals[nv++] = s->mass[i];
    for (int c = 0; c < 3; c++) vals[nv++] = s->x[3 * i + c];
    if (flags & IMDGPU_FMT_VELOCITY)
      for (int c = 0; c < 3; c++) vals[nv++] = s->p[3 * i + c] / s->mass[i];
    vals[nv++] = s->epot[i];
    if (flags & IMDGPU_FMT_EAM_RHO) vals[nv++] = s->eam_rho[i];
    for (int k = 0; k < nv; k++) l += snprintf(line + l, sizeof line - l, f, vals[k]);
    l += snprintf(line + l, sizeof line - l, "\n");
    if (buf && total + l <= cap) memcpy(buf + total, line, l);
    total += l;
  }
  *len = total;
  return IMDGPU_OK;
}
