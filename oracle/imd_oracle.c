/*
 * imd_oracle.c -- CPU restatement of IMD's force / neighbour-list / NVE / CG
 * hot path (itapmd/imd, src/imd_forces_nbl.c, src/potaccess.h,
 * src/imd_potential.c, src/imd_geom_3d.c, src/imd_comm_force_3d.c,
 * src/imd_fix_cells_3d.c, src/imd_integrate.c, src/imd_cg.c,
 * src/cg_utils.h).
 *
 * TEST INFRASTRUCTURE ONLY: the reference values for testing the GPU library and the timed
 * CPU baseline.  Never linked into the product.
 *
 * Build with -ffp-contract=off: the reference is compiled without fused
 * multiply-add, and r^2 / table-index / cell-index bits depend on it.
 */
#include "imd_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define OMIN(a, b) ((a) < (b) ? (a) : (b))
#define OMAX(a, b) ((a) > (b) ? (a) : (b))
#define SQR(a) ((a) * (a))

/* ------------------------------------------------------------------------ */
/* tables                                                                    */
/* ------------------------------------------------------------------------ */

static int g_interp = ORC_QUADRATIC;
void orc_set_interpolation(int mode) { g_interp = mode; }

static int alloc_info(orc_table_t *pt, int ncols) {
  pt->ncols = ncols;
  pt->table2 = NULL;
  pt->mode = g_interp;
  pt->maxsteps = 0;
  pt->begin = (double *)calloc(ncols, sizeof(double));
  pt->end = (double *)calloc(ncols, sizeof(double));
  pt->step = (double *)calloc(ncols, sizeof(double));
  pt->invstep = (double *)calloc(ncols, sizeof(double));
  pt->len = (int *)calloc(ncols, sizeof(int));
  pt->table = NULL;
  return (pt->begin && pt->end && pt->step && pt->invstep && pt->len) ? 0 : 1;
}

void orc_free_table(orc_table_t *pt) {
  free(pt->table2);
  free(pt->begin);
  free(pt->end);
  free(pt->step);
  free(pt->invstep);
  free(pt->len);
  free(pt->table);
  memset(pt, 0, sizeof(*pt));
}

/* init_threepoint (src/imd_potential.c:1256-1272): continue the last
 * interpolation polynomial into rows len and len+1. */
static void threepoint(orc_table_t *pt) {
  int nc = pt->ncols;
  for (int col = 0; col < nc; col++) {
    double *y = pt->table + col;
    int n = pt->len[col];
    if (n < 3) continue;
    y[n * nc] = 3 * y[(n - 1) * nc] - 3 * y[(n - 2) * nc] + y[(n - 3) * nc];
    y[(n + 1) * nc] =
        6 * y[(n - 1) * nc] - 8 * y[(n - 2) * nc] + 3 * y[(n - 3) * nc];
  }
}

/* init_fourpoint (src/imd_potential.c:1171-1187) */
static void fourpoint(orc_table_t *pt) {
  int nc = pt->ncols;
  for (int col = 0; col < nc; col++) {
    double *y = pt->table + col;
    int n = pt->len[col];
    if (n < 4) continue;
    y[n * nc] = 4 * y[(n - 1) * nc] - 6 * y[(n - 2) * nc] + 4 * y[(n - 3) * nc] - y[(n - 4) * nc];
    y[(n + 1) * nc] = 10 * y[(n - 1) * nc] - 20 * y[(n - 2) * nc] + 15 * y[(n - 3) * nc] -
                      4 * y[(n - 4) * nc];
  }
}

/* init_spline (src/imd_potential.c:1197-1246): natural spline at the left
 * end; zero slope at the right end for radial functions, natural otherwise */
static void spline(orc_table_t *pt, int radial) {
  int nc = pt->ncols, size = pt->maxsteps + 2;
  pt->table2 = (double *)calloc((size_t)nc * size, sizeof(double));
  double *u = (double *)calloc(size, sizeof(double));
  for (int col = 0; col < nc; col++) {
    double *y2 = pt->table2 + col, *y = pt->table + col;
    int n = pt->len[col];
    double step = pt->step[col], p, qn, un;
    y2[0] = u[0] = 0;
    for (int i = 1; i < n - 1; i++) {
      p = 0.5 * y2[(i - 1) * nc] + 2.0;
      y2[i * nc] = -0.5 / p;
      u[i] = (y[(i + 1) * nc] - 2 * y[i * nc] + y[(i - 1) * nc]) / step;
      u[i] = (6.0 * u[i] / (2 * step) - 0.5 * u[i - 1]) / p;
    }
    if (radial) {
      qn = 0.5;
      un = (3.0 / step) * (y[(n - 2) * nc] - y[(n - 1) * nc]) / step;
    } else {
      qn = un = 0.0;
    }
    y2[(n - 1) * nc] = (un - qn * u[n - 2]) / (qn * y2[(n - 2) * nc] + 1.0);
    for (int k = n - 2; k >= 0; k--) y2[k * nc] = y2[k * nc] * y2[(k + 1) * nc] + u[k];
    y[n * nc] = 2 * y[(n - 1) * nc] - y[(n - 2) * nc] + SQR(step) * y2[(n - 1) * nc];
    y2[n * nc] = 2 * y2[(n - 1) * nc] - y2[(n - 2) * nc];
  }
  free(u);
}

static void init_interp(orc_table_t *pt, int radial) {
  if (pt->mode == ORC_FOURPOINT) fourpoint(pt);
  else if (pt->mode == ORC_SPLINE) spline(pt, radial);
  else threepoint(pt);
}

/* format 1 (src/imd_potential.c:297-376): lines "r2 v_0 ... v_{ncols-1}",
 * end = r2 of the last nonzero value, len = its row + 1, shift by the value
 * of the last row. */
static int read_format1(orc_table_t *pt, FILE *in, int radial, double *cellsz,
                        char *err, int errlen) {
  int nc = pt->ncols, npot = 0, cap = 50;
  double r2 = 0.0, r2_start = 0.0, val;
  pt->table = (double *)malloc((size_t)nc * cap * sizeof(double));
  for (;;) {
    if (npot == cap) {
      cap += 50;
      pt->table = (double *)realloc(pt->table, (size_t)nc * cap * sizeof(double));
    }
    if (1 != fscanf(in, "%lf", &r2)) break;
    if (npot == 0) r2_start = r2;
    for (int i = 0; i < nc; i++) {
      if (1 != fscanf(in, "%lf", &val)) {
        snprintf(err, errlen, "Line incomplete in potential file.");
        return 1;
      }
      pt->table[npot * nc + i] = val;
      if (val != 0.0) {
        pt->end[i] = r2;
        pt->len[i] = npot + 1;
      }
    }
    npot++;
  }
  if (npot < 2) {
    snprintf(err, errlen, "table too short");
    return 1;
  }
  double r2_step = (r2 - r2_start) / (npot - 1);
  pt->maxsteps = cap;
  for (int i = 0; i < nc; i++) {
    pt->begin[i] = r2_start;
    pt->step[i] = r2_step;
    pt->invstep[i] = 1.0 / r2_step;
    double delta = pt->table[(npot - 1) * nc + i];
    if (radial && delta != 0.0)
      for (int k = 0; k < npot; k++) pt->table[k * nc + i] -= delta;
    if (radial) *cellsz = OMAX(*cellsz, pt->end[i]);
  }
  pt->table = (double *)realloc(pt->table, (size_t)nc * (cap + 2) * sizeof(double));
  for (int k = npot; k < cap + 2; k++)
    for (int i = 0; i < nc; i++) pt->table[k * nc + i] = 0.0;
  return 0;
}

/* format 2 (src/imd_potential.c:394-462): per column "begin end step", then
 * len values per column; shift radial columns by their last value. */
static int read_format2(orc_table_t *pt, FILE *in, int radial, double *cellsz,
                        char *err, int errlen) {
  int nc = pt->ncols;
  for (int i = 0; i < nc; i++) {
    if (3 != fscanf(in, "%lf %lf %lf", &pt->begin[i], &pt->end[i], &pt->step[i])) {
      snprintf(err, errlen, "Info line corrupt.");
      return 1;
    }
    if (radial) *cellsz = OMAX(*cellsz, pt->end[i]);
    pt->invstep[i] = 1.0 / pt->step[i];
    double numstep = 1 + (pt->end[i] - pt->begin[i]) / pt->step[i];
    pt->len[i] = (int)(numstep + 0.49);
    pt->maxsteps = OMAX(pt->maxsteps, pt->len[i]);
  }
  size_t tsize = (size_t)nc * (pt->maxsteps + 2);
  pt->table = (double *)calloc(tsize, sizeof(double));
  for (int i = 0; i < nc; i++)
    for (int k = 0; k < pt->len[i]; k++) {
      double val;
      if (1 != fscanf(in, "%lf", &val)) {
        snprintf(err, errlen, "wrong format in potential file.");
        return 1;
      }
      pt->table[k * nc + i] = val;
    }
  if (radial)
    for (int i = 0; i < nc; i++) {
      double delta = pt->table[(pt->len[i] - 1) * nc + i];
      if (delta != 0.0)
        for (int k = 0; k < pt->len[i]; k++) pt->table[k * nc + i] -= delta;
    }
  return 0;
}

/* read_pot_table (src/imd_potential.c:161-282): header "#F fmt ncols" ...
 * "#E"; no header means the build's default format. */
int orc_read_table(orc_table_t *pt, const char *fname, int ncols, int radial,
                   int default_format, double *cellsz, char *err, int errlen) {
  char buf[1024];
  int have_header = 0, have_format = 0, end_header = 0;
  int format = default_format, size = ncols;
  FILE *in = fopen(fname, "r");
  if (!in) {
    snprintf(err, errlen, "Could not open potential file %s", fname);
    return 1;
  }
  do {
    if (!fgets(buf, sizeof buf, in)) {
      snprintf(err, errlen, "Unexpected end of file in %s", fname);
      fclose(in);
      return 1;
    }
    if (buf[0] == '#') {
      have_header = 1;
      end_header = (buf[1] == 'E');
      if (buf[1] == 'F') {
        if (2 != sscanf(buf + 2, "%d%d", &format, &size)) {
          snprintf(err, errlen, "Corrupted format header line in file %s", fname);
          fclose(in);
          return 1;
        }
        if (size != ncols) {
          snprintf(err, errlen, "Wrong number of data columns in file %s", fname);
          fclose(in);
          return 1;
        }
        if (format != 1 && format != 2) {
          snprintf(err, errlen, "Unrecognized format specified for file %s", fname);
          fclose(in);
          return 1;
        }
        have_format = 1;
      }
    } else if (have_header) {
      snprintf(err, errlen, "Corrupted header in file %s", fname);
      fclose(in);
      return 1;
    } else {
      end_header = 1;
    }
  } while (!end_header);
  if (have_header && !have_format) {
    snprintf(err, errlen, "Format not specified in header of file %s", fname);
    fclose(in);
    return 1;
  }
  if (!have_header) rewind(in);
  if (alloc_info(pt, ncols)) {
    fclose(in);
    return 1;
  }
  int rc = (format == 1) ? read_format1(pt, in, radial, cellsz, err, errlen)
                         : read_format2(pt, in, radial, cellsz, err, errlen);
  fclose(in);
  if (rc) return rc;
  init_interp(pt, radial);
  return 0;
}

int orc_make_table(orc_table_t *pt, int ncols, const double *begin,
                   const double *end, const double *step, const double *vals,
                   const int *len, int radial, double *cellsz) {
  if (alloc_info(pt, ncols)) return 1;
  for (int i = 0; i < ncols; i++) {
    pt->begin[i] = begin[i];
    pt->end[i] = end[i];
    pt->step[i] = step[i];
    pt->invstep[i] = 1.0 / step[i];
    pt->len[i] = len[i];
    pt->maxsteps = OMAX(pt->maxsteps, len[i]);
    if (radial) *cellsz = OMAX(*cellsz, end[i]);
  }
  pt->table = (double *)calloc((size_t)ncols * (pt->maxsteps + 2), sizeof(double));
  long off = 0;
  for (int i = 0; i < ncols; i++) {
    for (int k = 0; k < len[i]; k++) pt->table[k * ncols + i] = vals[off + k];
    off += len[i];
  }
  if (radial)
    for (int i = 0; i < ncols; i++) {
      double delta = pt->table[(len[i] - 1) * ncols + i];
      if (delta != 0.0)
        for (int k = 0; k < len[i]; k++) pt->table[k * ncols + i] -= delta;
    }
  init_interp(pt, radial);
  return 0;
}

/* shared index computation of PAIR_INT2/VAL_FUNC2/DERIV_FUNC2
 * (src/potaccess.h:323-345) */
static inline void tab_row(const orc_table_t *pt, int col, int inc, double r2,
                           double *chi, double *istep, double *p0, double *p1,
                           double *p2, int *is_short) {
  double r2a = OMIN(r2, pt->end[col]);
  r2a = r2a - pt->begin[col];
  if (r2a < 0) {
    r2a = 0;
    *is_short = 1;
  }
  *istep = pt->invstep[col];
  r2a = r2a * (*istep);
  int k = (int)r2a;
  *chi = r2a - k;
  const double *ptr = pt->table + (long)k * inc + col;
  *p0 = ptr[0];
  *p1 = ptr[inc];
  *p2 = ptr[2 * inc];
}

static void pair_int_q(const orc_table_t *pt, int col, int inc, double r2,
                       double *pot, double *grad, int *is_short) {
  double chi, istep, p0, p1, p2;
  tab_row(pt, col, inc, r2, &chi, &istep, &p0, &p1, &p2, is_short);
  double dv = p1 - p0;
  double d2v = p2 - 2 * p1 + p0;
  *pot = p0 + chi * dv + 0.5 * chi * (chi - 1) * d2v;
  *grad = 2 * istep * (dv + (chi - 0.5) * d2v);
}

static double val_func_q(const orc_table_t *pt, int col, int inc, double r2,
                         int *is_short) {
  double chi, istep, p0, p1, p2;
  tab_row(pt, col, inc, r2, &chi, &istep, &p0, &p1, &p2, is_short);
  double dv = p1 - p0;
  double d2v = p2 - 2 * p1 + p0;
  return p0 + chi * dv + 0.5 * chi * (chi - 1) * d2v;
}

static double deriv_func_q(const orc_table_t *pt, int col, int inc, double r2,
                           int *is_short) {
  double chi, istep, p0, p1, p2;
  tab_row(pt, col, inc, r2, &chi, &istep, &p0, &p1, &p2, is_short);
  double dv = p1 - p0;
  double d2v = p2 - 2 * p1 + p0;
  return 2 * istep * (dv + (chi - 0.5) * d2v);
}

/* index of the 4-point and spline macros: r2a as for the quadratic one */
static double r2a_of(const orc_table_t *pt, int col, double r2, int *is_short) {
  double r2a = OMIN(r2, pt->end[col]);
  r2a = r2a - pt->begin[col];
  if (r2a < 0) {
    r2a = 0;
    *is_short = 1;
  }
  return r2a * pt->invstep[col];
}

/* PAIR_INT3 / VAL_FUNC3 / DERIV_FUNC3 (src/potaccess.h:365-410, :503-539,
 * :630-666): cubic through rows k-1..k+2, k = max(floor, 1) */
static void four_eval(const orc_table_t *pt, int col, int inc, double r2, double *pot,
                      double *grad, int *is_short) {
  double istep = pt->invstep[col];
  double r2a = r2a_of(pt, col, r2, is_short);
  int k = (int)r2a;
  if (k < 1) k = 1;
  double chi = r2a - k;
  double fac0 = -(1.0 / 6.0) * chi * (chi - 1.0) * (chi - 2.0);
  double fac1 = 0.5 * (chi * chi - 1.0) * (chi - 2.0);
  double fac2 = -0.5 * chi * (chi + 1.0) * (chi - 2.0);
  double fac3 = (1.0 / 6.0) * chi * (chi * chi - 1.0);
  double dfac0 = -(1.0 / 6.0) * ((3.0 * chi - 6.0) * chi + 2.0);
  double dfac1 = 0.5 * ((3.0 * chi - 4.0) * chi - 1.0);
  double dfac2 = -0.5 * ((3.0 * chi - 2.0) * chi - 2.0);
  double dfac3 = 1.0 / 6.0 * (3.0 * chi * chi - 1.0);
  const double *ptr = pt->table + (long)(k - 1) * inc + col;
  double p0 = ptr[0], p1 = ptr[inc], p2 = ptr[2 * inc], p3 = ptr[3 * inc];
  if (pot) *pot = fac0 * p0 + fac1 * p1 + fac2 * p2 + fac3 * p3;
  if (grad) *grad = 2 * istep * (dfac0 * p0 + dfac1 * p1 + dfac2 * p2 + dfac3 * p3);
}

/* PAIR_INT_SP / VAL_FUNC_SP / DERIV_FUNC_SP (src/potaccess.h:421-457,
 * :547-582, :675-710) */
static void spline_eval(const orc_table_t *pt, int col, int inc, double r2, double *pot,
                        double *grad, int *is_short) {
  double istep = pt->invstep[col], step = pt->step[col];
  double r2a = r2a_of(pt, col, r2, is_short);
  int k = (int)r2a;
  double b = r2a - k, a = 1.0 - b;
  k = k * inc + col;
  double p1 = pt->table[k], d21 = pt->table2[k];
  k += inc;
  double p2 = pt->table[k], d22 = pt->table2[k];
  double a2 = a * a - 1, b2 = b * b - 1, st6 = step / 6;
  if (pot) *pot = a * p1 + b * p2 + (a * a2 * d21 + b * b2 * d22) * st6 * step;
  if (grad) *grad = 2 * ((p2 - p1) * istep + ((3 * b2 + 2) * d22 - (3 * a2 + 2) * d21) * st6);
}

void orc_pair_int2(const orc_table_t *pt, int col, int inc, double r2, double *pot,
                   double *grad, int *is_short) {
  if (pt->mode == ORC_FOURPOINT) four_eval(pt, col, inc, r2, pot, grad, is_short);
  else if (pt->mode == ORC_SPLINE) spline_eval(pt, col, inc, r2, pot, grad, is_short);
  else pair_int_q(pt, col, inc, r2, pot, grad, is_short);
}
double orc_val_func2(const orc_table_t *pt, int col, int inc, double r2, int *is_short) {
  double v;
  if (pt->mode == ORC_FOURPOINT) four_eval(pt, col, inc, r2, &v, NULL, is_short);
  else if (pt->mode == ORC_SPLINE) spline_eval(pt, col, inc, r2, &v, NULL, is_short);
  else v = val_func_q(pt, col, inc, r2, is_short);
  return v;
}
double orc_deriv_func2(const orc_table_t *pt, int col, int inc, double r2, int *is_short) {
  double g;
  if (pt->mode == ORC_FOURPOINT) four_eval(pt, col, inc, r2, NULL, &g, is_short);
  else if (pt->mode == ORC_SPLINE) spline_eval(pt, col, inc, r2, NULL, &g, is_short);
  else g = deriv_func_q(pt, col, inc, r2, is_short);
  return g;
}

void orc_pair_int2_batch(const orc_table_t *pt, int col, int inc, int n,
                         const double *r2, double *pot, double *grad) {
  int is_short = 0;
  for (int i = 0; i < n; i++) orc_pair_int2(pt, col, inc, r2[i], pot + i, grad + i, &is_short);
}

/* ------------------------------------------------------------------------ */
/* system set-up                                                             */
/* ------------------------------------------------------------------------ */

int orc_init(orc_sys_t *s, int n) {
  /* keep caller-set parameters, reset everything else */
  s->n = n;
  s->number = (int *)calloc(n, sizeof(int));
  s->type = (int *)calloc(n, sizeof(int));
  s->mass = (double *)calloc(n, sizeof(double));
  s->x = (double *)calloc(3 * (size_t)n, sizeof(double));
  s->p = (double *)calloc(3 * (size_t)n, sizeof(double));
  s->f = (double *)calloc(3 * (size_t)n, sizeof(double));
  s->epot = (double *)calloc(n, sizeof(double));
  s->eam_rho = (double *)calloc(n, sizeof(double));
  s->eam_df = (double *)calloc(n, sizeof(double));
  s->nbl_pos = (double *)calloc(3 * (size_t)n, sizeof(double));
  s->old_x = (double *)calloc(3 * (size_t)n, sizeof(double));
  s->cg_g = (double *)calloc(3 * (size_t)n, sizeof(double));
  s->cg_h = (double *)calloc(3 * (size_t)n, sizeof(double));
  s->order = (int *)calloc(n, sizeof(int));
  s->tl = (int *)calloc((size_t)n + 1, sizeof(int));
  s->next = 0;
  s->next_cap = 0;
  s->ex = NULL;
  s->etype = s->esrc = s->eowner = NULL;
  s->eshift = s->ef = s->eepot = s->erho = s->edf = NULL;
  s->do_stress = 0;
  s->estress = NULL;
  s->stress = (double *)calloc(6 * (size_t)n, sizeof(double));
  s->tb = NULL;
  s->nb_cap = s->nb_len = 0;
  s->have_valid_nbl = 0;
  s->nbl_count = s->nfc = 0;
  s->cell_start = s->cell_cnt = s->cell_atoms = NULL;
  s->real_cells = s->cnbrs = NULL;
  s->old_alphamin = 0.1; /* static in linmin, src/imd_cg.c:99 */
  s->nactive = 3L * n;
  if (s->linmin_maxsteps <= 0) s->linmin_maxsteps = 100;
  if (s->linmin_tol <= 0) s->linmin_tol = 0.0002;
  if (s->linmin_dmax <= 0) s->linmin_dmax = 0.01;
  if (s->linmin_dmin <= 0) s->linmin_dmin = 0.001;
  if (s->cg_glimit <= 0) s->cg_glimit = 100;
  if (s->cg_zeps <= 0) s->cg_zeps = 1e-10;
  return (s->number && s->type && s->x && s->p && s->f && s->tl) ? 0 : 1;
}

void orc_free(orc_sys_t *s) {
  free(s->estress); free(s->stress);
  s->estress = s->stress = NULL;
  free(s->number); free(s->type); free(s->mass); free(s->x); free(s->p);
  free(s->f); free(s->epot); free(s->eam_rho); free(s->eam_df);
  free(s->nbl_pos); free(s->old_x); free(s->cg_g); free(s->cg_h);
  free(s->order); free(s->tl); free(s->tb); free(s->ex); free(s->etype);
  free(s->esrc); free(s->eowner); free(s->eshift); free(s->ef);
  free(s->eepot); free(s->erho); free(s->edf); free(s->cell_start);
  free(s->cell_cnt); free(s->cell_atoms); free(s->real_cells); free(s->cnbrs);
  orc_free_table(&s->pair);
  orc_free_table(&s->rho);
  orc_free_table(&s->embed);
}

/* vec_prod (src/imd_geom_3d.c:36-43) */
static void vec_prod(const double *u, const double *v, double *w) {
  w[0] = u[1] * v[2] - u[2] * v[1];
  w[1] = u[2] * v[0] - u[0] * v[2];
  w[2] = u[0] * v[1] - u[1] * v[0];
}
static inline double sprod(const double *a, const double *b) {
  return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}

/* make_box (src/imd_geom_3d.c:52-80): tbox, volume, squared heights */
static int make_box(orc_sys_t *s) {
  vec_prod(s->box[1], s->box[2], s->tbox[0]);
  vec_prod(s->box[2], s->box[0], s->tbox[1]);
  vec_prod(s->box[0], s->box[1], s->tbox[2]);
  s->volume = sprod(s->box[0], s->tbox[0]);
  if (s->volume == 0) return 1;
  for (int a = 0; a < 3; a++)
    for (int c = 0; c < 3; c++) s->tbox[a][c] /= s->volume;
  for (int a = 0; a < 3; a++) s->height[a] = 1.0 / sprod(s->tbox[a], s->tbox[a]);
  return 0;
}

/* init_cells (src/imd_geom_3d.c:113-206) with the NPT tolerance factor tol
 * (:128-133, 1 otherwise) on the list radius already set, and
 * make_cell_lists with AR (:823-947); min/max_height (may be NULL) get the
 * squared heights between which the grid stays (:196-206) */
static int init_cells(orc_sys_t *s, double tol, double *min_height, double *max_height) {
  for (int a = 0; a < 3; a++) {
    double scale = sqrt(tol * s->cellsz / s->height[a]);
    s->gdim[a] = (int)(1.0 / scale);
    if (s->gdim[a] < 1) return 2; /* "global_cell_dim too small" */
    s->cdim[a] = s->gdim[a] + 2;
    if (min_height) min_height[a] = s->cellsz * SQR(s->gdim[a]);
    if (max_height) max_height[a] = s->cellsz * SQR(s->gdim[a] + 1) * tol;
  }
  int cx = s->cdim[0], cy = s->cdim[1], cz = s->cdim[2];
  s->nallcells = cx * cy * cz;
  s->nreal_cells = s->gdim[0] * s->gdim[1] * s->gdim[2];
  free(s->real_cells);
  free(s->cnbrs);
  s->real_cells = (int *)malloc(sizeof(int) * s->nreal_cells);
  s->cnbrs = (int *)malloc(sizeof(int) * 14 * s->nreal_cells);
  int l = 0;
  for (int i = 1; i < cx - 1; i++)
    for (int j = 1; j < cy - 1; j++)
      for (int k = 1; k < cz - 1; k++) {
        int np = i * cy * cz + j * cz + k;
        int *nq = s->cnbrs + 14 * l;
        s->real_cells[l] = np;
        nq[0] = np;
        int nn = 1;
        for (int a = 0; a <= 1; a++)
          for (int b = -a; b <= 1; b++)
            for (int c = (a == 0 ? -b : -a); c <= 1; c++) {
              int r = i + a, t2 = j + b, u = k + c;
              int qq = r * cy * cz + t2 * cz + u;
              if (qq == np) continue;
              int gr = r - 1, gs = t2 - 1, gt = u - 1;
              int px = (gr < 0) ? -1 : (gr > s->gdim[0] - 1) ? 1 : 0;
              int py = (gs < 0) ? -1 : (gs > s->gdim[1] - 1) ? 1 : 0;
              int pz = (gt < 0) ? -1 : (gt > s->gdim[2] - 1) ? 1 : 0;
              if ((s->pbc[0] == 1 || px == 0) && (s->pbc[1] == 1 || py == 0) &&
                  (s->pbc[2] == 1 || pz == 0))
                nq[nn] = qq;
              else
                nq[nn] = -1;
              nn++;
            }
        l++;
      }
  free(s->cell_start);
  free(s->cell_cnt);
  s->cell_start = (int *)calloc(s->nallcells + 1, sizeof(int));
  s->cell_cnt = (int *)calloc(s->nallcells, sizeof(int));
  return 0;
}

/* make_box, the list margin added once (src/imd_geom_3d.c:122-126), then
 * init_cells */
int orc_setup_geometry(orc_sys_t *s) {
  if (make_box(s)) return 1;
  s->cellsz = SQR(sqrt((double)s->cellsz) + s->nbl_margin);
  return init_cells(s, 1.0, NULL, NULL);
}

/* cell_coord (src/imd_geom_3d.c:1054-1074) */
static void cell_coord(const orc_sys_t *s, const double *x, int *c) {
  for (int a = 0; a < 3; a++) {
    int v = (int)(s->gdim[a] * (x[0] * s->tbox[a][0] + x[1] * s->tbox[a][1] +
                                x[2] * s->tbox[a][2]));
    if (v >= s->gdim[a]) v = s->gdim[a] - 1;
    else if (v < 0) v = 0;
    c[a] = v;
  }
}

/* do_boundaries (src/imd_main_3d.c:1972-2010) */
static void wrap_atom(const orc_sys_t *s, double *x) {
  for (int a = 0; a < 3; a++) {
    if (s->pbc[a] != 1) continue;
    double i = -floor(x[0] * s->tbox[a][0] + x[1] * s->tbox[a][1] + x[2] * s->tbox[a][2]);
    x[0] += i * s->box[a][0];
    x[1] += i * s->box[a][1];
    x[2] += i * s->box[a][2];
  }
}

static void ensure_ext(orc_sys_t *s, int need) {
  if (need <= s->next_cap) return;
  int cap = need + need / 4 + 64;
  s->ex = (double *)realloc(s->ex, sizeof(double) * 3 * cap);
  s->eshift = (double *)realloc(s->eshift, sizeof(double) * 3 * cap);
  s->ef = (double *)realloc(s->ef, sizeof(double) * 3 * cap);
  s->etype = (int *)realloc(s->etype, sizeof(int) * cap);
  s->esrc = (int *)realloc(s->esrc, sizeof(int) * cap);
  s->eowner = (int *)realloc(s->eowner, sizeof(int) * cap);
  s->eepot = (double *)realloc(s->eepot, sizeof(double) * cap);
  s->erho = (double *)realloc(s->erho, sizeof(double) * cap);
  s->edf = (double *)realloc(s->edf, sizeof(double) * cap);
  s->estress = (double *)realloc(s->estress, sizeof(double) * 6 * cap);
  s->next_cap = cap;
}

/* One buffer-cell copy, copy_cell (src/imd_comm_force_3d.c:726-778):
 * the atoms of cell `from` (in order) get ghost images in cell `to`. */
static void copy_cell_ext(orc_sys_t *s, int from, int to, const double *v,
                          int **lists, int *cnt, int *ncap) {
  int nfrom = cnt[from];
  for (int i = 0; i < nfrom; i++) {
    int src = lists[from][i];
    int g = s->next++;
    ensure_ext(s, s->next);
    for (int a = 0; a < 3; a++) {
      s->eshift[3 * g + a] = v[a];
      s->ex[3 * g + a] = s->ex[3 * src + a] + v[a];
    }
    s->etype[g] = s->etype[src];
    s->esrc[g] = src;
    s->eowner[g] = s->eowner[src];
    if (cnt[to] == ncap[to]) {
      ncap[to] = ncap[to] * 2 + 8;
      lists[to] = (int *)realloc(lists[to], sizeof(int) * ncap[to]);
    }
    lists[to][cnt[to]++] = g;
  }
}

/* fix_cells + send_cells(copy_cell) + make_nblist: wrap, bin, ghosts, list */
int orc_rebuild(orc_sys_t *s) {
  int n = s->n, cx = s->cdim[0], cy = s->cdim[1], cz = s->cdim[2];
  int nall = s->nallcells;
  int **lists = (int **)calloc(nall, sizeof(int *));
  int *cnt = (int *)calloc(nall, sizeof(int));
  int *ncap = (int *)calloc(nall, sizeof(int));
  /* wrap and bin real atoms; in-cell order = atom index order */
  for (int i = 0; i < n; i++) {
    int c[3];
    wrap_atom(s, s->x + 3 * i);
    cell_coord(s, s->x + 3 * i, c);
    int lin = (c[0] + 1) * cy * cz + (c[1] + 1) * cz + (c[2] + 1);
    if (cnt[lin] == ncap[lin]) {
      ncap[lin] = ncap[lin] * 2 + 8;
      lists[lin] = (int *)realloc(lists[lin], sizeof(int) * ncap[lin]);
    }
    lists[lin][cnt[lin]++] = i;
  }
  /* ext arrays: reals first */
  s->next = n;
  ensure_ext(s, n);
  for (int i = 0; i < n; i++) {
    for (int a = 0; a < 3; a++) {
      s->ex[3 * i + a] = s->x[3 * i + a];
      s->eshift[3 * i + a] = 0.0;
    }
    s->etype[i] = s->type[i];
    s->esrc[i] = -1;
    s->eowner[i] = i;
  }
  /* ghost copies in send_cells order (src/imd_comm_force_3d.c:247-276,
   * :288-296, :320-327, :351-358): z, then y, then x (east only, AR) */
  double zero[3] = {0, 0, 0}, up[3], dn[3], no[3], so[3], ea[3];
  for (int a = 0; a < 3; a++) {
    up[a] = s->pbc[2] == 1 ? s->box[2][a] : 0.0;
    dn[a] = s->pbc[2] == 1 ? -s->box[2][a] : 0.0;
    no[a] = s->pbc[1] == 1 ? s->box[1][a] : 0.0;
    so[a] = s->pbc[1] == 1 ? -s->box[1][a] : 0.0;
    ea[a] = s->pbc[0] == 1 ? s->box[0][a] : 0.0;
  }
  (void)zero;
#define LIN(i, j, k) ((i) * cy * cz + (j) * cz + (k))
  for (int i = 1; i < cx - 1; i++)
    for (int j = 1; j < cy - 1; j++) {
      copy_cell_ext(s, LIN(i, j, 1), LIN(i, j, cz - 1), up, lists, cnt, ncap);
      copy_cell_ext(s, LIN(i, j, cz - 2), LIN(i, j, 0), dn, lists, cnt, ncap);
    }
  for (int i = 1; i < cx - 1; i++)
    for (int k = 0; k < cz; k++) {
      copy_cell_ext(s, LIN(i, 1, k), LIN(i, cy - 1, k), no, lists, cnt, ncap);
      copy_cell_ext(s, LIN(i, cy - 2, k), LIN(i, 0, k), so, lists, cnt, ncap);
    }
  for (int j = 0; j < cy; j++)
    for (int k = 0; k < cz; k++)
      copy_cell_ext(s, LIN(1, j, k), LIN(cx - 1, j, k), ea, lists, cnt, ncap);
#undef LIN
  /* CSR of cell contents */
  s->cell_start[0] = 0;
  for (int c = 0; c < nall; c++) {
    s->cell_cnt[c] = cnt[c];
    s->cell_start[c + 1] = s->cell_start[c] + cnt[c];
  }
  s->cell_atoms = (int *)realloc(s->cell_atoms, sizeof(int) * (s->cell_start[nall] + 1));
  for (int c = 0; c < nall; c++) {
    memcpy(s->cell_atoms + s->cell_start[c], lists[c], sizeof(int) * cnt[c]);
    free(lists[c]);
  }
  free(lists);
  free(cnt);
  free(ncap);

  /* make_nblist (src/imd_forces_nbl.c:136-273) */
  for (int i = 0; i < 3 * n; i++) s->nbl_pos[i] = s->x[i];
  if (s->nb_cap == 0) {
    s->nb_cap = 64L * n + 1000;
    s->tb = (int *)malloc(sizeof(int) * s->nb_cap);
  }
  long tn = 0;
  int nn = 0;
  s->tl[0] = 0;
  for (int c = 0; c < s->nreal_cells; c++) {
    int c1 = s->real_cells[c];
    const int *nq = s->cnbrs + 14 * c;
    for (int ii = 0; ii < s->cell_cnt[c1]; ii++) {
      int i = s->cell_atoms[s->cell_start[c1] + ii];
      double d1x = s->ex[3 * i], d1y = s->ex[3 * i + 1], d1z = s->ex[3 * i + 2];
      for (int m = 0; m < 14; m++) {
        int c2 = nq[m];
        if (c2 < 0) continue;
        int jstart = (c2 == c1) ? ii + 1 : 0;
        for (int jj = jstart; jj < s->cell_cnt[c2]; jj++) {
          int j = s->cell_atoms[s->cell_start[c2] + jj];
          double dx = s->ex[3 * j] - d1x;
          double dy = s->ex[3 * j + 1] - d1y;
          double dz = s->ex[3 * j + 2] - d1z;
          double r2 = dx * dx + dy * dy + dz * dz;
          if (r2 < s->cellsz) {
            if (tn == s->nb_cap) {
              s->nb_cap = s->nb_cap * 3 / 2 + 1000;
              s->tb = (int *)realloc(s->tb, sizeof(int) * s->nb_cap);
            }
            s->tb[tn++] = j;
          }
        }
      }
      s->order[nn] = i;
      s->tl[++nn] = (int)tn;
    }
  }
  s->nb_len = tn;
  s->have_valid_nbl = 1;
  s->nbl_count++;
  return 0;
}

/* send_cells(copy_cell) on a valid list: refresh ghost positions in
 * creation order so chained copies see their updated source. */
static void refresh_ghosts(orc_sys_t *s) {
  int n = s->n;
  for (int i = 0; i < n; i++)
    for (int a = 0; a < 3; a++) s->ex[3 * i + a] = s->x[3 * i + a];
  for (int g = n; g < s->next; g++) {
    int src = s->esrc[g];
    for (int a = 0; a < 3; a++) s->ex[3 * g + a] = s->ex[3 * src + a] + s->eshift[3 * g + a];
  }
}

/* STRESS_TENS for one pair (src/imd_forces_nbl.c:558-580, :1284-1303):
 * with the force halved "to avoid double counting", -d_a f_b goes to both
 * atoms; components xx yy zz yz zx xy. */
static void stress_pair(double *pp, double *sj, double dx, double dy, double dz, double fx,
                        double fy, double fz) {
  fx *= 0.5;
  fy *= 0.5;
  fz *= 0.5;
  const double v[6] = {dx * fx, dy * fy, dz * fz, dy * fz, dz * fx, dx * fy};
  for (int c = 0; c < 6; c++) {
    pp[c] -= v[c];
    sj[c] -= v[c];
  }
}

/* Neumaier's compensated summation (a published refinement of Kahan's).
 * IMD sums the energy and the virial of every pair into one running FP64
 * total, which loses about (terms x eps) relative: 1e-9 at 4 million atoms.
 * The compensated totals beside them are accurate to a few ulps and serve as
 * the reference for summation orders other than IMD's. */
static inline void csum_add(double acc[2], double v) {
  double t = acc[0] + v;
  if (fabs(acc[0]) >= fabs(v)) acc[1] += (acc[0] - t) + v;
  else acc[1] += (v - t) + acc[0];
  acc[0] = t;
}

/* calc_forces (src/imd_forces_nbl.c:281-1999), PAIR + EAM2 */
int orc_calc_forces(orc_sys_t *s) {
  int n = s->n, nt = s->ntypes, inc = nt * nt;
  int eam = (s->interaction == ORC_EAM2);
  if (!s->have_valid_nbl) orc_rebuild(s);
  else refresh_ghosts(s);

  s->tot_pot_energy = 0.0;
  s->virial = 0.0;
  s->vir_axial[0] = s->vir_axial[1] = s->vir_axial[2] = 0.0;
  double e_acc[2] = {0.0, 0.0}, v_acc[2] = {0.0, 0.0};
  s->nfc++;
  for (int g = 0; g < s->next; g++) {
    s->ef[3 * g] = s->ef[3 * g + 1] = s->ef[3 * g + 2] = 0.0;
    s->eepot[g] = 0.0;
    s->erho[g] = 0.0;
  }
  const int st = s->do_stress;  /* do_press_calc */
  if (st)
    for (long g = 0; g < 6L * s->next; g++) s->estress[g] = 0.0;
  const double *ex = s->ex;
  /* loop 1: pair + host electron density (:423-981) */
  for (int nn = 0; nn < n; nn++) {
    int i = s->order[nn];
    double d1x = ex[3 * i], d1y = ex[3 * i + 1], d1z = ex[3 * i + 2];
    double ffx = 0, ffy = 0, ffz = 0, ee = 0, eam_r = 0;
    double pp[6] = {0, 0, 0, 0, 0, 0};
    int it = s->etype[i];
    for (int m = s->tl[nn]; m < s->tl[nn + 1]; m++) {
      int j = s->tb[m];
      double dx = ex[3 * j] - d1x, dy = ex[3 * j + 1] - d1y, dz = ex[3 * j + 2] - d1z;
      double r2 = dx * dx + dy * dy + dz * dz;
      int jt = s->etype[j];
      int col = it * nt + jt, col2 = jt * nt + it;
      if (r2 <= s->pair.end[col]) {
        double pot, grad;
        orc_pair_int2(&s->pair, col, inc, r2, &pot, &grad, &s->is_short);
        s->tot_pot_energy += pot;
        csum_add(e_acc, pot);
        double fx = dx * grad, fy = dy * grad, fz = dz * grad;
        s->ef[3 * j] -= fx;
        s->ef[3 * j + 1] -= fy;
        s->ef[3 * j + 2] -= fz;
        ffx += fx;
        ffy += fy;
        ffz += fz;
        pot *= 0.5;
        ee += pot;
        s->eepot[j] += pot;
        s->virial -= r2 * grad;
        csum_add(v_acc, -(r2 * grad));
        s->vir_axial[0] -= dx * fx;
        s->vir_axial[1] -= dy * fy;
        s->vir_axial[2] -= dz * fz;
        if (st) stress_pair(pp, s->estress + 6 * j, dx, dy, dz, fx, fy, fz);
      }
      if (eam) {
        double rho_h = 0.0;
        if (r2 < s->rho.end[col]) {
          rho_h = orc_val_func2(&s->rho, col, inc, r2, &s->is_short);
          eam_r += rho_h;
        }
        if (it == jt) {
          if (r2 < s->rho.end[col]) s->erho[j] += rho_h;
        } else {
          if (r2 < s->rho.end[col2]) {
            rho_h = orc_val_func2(&s->rho, col2, inc, r2, &s->is_short);
            s->erho[j] += rho_h;
          }
        }
      }
    }
    s->ef[3 * i] += ffx;
    s->ef[3 * i + 1] += ffy;
    s->ef[3 * i + 2] += ffz;
    s->eepot[i] += ee;
    if (eam) s->erho[i] += eam_r;
    if (st)
      for (int c = 0; c < 6; c++) s->estress[6 * i + c] += pp[c];
  }
  if (eam) {
    /* send_forces(add_rho) (:1076): fold ghosts into sources, reverse order */
    for (int g = s->next - 1; g >= n; g--) s->erho[s->esrc[g]] += s->erho[g];
    /* embedding energy (:1079-1112) */
    for (int nn = 0; nn < n; nn++) {
      int i = s->order[nn];
      double pot, df;
      int idummy = 0;
      orc_pair_int2(&s->embed, s->etype[i], nt, s->erho[i], &pot, &df, &idummy);
      s->edf[i] = df;
      s->eepot[i] += pot;
      s->tot_pot_energy += pot;
      csum_add(e_acc, pot);
    }
    /* send_cells(copy_dF) (:1115) */
    for (int g = n; g < s->next; g++) s->edf[g] = s->edf[s->esrc[g]];
    /* loop 2: EAM forces (:1117-1323) */
    for (int nn = 0; nn < n; nn++) {
      int i = s->order[nn];
      double d1x = ex[3 * i], d1y = ex[3 * i + 1], d1z = ex[3 * i + 2];
      double ffx = 0, ffy = 0, ffz = 0;
      double pp[6] = {0, 0, 0, 0, 0, 0};
      int it = s->etype[i];
      for (int m = s->tl[nn]; m < s->tl[nn + 1]; m++) {
        int j = s->tb[m];
        double dx = ex[3 * j] - d1x, dy = ex[3 * j + 1] - d1y, dz = ex[3 * j + 2] - d1z;
        double r2 = dx * dx + dy * dy + dz * dz;
        int jt = s->etype[j];
        int col1 = jt * nt + it, col2 = it * nt + jt;
        if ((r2 < s->rho.end[col1]) || (r2 < s->rho.end[col2])) {
          double rho_i_strich, rho_j_strich;
          rho_i_strich = orc_deriv_func2(&s->rho, col1, inc, r2, &s->is_short);
          if (col1 == col2)
            rho_j_strich = rho_i_strich;
          else
            rho_j_strich = orc_deriv_func2(&s->rho, col2, inc, r2, &s->is_short);
          double grad = 0.5 * (s->edf[i] * rho_j_strich + s->edf[j] * rho_i_strich);
          double fx = dx * grad, fy = dy * grad, fz = dz * grad;
          s->ef[3 * j] -= fx;
          s->ef[3 * j + 1] -= fy;
          s->ef[3 * j + 2] -= fz;
          ffx += fx;
          ffy += fy;
          ffz += fz;
          s->virial -= dx * fx + dy * fy + dz * fz;
          csum_add(v_acc, -(dx * fx + dy * fy + dz * fz));
          s->vir_axial[0] -= dx * fx;
          s->vir_axial[1] -= dy * fy;
          s->vir_axial[2] -= dz * fz;
          if (st) stress_pair(pp, s->estress + 6 * j, dx, dy, dz, fx, fy, fz);
        }
      }
      s->ef[3 * i] += ffx;
      s->ef[3 * i + 1] += ffy;
      s->ef[3 * i + 2] += ffz;
      if (st)
        for (int c = 0; c < 6; c++) s->estress[6 * i + c] += pp[c];
    }
  }
  /* send_forces(add_forces) (:1997) */
  for (int g = s->next - 1; g >= n; g--) {
    int src = s->esrc[g];
    s->ef[3 * src] += s->ef[3 * g];
    s->ef[3 * src + 1] += s->ef[3 * g + 1];
    s->ef[3 * src + 2] += s->ef[3 * g + 2];
    s->eepot[src] += s->eepot[g];
    if (st)
      for (int c = 0; c < 6; c++) s->estress[6 * src + c] += s->estress[6 * g + c];
  }
  if (st) {
    /* PRESSTENS of the real atoms; calc_tot_presstens in cell order */
    for (int c = 0; c < 6; c++) s->tot_stress[c] = 0.0;
    for (int i = 0; i < n; i++)
      for (int c = 0; c < 6; c++) s->stress[6 * i + c] = s->estress[6 * i + c];
    for (int nn = 0; nn < n; nn++)
      for (int c = 0; c < 6; c++) s->tot_stress[c] += s->stress[6 * s->order[nn] + c];
  }
  for (int i = 0; i < n; i++) {
    s->f[3 * i] = s->ef[3 * i];
    s->f[3 * i + 1] = s->ef[3 * i + 1];
    s->f[3 * i + 2] = s->ef[3 * i + 2];
    s->epot[i] = s->eepot[i];
    if (eam) {
      s->eam_rho[i] = s->erho[i];
      s->eam_df[i] = s->edf[i];
    }
  }
  s->tot_pot_energy_c = e_acc[0] + e_acc[1];
  s->virial_c = v_acc[0] + v_acc[1];
  return 0;
}

static inline double restr(const orc_sys_t *s, int t, int a) {
  return s->restrictions ? s->restrictions[3 * t + a] : 1.0;
}

/* move_atoms_nve (src/imd_integrate.c:32-497), plain NVE branch */
void orc_move_atoms_nve(orc_sys_t *s) {
  double ekin = 0.0, fnorm = 0.0, fmax2 = 0.0;
  double dt = s->timestep;
  for (int nn = 0; nn < s->n; nn++) {
    int i = s->order[nn];
    double *p = s->p + 3 * i, *f = s->f + 3 * i, *x = s->x + 3 * i;
    double kin1 = p[0] * p[0] + p[1] * p[1] + p[2] * p[2];
    int t = s->type[i];
    f[0] *= restr(s, t, 0);
    f[1] *= restr(s, t, 1);
    f[2] *= restr(s, t, 2);
    fnorm += f[0] * f[0] + f[1] * f[1] + f[2] * f[2];
    fmax2 = OMAX(SQR(f[0]), fmax2);
    fmax2 = OMAX(SQR(f[1]), fmax2);
    fmax2 = OMAX(SQR(f[2]), fmax2);
    p[0] += dt * f[0];
    p[1] += dt * f[1];
    p[2] += dt * f[2];
    double kin2 = p[0] * p[0] + p[1] * p[1] + p[2] * p[2];
    ekin += (kin1 + kin2) / (4 * s->mass[i]);
    double tmp = dt / s->mass[i];
    x[0] += tmp * p[0];
    x[1] += tmp * p[1];
    x[2] += tmp * p[2];
  }
  s->tot_kin_energy = ekin;
  s->fnorm = fnorm;
  s->f_max2 = fmax2;
}

/* move_atoms_nvt (src/imd_integrate.c:891-1150), Nose-Hoover thermostat */
void orc_move_atoms_nvt(orc_sys_t *s) {
  double e1 = 0.0, e2 = 0.0, fnorm = 0.0, fmax2 = 0.0;
  double dt = s->timestep;
  double reibung = 1.0 - s->eta * dt / 2.0;
  double eins_d_reib = 1.0 / (1.0 + s->eta * dt / 2.0);
  for (int nn = 0; nn < s->n; nn++) {
    int i = s->order[nn];
    double *p = s->p + 3 * i, *f = s->f + 3 * i, *x = s->x + 3 * i;
    double m = s->mass[i];
    e1 += (p[0] * p[0] + p[1] * p[1] + p[2] * p[2]) / m;
    int t = s->type[i];
    f[0] *= restr(s, t, 0);
    f[1] *= restr(s, t, 1);
    f[2] *= restr(s, t, 2);
    fnorm += f[0] * f[0] + f[1] * f[1] + f[2] * f[2];
    fmax2 = OMAX(SQR(f[0]), fmax2);
    fmax2 = OMAX(SQR(f[1]), fmax2);
    fmax2 = OMAX(SQR(f[2]), fmax2);
    for (int a = 0; a < 3; a++) p[a] = (p[a] * reibung + dt * f[a]) * eins_d_reib * restr(s, t, a);
    e2 += (p[0] * p[0] + p[1] * p[1] + p[2] * p[2]) / m;
    double tmp = dt / m;
    x[0] += tmp * p[0];
    x[1] += tmp * p[1];
    x[2] += tmp * p[2];
  }
  s->tot_kin_energy = (e1 + e2) / 4.0;
  s->fnorm = fnorm;
  s->f_max2 = fmax2;
  double ttt = s->nactive * s->temperature;
  s->eta += dt * (e2 / ttt - 1.0) * s->isq_tau_eta;
}

/* move_atoms_mik (src/imd_integrate.c:675-873): a momentum that points
 * against the force is set to zero (microconvergence) */
void orc_move_atoms_mik(orc_sys_t *s) {
  double ekin = 0.0, fnorm = 0.0, fmax2 = 0.0;
  double dt = s->timestep;
  for (int nn = 0; nn < s->n; nn++) {
    int i = s->order[nn];
    double *p = s->p + 3 * i, *f = s->f + 3 * i, *x = s->x + 3 * i;
    double kin1 = p[0] * p[0] + p[1] * p[1] + p[2] * p[2];
    int t = s->type[i];
    f[0] *= restr(s, t, 0);
    f[1] *= restr(s, t, 1);
    f[2] *= restr(s, t, 2);
    fnorm += f[0] * f[0] + f[1] * f[1] + f[2] * f[2];
    fmax2 = OMAX(SQR(f[0]), fmax2);
    fmax2 = OMAX(SQR(f[1]), fmax2);
    fmax2 = OMAX(SQR(f[2]), fmax2);
    p[0] += dt * f[0];
    p[1] += dt * f[1];
    p[2] += dt * f[2];
    if (0.0 > p[0] * f[0] + p[1] * f[1] + p[2] * f[2]) {
      p[0] = p[1] = p[2] = 0.0;
    } else {
      double tmp = dt / s->mass[i];
      x[0] += tmp * p[0];
      x[1] += tmp * p[1];
      x[2] += tmp * p[2];
    }
    double kin2 = p[0] * p[0] + p[1] * p[1] + p[2] * p[2];
    ekin += (kin1 + kin2) / (4.0 * s->mass[i]);
  }
  s->tot_kin_energy = ekin;
  s->fnorm = fnorm;
  s->f_max2 = fmax2;
}

/* ------------------------------------------------------------------------ */
/* GLOK / FIRE (src/imd_main_3d.c:972-1055, src/imd_integrate.c:297-316)     */
/* ------------------------------------------------------------------------ */

/* INIT values of src/globals.h:580-600 */
void orc_glok_defaults(orc_glok_t *g) {
  memset(g, 0, sizeof *g);
  g->glok_ekin_threshold = 100.0;
  g->glok_fmaxcrit = 10000.0;
  g->glok_mixdec = 1.0;
  g->glok_incfac = 1.02;
  g->glok_decfac = 0.5;
  g->glok_minsteps = 5;
}

/* update_glok (src/imd_main_3d.c:972-1055).  With ADAPTGLOK the loop that
 * steps the positions back by half a step and zeroes the momenta is the
 * else branch of `if (glok_int > glok_minsteps) mix = glok_mix;` (the
 * preprocessor lines at :1030-1035 leave the `else` without a statement of
 * its own); without ADAPTGLOK it always runs. */
void orc_update_glok(orc_sys_t *s, orc_glok_t *g, int steps) {
  const int n = s->n;
  if (steps == g->steps_min) {
    g->glok_start = g->steps_min;
    if (g->mix_on) g->mix = g->glok_mix;
  }
  g->glok_int = steps - g->glok_start;
  if (g->glok_int == 0)
    for (int i = 0; i < 3 * n; i++) s->p[i] = 0.0;
  if (g->adapt && g->nPxF >= g->min_nPxF && g->glok_int > g->glok_minsteps) {
    s->timestep = (s->timestep * g->glok_incfac > g->glok_maxtimestep)
                      ? g->glok_maxtimestep : s->timestep * g->glok_incfac;
    if (g->mix_on) g->mix *= g->glok_mixdec;
  }
  if (g->mix_on && s->fnorm >= 1e-20) g->mixforcescalefac = sqrt(g->pnorm / s->fnorm);
  const double nact = g->nactive > 0 ? (double)g->nactive : 3.0 * n;
  const double ekin = 2 * s->tot_kin_energy / nact;
  if ((g->PxF < 0.0) || (ekin > g->glok_ekin_threshold) || (sqrt(s->f_max2) >= g->glok_fmaxcrit)) {
    int back = 1;
    if (g->adapt) {
      if (steps > g->glok_minsteps && g->PxF < 0.0) {
        g->nPxF++;
        if (s->timestep > g->glok_maxtimestep / 50.0) s->timestep *= g->glok_decfac;
      }
      if (g->glok_int > g->glok_minsteps) {
        g->mix = g->glok_mix;
        back = 0;
      }
    }
    if (back)
      for (int nn = 0; nn < n; nn++) {
        int i = s->order[nn];
        for (int a = 0; a < 3; a++) {
          s->x[3 * i + a] -= 0.5 * s->timestep / s->mass[i] * s->p[3 * i + a];
          s->p[3 * i + a] = 0.0;
        }
      }
    g->glok_start = steps;
  }
}

/* move_atoms_nve (src/imd_integrate.c:32-497) with the GLOK and MIX
 * branches: the global P.F and |P/m|^2 after the momentum update, then the
 * momenta turned towards the forces by `mix` */
void orc_move_atoms_glok(orc_sys_t *s, orc_glok_t *g) {
  double ekin = 0.0, fnorm = 0.0, fmax2 = 0.0, pxf = 0.0, pnorm = 0.0;
  double dt = s->timestep;
  for (int nn = 0; nn < s->n; nn++) {
    int i = s->order[nn];
    double *p = s->p + 3 * i, *f = s->f + 3 * i, *x = s->x + 3 * i;
    double m = s->mass[i];
    double kin1 = p[0] * p[0] + p[1] * p[1] + p[2] * p[2];
    int t = s->type[i];
    f[0] *= restr(s, t, 0);
    f[1] *= restr(s, t, 1);
    f[2] *= restr(s, t, 2);
    fnorm += f[0] * f[0] + f[1] * f[1] + f[2] * f[2];
    fmax2 = OMAX(SQR(f[0]), fmax2);
    fmax2 = OMAX(SQR(f[1]), fmax2);
    fmax2 = OMAX(SQR(f[2]), fmax2);
    p[0] += dt * f[0];
    p[1] += dt * f[1];
    p[2] += dt * f[2];
    pxf += (p[0] * f[0] + p[1] * f[1] + p[2] * f[2]) / m;
    pnorm += (p[0] * p[0] + p[1] * p[1] + p[2] * p[2]) / m / m;
    if (g->mix_on)
      for (int a = 0; a < 3; a++)
        p[a] = (1.0 - g->mix) * p[a] + g->mix * f[a] * g->mixforcescalefac * m;
    double kin2 = p[0] * p[0] + p[1] * p[1] + p[2] * p[2];
    ekin += (kin1 + kin2) / (4 * m);
    double tmp = dt / m;
    x[0] += tmp * p[0];
    x[1] += tmp * p[1];
    x[2] += tmp * p[2];
  }
  s->tot_kin_energy = ekin;
  s->fnorm = fnorm;
  s->f_max2 = fmax2;
  g->pnorm = pnorm;
  g->PxF = pxf / (sqrt(fnorm) * sqrt(pnorm));
}

int orc_glok_steps(orc_sys_t *s, orc_glok_t *g, int step0, int nsteps, double *out) {
  for (int st = 0; st < nsteps; st++) {
    int rc = orc_calc_forces(s);
    if (rc < 0) return rc;
    double ep = s->tot_pot_energy;
    orc_update_glok(s, g, step0 + st);
    orc_move_atoms_glok(s, g);
    if (out) {
      double *o = out + 8 * (size_t)st;
      o[0] = ep;
      o[1] = s->tot_kin_energy;
      o[2] = s->fnorm;
      o[3] = s->f_max2;
      o[4] = s->timestep;
      o[5] = g->mix;
      o[6] = g->PxF;
      o[7] = g->glok_start;
    }
    orc_check_nblist(s);
  }
  return 0;
}

/* ------------------------------------------------------------------------ */
/* NPT, isotropic (src/imd_integrate.c:1403-1447, :1475-1728)                 */
/* ------------------------------------------------------------------------ */

void orc_npt_defaults(orc_npt_t *np) {
  memset(np, 0, sizeof *np);
  np->cell_size_tolerance = 0.05;   /* src/globals.h:570 */
}

int orc_npt_begin(orc_sys_t *s, orc_npt_t *np) {
  if (make_box(s)) return 1;
  np->volume_init = s->volume;
  int rc = init_cells(s, SQR(1.0 + np->cell_size_tolerance), np->min_height, np->max_height);
  s->have_valid_nbl = 0;
  return rc;
}

/* The buffer-cell copies of the next calc_forces use the box as it is then
 * (send_cells, src/imd_comm_force_3d.c:247-358): each ghost's copy vector
 * is one of 0, +-box_x, +-box_y, +-box_z of the old box, and becomes the
 * same vector of the new box. */
static void rescale_ghost_shifts(orc_sys_t *s, double old[3][3]) {
  for (int g = s->n; g < s->next; g++) {
    double *v = s->eshift + 3 * g;
    for (int a = 0; a < 3; a++) {
      int hit = 0;
      if (v[0] == old[a][0] && v[1] == old[a][1] && v[2] == old[a][2]) hit = 1;
      else if (v[0] == -old[a][0] && v[1] == -old[a][1] && v[2] == -old[a][2]) hit = -1;
      if (hit) {
        for (int c = 0; c < 3; c++) v[c] = hit > 0 ? s->box[a][c] : -s->box[a][c];
        break;
      }
    }
  }
}

int orc_move_atoms_npt_iso(orc_sys_t *s, orc_npt_t *np, int steps) {
  const int n = s->n;
  const double dt = s->timestep;
  const double nact = np->nactive > 0 ? (double)np->nactive : 3.0 * n;
  double Ekin_new = 0.0, fnorm = 0.0, fmax2 = 0.0;
  if (steps == np->steps_min) {
    /* calc_dyn_pressure: twice the kinetic energy, per component */
    double dx = 0.0, dy = 0.0, dz = 0.0;
    for (int nn = 0; nn < n; nn++) {
      int i = s->order[nn];
      const double *p = s->p + 3 * i;
      double tmp = 1.0 / s->mass[i];
      dx += p[0] * p[0] * tmp;
      dy += p[1] * p[1] * tmp;
      dz += p[2] * p[2] * tmp;
    }
    np->Ekin_old = dx + dy;
    np->Ekin_old += dz;
    if (np->isq_tau_xi == 0.0) np->xi = 0.0;
  }
  np->pressure = (np->Ekin_old + s->virial) / (3 * s->volume);
  np->xi_old = np->xi;
  np->xi += dt * (np->pressure - np->pressure_ext) * s->volume * np->isq_tau_xi / nact;
  double pfric = 1.0 - (np->xi_old + np->eta) * dt / 2.0;
  double pifric = 1.0 / (1.0 + (np->xi + np->eta) * dt / 2.0);
  double rfric = 1.0 + (np->xi) * dt / 2.0;
  double rifric = 1.0 / (1.0 - (np->xi) * dt / 2.0);
  for (int nn = 0; nn < n; nn++) {
    int i = s->order[nn];
    double *p = s->p + 3 * i, *f = s->f + 3 * i, *x = s->x + 3 * i;
    fnorm += f[0] * f[0] + f[1] * f[1] + f[2] * f[2];
    fmax2 = OMAX(SQR(f[0]), fmax2);
    fmax2 = OMAX(SQR(f[1]), fmax2);
    fmax2 = OMAX(SQR(f[2]), fmax2);
    for (int a = 0; a < 3; a++) p[a] = (pfric * p[a] + dt * f[a]) * pifric;
    Ekin_new += (p[0] * p[0] + p[1] * p[1] + p[2] * p[2]) / s->mass[i];
    double tmp = dt / s->mass[i];
    for (int a = 0; a < 3; a++) x[a] = (rfric * x[a] + p[a] * tmp) * rifric;
  }
  s->fnorm = fnorm;
  s->f_max2 = fmax2;
  s->tot_kin_energy = (np->Ekin_old + Ekin_new) / 4.0;
  double ttt = nact * np->temperature;
  np->eta += dt * (Ekin_new / ttt - 1.0) * np->isq_tau_eta;
  np->Ekin_old = Ekin_new;
  /* the box */
  ttt = (1.0 + np->xi * dt / 2.0) / (1.0 - np->xi * dt / 2.0);
  if (ttt < 0) return -1;   /* "box size has become negative!" */
  double old[3][3];
  memcpy(old, s->box, sizeof old);
  for (int a = 0; a < 3; a++)
    for (int c = 0; c < 3; c++) s->box[a][c] *= ttt;
  if (make_box(s)) return -2;
  if (s->volume > 8 * np->volume_init) return -4;   /* src/imd_geom_3d.c:93-97 */
  rescale_ghost_shifts(s, old);
  int out = 0;
  for (int a = 0; a < 3; a++)
    if (s->height[a] < np->min_height[a] || s->height[a] > np->max_height[a]) out = 1;
  if (out) {
    if (init_cells(s, SQR(1.0 + np->cell_size_tolerance), np->min_height, np->max_height))
      return -3;
    s->have_valid_nbl = 0;
  }
  if (steps == np->steps_min) {
    if (np->use_curr_pressure == 1) {
      np->pressure_ext = np->pressure;
      np->use_curr_pressure = 0;
    }
    np->d_pressure = (np->pressure_end - np->pressure_ext) / (np->steps_max - np->steps_min);
  }
  np->pressure_ext += np->d_pressure;
  return 0;
}

int orc_npt_steps(orc_sys_t *s, orc_npt_t *np, int step0, int nsteps, double *out) {
  for (int st = 0; st < nsteps; st++) {
    int rc = orc_calc_forces(s);
    if (rc < 0) return rc;
    double ep = s->tot_pot_energy;
    if ((rc = orc_move_atoms_npt_iso(s, np, step0 + st))) return rc;
    if (out) {
      double *o = out + 8 * (size_t)st;
      o[0] = ep;
      o[1] = s->tot_kin_energy;
      o[2] = np->xi;
      o[3] = np->eta;
      o[4] = np->pressure;
      o[5] = s->volume;
      o[6] = s->box[0][0];
      o[7] = np->pressure_ext;
    }
    orc_check_nblist(s);
  }
  return 0;
}

/* ------------------------------------------------------------------------ */
/* NPT, per axis (src/imd_integrate.c:1747-1960)                              */
/* ------------------------------------------------------------------------ */

void orc_npt_axial_defaults(orc_npt_axial_t *np) {
  memset(np, 0, sizeof *np);
  np->cell_size_tolerance = 0.05;
  np->relax_dirs[0] = np->relax_dirs[1] = np->relax_dirs[2] = 1;   /* einsivektor */
}

int orc_npt_axial_begin(orc_sys_t *s, orc_npt_axial_t *np) {
  if (make_box(s)) return 1;
  np->volume_init = s->volume;
  int rc = init_cells(s, SQR(1.0 + np->cell_size_tolerance), np->min_height, np->max_height);
  s->have_valid_nbl = 0;
  return rc;
}

int orc_move_atoms_npt_axial(orc_sys_t *s, orc_npt_axial_t *np, int steps) {
  const int n = s->n;
  const double dt = s->timestep;
  const double nact = np->nactive > 0 ? (double)np->nactive : 3.0 * n;
  double Ekin_new = 0.0, fnorm = 0.0, fmax2 = 0.0;
  double pfric[3], pifric[3], rfric[3], rifric[3];
  if (steps == np->steps_min) {
    /* calc_dyn_pressure (src/imd_integrate.c:1403-1447) */
    double d[3] = {0.0, 0.0, 0.0};
    for (int nn = 0; nn < n; nn++) {
      int i = s->order[nn];
      const double *p = s->p + 3 * i;
      double tmp = 1.0 / s->mass[i];
      for (int a = 0; a < 3; a++) d[a] += p[a] * p[a] * tmp;
    }
    for (int a = 0; a < 3; a++) np->dyn_stress[a] = d[a];
    np->Ekin_old = d[0] + d[1];
    np->Ekin_old += d[2];
    if (np->isq_tau_xi == 0.0) np->xi[0] = np->xi[1] = np->xi[2] = 0.0;
    for (int a = 0; a < 3; a++) np->xi[a] *= np->relax_dirs[a];
  }
  for (int a = 0; a < 3; a++) {
    np->stress[a] = (np->dyn_stress[a] + s->vir_axial[a]) / s->volume;
    np->dyn_stress[a] = 0.0;
  }
  double ttt = dt * s->volume * np->isq_tau_xi / nact;
  for (int a = 0; a < 3; a++) {
    np->xi_old[a] = np->xi[a];
    np->xi[a] += ttt * (np->stress[a] - np->pressure_ext[a]) * np->relax_dirs[a];
  }
  for (int a = 0; a < 3; a++) {
    pfric[a] = 1.0 - (np->xi_old[a] + np->eta) * dt / 2.0;
    pifric[a] = 1.0 / (1.0 + (np->xi[a] + np->eta) * dt / 2.0);
    rfric[a] = 1.0 + (np->xi[a]) * dt / 2.0;
    rifric[a] = 1.0 / (1.0 - (np->xi[a]) * dt / 2.0);
  }
  for (int nn = 0; nn < n; nn++) {
    int i = s->order[nn];
    double *p = s->p + 3 * i, *f = s->f + 3 * i, *x = s->x + 3 * i;
    double tmp = 1.0 / s->mass[i];
    fnorm += f[0] * f[0] + f[1] * f[1] + f[2] * f[2];
    fmax2 = OMAX(SQR(f[0]), fmax2);
    fmax2 = OMAX(SQR(f[1]), fmax2);
    fmax2 = OMAX(SQR(f[2]), fmax2);
    for (int a = 0; a < 3; a++) p[a] = (pfric[a] * p[a] + dt * f[a]) * pifric[a];
    int t = s->type[i];
    for (int a = 0; a < 3; a++) p[a] *= restr(s, t, a);
    for (int a = 0; a < 3; a++) np->dyn_stress[a] += p[a] * p[a] * tmp;
    Ekin_new += (p[0] * p[0] + p[1] * p[1] + p[2] * p[2]) * tmp;
    tmp *= dt;
    for (int a = 0; a < 3; a++) x[a] = (rfric[a] * x[a] + p[a] * tmp) * rifric[a];
  }
  s->fnorm = fnorm;
  s->f_max2 = fmax2;
  s->tot_kin_energy = (np->Ekin_old + Ekin_new) / 4.0;
  ttt = nact * np->temperature;
  np->eta += dt * (Ekin_new / ttt - 1.0) * np->isq_tau_eta;
  np->Ekin_old = Ekin_new;
  /* the box, row a scaled by its own factor */
  double tvec[3];
  for (int a = 0; a < 3; a++) tvec[a] = (1.0 + np->xi[a] * dt / 2.0) / (1.0 - np->xi[a] * dt / 2.0);
  if (tvec[0] < 0 || tvec[1] < 0 || tvec[2] < 0) return -1;   /* "box size has become negative!" */
  double old[3][3];
  memcpy(old, s->box, sizeof old);
  for (int a = 0; a < 3; a++)
    for (int c = 0; c < 3; c++) s->box[a][c] *= tvec[a];
  if (make_box(s)) return -2;
  if (s->volume > 8 * np->volume_init) return -4;
  rescale_ghost_shifts(s, old);
  int out = 0;
  for (int a = 0; a < 3; a++)
    if (s->height[a] < np->min_height[a] || s->height[a] > np->max_height[a]) out = 1;
  if (out) {
    if (init_cells(s, SQR(1.0 + np->cell_size_tolerance), np->min_height, np->max_height))
      return -3;
    s->have_valid_nbl = 0;
  }
  if (steps == np->steps_min) {
    if (np->use_curr_pressure == 1) {
      for (int a = 0; a < 3; a++) np->pressure_ext[a] = np->stress[a];
      np->use_curr_pressure = 0;
    }
    for (int a = 0; a < 3; a++)
      np->d_pressure[a] = (np->pressure_end[a] - np->pressure_ext[a]) / (np->steps_max - np->steps_min);
  }
  for (int a = 0; a < 3; a++) np->pressure_ext[a] += np->d_pressure[a];
  return 0;
}

int orc_npt_axial_steps(orc_sys_t *s, orc_npt_axial_t *np, int step0, int nsteps, double *out) {
  for (int st = 0; st < nsteps; st++) {
    int rc = orc_calc_forces(s);
    if (rc < 0) return rc;
    double ep = s->tot_pot_energy;
    if ((rc = orc_move_atoms_npt_axial(s, np, step0 + st))) return rc;
    if (out) {
      double *o = out + 12 * (size_t)st;
      o[0] = ep;
      o[1] = s->tot_kin_energy;
      for (int a = 0; a < 3; a++) o[2 + a] = np->xi[a];
      o[5] = np->eta;
      for (int a = 0; a < 3; a++) o[6 + a] = np->stress[a];
      for (int a = 0; a < 3; a++) o[9 + a] = s->box[a][a];
    }
    orc_check_nblist(s);
  }
  return 0;
}

/* check_nblist (src/imd_forces_nbl.c:2007-2037) */
void orc_check_nblist(orc_sys_t *s) {
  double max1 = 0.0;
  for (int i = 0; i < s->n; i++) {
    double dx = s->x[3 * i] - s->nbl_pos[3 * i];
    double dy = s->x[3 * i + 1] - s->nbl_pos[3 * i + 1];
    double dz = s->x[3 * i + 2] - s->nbl_pos[3 * i + 2];
    double r2 = dx * dx + dy * dy + dz * dz;
    if (r2 > max1) max1 = r2;
  }
  if (max1 > SQR(0.5 * s->nbl_margin)) s->have_valid_nbl = 0;
}

int orc_md_steps(orc_sys_t *s, int nsteps, int ensemble, double *epot_out,
                 double *ekin_out, double *extra_out) {
  for (int st = 0; st < nsteps; st++) {
    orc_calc_forces(s);
    if (epot_out) epot_out[st] = s->tot_pot_energy;
    if (ensemble == 1) orc_move_atoms_nvt(s);
    else if (ensemble == 2) orc_move_atoms_mik(s);
    else orc_move_atoms_nve(s);
    if (ekin_out) ekin_out[st] = s->tot_kin_energy;
    if (extra_out) extra_out[st] = (ensemble == 1) ? s->eta : s->fnorm;
    orc_check_nblist(s);
  }
  return 0;
}

int orc_nve_steps(orc_sys_t *s, int nsteps, double *epot_out, double *ekin_out) {
  for (int st = 0; st < nsteps; st++) {
    orc_calc_forces(s);
    if (epot_out) epot_out[st] = s->tot_pot_energy;
    orc_move_atoms_nve(s);
    if (ekin_out) ekin_out[st] = s->tot_kin_energy;
    orc_check_nblist(s);
  }
  return 0;
}

/* ------------------------------------------------------------------------ */
/* CG (src/imd_cg.c, src/cg_utils.h, move_atoms_cg src/imd_integrate.c:2881) */
/* ------------------------------------------------------------------------ */

static void move_atoms_cg(orc_sys_t *s, double alpha) {
  for (int i = 0; i < 3 * s->n; i++) s->x[i] = s->old_x[i] + alpha * s->cg_h[i];
}

static void calc_fnorm(orc_sys_t *s) {
  double t = 0.0;
  for (int nn = 0; nn < s->n; nn++) {
    int i = s->order[nn];
    double *f = s->f + 3 * i;
    int ty = s->type[i];
    f[0] *= restr(s, ty, 0);
    f[1] *= restr(s, ty, 1);
    f[2] *= restr(s, ty, 2);
    t += f[0] * f[0] + f[1] * f[1] + f[2] * f[2];
  }
  s->fnorm = t;
}

static void calc_fnorm_g_h(orc_sys_t *s) {
  double t = 0.0, fm = 0.0;
  for (int nn = 0; nn < s->n; nn++) {
    int i = s->order[nn];
    double *f = s->f + 3 * i;
    int ty = s->type[i];
    f[0] *= restr(s, ty, 0);
    f[1] *= restr(s, ty, 1);
    f[2] *= restr(s, ty, 2);
    t += f[0] * f[0] + f[1] * f[1] + f[2] * f[2];
    for (int a = 0; a < 3; a++) {
      s->old_x[3 * i + a] = s->x[3 * i + a];
      s->cg_h[3 * i + a] = f[a];
      s->cg_g[3 * i + a] = f[a];
    }
    fm = OMAX(SQR(f[0]), fm);
    fm = OMAX(SQR(f[1]), fm);
    fm = OMAX(SQR(f[2]), fm);
  }
  s->fnorm = t;
  s->f_max2 = fm;
}

static void cg_calcgamma(orc_sys_t *s) {
  double gg = 0.0, dgg = 0.0;
  for (int nn = 0; nn < s->n; nn++) {
    int i = s->order[nn];
    const double *g = s->cg_g + 3 * i, *f = s->f + 3 * i;
    gg += g[0] * g[0] + g[1] * g[1] + g[2] * g[2];
    if (s->cg_fr == 1) {
      dgg += f[0] * f[0] + f[1] * f[1] + f[2] * f[2];
    } else {
      double tx = f[0] - g[0], ty = f[1] - g[1], tz = f[2] - g[2];
      dgg += f[0] * tx + f[1] * ty + f[2] * tz;
    }
  }
  s->cg_gamma = dgg / gg;
}

static void set_hg(orc_sys_t *s) {
  double fm = 0.0;
  for (int nn = 0; nn < s->n; nn++) {
    int i = s->order[nn];
    for (int a = 0; a < 3; a++) {
      s->old_x[3 * i + a] = s->x[3 * i + a];
      s->cg_g[3 * i + a] = s->f[3 * i + a];
      s->cg_h[3 * i + a] = s->f[3 * i + a] + s->cg_gamma * s->cg_h[3 * i + a];
    }
    fm = OMAX(SQR(s->f[3 * i]), fm);
    fm = OMAX(SQR(s->f[3 * i + 1]), fm);
    fm = OMAX(SQR(s->f[3 * i + 2]), fm);
  }
  s->f_max2 = fm;
}

static double fonedim(orc_sys_t *s, double alpha) {
  move_atoms_cg(s, alpha);
  orc_check_nblist(s);
  orc_calc_forces(s);
  calc_fnorm(s);
  return s->tot_pot_energy;
}

#define CGOLD 0.3819660
#define GOLD 1.618034
#define TINY 1.0e-20
#define SHFT(a, b, c, d) \
  (a) = (b);             \
  (b) = (c);             \
  (c) = (d);
#define SIGN(a, b) ((b) >= 0.0 ? fabs(a) : -fabs(a))

/* brent (src/cg_utils.h:34-114), IMD's variant: a=ax, b=bx, x=w=v=bx */
static int brent(orc_sys_t *s, double ax, double bx, double cx, double fa,
                 double fb, double fc, double *alphamin) {
  (void)fa; (void)fc;
  double a, b, etemp, fu, fv, fw, fx, p, q, r, tol1, tol2, u, v, w, x, xm;
  double e = 0.0, d = 0.0, tol = s->linmin_tol;
  a = ax;
  b = s->cg_brent_full ? cx : bx;
  x = w = v = bx;
  fw = fv = fx = fb;
  for (int iter = 1; iter <= s->linmin_maxsteps; iter++) {
    xm = 0.5 * (a + b);
    tol1 = tol * fabs(x) + s->cg_zeps;
    tol2 = 2.0 * tol1;
    if (fabs(x - xm) <= (tol2 - 0.5 * (b - a))) {
      *alphamin = x;
      return iter;
    }
    if (fabs(e) > tol1) {
      r = (x - w) * (fx - fv);
      q = (x - v) * (fx - fw);
      p = (x - v) * q - (x - w) * r;
      q = 2.0 * (q - r);
      if (q > 0.0) p = -p;
      q = fabs(q);
      etemp = e;
      e = d;
      if (fabs(p) >= fabs(0.5 * q * etemp) || p <= q * (a - x) || p >= q * (b - x)) {
        e = (x >= xm) ? (a - x) : (b - x);
        d = CGOLD * e;
      } else {
        d = p / q;
        u = x + d;
        if ((u - a < tol2) || (b - u < tol2)) d = SIGN(tol1, xm - x);
      }
    } else {
      e = (x >= xm) ? (a - x) : (b - x);
      d = CGOLD * e;
    }
    u = ((fabs(d) >= tol1) ? (x + d) : (x + SIGN(tol1, d)));
    fu = fonedim(s, u);
    if (fu <= fx) {
      if (u >= x) a = x;
      else b = x;
      SHFT(v, w, x, u)
      SHFT(fv, fw, fx, fu)
    } else {
      if (u < x) a = u;
      else b = u;
      if ((fu <= fw) || (w == x)) {
        v = w;
        fv = fw;
        w = u;
        fw = fu;
      } else if ((fu <= fv) || (v == x) || (v == w)) {
        v = u;
        fv = fu;
      }
    }
  }
  return -1; /* "Too many iterations in brent" */
}

/* mnbrak (src/cg_utils.h:119-194) */
static int mnbrak(orc_sys_t *s, double *ax, double *bx, double *cx, double *fa,
                  double *fb, double *fc) {
  double ulim, u, r, q, fu, dum;
  int ctf;
  if (*fb > *fa) {
    SHFT(dum, *ax, *bx, dum)
    SHFT(dum, *fb, *fa, dum)
  }
  *cx = (*bx) + GOLD * (*bx - *ax);
  if ((*bx - *ax) <= 1e-4) *cx = (*bx) + 0.05;
  if (*cx < 0.0) *cx = (*bx) - 1.0 / GOLD * (*bx - *ax);
  if (*cx >= 1.0) *cx = 1.0;
  *fc = fonedim(s, *cx);
  ctf = 1;
  while (*fb >= *fc) {
    r = (*bx - *ax) * (*fb - *fc);
    q = (*bx - *cx) * (*fb - *fa);
    u = (*bx) - ((*bx - *cx) * q - (*bx - *ax) * r) /
                    (2.0 * SIGN(OMAX(fabs(q - r), TINY), q - r));
    ulim = (*bx) + s->cg_glimit * (*cx - *bx);
    if ((*bx - u) * (u - *cx) > 0.0) {
      fu = fonedim(s, u);
      ctf++;
      if (fu < *fc) {
        *ax = (*bx);
        *bx = u;
        *fa = (*fb);
        *fb = fu;
        return ctf;
      } else if (fu > *fb) {
        *cx = u;
        *fc = fu;
        return ctf;
      }
      u = (*cx) + GOLD * (*cx - *bx);
      fu = fonedim(s, u);
      ctf++;
    } else if ((*cx - u) * (u - ulim) > 0.0) {
      fu = fonedim(s, u);
      ctf++;
      if (fu < *fc) {
        SHFT(*bx, *cx, u, *cx + GOLD * (*cx - *bx))
        SHFT(*fb, *fc, fu, fonedim(s, u))
        ctf++;
      }
    } else if ((u - ulim) * (ulim - *cx) >= 0.0) {
      u = ulim;
      fu = fonedim(s, u);
      ctf++;
    } else {
      u = (*cx) + GOLD * (*cx - *bx);
      fu = fonedim(s, u);
      ctf++;
    }
    SHFT(*ax, *bx, *cx, u)
    SHFT(*fa, *fb, *fc, fu)
  }
  return ctf;
}

/* linmin (src/imd_cg.c:96-200) */
static int linmin(orc_sys_t *s) {
  double alpha_a, alpha_b, alpha_c, fa, fb, fc, dum, alphamin = 0.0;
  double f_max = sqrt(s->f_max2);
  if (f_max > 100 * s->linmin_dmax)
    alpha_b = s->linmin_dmax / f_max;
  else if (s->old_alphamin < s->linmin_dmin)
    alpha_b = 0.05;
  else
    alpha_b = 2.0 * s->old_alphamin;
  alpha_c = 2.0 * alpha_b;
  alpha_a = 0.0;
  fa = s->old_cg_poteng;
  fb = fonedim(s, alpha_b);
  int iter1 = mnbrak(s, &alpha_a, &alpha_b, &alpha_c, &fa, &fb, &fc);
  if (alpha_a > alpha_b) {
    SHFT(dum, alpha_a, alpha_b, dum)
    SHFT(dum, fa, fb, dum)
  }
  if (alpha_b > alpha_c) {
    SHFT(dum, alpha_b, alpha_c, dum)
    SHFT(dum, fb, fc, dum)
  }
  if (alpha_a > alpha_b) {
    SHFT(dum, alpha_a, alpha_b, dum)
    SHFT(dum, fa, fb, dum)
  }
  int iter2 = brent(s, alpha_a, alpha_b, alpha_c, fa, fb, fc, &alphamin);
  if (iter2 < 0) return -1;
  s->old_alphamin = alphamin;
  return iter1 + iter2;
}

int orc_reset_cg(orc_sys_t *s) {
  orc_calc_forces(s);
  calc_fnorm_g_h(s);
  s->cg_poteng = s->tot_pot_energy;
  s->old_cg_poteng = s->cg_poteng;
  return 0;
}

int orc_cg_step(orc_sys_t *s, int steps) {
  if (s->cg_reset_int > 0 && 0 == steps % s->cg_reset_int) orc_reset_cg(s);
  s->cg_poteng = s->tot_pot_energy;
  s->old_cg_poteng = s->cg_poteng;
  if (linmin(s) < 0) return -1;
  cg_calcgamma(s);
  set_hg(s);
  return 0;
}

double orc_max_atom_force(const orc_sys_t *s) {
  double m = 0.0;
  for (int i = 0; i < s->n; i++) {
    const double *f = s->f + 3 * i;
    double v = f[0] * f[0] + f[1] * f[1] + f[2] * f[2];
    if (v > m) m = v;
  }
  return sqrt(m);
}

/* main_loop with ensemble cg (src/imd_main_3d.c:140, :393, :760, :769),
 * stopping on the max per-atom force. */
int orc_cg_relax(orc_sys_t *s, double fmax, int maxsteps, double *fmax_out) {
  orc_reset_cg(s);
  double fm = orc_max_atom_force(s);
  int steps = 0;
  while (fm > fmax && steps < maxsteps) {
    steps++;
    if (orc_cg_step(s, steps) < 0) return -1;
    fm = orc_max_atom_force(s);
    orc_check_nblist(s);
  }
  if (fmax_out) *fmax_out = fm;
  return steps;
}

/* neighbour pairs of the current list with ghost image shifts */
long orc_pairs(const orc_sys_t *s, long cap, int *ni, int *nj, int *shift, double *r2) {
  long cnt = 0;
  int n = s->n;
  for (int nn = 0; nn < n; nn++) {
    int i = s->order[nn];
    for (int m = s->tl[nn]; m < s->tl[nn + 1]; m++) {
      int j = s->tb[m];
      if (cnt < cap) {
        ni[cnt] = s->number[i];
        nj[cnt] = s->number[s->eowner[j]];
        /* image shift in box vectors: solve from the position difference */
        int o = s->eowner[j];
        for (int a = 0; a < 3; a++) {
          double d[3] = {s->ex[3 * j] - s->ex[3 * o], s->ex[3 * j + 1] - s->ex[3 * o + 1],
                         s->ex[3 * j + 2] - s->ex[3 * o + 2]};
          shift[3 * cnt + a] = (int)lround(sprod(d, s->tbox[a]));
        }
        double dx = s->ex[3 * j] - s->ex[3 * i], dy = s->ex[3 * j + 1] - s->ex[3 * i + 1],
               dz = s->ex[3 * j + 2] - s->ex[3 * i + 2];
        r2[cnt] = dx * dx + dy * dy + dz * dz;
      }
      cnt++;
    }
  }
  return cnt;
}
