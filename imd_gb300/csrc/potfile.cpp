// potfile.cpp -- host reader of IMD potential tables for libimdgpu.
//
// Reads the two file formats of read_pot_table (src/imd_potential.c:161-282;
// format 1 :297-376, format 2 :394-462) into the pot_table_t layout
// (src/types.h:416-428) and applies init_threepoint (:1256-1272).  In the
// IMD cuda target IMD's own reader fills pot_table_t and passes it through
// imdgpu_set_table(); this reader serves standalone callers.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "hosttab.h"

namespace imdgpu {

static void threepoint(HostTable &t) {
  const int nc = t.ncols;
  for (int col = 0; col < nc; col++) {
    double *y = t.table.data() + col;
    const int n = t.len[col];
    if (n < 3) continue;
    y[n * nc] = 3 * y[(n - 1) * nc] - 3 * y[(n - 2) * nc] + y[(n - 3) * nc];
    y[(n + 1) * nc] = 6 * y[(n - 1) * nc] - 8 * y[(n - 2) * nc] + 3 * y[(n - 3) * nc];
  }
}

// init_fourpoint (src/imd_potential.c:1171-1187)
static void fourpoint(HostTable &t) {
  const int nc = t.ncols;
  for (int col = 0; col < nc; col++) {
    double *y = t.table.data() + col;
    const int n = t.len[col];
    if (n < 4) continue;
    y[n * nc] = 4 * y[(n - 1) * nc] - 6 * y[(n - 2) * nc] + 4 * y[(n - 3) * nc] - y[(n - 4) * nc];
    y[(n + 1) * nc] =
        10 * y[(n - 1) * nc] - 20 * y[(n - 2) * nc] + 15 * y[(n - 3) * nc] - 4 * y[(n - 4) * nc];
  }
}

// init_spline (src/imd_potential.c:1197-1246): natural at the left end, zero
// slope at the right end of radial functions, natural otherwise
static void spline(HostTable &t, int radial) {
  const int nc = t.ncols, size = t.maxsteps + 2;
  t.table2.assign((size_t)nc * size, 0.0);
  std::vector<double> u(size, 0.0);
  for (int col = 0; col < nc; col++) {
    double *y2 = t.table2.data() + col, *y = t.table.data() + col;
    const int n = t.len[col];
    const double step = t.step[col];
    double p, qn, un;
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
    y[n * nc] = 2 * y[(n - 1) * nc] - y[(n - 2) * nc] + step * step * y2[(n - 1) * nc];
    y2[n * nc] = 2 * y2[(n - 1) * nc] - y2[(n - 2) * nc];
  }
}

void init_interpolation(HostTable &t, int radial, int mode) {
  t.mode = mode;
  if (mode == 1) fourpoint(t);
  else if (mode == 2) spline(t, radial);
  else threepoint(t);
}

int read_table_file(const char *fname, int ncols, int radial, int default_format,
                    HostTable &t, double &cellsz, std::string &err, int mode) {
  FILE *in = std::fopen(fname, "r");
  if (!in) {
    err = std::string("Could not open potential file ") + fname;
    return 1;
  }
  char buf[1024];
  int have_header = 0, have_format = 0, end_header = 0;
  int format = default_format, size = ncols;
  do {
    if (!std::fgets(buf, sizeof buf, in)) {
      err = std::string("Unexpected end of file in ") + fname;
      std::fclose(in);
      return 1;
    }
    if (buf[0] == '#') {
      have_header = 1;
      end_header = (buf[1] == 'E');
      if (buf[1] == 'F') {
        if (2 != std::sscanf(buf + 2, "%d%d", &format, &size)) {
          err = std::string("Corrupted format header line in file ") + fname;
          std::fclose(in);
          return 1;
        }
        if (size != ncols) {
          err = std::string("Wrong number of data columns in file ") + fname;
          std::fclose(in);
          return 1;
        }
        if (format != 1 && format != 2) {
          err = std::string("Unrecognized format specified for file ") + fname;
          std::fclose(in);
          return 1;
        }
        have_format = 1;
      }
    } else if (have_header) {
      err = std::string("Corrupted header in file ") + fname;
      std::fclose(in);
      return 1;
    } else {
      end_header = 1;
    }
  } while (!end_header);
  if (have_header && !have_format) {
    err = std::string("Format not specified in header of file ") + fname;
    std::fclose(in);
    return 1;
  }
  if (!have_header) std::rewind(in);

  t.ncols = ncols;
  t.begin.assign(ncols, 0.0);
  t.end.assign(ncols, 0.0);
  t.step.assign(ncols, 0.0);
  t.invstep.assign(ncols, 0.0);
  t.len.assign(ncols, 0);
  t.maxsteps = 0;
  if (format == 1) {
    std::vector<double> rows;
    double r2 = 0.0, r2_start = 0.0, val;
    int npot = 0;
    for (;;) {
      if (1 != std::fscanf(in, "%lf", &r2)) break;
      if (npot == 0) r2_start = r2;
      for (int i = 0; i < ncols; i++) {
        if (1 != std::fscanf(in, "%lf", &val)) {
          err = "Line incomplete in potential file.";
          std::fclose(in);
          return 1;
        }
        rows.push_back(val);
        if (val != 0.0) {
          t.end[i] = r2;
          t.len[i] = npot + 1;
        }
      }
      npot++;
    }
    if (npot < 3) {
      err = "potential table too short";
      std::fclose(in);
      return 1;
    }
    const double r2_step = (r2 - r2_start) / (npot - 1);
    t.maxsteps = npot;
    t.table.assign((size_t)ncols * (npot + 2), 0.0);
    std::memcpy(t.table.data(), rows.data(), rows.size() * sizeof(double));
    for (int i = 0; i < ncols; i++) {
      t.begin[i] = r2_start;
      t.step[i] = r2_step;
      t.invstep[i] = 1.0 / r2_step;
      const double delta = t.table[(size_t)(npot - 1) * ncols + i];
      if (radial && delta != 0.0)
        for (int k = 0; k < npot; k++) t.table[(size_t)k * ncols + i] -= delta;
      if (radial) cellsz = std::fmax(cellsz, t.end[i]);
    }
  } else {
    for (int i = 0; i < ncols; i++) {
      if (3 != std::fscanf(in, "%lf %lf %lf", &t.begin[i], &t.end[i], &t.step[i])) {
        err = "Info line corrupt.";
        std::fclose(in);
        return 1;
      }
      if (radial) cellsz = (cellsz > t.end[i]) ? cellsz : t.end[i];
      t.invstep[i] = 1.0 / t.step[i];
      const double numstep = 1 + (t.end[i] - t.begin[i]) / t.step[i];
      t.len[i] = (int)(numstep + 0.49);
      if (t.len[i] > t.maxsteps) t.maxsteps = t.len[i];
    }
    t.table.assign((size_t)ncols * (t.maxsteps + 2), 0.0);
    for (int i = 0; i < ncols; i++)
      for (int k = 0; k < t.len[i]; k++) {
        double val;
        if (1 != std::fscanf(in, "%lf", &val)) {
          err = std::string("wrong format in file ") + fname;
          std::fclose(in);
          return 1;
        }
        t.table[(size_t)k * ncols + i] = val;
      }
    if (radial)
      for (int i = 0; i < ncols; i++) {
        const double delta = t.table[(size_t)(t.len[i] - 1) * ncols + i];
        if (delta != 0.0)
          for (int k = 0; k < t.len[i]; k++) t.table[(size_t)k * ncols + i] -= delta;
      }
  }
  std::fclose(in);
  for (int i = 0; i < ncols; i++)
    if (t.len[i] < 3) {
      err = std::string("column with fewer than 3 values in ") + fname;
      return 1;
    }
  init_interpolation(t, radial, mode);
  t.radial = radial;
  return 0;
}

}  // namespace imdgpu
