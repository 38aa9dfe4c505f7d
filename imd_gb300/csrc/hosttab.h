// hosttab.h -- host copy of one pot_table_t (src/types.h:416-428).
#pragma once

#include <string>
#include <vector>

namespace imdgpu {

struct HostTable {
  int ncols = 0;
  int maxsteps = 0;  // rows = maxsteps + 2
  int radial = 1;
  std::vector<double> begin, end, step, invstep;
  std::vector<int> len;
  std::vector<double> table;  // table[k * ncols + col]
  std::vector<double> table2; // spline second derivatives (same layout)
  int mode = 0;               // 0 quadratic (3-point), 1 4-point, 2 spline
};

// read_pot_table and the initialisation of the interpolation `mode`
// (init_threepoint / init_fourpoint / init_spline)
int read_table_file(const char *fname, int ncols, int radial, int default_format,
                    HostTable &t, double &cellsz, std::string &err, int mode = 0);
// init_threepoint / init_fourpoint / init_spline on a table already read
void init_interpolation(HostTable &t, int radial, int mode);

}  // namespace imdgpu
