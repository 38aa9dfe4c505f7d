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
};

int read_table_file(const char *fname, int ncols, int radial, int default_format,
                    HostTable &t, double &cellsz, std::string &err);

}  // namespace imdgpu
