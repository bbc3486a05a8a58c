// SNAP coefficient / parameter file reader (force_snap_neigh_impl.h:341-587).
#pragma once
#include <string>
#include <vector>

namespace emdhost {

struct SnapFiles {
  int ncoeffall = 0;
  std::vector<double> radelem, wjelem;  // per element in the pair_coeff element list
  std::vector<double> coeffelem;        // nelements x ncoeffall, row-major
  double rcutfac = 0, rfac0 = 0.99363, rmin0 = 0.0;
  int twojmax = 0, diagonalstyle = 3, switchflag = 1, bzeroflag = 1, quadraticflag = 0;
};

SnapFiles read_snap_files(const char* coefffile, const char* paramfile, const std::vector<std::string>& elements);

}  // namespace emdhost
