// SNAP file parsing with the reference's rules (force_snap_neigh_impl.h:341-587):
//  * .snapcoeff: the first line that has no '#' and is not blank holds
//    "nelemfile ncoeffall"; each element block is "name radius weight"
//    followed by ncoeffall lines whose first word is a coefficient; blocks of
//    elements not named in pair_coeff (or repeated) are skipped.  As in the
//    reference, radius and weight of the last block read are assigned to
//    every element (it deep-copies into the whole radelem / wjelem views).
//  * .snapparam: lines containing '#' and blank lines are skipped; keywords
//    rcutfac and twojmax are required; rfac0, rmin0, diagonalstyle,
//    switchflag, bzeroflag, quadraticflag are optional.
#include "snap_params.h"

#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "emd_host.h"

namespace emdhost {

SnapFiles read_snap_files(const char* coefffile, const char* paramfile, const std::vector<std::string>& elements) {
  SnapFiles s;
  const int nelements = int(elements.size());
  FILE* fp = fopen(coefffile, "r");
  if (!fp) throw HostError(std::string("Cannot open SNAP coefficient file ") + coefffile);
  char line[1024];
  bool header = false;
  while (fgets(line, sizeof(line), fp)) {
    char* p = strchr(line, '#');
    if (p) continue;
    if (line[0] != '\n') {
      header = true;
      break;
    }
  }
  if (!header) {
    fclose(fp);
    throw HostError("Incorrect format in SNAP coefficient file");
  }
  const char* delim = "' \t\n\r\f";
  char* w0 = strtok(line, delim);
  char* w1 = strtok(nullptr, delim);
  if (!w0 || !w1) {
    fclose(fp);
    throw HostError("Incorrect format in SNAP coefficient file");
  }
  const int nelemfile = atoi(w0);
  s.ncoeffall = atoi(w1);
  s.radelem.assign(size_t(nelements), 0.0);
  s.wjelem.assign(size_t(nelements), 0.0);
  s.coeffelem.assign(size_t(nelements) * s.ncoeffall, 0.0);
  std::vector<int> found(size_t(nelements), 0);
  for (int ielemfile = 0; ielemfile < nelemfile; ielemfile++) {
    if (!fgets(line, sizeof(line), fp)) {
      fclose(fp);
      throw HostError("Incorrect format in SNAP coefficient file");
    }
    char* e = strtok(line, delim);
    char* r = strtok(nullptr, delim);
    char* wj = strtok(nullptr, delim);
    if (!e || !r || !wj) {
      fclose(fp);
      throw HostError("Incorrect format in SNAP coefficient file");
    }
    int ielem = 0;
    for (; ielem < nelements; ielem++)
      if (elements[size_t(ielem)] == e) break;
    if (ielem == nelements || found[size_t(ielem)]) {
      for (int k = 0; k < s.ncoeffall; k++)
        if (!fgets(line, sizeof(line), fp)) break;
      continue;
    }
    found[size_t(ielem)] = 1;
    const double radtmp = atof(r), wjtmp = atof(wj);
    for (int k = 0; k < nelements; k++) {
      s.radelem[size_t(k)] = radtmp;
      s.wjelem[size_t(k)] = wjtmp;
    }
    for (int icoeff = 0; icoeff < s.ncoeffall; icoeff++) {
      if (!fgets(line, sizeof(line), fp)) {
        fclose(fp);
        throw HostError("Incorrect format in SNAP coefficient file");
      }
      char* c = strtok(line, delim);
      s.coeffelem[size_t(ielem) * s.ncoeffall + icoeff] = c ? atof(c) : 0.0;
    }
  }
  fclose(fp);

  fp = fopen(paramfile, "r");
  if (!fp) throw HostError(std::string("Cannot open SNAP parameter file ") + paramfile);
  bool have_rcutfac = false, have_twojmax = false;
  while (fgets(line, sizeof(line), fp)) {
    if (strchr(line, '#')) continue;
    if (line[0] == '\n') continue;
    char* key = strtok(line, delim);
    char* val = strtok(nullptr, delim);
    if (!key) continue;
    if (!val) {
      fclose(fp);
      throw HostError("Incorrect format in SNAP parameter file");
    }
    const std::string k = key;
    if (k == "rcutfac") {
      s.rcutfac = atof(val);
      have_rcutfac = true;
    } else if (k == "twojmax") {
      s.twojmax = atoi(val);
      have_twojmax = true;
    } else if (k == "rfac0") s.rfac0 = atof(val);
    else if (k == "rmin0") s.rmin0 = atof(val);
    else if (k == "diagonalstyle") s.diagonalstyle = atoi(val);
    else if (k == "switchflag") s.switchflag = atoi(val);
    else if (k == "bzeroflag") s.bzeroflag = atoi(val);
    else if (k == "quadraticflag") s.quadraticflag = atoi(val);
    else {
      fclose(fp);
      throw HostError("Incorrect SNAP parameter file");
    }
  }
  fclose(fp);
  if (!have_rcutfac || !have_twojmax) throw HostError("Incorrect SNAP parameter file");
  if (s.diagonalstyle != 3) throw HostError("SNAP: only diagonalstyle 3 is supported (as SNA::build_indexlist)");
  if (s.quadraticflag) throw HostError("SNAP: quadraticflag is not supported (the reference force is linear)");
  return s;
}

}  // namespace emdhost
