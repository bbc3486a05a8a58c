// ref_probe: golden-vector probe built from ExaMiniMD's own sources (through
// the serial Kokkos-subset shim).  TEST INFRASTRUCTURE ONLY.
//
//   ref_probe OUT.bin [ExaMiniMD command line ...]
//
// Runs ExaMiniMD::init (examinimd.cpp:60-174) -- lattice, exchange, sorted
// binning, six-phase halo, ghost binning, neighbour list, initial forces --
// and writes the reference's own intermediate arrays: the binning
// (bincount / binoffsets / permute_vector of binning.h:50-59), all particles
// including ghosts, the neighbour rows (NeighListCSR / NeighList2D) and the
// forces.  Record format: name[32], type char ('i' int32 / 'd' f64),
// int64 count, payload.
#include <cstdio>
#include <cstring>
#include <vector>

#include <examinimd.h>
#include <neighbor_2d.h>
#include <neighbor_csr.h>
#include <neighbor_csr_map_constr.h>

static void rec(FILE* fp, const char* name, char t, long long n, const void* p) {
  char nm[32] = {0};
  strncpy(nm, name, 31);
  fwrite(nm, 1, 32, fp);
  fwrite(&t, 1, 1, fp);
  fwrite(&n, sizeof(long long), 1, fp);
  fwrite(p, t == 'i' ? 4 : 8, size_t(n), fp);
}

int main(int argc, char* argv[]) {
  if (argc < 2) {
    fprintf(stderr, "usage: ref_probe OUT.bin [ExaMiniMD args]\n");
    return 2;
  }
  const char* out = argv[1];
  argv[1] = argv[0];
  int eargc = argc - 1;
  char** eargv = argv + 1;
  Kokkos::initialize(eargc, eargv);
  {
    ExaMiniMD e;
    e.init(eargc, eargv);
    System* s = e.system;
    FILE* fp = fopen(out, "wb");
    if (!fp) return 3;
    const int nl = s->N_local, ng = s->N_ghost, nt = nl + ng;
    int counts[2] = {nl, ng};
    rec(fp, "counts", 'i', 2, counts);
    int nbin[4] = {e.binning->nbinx, e.binning->nbiny, e.binning->nbinz, e.binning->nhalo};
    rec(fp, "nbin", 'i', 4, nbin);
    const long long nb = (long long)nbin[0] * nbin[1] * nbin[2];
    std::vector<int> bc(nb), bo(nb);
    for (int x = 0; x < nbin[0]; x++)
      for (int y = 0; y < nbin[1]; y++)
        for (int z = 0; z < nbin[2]; z++) {
          bc[(size_t(x) * nbin[1] + y) * nbin[2] + z] = e.binning->bincount(x, y, z);
          bo[(size_t(x) * nbin[1] + y) * nbin[2] + z] = e.binning->binoffsets(x, y, z);
        }
    rec(fp, "bincount", 'i', nb, bc.data());
    rec(fp, "binoffsets", 'i', nb, bo.data());
    std::vector<int> perm(e.binning->permute_vector.extent(0));
    for (size_t k = 0; k < perm.size(); k++) perm[k] = e.binning->permute_vector(k);
    rec(fp, "permute", 'i', (long long)perm.size(), perm.data());
    double bounds[6] = {e.binning->minx, e.binning->maxx, e.binning->miny, e.binning->maxy, e.binning->minz, e.binning->maxz};
    rec(fp, "bounds", 'd', 6, bounds);
    std::vector<double> x(3 * size_t(nt)), v(3 * size_t(nt)), f(3 * size_t(nt));
    std::vector<int> id(nt), type(nt);
    for (int i = 0; i < nt; i++) {
      for (int d = 0; d < 3; d++) {
        x[3 * size_t(i) + d] = s->x(i, d);
        v[3 * size_t(i) + d] = s->v(i, d);
        f[3 * size_t(i) + d] = s->f(i, d);
      }
      id[i] = s->id(i);
      type[i] = s->type(i);
    }
    rec(fp, "x", 'd', 3LL * nt, x.data());
    rec(fp, "v", 'd', 3LL * nt, v.data());
    rec(fp, "f", 'd', 3LL * nt, f.data());
    rec(fp, "id", 'i', nt, id.data());
    rec(fp, "type", 'i', nt, type.data());
    std::vector<int> num(nl), ent;
    if (e.input->neighbor_type == NEIGH_CSR) {
      auto list = ((NeighborCSR<t_neigh_mem_space>*)e.neighbor)->get_neigh_list();
      for (int i = 0; i < nl; i++) {
        auto row = list.get_neighs(i);
        num[i] = row.get_num_neighs();
        for (int k = 0; k < num[i]; k++) ent.push_back(row(k));
      }
    } else if (e.input->neighbor_type == NEIGH_CSR_MAPCONSTR) {
      // the same CSR container, rows in the hash map's order
      auto list = ((NeighborCSRMapConstr<t_neigh_mem_space>*)e.neighbor)->get_neigh_list();
      for (int i = 0; i < nl; i++) {
        auto row = list.get_neighs(i);
        num[i] = row.get_num_neighs();
        for (int k = 0; k < num[i]; k++) ent.push_back(row(k));
      }
    } else {
      auto list = ((Neighbor2D<t_neigh_mem_space>*)e.neighbor)->get_neigh_list();
      int mx = list.maxneighs;
      rec(fp, "maxneighs", 'i', 1, &mx);
      for (int i = 0; i < nl; i++) {
        auto row = list.get_neighs(i);
        num[i] = row.get_num_neighs();
        for (int k = 0; k < num[i]; k++) ent.push_back(row(k));
      }
    }
    rec(fp, "num_neighs", 'i', nl, num.data());
    rec(fp, "neighs", 'i', (long long)ent.size(), ent.data());
    fclose(fp);
  }
  Kokkos::finalize();
  return 0;
}
