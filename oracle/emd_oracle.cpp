// CPU oracle for the ExaMiniMD hot path -- TEST INFRASTRUCTURE ONLY (see
// emd_oracle.h).  A serial restatement of the reference functions; every
// function names the ExaMiniMD file:line it follows.  Compiled with
// -ffp-contract=off so no multiply-add is fused on any host.
#include "emd_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

const double MY_PI = 3.14159265358979323846;

struct OrcErr : std::runtime_error {
  explicit OrcErr(const std::string& m) : std::runtime_error(m) {}
};

// ------------------------------------------------------------------ SNA
// SNA (sna.h:68-211, sna_impl.hpp): tables and per-atom kernels in the
// reference formulation (U, Z, dU, dB).
struct Sna {
  int twojmax = 0, jdim = 0;
  double rfac0 = 0, rmin0 = 0, wself = 1.0;
  int switch_flag = 1;
  struct Idx {
    int j1, j2, j;
  };
  std::vector<Idx> idxj, idxj_full;
  std::vector<double> cg, rootpq;
  int ncoeff = 0;
  // per-atom working arrays
  std::vector<double> utot_r, utot_i, u_r, u_i, z_r, z_i, du_r, du_i, dbarray;

  size_t i3(int j, int a, int b) const { return (size_t(j) * jdim + a) * jdim + b; }
  size_t i5(int a, int b, int c, int d, int e) const {
    return (((size_t(a) * jdim + b) * jdim + c) * jdim + d) * jdim + e;
  }
  size_t i4(int j, int mb, int ma, int k) const { return ((size_t(j) * jdim + mb) * jdim + ma) * 3 + k; }

  static double factorial(int n) {  // sna_impl.hpp:977-983
    double r = 1.0;
    for (int i = 1; i <= n; i++) r *= 1.0 * i;
    return r;
  }
  static double deltacg(int j1, int j2, int j) {  // sna_impl.hpp:989-996
    double sfaccg = factorial((j1 + j2 + j) / 2 + 1);
    return std::sqrt(factorial((j1 + j2 - j) / 2) * factorial((j1 - j2 + j) / 2) * factorial((-j1 + j2 + j) / 2) /
                     sfaccg);
  }

  void init(int twojmax_, double rfac0_, double rmin0_, int switch_flag_) {
    twojmax = twojmax_;
    jdim = twojmax + 1;
    rfac0 = rfac0_;
    rmin0 = rmin0_;
    switch_flag = switch_flag_;
    // build_indexlist (sna_impl.hpp:88-139), diagonalstyle 3
    idxj.clear();
    idxj_full.clear();
    for (int j1 = 0; j1 <= twojmax; j1++)
      for (int j2 = 0; j2 <= j1; j2++)
        for (int j = std::abs(j1 - j2); j <= std::min(twojmax, j1 + j2); j += 2) {
          if (j >= j1) idxj.push_back({j1, j2, j});
          idxj_full.push_back({j1, j2, j});
        }
    ncoeff = int(idxj.size());
    // init_clebsch_gordan (sna_impl.hpp:1003-1046), VMK 8.2.1(3)
    cg.assign(size_t(jdim) * jdim * jdim * jdim * jdim, 0.0);
    for (int j1 = 0; j1 <= twojmax; j1++)
      for (int j2 = 0; j2 <= twojmax; j2++)
        for (int j = std::abs(j1 - j2); j <= std::min(twojmax, j1 + j2); j += 2)
          for (int m1 = 0; m1 <= j1; m1++) {
            const int aa2 = 2 * m1 - j1;
            for (int m2 = 0; m2 <= j2; m2++) {
              const int bb2 = 2 * m2 - j2;
              const int m = (aa2 + bb2 + j) / 2;
              if (m < 0 || m > j) continue;
              double sum = 0.0;
              for (int z = std::max(0, std::max(-(j - j2 + aa2) / 2, -(j - j1 - bb2) / 2));
                   z <= std::min((j1 + j2 - j) / 2, std::min((j1 - aa2) / 2, (j2 + bb2) / 2)); z++) {
                const int ifac = z % 2 ? -1 : 1;
                sum += ifac / (factorial(z) * factorial((j1 + j2 - j) / 2 - z) * factorial((j1 - aa2) / 2 - z) *
                               factorial((j2 + bb2) / 2 - z) * factorial((j - j2 + aa2) / 2 + z) *
                               factorial((j - j1 - bb2) / 2 + z));
              }
              const int cc2 = 2 * m - j;
              const double dcg = deltacg(j1, j2, j);
              const double sfaccg = std::sqrt(factorial((j1 + aa2) / 2) * factorial((j1 - aa2) / 2) *
                                              factorial((j2 + bb2) / 2) * factorial((j2 - bb2) / 2) *
                                              factorial((j + cc2) / 2) * factorial((j - cc2) / 2) * (j + 1));
              cg[i5(j1, j2, j, m1, m2)] = sum * dcg * sfaccg;
            }
          }
    // init_rootpqarray (sna_impl.hpp:1054-1061)
    rootpq.assign(size_t(jdim + 1) * (jdim + 1), 0.0);
    for (int p = 1; p <= twojmax; p++)
      for (int q = 1; q <= twojmax; q++) rootpq[size_t(p) * (jdim + 1) + q] = std::sqrt(static_cast<double>(p) / q);
    const size_t n3 = size_t(jdim) * jdim * jdim;
    utot_r.assign(n3, 0.0);
    utot_i.assign(n3, 0.0);
    u_r.assign(n3, 0.0);
    u_i.assign(n3, 0.0);
    z_r.assign(n3 * jdim * jdim, 0.0);
    z_i.assign(n3 * jdim * jdim, 0.0);
    du_r.assign(n3 * 3, 0.0);
    du_i.assign(n3 * 3, 0.0);
    dbarray.assign(n3 * 3, 0.0);
  }
  double rpq(int p, int q) const { return rootpq[size_t(p) * (jdim + 1) + q]; }

  double compute_sfac(double r, double rcut) const {  // sna_impl.hpp:1099-1111
    if (switch_flag == 0) return 1.0;
    if (switch_flag == 1) {
      if (r <= rmin0) return 1.0;
      else if (r > rcut) return 0.0;
      else {
        double rcutfac = MY_PI / (rcut - rmin0);
        return 0.5 * (std::cos((r - rmin0) * rcutfac) + 1.0);
      }
    }
    return 0.0;
  }
  double compute_dsfac(double r, double rcut) const {  // sna_impl.hpp:1116-1128
    if (switch_flag == 0) return 0.0;
    if (switch_flag == 1) {
      if (r <= rmin0) return 0.0;
      else if (r > rcut) return 0.0;
      else {
        double rcutfac = MY_PI / (rcut - rmin0);
        return -0.5 * std::sin((r - rmin0) * rcutfac) * rcutfac;
      }
    }
    return 0.0;
  }

  // compute_uarray (sna_impl.hpp:642-720)
  void compute_uarray(double x, double y, double z, double z0, double r) {
    const double r0inv = 1.0 / std::sqrt(r * r + z0 * z0);
    const double a_r = r0inv * z0, a_i = -r0inv * z, b_r = r0inv * y, b_i = -r0inv * x;
    u_r[i3(0, 0, 0)] = 1.0;
    u_i[i3(0, 0, 0)] = 0.0;
    for (int j = 1; j <= twojmax; j++) {
      for (int mb = 0; mb < (j + 2) / 2; mb++) {
        u_r[i3(j, 0, mb)] = 0.0;
        u_i[i3(j, 0, mb)] = 0.0;
        for (int ma = 0; ma < j; ma++) {
          double rootpq = rpq(j - ma, j - mb);
          u_r[i3(j, ma, mb)] += rootpq * (a_r * u_r[i3(j - 1, ma, mb)] + a_i * u_i[i3(j - 1, ma, mb)]);
          u_i[i3(j, ma, mb)] += rootpq * (a_r * u_i[i3(j - 1, ma, mb)] - a_i * u_r[i3(j - 1, ma, mb)]);
          rootpq = rpq(ma + 1, j - mb);
          u_r[i3(j, ma + 1, mb)] = -rootpq * (b_r * u_r[i3(j - 1, ma, mb)] + b_i * u_i[i3(j - 1, ma, mb)]);
          u_i[i3(j, ma + 1, mb)] = -rootpq * (b_r * u_i[i3(j - 1, ma, mb)] - b_i * u_r[i3(j - 1, ma, mb)]);
        }
      }
      for (int mb = 0; mb < (j + 2) / 2; mb++) {
        const int mbpar = (mb) % 2 == 0 ? 1 : -1;
        int mapar = -mbpar;
        for (int ma = 0; ma <= j; ma++) {
          mapar = -mapar;
          if (mapar == 1) {
            u_r[i3(j, j - ma, j - mb)] = u_r[i3(j, ma, mb)];
            u_i[i3(j, j - ma, j - mb)] = -u_i[i3(j, ma, mb)];
          } else {
            u_r[i3(j, j - ma, j - mb)] = -u_r[i3(j, ma, mb)];
            u_i[i3(j, j - ma, j - mb)] = u_i[i3(j, ma, mb)];
          }
        }
      }
    }
  }

  // compute_ui (sna_impl.hpp:153-190) with zero/addself/add_uarraytot (575-635)
  void compute_ui(const std::vector<double>& rij, const std::vector<double>& wj, const std::vector<double>& rcutij,
                  int jnum) {
    std::fill(utot_r.begin(), utot_r.end(), 0.0);
    std::fill(utot_i.begin(), utot_i.end(), 0.0);
    for (int j = 0; j <= twojmax; j++)
      for (int ma = 0; ma <= j; ma++) {
        utot_r[i3(j, ma, ma)] = wself;
        utot_i[i3(j, ma, ma)] = 0.0;
      }
    for (int n = 0; n < jnum; n++) {
      const double x = rij[3 * n], y = rij[3 * n + 1], z = rij[3 * n + 2];
      const double rsq = x * x + y * y + z * z;
      const double r = std::sqrt(rsq);
      const double theta0 = (r - rmin0) * rfac0 * MY_PI / (rcutij[n] - rmin0);
      const double z0 = r / std::tan(theta0);
      compute_uarray(x, y, z, z0, r);
      const double sfac = compute_sfac(r, rcutij[n]) * wj[n];
      for (size_t k = 0; k < utot_r.size(); k++) {
        utot_r[k] += sfac * u_r[k];
        utot_i[k] += sfac * u_i[k];
      }
    }
  }

  // compute_zi (sna_impl.hpp:197-283)
  void compute_zi() {
    for (const Idx& t : idxj_full) {
      const int j1 = t.j1, j2 = t.j2, j = t.j;
      const int bound = (j + 2) / 2;
      for (int mbma = 0; mbma < (j + 1) * bound; mbma++) {
        const int ma = mbma % (j + 1);
        const int mb = mbma / (j + 1);
        double zr = 0.0, zi = 0.0;
        for (int ma1 = std::max(0, (2 * ma - j - j2 + j1) / 2); ma1 <= std::min(j1, (2 * ma - j + j2 + j1) / 2);
             ma1++) {
          double sumb1_r = 0.0, sumb1_i = 0.0;
          const int ma2 = (2 * ma - j - (2 * ma1 - j1) + j2) / 2;
          for (int mb1 = std::max(0, (2 * mb - j - j2 + j1) / 2); mb1 <= std::min(j1, (2 * mb - j + j2 + j1) / 2);
               mb1++) {
            const int mb2 = (2 * mb - j - (2 * mb1 - j1) + j2) / 2;
            const double cga = cg[i5(j1, j2, j, mb1, mb2)];
            const double u1r = utot_r[i3(j1, ma1, mb1)], u1i = utot_i[i3(j1, ma1, mb1)];
            const double u2r = utot_r[i3(j2, ma2, mb2)], u2i = utot_i[i3(j2, ma2, mb2)];
            sumb1_r += cga * (u1r * u2r - u1i * u2i);
            sumb1_i += cga * (u1r * u2i + u1i * u2r);
          }
          const double cga = cg[i5(j1, j2, j, ma1, ma2)];
          zr += sumb1_r * cga;
          zi += sumb1_i * cga;
        }
        z_r[i5(j1, j2, j, mb, ma)] = zr;
        z_i[i5(j1, j2, j, mb, ma)] = zi;
      }
    }
  }

  // compute_duidrj + compute_duarray (sna_impl.hpp:291-321, 729-893)
  void compute_duidrj(const double* rij, double wj, double rcut) {
    const double x = rij[0], y = rij[1], z = rij[2];
    const double rsq = x * x + y * y + z * z;
    const double r = std::sqrt(rsq);
    const double rscale0 = rfac0 * MY_PI / (rcut - rmin0);
    const double theta0 = (r - rmin0) * rscale0;
    const double cs = std::cos(theta0), sn = std::sin(theta0);
    const double z0 = r * cs / sn;
    const double dz0dr = z0 / r - (r * rscale0) * (rsq + z0 * z0) / rsq;
    compute_duarray(x, y, z, z0, r, dz0dr, wj, rcut);
  }

  void compute_duarray(double x, double y, double z, double z0, double r, double dz0dr, double wj, double rcut) {
    double da_r[3], da_i[3], db_r[3], db_i[3], dz0[3], dr0inv[3];
    const double rinv = 1.0 / r;
    const double ux = x * rinv, uy = y * rinv, uz = z * rinv;
    const double r0inv = 1.0 / std::sqrt(r * r + z0 * z0);
    const double a_r = z0 * r0inv, a_i = -z * r0inv, b_r = y * r0inv, b_i = -x * r0inv;
    const double dr0invdr = -std::pow(r0inv, 3.0) * (r + z0 * dz0dr);
    dr0inv[0] = dr0invdr * ux;
    dr0inv[1] = dr0invdr * uy;
    dr0inv[2] = dr0invdr * uz;
    dz0[0] = dz0dr * ux;
    dz0[1] = dz0dr * uy;
    dz0[2] = dz0dr * uz;
    for (int k = 0; k < 3; k++) {
      da_r[k] = dz0[k] * r0inv + z0 * dr0inv[k];
      da_i[k] = -z * dr0inv[k];
    }
    da_i[2] += -r0inv;
    for (int k = 0; k < 3; k++) {
      db_r[k] = y * dr0inv[k];
      db_i[k] = -x * dr0inv[k];
    }
    db_i[0] += -r0inv;
    db_r[1] += r0inv;
    u_r[i3(0, 0, 0)] = 1.0;
    u_i[i3(0, 0, 0)] = 0.0;
    for (int k = 0; k < 3; k++) {
      du_r[i4(0, 0, 0, k)] = 0.0;
      du_i[i4(0, 0, 0, k)] = 0.0;
    }
    for (int j = 1; j <= twojmax; j++) {
      for (int mb = 0; mb < (j + 2) / 2; mb++) {
        u_r[i3(j, 0, mb)] = 0.0;
        u_i[i3(j, 0, mb)] = 0.0;
        for (int k = 0; k < 3; k++) {
          du_r[i4(j, mb, 0, k)] = 0.0;
          du_i[i4(j, mb, 0, k)] = 0.0;
        }
        for (int ma = 0; ma < j; ma++) {
          double rootpq = rpq(j - ma, j - mb);
          const double ur = u_r[i3(j - 1, ma, mb)], ui = u_i[i3(j - 1, ma, mb)];
          u_r[i3(j, ma, mb)] += rootpq * (a_r * ur + a_i * ui);
          u_i[i3(j, ma, mb)] += rootpq * (a_r * ui - a_i * ur);
          for (int k = 0; k < 3; k++) {
            const double dur = du_r[i4(j - 1, mb, ma, k)], dui = du_i[i4(j - 1, mb, ma, k)];
            du_r[i4(j, mb, ma, k)] += rootpq * (da_r[k] * ur + da_i[k] * ui + a_r * dur + a_i * dui);
            du_i[i4(j, mb, ma, k)] += rootpq * (da_r[k] * ui - da_i[k] * ur + a_r * dui - a_i * dur);
          }
          rootpq = rpq(ma + 1, j - mb);
          u_r[i3(j, ma + 1, mb)] = -rootpq * (b_r * ur + b_i * ui);
          u_i[i3(j, ma + 1, mb)] = -rootpq * (b_r * ui - b_i * ur);
          for (int k = 0; k < 3; k++) {
            const double dur = du_r[i4(j - 1, mb, ma, k)], dui = du_i[i4(j - 1, mb, ma, k)];
            du_r[i4(j, mb, ma + 1, k)] = -rootpq * (db_r[k] * ur + db_i[k] * ui + b_r * dur + b_i * dui);
            du_i[i4(j, mb, ma + 1, k)] = -rootpq * (db_r[k] * ui - db_i[k] * ur + b_r * dui - b_i * dur);
          }
        }
      }
      for (int mb = 0; mb < (j + 2) / 2; mb++) {
        const int mbpar = (mb) % 2 == 0 ? 1 : -1;
        int mapar = -mbpar;
        for (int ma = 0; ma <= j; ma++) {
          mapar = -mapar;
          if (mapar == 1) {
            u_r[i3(j, j - ma, j - mb)] = u_r[i3(j, ma, mb)];
            u_i[i3(j, j - ma, j - mb)] = -u_i[i3(j, ma, mb)];
            for (int k = 0; k < 3; k++) {
              du_r[i4(j, j - mb, j - ma, k)] = du_r[i4(j, mb, ma, k)];
              du_i[i4(j, j - mb, j - ma, k)] = -du_i[i4(j, mb, ma, k)];
            }
          } else {
            u_r[i3(j, j - ma, j - mb)] = -u_r[i3(j, ma, mb)];
            u_i[i3(j, j - ma, j - mb)] = u_i[i3(j, ma, mb)];
            for (int k = 0; k < 3; k++) {
              du_r[i4(j, j - mb, j - ma, k)] = -du_r[i4(j, mb, ma, k)];
              du_i[i4(j, j - mb, j - ma, k)] = du_i[i4(j, mb, ma, k)];
            }
          }
        }
      }
    }
    double sfac = compute_sfac(r, rcut), dsfac = compute_dsfac(r, rcut);
    sfac *= wj;
    dsfac *= wj;
    const double uk[3] = {ux, uy, uz};
    for (int j = 0; j <= twojmax; j++)
      for (int mb = 0; mb <= j; mb++)
        for (int ma = 0; ma <= j; ma++)
          for (int k = 0; k < 3; k++) {
            du_r[i4(j, mb, ma, k)] = dsfac * u_r[i3(j, ma, mb)] * uk[k] + sfac * du_r[i4(j, mb, ma, k)];
            du_i[i4(j, mb, ma, k)] = dsfac * u_i[i3(j, ma, mb)] * uk[k] + sfac * du_i[i4(j, mb, ma, k)];
          }
  }

  // one half-range contraction sum_{mb,ma} Re(conj(dU_jj) Z(a,b,c)) with the
  // middle-column weights of compute_dbidrj (sna_impl.hpp:384-413)
  void zdu_sum(int jj, int a, int b, int c, double s[3]) const {
    s[0] = s[1] = s[2] = 0.0;
    for (int mb = 0; 2 * mb < jj; mb++)
      for (int ma = 0; ma <= jj; ma++) {
        const double zr = z_r[i5(a, b, c, mb, ma)], zi = z_i[i5(a, b, c, mb, ma)];
        for (int k = 0; k < 3; k++) s[k] += (du_r[i4(jj, mb, ma, k)] * zr + du_i[i4(jj, mb, ma, k)] * zi);
      }
    if (jj % 2 == 0) {
      const int mb = jj / 2;
      for (int ma = 0; ma <= mb; ma++) {
        const double factor = ma == mb ? 0.5 : 1.0;
        const double zr = z_r[i5(a, b, c, mb, ma)] * factor, zi = z_i[i5(a, b, c, mb, ma)] * factor;
        for (int k = 0; k < 3; k++) s[k] += (du_r[i4(jj, mb, ma, k)] * zr + du_i[i4(jj, mb, ma, k)] * zi);
      }
    }
  }

  // compute_dbidrj + copy_dbi2dbvec (sna_impl.hpp:330-570) -> dbvec[ncoeff][3]
  void compute_dbidrj(std::vector<double>& dbvec) const {
    dbvec.assign(size_t(ncoeff) * 3, 0.0);
    for (int JJ = 0; JJ < ncoeff; JJ++) {
      const int j1 = idxj[JJ].j1, j2 = idxj[JJ].j2, j = idxj[JJ].j;
      double dbdr[3] = {0, 0, 0}, s[3];
      int a, b, c;
      if (j1 >= j2) { a = j1; b = j2; c = j; } else { a = j2; b = j1; c = j; }
      zdu_sum(j, a, b, c, s);
      for (int k = 0; k < 3; k++) dbdr[k] += s[k] * 2.0;
      const double j1fac = (j + 1) / (j1 + 1.0);
      if (j >= j2) { a = j; b = j2; c = j1; } else { a = j2; b = j; c = j1; }
      zdu_sum(j1, a, b, c, s);
      for (int k = 0; k < 3; k++) dbdr[k] += s[k] * 2.0 * j1fac;
      const double j2fac = (j + 1) / (j2 + 1.0);
      if (j1 >= j) { a = j1; b = j; c = j2; } else { a = j; b = j1; c = j2; }
      zdu_sum(j2, a, b, c, s);
      for (int k = 0; k < 3; k++) dbdr[k] += s[k] * 2.0 * j2fac;
      for (int k = 0; k < 3; k++) dbvec[size_t(JJ) * 3 + k] = dbdr[k];
    }
  }

  // B(j1,j2,j) = sum_{ma,mb} conj(U_j) Z(j1,j2,j) over the full square,
  // evaluated as 2 Re of the half range (the energy ExaMiniMD does not compute)
  void compute_bi(std::vector<double>& bvec) const {
    bvec.assign(size_t(ncoeff), 0.0);
    for (int JJ = 0; JJ < ncoeff; JJ++) {
      const int j1 = idxj[JJ].j1, j2 = idxj[JJ].j2, j = idxj[JJ].j;
      double sumzu = 0.0;
      for (int mb = 0; 2 * mb < j; mb++)
        for (int ma = 0; ma <= j; ma++)
          sumzu += utot_r[i3(j, ma, mb)] * z_r[i5(j1, j2, j, mb, ma)] + utot_i[i3(j, ma, mb)] * z_i[i5(j1, j2, j, mb, ma)];
      if (j % 2 == 0) {
        const int mb = j / 2;
        for (int ma = 0; ma < mb; ma++)
          sumzu += utot_r[i3(j, ma, mb)] * z_r[i5(j1, j2, j, mb, ma)] + utot_i[i3(j, ma, mb)] * z_i[i5(j1, j2, j, mb, ma)];
        sumzu += 0.5 * (utot_r[i3(j, mb, mb)] * z_r[i5(j1, j2, j, mb, mb)] +
                        utot_i[i3(j, mb, mb)] * z_i[i5(j1, j2, j, mb, mb)]);
      }
      bvec[size_t(JJ)] = 2.0 * sumzu;
    }
  }
};

}  // namespace

struct orc_ctx {
  std::string err;
  int threads = 1;
  // System (system.h:57-143)
  int ntypes = 1;
  std::vector<double> mass;
  double boltz = 0, mvv2e = 0, dt = 0;
  double domain[3] = {0, 0, 0}, lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
  int N_local = 0, N_ghost = 0;
  std::vector<double> x, v, f, q;
  std::vector<int> type, id;
  // CommSerial
  double comm_depth = 0;
  int num_ghost[6] = {0, 0, 0, 0, 0, 0};
  std::vector<int> pack[6];
  // BinningKKSort
  int nbin[3] = {0, 0, 0}, nhalo = 0, bin_first = 0, bin_n = 0;
  double bmin[3] = {0, 0, 0}, bmax[3] = {0, 0, 0};
  std::vector<int> bincount, binoffsets, permute;
  // Neighbor
  int kind = 0, newton = 0, half = 0, maxneighs = 16;
  double cut = 0;
  int rows = 0;
  std::vector<int> num_neighs, offsets, entries, neighs2d;
  // LJ
  int lj_nt = 0, lj_half = 0;
  std::vector<double> lj1, lj2, cutsq;
  // SNAP
  bool snap_ready = false;
  Sna sna;
  std::vector<double> radelem, wjelem, beta;
  int ncoeffall = 0;
  std::vector<int> snap_map;
  double rcutfac = 0, rcutmax = 0;

  int total() const { return N_local + N_ghost; }
  void grow(int n) {
    if (int(type.size()) >= n) return;
    x.resize(3 * size_t(n), 0.0);
    v.resize(3 * size_t(n), 0.0);
    f.resize(3 * size_t(n), 0.0);
    q.resize(size_t(n), 0.0);
    type.resize(size_t(n), 0);
    id.resize(size_t(n), 0);
  }
  int row_len(int i) const { return num_neighs[size_t(i)]; }
  int row_at(int i, int k) const {
    return kind == 0 ? entries[size_t(offsets[size_t(i)]) + k] : neighs2d[size_t(i) * maxneighs + k];
  }
};

#define ORC_TRY \
  if (!c) return 1; \
  try {
#define ORC_END                        \
  }                                    \
  catch (const std::exception& e) {    \
    c->err = e.what();                 \
    return 1;                          \
  }                                    \
  return 0;

extern "C" {

orc_ctx* orc_create(void) { return new orc_ctx(); }
void orc_destroy(orc_ctx* c) { delete c; }
const char* orc_last_error(orc_ctx* c) { return c ? c->err.c_str() : "null"; }
void orc_set_threads(orc_ctx* c, int n) {
  if (c) c->threads = n < 1 ? 1 : n;
}

int orc_system_init(orc_ctx* c, int ntypes, const double* mass, double boltz, double mvv2e, double dt,
                    const double domain[3], const double sub_lo[3], const double sub_hi[3]) {
  ORC_TRY
  c->ntypes = ntypes;
  c->mass.assign(mass, mass + ntypes);
  c->boltz = boltz;
  c->mvv2e = mvv2e;
  c->dt = dt;
  for (int d = 0; d < 3; d++) {
    c->domain[d] = domain[d];
    c->lo[d] = sub_lo[d];
    c->hi[d] = sub_hi[d];
  }
  ORC_END
}

int orc_system_set_local(orc_ctx* c, int n, const double* x, const double* v, const double* f, const int* type,
                         const int* id, const double* q) {
  ORC_TRY
  c->type.clear();
  c->grow(n);
  c->N_local = n;
  c->N_ghost = 0;
  for (int i = 0; i < n; i++) {
    for (int d = 0; d < 3; d++) {
      c->x[3 * size_t(i) + d] = x[3 * size_t(i) + d];
      c->v[3 * size_t(i) + d] = v ? v[3 * size_t(i) + d] : 0.0;
      c->f[3 * size_t(i) + d] = f ? f[3 * size_t(i) + d] : 0.0;
    }
    c->type[size_t(i)] = type[i];
    c->id[size_t(i)] = id[i];
    c->q[size_t(i)] = q ? q[i] : 0.0;
  }
  ORC_END
}

int orc_system_get(orc_ctx* c, int first, int count, double* x, double* v, double* f, int* type, int* id,
                   double* q) {
  ORC_TRY
  if (first < 0 || first + count > c->total()) throw OrcErr("orc_system_get: range");
  for (int k = 0; k < count; k++) {
    const size_t i = size_t(first + k);
    for (int d = 0; d < 3; d++) {
      if (x) x[3 * k + d] = c->x[3 * i + d];
      if (v) v[3 * k + d] = c->v[3 * i + d];
      if (f) f[3 * k + d] = c->f[3 * i + d];
    }
    if (type) type[k] = c->type[i];
    if (id) id[k] = c->id[i];
    if (q) q[k] = c->q[i];
  }
  ORC_END
}

int orc_system_info(orc_ctx* c, int* n_local, int* n_ghost) {
  ORC_TRY
  if (n_local) *n_local = c->N_local;
  if (n_ghost) *n_ghost = c->N_ghost;
  ORC_END
}

// Kokkos::deep_copy(system->f, 0.0) (examinimd.cpp:138, 232)
int orc_zero_forces(orc_ctx* c) {
  ORC_TRY
  std::fill(c->f.begin(), c->f.end(), 0.0);
  ORC_END
}

// Input::create_lattice (input.cpp:460-792) with LAMMPS_RandomVelocityGeom
// (input.h:66-133).  The hash reads bytes as signed char (x86-64 behaviour).
int orc_create_lattice(orc_ctx* c, int style, double a, const double off[3], int nx, int ny, int nz, double t_target,
                       int seed) {
  ORC_TRY
  c->domain[0] = a * nx;
  c->domain[1] = a * ny;
  c->domain[2] = a * nz;
  for (int d = 0; d < 3; d++) {  // Comm::create_domain_decomposition (comm.cpp:58-65)
    c->lo[d] = 0.0;
    c->hi[d] = c->domain[d];
  }
  std::vector<double> basis;
  if (style == 0) basis = {0, 0, 0};
  else if (style == 1) basis = {0, 0, 0, 0.5, 0.5, 0.0, 0.5, 0.0, 0.5, 0.0, 0.5, 0.5};
  else basis = {0, 0, 0, 0.5, 0.5, 0.5};
  const int nb = int(basis.size() / 3);
  const int xs = int(c->lo[0] / c->domain[0] * nx - 0.5), ys = int(c->lo[1] / c->domain[1] * ny - 0.5),
            zs = int(c->lo[2] / c->domain[2] * nz - 0.5);
  const int xe = int(c->hi[0] / c->domain[0] * nx + 0.5), ye = int(c->hi[1] / c->domain[1] * ny + 0.5),
            ze = int(c->hi[2] / c->domain[2] * nz + 0.5);
  std::vector<double> X;
  std::vector<int> T, I;
  srand(1);
  int n = 0;
  for (int iz = zs; iz <= ze; iz++)
    for (int iy = ys; iy <= ye; iy++)
      for (int ix = xs; ix <= xe; ix++)
        for (int k = 0; k < nb; k++) {
          double xt, yt, zt;
          if (style == 0) {
            xt = a * (ix + off[0]);
            yt = a * (iy + off[1]);
            zt = a * (iz + off[2]);
          } else {
            xt = a * (1.0 * ix + (basis[3 * k] + off[0]));
            yt = a * (1.0 * iy + (basis[3 * k + 1] + off[1]));
            zt = a * (1.0 * iz + (basis[3 * k + 2] + off[2]));
          }
          if (xt >= c->lo[0] && yt >= c->lo[1] && zt >= c->lo[2] && xt < c->hi[0] && yt < c->hi[1] && zt < c->hi[2]) {
            X.push_back(xt);
            X.push_back(yt);
            X.push_back(zt);
            T.push_back(rand() % c->ntypes);
            I.push_back(++n);
          }
        }
  std::vector<double> V(X.size());
  double tm = 0, px = 0, py = 0, pz = 0;
  for (int i = 0; i < n; i++) {
    unsigned int hash = 0;
    const signed char* s = reinterpret_cast<const signed char*>(&seed);
    for (int k = 0; k < 4; k++) {
      hash += s[k];
      hash += (hash << 10);
      hash ^= (hash >> 6);
    }
    double xi[3] = {X[3 * size_t(i)], X[3 * size_t(i) + 1], X[3 * size_t(i) + 2]};
    s = reinterpret_cast<const signed char*>(xi);
    for (int k = 0; k < 24; k++) {
      hash += s[k];
      hash += (hash << 10);
      hash ^= (hash >> 6);
    }
    hash += (hash << 3);
    hash ^= (hash >> 11);
    hash += (hash << 15);
    int st = int(hash & 0x7ffffff);
    if (!st) st = 1;
    auto uniform = [&st]() {
      const int k = st / 127773;
      st = 16807 * (st - k * 127773) - 2836 * k;
      if (st < 0) st += 2147483647;
      return (1.0 / 2147483647) * st;
    };
    for (int k = 0; k < 5; k++) uniform();
    const double m = c->mass[size_t(T[size_t(i)])];
    const double vx = uniform() - 0.5, vy = uniform() - 0.5, vz = uniform() - 0.5;
    V[3 * size_t(i)] = vx / std::sqrt(m);
    V[3 * size_t(i) + 1] = vy / std::sqrt(m);
    V[3 * size_t(i) + 2] = vz / std::sqrt(m);
    tm += m;
    px += m * V[3 * size_t(i)];
    py += m * V[3 * size_t(i) + 1];
    pz += m * V[3 * size_t(i) + 2];
  }
  const double sx = px / tm, sy = py / tm, sz = pz / tm;
  for (int i = 0; i < n; i++) {
    V[3 * size_t(i)] -= sx;
    V[3 * size_t(i) + 1] -= sy;
    V[3 * size_t(i) + 2] -= sz;
  }
  double Ts = 0;  // Temperature::compute (property_temperature.cpp:43-62), serial order
  for (int i = 0; i < n; i++) {
    const size_t b = 3 * size_t(i);
    Ts += (V[b] * V[b] + V[b + 1] * V[b + 1] + V[b + 2] * V[b + 2]) * c->mass[size_t(T[size_t(i)])];
  }
  const double Tcur = Ts * (c->mvv2e / (1.0 * (3 * n - 3) * c->boltz));
  const double scale = std::sqrt(t_target / Tcur);
  for (auto& e : V) e *= scale;
  std::vector<double> Q(static_cast<size_t>(n), 0.0);
  return orc_system_set_local(c, n, X.data(), V.data(), nullptr, T.data(), I.data(), Q.data());
  ORC_END
}

// IntegratorNVE (integrator_nve.cpp:41-121)
int orc_nve_initial(orc_ctx* c) {
  ORC_TRY
  const double dtv = c->dt, dtf = 0.5 * c->dt / c->mvv2e;
  const int n = c->N_local;
#pragma omp parallel for num_threads(c->threads) schedule(static)
  for (int i = 0; i < n; i++) {
    const size_t b = 3 * size_t(i);
    const double dtfm = dtf / c->mass[size_t(c->type[size_t(i)])];
    c->v[b] += dtfm * c->f[b];
    c->v[b + 1] += dtfm * c->f[b + 1];
    c->v[b + 2] += dtfm * c->f[b + 2];
    c->x[b] += dtv * c->v[b];
    c->x[b + 1] += dtv * c->v[b + 1];
    c->x[b + 2] += dtv * c->v[b + 2];
  }
  ORC_END
}

int orc_nve_final(orc_ctx* c) {
  ORC_TRY
  const double dtf = 0.5 * c->dt / c->mvv2e;
  const int n = c->N_local;
#pragma omp parallel for num_threads(c->threads) schedule(static)
  for (int i = 0; i < n; i++) {
    const size_t b = 3 * size_t(i);
    const double dtfm = dtf / c->mass[size_t(c->type[size_t(i)])];
    c->v[b] += dtfm * c->f[b];
    c->v[b + 1] += dtfm * c->f[b + 1];
    c->v[b + 2] += dtfm * c->f[b + 2];
  }
  ORC_END
}

// CommSerial (comm_serial.cpp:41-127, comm_serial.h:95-213)
int orc_comm_init(orc_ctx* c, double depth) {
  ORC_TRY
  c->comm_depth = depth;
  ORC_END
}

int orc_comm_exchange(orc_ctx* c) {
  ORC_TRY
  for (int i = 0; i < c->N_local; i++)
    for (int d = 0; d < 3; d++) {
      double& xd = c->x[3 * size_t(i) + d];
      const double x0 = xd;
      if (x0 > c->domain[d]) xd -= c->domain[d];
      if (x0 < 0) xd += c->domain[d];
    }
  ORC_END
}

int orc_comm_exchange_halo(orc_ctx* c, int* n_ghost) {
  ORC_TRY
  const int N_local = c->N_local;
  int N_ghost = 0;
  for (int phase = 0; phase < 6; phase++) {
    const int d = phase / 2;
    const int nparticles = N_local + N_ghost - ((phase % 2 == 1) ? c->num_ghost[phase - 1] : 0);
    std::vector<int>& pk = c->pack[phase];
    pk.clear();
    for (int i = 0; i < nparticles; i++) {
      const double xd = c->x[3 * size_t(i) + d];
      const bool sel = phase % 2 == 0 ? (xd >= c->hi[d] - c->comm_depth) : (xd <= c->lo[d] + c->comm_depth);
      if (sel) pk.push_back(i);
    }
    const int count = int(pk.size());
    c->grow(N_local + N_ghost + count);
    for (int k = 0; k < count; k++) {
      const size_t s = size_t(pk[size_t(k)]), t = size_t(N_local + N_ghost + k);
      for (int e = 0; e < 3; e++) {
        c->x[3 * t + e] = c->x[3 * s + e];
        c->v[3 * t + e] = c->v[3 * s + e];
      }
      if (phase % 2 == 0) c->x[3 * t + d] -= c->domain[d];
      else c->x[3 * t + d] += c->domain[d];
      c->q[t] = c->q[s];
      c->id[t] = c->id[s];
      c->type[t] = c->type[s];
    }
    c->num_ghost[phase] = count;
    N_ghost += count;
  }
  c->N_ghost = N_ghost;
  if (n_ghost) *n_ghost = N_ghost;
  ORC_END
}

int orc_comm_update_halo(orc_ctx* c) {
  ORC_TRY
  int N_ghost = 0;
  for (int phase = 0; phase < 6; phase++) {
    const int d = phase / 2;
    for (int k = 0; k < c->num_ghost[phase]; k++) {
      const size_t s = size_t(c->pack[phase][size_t(k)]), t = size_t(c->N_local + N_ghost + k);
      for (int e = 0; e < 3; e++) c->x[3 * t + e] = c->x[3 * s + e];
      if (phase % 2 == 0) c->x[3 * t + d] -= c->domain[d];
      else c->x[3 * t + d] += c->domain[d];
    }
    N_ghost += c->num_ghost[phase];
  }
  ORC_END
}

int orc_comm_update_force(orc_ctx* c) {
  ORC_TRY
  int offs[6];
  offs[0] = c->N_local;
  for (int p = 1; p < 6; p++) offs[p] = offs[p - 1] + c->num_ghost[p - 1];
  for (int phase = 5; phase >= 0; phase--)
    for (int k = 0; k < c->num_ghost[phase]; k++) {
      const size_t i = size_t(c->pack[phase][size_t(k)]), g = size_t(offs[phase] + k);
      c->f[3 * i] += c->f[3 * g];
      c->f[3 * i + 1] += c->f[3 * g + 1];
      c->f[3 * i + 2] += c->f[3 * g + 2];
    }
  ORC_END
}

int orc_comm_get_ghosts(orc_ctx* c, int num_ghost[6], int* pack) {
  ORC_TRY
  size_t o = 0;
  for (int p = 0; p < 6; p++) {
    if (num_ghost) num_ghost[p] = c->num_ghost[p];
    if (pack)
      for (int v : c->pack[p]) pack[o++] = v;
  }
  ORC_END
}

// BinningKKSort::create_binning (binning_kksort.cpp:71-140) with the serial
// BinSort semantics (counting sort, ascending index inside a bin).
int orc_binning_create(orc_ctx* c, double dx_in, double dy_in, double dz_in, int halo, int do_local, int do_ghost,
                       int sort, int nbin_out[3]) {
  ORC_TRY
  if (!(do_local || do_ghost)) return 0;
  const int first = do_local ? 0 : c->N_local;
  const int last = do_ghost ? c->N_local + c->N_ghost : c->N_local;
  const int n = last - first;
  const double sub[3] = {c->hi[0] - c->lo[0], c->hi[1] - c->lo[1], c->hi[2] - c->lo[2]};
  const double din[3] = {dx_in, dy_in, dz_in};
  int nb[3];
  double dxyz[3];
  for (int d = 0; d < 3; d++) {
    nb[d] = int(sub[d] / din[d]);
    if (nb[d] == 0) nb[d] = 1;
    dxyz[d] = sub[d] / nb[d];
    nb[d] += 2 * halo;
  }
  const double eps = dxyz[0] / 1000;
  double mul[3];
  for (int d = 0; d < 3; d++) {
    c->bmin[d] = -dxyz[d] * halo - eps + c->lo[d];
    c->bmax[d] = dxyz[d] * halo + eps + c->hi[d];
    mul[d] = double(nb[d]) / (c->bmax[d] - c->bmin[d]);
    c->nbin[d] = nb[d];
  }
  c->nhalo = halo;
  c->bin_first = first;
  c->bin_n = n;
  const int nbins = nb[0] * nb[1] * nb[2];
  std::vector<int> binof(static_cast<size_t>(n));
  c->bincount.assign(size_t(nbins), 0);
  for (int r = 0; r < n; r++) {
    const size_t i = size_t(first + r);
    int ix = int((c->x[3 * i] - c->bmin[0]) * mul[0]);
    int iy = int((c->x[3 * i + 1] - c->bmin[1]) * mul[1]);
    int iz = int((c->x[3 * i + 2] - c->bmin[2]) * mul[2]);
    if (ix < 0 || ix >= nb[0] || iy < 0 || iy >= nb[1] || iz < 0 || iz >= nb[2])
      throw OrcErr("orc_binning_create: particle outside the binned box");
    binof[size_t(r)] = (ix * nb[1] + iy) * nb[2] + iz;
    c->bincount[size_t(binof[size_t(r)])]++;
  }
  c->binoffsets.assign(size_t(nbins), 0);
  int off = 0;
  for (int b = 0; b < nbins; b++) {
    c->binoffsets[size_t(b)] = off;
    off += c->bincount[size_t(b)];
  }
  std::vector<int> fill(static_cast<size_t>(nbins), 0);
  c->permute.assign(size_t(n), 0);
  for (int r = 0; r < n; r++) {
    const int b = binof[size_t(r)];
    c->permute[size_t(c->binoffsets[size_t(b)] + fill[size_t(b)]++)] = r;
  }
  if (sort) {
    auto reorder3 = [&](std::vector<double>& a) {
      std::vector<double> t(3 * size_t(n));
      for (int r = 0; r < n; r++)
        for (int e = 0; e < 3; e++) t[3 * size_t(r) + e] = a[3 * size_t(first + c->permute[size_t(r)]) + e];
      std::copy(t.begin(), t.end(), a.begin() + 3 * size_t(first));
    };
    auto reorder1 = [&](auto& a) {
      auto t = a;
      for (int r = 0; r < n; r++) t[size_t(first + r)] = a[size_t(first + c->permute[size_t(r)])];
      a.swap(t);
    };
    reorder3(c->x);
    reorder3(c->v);
    reorder3(c->f);
    reorder1(c->type);
    reorder1(c->id);
    reorder1(c->q);
  }
  if (nbin_out)
    for (int d = 0; d < 3; d++) nbin_out[d] = nb[d];
  ORC_END
}

int orc_binning_get(orc_ctx* c, int* bincount, int* binoffsets, int* permute, double bounds[6]) {
  ORC_TRY
  if (bincount) std::copy(c->bincount.begin(), c->bincount.end(), bincount);
  if (binoffsets) std::copy(c->binoffsets.begin(), c->binoffsets.end(), binoffsets);
  if (permute) std::copy(c->permute.begin(), c->permute.end(), permute);
  if (bounds)
    for (int d = 0; d < 3; d++) {
      bounds[2 * d] = c->bmin[d];
      bounds[2 * d + 1] = c->bmax[d];
    }
  ORC_END
}

// NeighborCSR / Neighbor2D (neighbor_csr.h:176-435, neighbor_2d.h:175-331)
int orc_neigh_init(orc_ctx* c, int kind, double cut, int newton) {
  ORC_TRY
  c->kind = kind;
  c->cut = cut;
  c->newton = newton;
  c->maxneighs = 16;
  ORC_END
}

namespace {
// the row of owned atom i in the reference's append order (interior bins only)
void build_row(const orc_ctx* c, int i, std::vector<int>& row) {
  row.clear();
  const int nby = c->nbin[1], nbz = c->nbin[2], h = c->nhalo;
  // locate i's bin from its position, as the binning did
  const double* xi = &c->x[3 * size_t(i)];
  double mul[3];
  for (int d = 0; d < 3; d++) mul[d] = double(c->nbin[d]) / (c->bmax[d] - c->bmin[d]);
  const int bx = int((xi[0] - c->bmin[0]) * mul[0]), by = int((xi[1] - c->bmin[1]) * mul[1]),
            bz = int((xi[2] - c->bmin[2]) * mul[2]);
  if (bx < h || bx >= c->nbin[0] - h || by < h || by >= nby - h || bz < h || bz >= nbz - h) return;
  const double cutsq = c->cut * c->cut;
  for (int bxj = bx - 1; bxj < bx + 2; bxj++)
    for (int byj = by - 1; byj < by + 2; byj++)
      for (int bzj = bz - 1; bzj < bz + 2; bzj++) {
        const int b = (bxj * nby + byj) * nbz + bzj;
        const int off = c->binoffsets[size_t(b)], cnt = c->bincount[size_t(b)];
        for (int k = 0; k < cnt; k++) {
          const int j = c->permute[size_t(off + k)];
          const double* xj = &c->x[3 * size_t(j)];
          if (c->half) {
            const bool above = (xj[0] > xi[0]) || ((xj[0] == xi[0]) && ((xj[1] > xi[1]) || ((xj[1] == xi[1]) && (xj[2] > xi[2]))));
            if (((j == i) || (j < c->N_local || c->newton)) && !above) continue;
            const double dx = xi[0] - xj[0], dy = xi[1] - xj[1], dz = xi[2] - xj[2];
            if (dx * dx + dy * dy + dz * dz <= cutsq) row.push_back(j);
          } else {
            const double dx = xi[0] - xj[0], dy = xi[1] - xj[1], dz = xi[2] - xj[2];
            if ((dx * dx + dy * dy + dz * dz <= cutsq) && (i != j)) row.push_back(j);
          }
        }
      }
}
}  // namespace

int orc_neigh_create(orc_ctx* c, int half, long long* total) {
  ORC_TRY
  if (c->bin_first != 0 || c->bin_n != c->N_local + c->N_ghost)
    throw OrcErr("orc_neigh_create: needs a binning of owned and ghost particles");
  c->half = half;
  const int n = c->N_local;
  c->rows = n;
  std::vector<std::vector<int>> rows(static_cast<size_t>(n));
#pragma omp parallel for num_threads(c->threads) schedule(dynamic, 256)
  for (int i = 0; i < n; i++) build_row(c, i, rows[size_t(i)]);
  c->num_neighs.assign(size_t(n), 0);
  long long tot = 0;
  for (int i = 0; i < n; i++) {
    c->num_neighs[size_t(i)] = int(rows[size_t(i)].size());
    tot += c->num_neighs[size_t(i)];
  }
  if (c->kind == 0) {
    c->offsets.assign(size_t(n) + 1, 0);
    for (int i = 0; i < n; i++) c->offsets[size_t(i) + 1] = c->offsets[size_t(i)] + c->num_neighs[size_t(i)];
    c->entries.resize(size_t(tot));
    for (int i = 0; i < n; i++)
      std::copy(rows[size_t(i)].begin(), rows[size_t(i)].end(), c->entries.begin() + c->offsets[size_t(i)]);
  } else {
    // neighbor_2d.h:304-330: regrow to 1.2x the reported row length; the
    // serial reference reports the last overflowing row in loop order
    while (true) {
      int report = -1;
      // loop order of the reference: interior bins, atoms of each bin
      for (size_t r = 0; r < c->permute.size(); r++) {
        const int i = c->permute[r];
        if (i < n && c->num_neighs[size_t(i)] > c->maxneighs) report = c->num_neighs[size_t(i)];
      }
      if (report < 0) break;
      c->maxneighs = int(report * 1.2);
    }
    c->neighs2d.assign(size_t(n) * c->maxneighs, 0);
    for (int i = 0; i < n; i++)
      std::copy(rows[size_t(i)].begin(), rows[size_t(i)].end(), c->neighs2d.begin() + size_t(i) * c->maxneighs);
  }
  if (total) *total = tot;
  ORC_END
}

int orc_neigh_get(orc_ctx* c, int* num_neighs, int* entries) {
  ORC_TRY
  size_t o = 0;
  for (int i = 0; i < c->rows; i++) {
    if (num_neighs) num_neighs[i] = c->num_neighs[size_t(i)];
    if (entries)
      for (int k = 0; k < c->num_neighs[size_t(i)]; k++) entries[o++] = c->row_at(i, k);
  }
  ORC_END
}

int orc_neigh_maxneighs(orc_ctx* c, int* m) {
  ORC_TRY
  *m = c->kind == 1 ? c->maxneighs : 0;
  ORC_END
}

// ForceLJNeigh (force_lj_neigh_impl.h:57-343)
int orc_lj_init(orc_ctx* c, int ntypes, const double* lj1, const double* lj2, const double* cutsq, int half) {
  ORC_TRY
  const size_t nt2 = size_t(ntypes) * ntypes;
  c->lj_nt = ntypes;
  c->lj1.assign(lj1, lj1 + nt2);
  c->lj2.assign(lj2, lj2 + nt2);
  c->cutsq.assign(cutsq, cutsq + nt2);
  c->lj_half = half;
  ORC_END
}

int orc_lj_compute(orc_ctx* c) {
  ORC_TRY
  const int n = c->N_local;
  if (!c->lj_half) {
    // TagFullNeigh (force_lj_neigh_impl.h:164-206)
#pragma omp parallel for num_threads(c->threads) schedule(dynamic, 512)
    for (int i = 0; i < n; i++) {
      const double* xi = &c->x[3 * size_t(i)];
      const int ti = c->type[size_t(i)];
      double fx = 0, fy = 0, fz = 0;
      for (int k = 0; k < c->row_len(i); k++) {
        const int j = c->row_at(i, k);
        const double* xj = &c->x[3 * size_t(j)];
        const double dx = xi[0] - xj[0], dy = xi[1] - xj[1], dz = xi[2] - xj[2];
        const size_t tp = size_t(ti) * c->lj_nt + c->type[size_t(j)];
        const double rsq = dx * dx + dy * dy + dz * dz;
        if (rsq < c->cutsq[tp]) {
          const double r2inv = 1.0 / rsq;
          const double r6inv = r2inv * r2inv * r2inv;
          const double fpair = (r6inv * (c->lj1[tp] * r6inv - c->lj2[tp])) * r2inv;
          fx += dx * fpair;
          fy += dy * fpair;
          fz += dz * fpair;
        }
      }
      c->f[3 * size_t(i)] += fx;
      c->f[3 * size_t(i) + 1] += fy;
      c->f[3 * size_t(i) + 2] += fz;
    }
  } else {
    // TagHalfNeigh (force_lj_neigh_impl.h:211-254), serial order
    for (int i = 0; i < n; i++) {
      const double* xi = &c->x[3 * size_t(i)];
      const int ti = c->type[size_t(i)];
      double fx = 0, fy = 0, fz = 0;
      for (int k = 0; k < c->row_len(i); k++) {
        const int j = c->row_at(i, k);
        const double* xj = &c->x[3 * size_t(j)];
        const double dx = xi[0] - xj[0], dy = xi[1] - xj[1], dz = xi[2] - xj[2];
        const size_t tp = size_t(ti) * c->lj_nt + c->type[size_t(j)];
        const double rsq = dx * dx + dy * dy + dz * dz;
        if (rsq < c->cutsq[tp]) {
          const double r2inv = 1.0 / rsq;
          const double r6inv = r2inv * r2inv * r2inv;
          const double fpair = (r6inv * (c->lj1[tp] * r6inv - c->lj2[tp])) * r2inv;
          fx += dx * fpair;
          fy += dy * fpair;
          fz += dz * fpair;
          c->f[3 * size_t(j)] -= dx * fpair;
          c->f[3 * size_t(j) + 1] -= dy * fpair;
          c->f[3 * size_t(j) + 2] -= dz * fpair;
        }
      }
      c->f[3 * size_t(i)] += fx;
      c->f[3 * size_t(i) + 1] += fy;
      c->f[3 * size_t(i) + 2] += fz;
    }
  }
  ORC_END
}

}  // extern "C"

// Shifted LJ energy over the list, every pair term in the reference's order
// (TagFullNeighPE / TagHalfNeighPE, force_lj_neigh_impl.h:259-343).  Acc is
// the reduction: a plain running double, the reference's serial
// parallel_reduce, or a compensated one.
template <class Acc>
static void lj_energy_terms(const orc_ctx* c, Acc& PE) {
  const int n = c->N_local;
  for (int i = 0; i < n; i++) {
    const double* xi = &c->x[3 * size_t(i)];
    const int ti = c->type[size_t(i)];
    for (int k = 0; k < c->row_len(i); k++) {
      const int j = c->row_at(i, k);
      const double* xj = &c->x[3 * size_t(j)];
      const double dx = xi[0] - xj[0], dy = xi[1] - xj[1], dz = xi[2] - xj[2];
      const size_t tp = size_t(ti) * c->lj_nt + c->type[size_t(j)];
      const double rsq = dx * dx + dy * dy + dz * dz;
      if (rsq < c->cutsq[tp]) {
        const double lj1 = c->lj1[tp], lj2 = c->lj2[tp];
        const double r2inv = 1.0 / rsq;
        const double r6inv = r2inv * r2inv * r2inv;
        const double r2invc = 1.0 / c->cutsq[tp];
        const double r6invc = r2invc * r2invc * r2invc;
        if (!c->lj_half) {  // TagFullNeighPE (force_lj_neigh_impl.h:259-296)
          PE += 0.5 * r6inv * (0.5 * lj1 * r6inv - lj2) / 6.0;
          PE -= 0.5 * r6invc * (0.5 * lj1 * r6invc - lj2) / 6.0;
        } else {  // TagHalfNeighPE (force_lj_neigh_impl.h:301-343)
          const double fac = j < n ? 1.0 : 0.5;
          PE += fac * r6inv * (0.5 * lj1 * r6inv - lj2) / 6.0;
          PE -= fac * r6invc * (0.5 * lj1 * r6invc - lj2) / 6.0;
        }
      }
    }
  }
}

// Neumaier's compensated sum (an improved Kahan sum): the running error of
// every addition is carried exactly (two-sum) in a second double, so the
// total is within about one rounding of the exact sum of the terms.
struct CompensatedSum {
  double s = 0.0, comp = 0.0;
  void add(double v) {
    const double t = s + v;
    if (std::fabs(s) >= std::fabs(v)) comp += (s - t) + v;
    else comp += (v - t) + s;
    s = t;
  }
  CompensatedSum& operator+=(double v) {
    add(v);
    return *this;
  }
  CompensatedSum& operator-=(double v) {
    add(-v);
    return *this;
  }
  double value() const { return s + comp; }
};

extern "C" {

int orc_lj_energy(orc_ctx* c, double* pe) {
  ORC_TRY
  double PE = 0.0;
  lj_energy_terms(c, PE);
  *pe = PE;
  ORC_END
}

// The same terms summed with compensation: a test-side value of the energy
// free of the serial sum's rounding (about 1e-11 relative at 32,000 atoms,
// 2.5 million pair terms), against which a differently ordered sum is judged.
int orc_lj_energy_compensated(orc_ctx* c, double* pe) {
  ORC_TRY
  CompensatedSum PE;
  lj_energy_terms(c, PE);
  *pe = PE.value();
  ORC_END
}

// ForceSNAP::init_coeff (force_snap_neigh_impl.h:228-336)
int orc_snap_init(orc_ctx* c, int twojmax, double rfac0, double rmin0, int switchflag, double rcutfac, int nelem,
                  const double* radelem, const double* wjelem, const double* beta, int ncoeffall, int ntypes,
                  const int* map) {
  ORC_TRY
  c->sna.init(twojmax, rfac0, rmin0, switchflag);
  if (c->sna.ncoeff != ncoeffall - 1) throw OrcErr("Incorrect SNAP parameter file");
  c->radelem.assign(radelem, radelem + nelem);
  c->wjelem.assign(wjelem, wjelem + nelem);
  c->beta.assign(beta, beta + size_t(nelem) * ncoeffall);
  c->ncoeffall = ncoeffall;
  c->snap_map.assign(map, map + ntypes);
  c->rcutfac = rcutfac;
  c->rcutmax = 0.0;
  for (int e = 0; e < nelem; e++) c->rcutmax = std::max(2.0 * c->radelem[size_t(e)] * rcutfac, c->rcutmax);
  c->snap_ready = true;
  ORC_END
}

namespace {
// inside list of atom i (force_snap_neigh_impl.h:612-656)
void snap_inside(const orc_ctx* c, int i, std::vector<double>& rij, std::vector<int>& inside, std::vector<double>& wj,
                 std::vector<double>& rcutij) {
  rij.clear();
  inside.clear();
  wj.clear();
  rcutij.clear();
  const double* xi = &c->x[3 * size_t(i)];
  const int ei = c->snap_map[size_t(c->type[size_t(i)])];
  const double radi = c->radelem[size_t(ei)];
  const double cutsq = c->rcutmax * c->rcutmax;
  for (int k = 0; k < c->row_len(i); k++) {
    const int j = c->row_at(i, k);
    const double* xj = &c->x[3 * size_t(j)];
    const double dx = xj[0] - xi[0], dy = xj[1] - xi[1], dz = xj[2] - xi[2];
    const double rsq = dx * dx + dy * dy + dz * dz;
    const int ej = c->snap_map[size_t(c->type[size_t(j)])];
    if (rsq < cutsq) {
      rij.push_back(dx);
      rij.push_back(dy);
      rij.push_back(dz);
      inside.push_back(j);
      wj.push_back(c->wjelem[size_t(ej)]);
      rcutij.push_back((radi + c->radelem[size_t(ej)]) * c->rcutfac);
    }
  }
}
}  // namespace

// ForceSNAP::compute / operator() (force_snap_neigh_impl.h:160-208, 591-724)
// One atom of ForceSNAP::operator() (force_snap_neigh_impl.h:591-724): its
// pair forces f_ij added to i and subtracted from j in `f`.
static void snap_atom(orc_ctx* c, Sna& sna, int i, std::vector<double>& rij, std::vector<int>& inside,
                      std::vector<double>& wj, std::vector<double>& rcutij, std::vector<double>& dbvec, double* f) {
  snap_inside(c, i, rij, inside, wj, rcutij);
  const int ninside = int(inside.size());
  sna.compute_ui(rij, wj, rcutij, ninside);
  sna.compute_zi();
  const double* coeffi = &c->beta[size_t(c->snap_map[size_t(c->type[size_t(i)])]) * c->ncoeffall];
  for (int jj = 0; jj < ninside; jj++) {
    const int j = inside[size_t(jj)];
    sna.compute_duidrj(&rij[3 * size_t(jj)], wj[size_t(jj)], rcutij[size_t(jj)]);
    sna.compute_dbidrj(dbvec);
    double fij[3] = {0.0, 0.0, 0.0};
    for (int k = 1; k <= sna.ncoeff; k++) {
      const double bgb = coeffi[k];
      fij[0] += bgb * dbvec[3 * size_t(k - 1)];
      fij[1] += bgb * dbvec[3 * size_t(k - 1) + 1];
      fij[2] += bgb * dbvec[3 * size_t(k - 1) + 2];
    }
    const double dx = rij[3 * size_t(jj)], dy = rij[3 * size_t(jj) + 1], dz = rij[3 * size_t(jj) + 2];
    const double fdivr = -1.5e6 / std::pow(dx * dx + dy * dy + dz * dz, 7.0);
    fij[0] += dx * fdivr;
    fij[1] += dy * fdivr;
    fij[2] += dz * fdivr;
    for (int d = 0; d < 3; d++) {
      f[3 * size_t(i) + d] += fij[d];
      f[3 * size_t(j) + d] -= fij[d];
    }
  }
}

int orc_snap_compute(orc_ctx* c) {
  ORC_TRY
  if (!c->snap_ready) throw OrcErr("orc_snap_compute: not initialised");
  if (c->threads > 1) {
    // OpenMP over atoms (the CPU baseline): each thread its own SNA state and
    // force buffer, added to f in thread order afterwards.  Serial (one
    // thread) keeps the reference's order of the f_j subtractions.
    const int T = c->threads;
    const size_t nall = size_t(c->N_local + c->N_ghost);
    std::vector<Sna> snas(size_t(T), c->sna);
    std::vector<std::vector<double>> fb(size_t(T), std::vector<double>(3 * nall, 0.0));
#pragma omp parallel num_threads(T)
    {
      const int t = omp_get_thread_num();
      std::vector<double> rij, wj, rcutij, dbvec;
      std::vector<int> inside;
#pragma omp for schedule(dynamic, 8)
      for (int i = 0; i < c->N_local; i++) snap_atom(c, snas[size_t(t)], i, rij, inside, wj, rcutij, dbvec,
                                                     fb[size_t(t)].data());
    }
    for (int t = 0; t < T; t++)
      for (size_t k = 0; k < 3 * nall; k++) c->f[k] += fb[size_t(t)][k];
    return 0;
  }
  std::vector<double> rij, wj, rcutij, dbvec;
  std::vector<int> inside;
  Sna& sna = c->sna;
  for (int i = 0; i < c->N_local; i++) {
    snap_inside(c, i, rij, inside, wj, rcutij);
    const int ninside = int(inside.size());
    sna.compute_ui(rij, wj, rcutij, ninside);
    sna.compute_zi();
    const double* coeffi = &c->beta[size_t(c->snap_map[size_t(c->type[size_t(i)])]) * c->ncoeffall];
    for (int jj = 0; jj < ninside; jj++) {
      const int j = inside[size_t(jj)];
      sna.compute_duidrj(&rij[3 * size_t(jj)], wj[size_t(jj)], rcutij[size_t(jj)]);
      sna.compute_dbidrj(dbvec);
      double fij[3] = {0.0, 0.0, 0.0};
      for (int k = 1; k <= sna.ncoeff; k++) {
        const double bgb = coeffi[k];
        fij[0] += bgb * dbvec[3 * size_t(k - 1)];
        fij[1] += bgb * dbvec[3 * size_t(k - 1) + 1];
        fij[2] += bgb * dbvec[3 * size_t(k - 1) + 2];
      }
      const double dx = rij[3 * size_t(jj)], dy = rij[3 * size_t(jj) + 1], dz = rij[3 * size_t(jj) + 2];
      const double fdivr = -1.5e6 / std::pow(dx * dx + dy * dy + dz * dz, 7.0);
      fij[0] += dx * fdivr;
      fij[1] += dy * fdivr;
      fij[2] += dz * fdivr;
      for (int d = 0; d < 3; d++) {
        c->f[3 * size_t(i) + d] += fij[d];
        c->f[3 * size_t(j) + d] -= fij[d];
      }
    }
  }
  ORC_END
}

int orc_snap_bispectrum(orc_ctx* c, double* b) {
  ORC_TRY
  if (!c->snap_ready) throw OrcErr("orc_snap_bispectrum: not initialised");
  std::vector<double> rij, wj, rcutij, bvec;
  std::vector<int> inside;
  for (int i = 0; i < c->N_local; i++) {
    snap_inside(c, i, rij, inside, wj, rcutij);
    c->sna.compute_ui(rij, wj, rcutij, int(inside.size()));
    c->sna.compute_zi();
    c->sna.compute_bi(bvec);
    std::copy(bvec.begin(), bvec.end(), b + size_t(i) * c->sna.ncoeff);
  }
  ORC_END
}

int orc_snap_energy(orc_ctx* c, double* pe) {
  ORC_TRY
  const int nc = c->sna.ncoeff;
  std::vector<double> B(size_t(c->N_local) * nc);
  if (orc_snap_bispectrum(c, B.data())) return 1;
  std::vector<double> rij, wj, rcutij;
  std::vector<int> inside;
  double E = 0.0;
  for (int i = 0; i < c->N_local; i++) {
    const double* coeffi = &c->beta[size_t(c->snap_map[size_t(c->type[size_t(i)])]) * c->ncoeffall];
    double ei = coeffi[0];
    for (int k = 1; k <= nc; k++) ei += coeffi[k] * B[size_t(i) * nc + k - 1];
    snap_inside(c, i, rij, inside, wj, rcutij);
    for (size_t jj = 0; jj < inside.size(); jj++) {
      const double rsq = rij[3 * jj] * rij[3 * jj] + rij[3 * jj + 1] * rij[3 * jj + 1] + rij[3 * jj + 2] * rij[3 * jj + 2];
      ei += 1.25e5 / std::pow(rsq, 6.0);
    }
    E += ei;
  }
  *pe = E;
  ORC_END
}

int orc_snap_ncoeff(orc_ctx* c, int* n) {
  ORC_TRY
  *n = c->sna.ncoeff;
  ORC_END
}

// Temperature / KinE functor (property_temperature.h:54-57), serial order
int orc_thermo_mv2(orc_ctx* c, double* mv2) {
  ORC_TRY
  double T = 0.0;
  for (int i = 0; i < c->N_local; i++) {
    const size_t b = 3 * size_t(i);
    T += (c->v[b] * c->v[b] + c->v[b + 1] * c->v[b + 1] + c->v[b + 2] * c->v[b + 2]) * c->mass[size_t(c->type[size_t(i)])];
  }
  *mv2 = T;
  ORC_END
}

}  // extern "C"
