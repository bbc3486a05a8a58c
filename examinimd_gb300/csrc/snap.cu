// ForceSNAP host side: tables, launches and the adjoint reduction
// (force_snap_neigh_impl.h:160-724, sna_impl.hpp).  The kernel is in
// snap_kernel.cuh; the mixed-form instantiation is compiled in snap_mixed.cu.
#include <algorithm>
#include <cmath>
#include <vector>

#include "snap_kernel.cuh"

namespace emd {

void snap_mixed_launch(const snapk::SnapArgs& A, size_t smem, cudaStream_t s);

namespace {

using namespace snapk;

struct SnapHost {
  SnapDev d;
  int precision = EMD_PREC_FP64;
  DevBuf<int> trip, cg_off, jobs, tjob_off, yred_off, yred_job, map;
  DevBuf<int4> zord;
  DevBuf<int> inside_max;  // k_snap_inside_max's result
  DevBuf<double> cg, cY, beta0, radelem, wjelem, eatom, invf, yscale;
  DevBuf<float> cg_f, cY_f, yscale_f;
  // adjoint: per-atom columns, their per-element sums, the loss gradient dL/dF
  DevBuf<double> adj, adj_sum, adj_g;
  // coefficient k's three dB/dr terms: full triples and factors (the cY fold)
  std::vector<int> k_t1, k_t2, k_t3;
  std::vector<double> k_f2, k_f3;
  std::vector<int> k_j;  // (j1, j2, j) of coefficient k
  // U_tot and Z jobs of the last FP64 force pass, kept for an adjoint on the
  // same positions and list (emd_snap_keep_for_adjoint)
  bool keep_on = false, keep_valid = false;
  unsigned long long keep_xver = 0;
  long long keep_builds = -1;
  int keep_n = -1;
  DevBuf<double> keep_u, keep_z;
};


// ---------------------------------------------------------------- host tables
double factorial(int n) {
  double r = 1.0;
  for (int i = 1; i <= n; i++) r *= 1.0 * i;
  return r;
}
double deltacg(int j1, int j2, int j) {
  const double s = factorial((j1 + j2 + j) / 2 + 1);
  return std::sqrt(factorial((j1 + j2 - j) / 2) * factorial((j1 - j2 + j) / 2) * factorial((-j1 + j2 + j) / 2) / s);
}
// Clebsch-Gordan coefficient by the quasi-binomial formula of Varshalovich,
// Moskalev, Khersonskii 8.2.1(3) in twice-angular-momentum integers (the
// table SNA::init_clebsch_gordan builds, sna_impl.hpp:1003-1046)
double clebsch_gordan(int j1, int j2, int j, int m1, int m2) {
  const int aa2 = 2 * m1 - j1, bb2 = 2 * m2 - j2;
  const int m = (aa2 + bb2 + j) / 2;
  if (m < 0 || m > j) return 0.0;
  double sum = 0.0;
  for (int z = std::max(0, std::max(-(j - j2 + aa2) / 2, -(j - j1 - bb2) / 2));
       z <= std::min((j1 + j2 - j) / 2, std::min((j1 - aa2) / 2, (j2 + bb2) / 2)); z++) {
    const int ifac = z % 2 ? -1 : 1;
    sum += ifac / (factorial(z) * factorial((j1 + j2 - j) / 2 - z) * factorial((j1 - aa2) / 2 - z) *
                   factorial((j2 + bb2) / 2 - z) * factorial((j - j2 + aa2) / 2 + z) * factorial((j - j1 - bb2) / 2 + z));
  }
  const int cc2 = 2 * m - j;
  return sum * deltacg(j1, j2, j) *
         std::sqrt(factorial((j1 + aa2) / 2) * factorial((j1 - aa2) / 2) * factorial((j2 + bb2) / 2) *
                   factorial((j2 - bb2) / 2) * factorial((j + cc2) / 2) * factorial((j - cc2) / 2) * (j + 1));
}

// The Z jobs as descriptors (see SnapDev::zord), ordered for
// balance: sorted by inner-loop count, longest first, in chunks of 32 (a warp
// gets jobs of one length); chunk c goes to round c / 8 and, alternating
// direction from round to round, to warp c % 8 or 7 - c % 8.
std::vector<int4> zjob_order(const std::vector<int>& trip, const std::vector<int>& cg_off, const std::vector<int>& jobs) {
  const int nj = int(jobs.size());
  std::vector<int4> desc(static_cast<size_t>(nj));
  std::vector<int> cost(static_cast<size_t>(nj));
  for (int jb = 0; jb < nj; ++jb) {
    const int code = jobs[size_t(jb)], t = code >> 8, ma = (code >> 4) & 15, mb = code & 15;
    const int j1 = trip[3 * size_t(t)], j2 = trip[3 * size_t(t) + 1], j = trip[3 * size_t(t) + 2];
    const int ma1lo = std::max(0, (2 * ma - j - j2 + j1) / 2), ma1hi = std::min(j1, (2 * ma - j + j2 + j1) / 2);
    const int mb1lo = std::max(0, (2 * mb - j - j2 + j1) / 2), mb1hi = std::min(j1, (2 * mb - j + j2 + j1) / 2);
    int na = std::max(0, ma1hi - ma1lo + 1), nb = std::max(0, mb1hi - mb1lo + 1);
    const int ma2 = (2 * ma - j - (2 * ma1lo - j1) + j2) / 2, mb2 = (2 * mb - j - (2 * mb1lo - j1) + j2) / 2;
    const int uo1 = j1 * (j1 + 1) * (2 * j1 + 1) / 6, uo2 = j2 * (j2 + 1) * (2 * j2 + 1) / 6;
    int u1 = uo1 + ma1lo * (j1 + 1) + mb1lo, u2 = uo2 + ma2 * (j2 + 1) + mb2;
    int ci = cg_off[size_t(t)] + mb1lo * (j2 + 1) + mb2, co = cg_off[size_t(t)] + ma1lo * (j2 + 1) + ma2;
    if (na == 0 || nb == 0) na = nb = u1 = u2 = ci = co = 0;  // Z = 0, nothing read
    require(u1 >= 0 && u2 >= 0 && ci >= 0 && co >= 0 && u1 < 65536 && u2 < 65536 && ci < 65536 && co < 65536 &&
                na < 256 && nb < 256,
            EMD_ERR_ARG,
            "SNAP: Z job tables exceed their packed fields");
    desc[size_t(jb)] = int4{jb, int(unsigned(u1) | (unsigned(u2) << 16)), int(unsigned(ci) | (unsigned(co) << 16)),
                            int(unsigned(na) | (unsigned(nb) << 8) | (unsigned(j1 + 1) << 16) | (unsigned(j2 + 1) << 24))};
    cost[size_t(jb)] = na * (nb + 1);
  }
  std::vector<int> idx(static_cast<size_t>(nj));
  for (int k = 0; k < nj; ++k) idx[size_t(k)] = k;
  // longest first; within one length, jobs of equal row counts together, so
  // a warp's lanes run the same inner loops (no divergence between na x nb
  // splits of one length)
  std::stable_sort(idx.begin(), idx.end(), [&](int x, int y) {
    if (cost[size_t(x)] != cost[size_t(y)]) return cost[size_t(x)] > cost[size_t(y)];
    return (desc[size_t(x)].w & 0xff) > (desc[size_t(y)].w & 0xff);
  });
  const int nchunk = (nj + 31) / 32, nround = (nchunk + SNAP_WARPS - 1) / SNAP_WARPS;
  std::vector<int4> out(size_t(nround) * SNAP_THREADS, int4{-1, 0, 0, 0});
  for (int c = 0; c < nchunk; ++c) {
    const int r = c / SNAP_WARPS, p = c % SNAP_WARPS, w = (r & 1) ? SNAP_WARPS - 1 - p : p;
    for (int l = 0; l < 32 && 32 * c + l < nj; ++l)
      out[size_t(r) * SNAP_THREADS + 32 * size_t(w) + l] = desc[size_t(idx[size_t(32 * c + l)])];
  }
  return out;
}

// bytes of the `work` region: the neighbour slots' half layers (B), Z jobs
// (C), the forward layers and adjoints of d_reverse (D), or the fitting
// adjoint's per-warp U and dU layers
size_t snap_work_bytes(const SnapDev& S, int real_bytes) {
  const int L2 = S.L * S.L, J = S.twojmax;
  const size_t wB = 2 * sizeof(double) * size_t(SNAP_WARPS) * BG * size_t(S.bh_even + S.bh_odd);
  const size_t wC = 2 * size_t(real_bytes) * size_t(S.njobs);
  size_t wD = 2 * size_t(real_bytes) * size_t(SNAP_WARPS) * 2 * size_t(drev_words(J));
  if (real_bytes == int(sizeof(double)))  // the fitting adjoint's U and tangent layers
    wD = std::max(wD, 2 * sizeof(double) * size_t(SNAP_WARPS) * 4 * L2);
  return (std::max(wB, std::max(wC, wD)) + 15) & ~size_t(15);
}

// the adjoint's extra shared memory after `work`: kept Z, per-warp D partials, D
size_t snap_adjoint_bytes(const SnapDev& S) {
  return 2 * sizeof(double) * (size_t(S.njobs) + size_t(SNAP_WARPS + 1) * S.nyh);
}

// the kernel's shared-memory carve-up (k_snap), for `cap` inside neighbours
size_t snap_smem_bytes(const SnapDev& S, int cap, int real_bytes) {
  const bool f64 = real_bytes == int(sizeof(double));
  const size_t nd = f64 ? size_t(ND_FIELDS) : size_t(ND_MIXED), nr = f64 ? 0 : size_t(NR_MIXED);
  size_t b = 0;
  b += sizeof(double) * 5 * size_t(cap);                                // r, w, rcut
  b += 2 * sizeof(double) * size_t(S.nuf);                              // utot
  b += 2 * size_t(real_bytes) * size_t(S.nyh);                          // ytot
  if (!f64) b += 2 * size_t(real_bytes) * size_t(S.nuf);               // FP32 U_tot
  b += sizeof(int) * size_t((cap + 3) & ~3);                            // inside j
  b += sizeof(double) * 4 * SNAP_WARPS;                                 // reductions
  b += sizeof(double) * nd * size_t(cap);                               // FP64 per-neighbour fields
  b += sizeof(double) * ((nr * size_t(cap) + 1) / 2);                   // FP32 per-neighbour fields
  b += snap_work_bytes(S, real_bytes);
  return b + 64;
}

// the largest number of inside neighbours (r^2 < rcutmax^2) over the owned
// atoms: the kernel's per-neighbour shared arrays are sized by it
__global__ void __launch_bounds__(256) k_snap_inside_max(const double4_32a* __restrict__ x4, ListView L, int n,
                                                         double cutsq, int* out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  int cnt = 0;
  if (i < n) {
    const double4_32a xi = x4[i];
    const Row<false> rowc(L, i);
    const Row<true> row2(L, i);
    const bool two_d = L.stride != 0;
    for (int k = 0; k < rowc.n; ++k) {
      const int j = two_d ? row2[k] : rowc[k];
      const double4_32a xj = x4[j];
      const double dx = xj.x - xi.x, dy = xj.y - xi.y, dz = xj.z - xi.z;
      cnt += (dx * dx + dy * dy + dz * dz) < cutsq;
    }
  }
  cnt = __reduce_max_sync(FULL_MASK, cnt);
  if ((threadIdx.x & 31) == 0 && cnt > 0) atomicMax(out, cnt);
}

// per-element column sums of the adjoint's per-atom outputs (fixed order)
__global__ void __launch_bounds__(256) k_adj_reduce(const double* __restrict__ adj, int n, int ncols,
                                                    const int* __restrict__ type, const int* __restrict__ map,
                                                    double* __restrict__ out) {
  __shared__ double sh[8];
  const int col = blockIdx.x, e = blockIdx.y;
  const double* a = adj + size_t(col) * n;
  double acc = 0.0;
  for (int i = threadIdx.x; i < n; i += 256)
    if (map[type[i]] == e) acc += a[i];
  const double t = block_sum(acc, sh);
  if (threadIdx.x == 0) out[size_t(e) * ncols + col] = t;
}

}  // namespace

void free_snap(Ctx& c) {
  if (!c.snap) return;
  SnapHost* h = static_cast<SnapHost*>(c.snap);
  for (auto* b : {&h->trip, &h->cg_off, &h->jobs, &h->tjob_off, &h->yred_off, &h->yred_job, &h->map}) b->release();
  h->zord.release();
  h->inside_max.release();
  for (auto* b : {&h->cg, &h->cY, &h->beta0, &h->radelem, &h->wjelem, &h->eatom, &h->adj, &h->adj_sum,
                  &h->adj_g, &h->invf, &h->yscale, &h->keep_u, &h->keep_z})
    b->release();
  for (auto* b : {&h->cg_f, &h->cY_f, &h->yscale_f}) b->release();
  delete h;
  c.snap = nullptr;
}

static void upload_i(Ctx& c, DevBuf<int>& b, const std::vector<int>& v) {
  b.reserve(v.size() + 1, c.stream);
  EMD_CUDA(cudaMemcpyAsync(b.p, v.data(), sizeof(int) * v.size(), cudaMemcpyHostToDevice, c.stream));
}
template <class T>
static void upload(Ctx& c, DevBuf<T>& b, const std::vector<T>& v) {
  b.reserve(v.size() + 1, c.stream);
  EMD_CUDA(cudaMemcpyAsync(b.p, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice, c.stream));
}

// Y's coefficients: beta_k folded onto the full triples of compute_dbidrj's
// three terms (sna_impl.hpp:330-570), per element, with beta_0 apart
void snap_fold_beta(const SnapHost& h, int nfull, int nelem, int ncoeffall, const double* beta,
                    std::vector<double>& cY, std::vector<double>& beta0) {
  cY.assign(size_t(nelem) * nfull, 0.0);
  beta0.assign(static_cast<size_t>(nelem), 0.0);
  for (int e = 0; e < nelem; ++e) {
    const double* be = beta + size_t(e) * ncoeffall;
    beta0[size_t(e)] = be[0];
    double* ce = &cY[size_t(e) * nfull];
    for (size_t k = 0; k < h.k_t1.size(); ++k) {
      const int j1 = h.k_j[3 * k], j2 = h.k_j[3 * k + 1], j = h.k_j[3 * k + 2];
      const double bk = be[k + 1];
      ce[h.k_t1[k]] += bk;
      ce[h.k_t2[k]] += bk * (j + 1) / (j1 + 1.0);
      ce[h.k_t3[k]] += bk * (j + 1) / (j2 + 1.0);
    }
  }
}

// cap for the kernel's per-neighbour arrays: the largest inside count
static int snap_cap(Ctx& c, SnapHost* h) {
  const int n = c.N_local;
  h->inside_max.reserve(1, c.stream);
  EMD_CUDA(cudaMemsetAsync(h->inside_max.p, 0, sizeof(int), c.stream));
  {
    TimedLaunch t(c, "snap_inside_max");
    k_snap_inside_max<<<blocks_for(n, 256), 256, 0, c.stream>>>(c.x4.p, list_view(c), n, h->d.cutsq,
                                                                 h->inside_max.p);
    EMD_CHECK_LAUNCH();
  }
  EMD_CUDA(cudaMemcpyAsync(c.h_int, h->inside_max.p, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
  EMD_CUDA(cudaStreamSynchronize(c.stream));
  return std::max(1, c.h_int[0]);
}

static void snap_launch(Ctx& c, bool energy) {
  SnapHost* h = static_cast<SnapHost*>(c.snap);
  require(h != nullptr, EMD_ERR_STATE, "SNAP not initialised");
  require(c.neigh_ready && c.neigh_rows == c.N_local && !c.half_neigh, EMD_ERR_STATE,
          "SNAP needs a current full neighbour list");
  require(!c.neigh_packed, EMD_ERR_STATE, "SNAP reads plain neighbour rows");
  const int n = c.N_local;
  if (n == 0) return;
  if (!energy) {
    materialize_kick(c);  // the forces are about to be overwritten
    materialize_zero(c, true, true);
  }
  SnapArgs A;
  A.S = h->d;
  A.x4 = c.x4.p;
  A.type = c.type.p;
  A.f = c.f.p;
  A.L = list_view(c);
  A.n_local = n;
  A.cap = snap_cap(c, h);
  A.status = c.d_status;
  A.eatom = nullptr;
  const bool fp64 = h->precision == EMD_PREC_FP64 || energy;
  const size_t smem = snap_smem_bytes(h->d, A.cap, fp64 ? 8 : 4);
  require(smem <= 227 * 1024, EMD_ERR_ARG, "SNAP: neighbour rows too long for one atom's shared memory");
  A.g = nullptr;
  A.ghost_owner = nullptr;
  A.newton = 0;
  A.adj = nullptr;
  A.work_bytes = snap_work_bytes(h->d, fp64 ? 8 : 4);
  if (energy) {
    h->eatom.reserve(size_t(n), c.stream);
    A.eatom = h->eatom.p;
    auto k = k_snap<double, 1>;
    EMD_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    TimedLaunch t(c, "snap_energy");
    k<<<n, SNAP_THREADS, smem, c.stream>>>(A);
    EMD_CHECK_LAUNCH();
    return;
  }
  if (fp64) {
    // asked for (emd_snap_request_energy): the per-atom energies in the same pass
    const bool fused = c.snap_energy_request;
    if (fused) {
      h->eatom.reserve(size_t(n), c.stream);
      A.eatom = h->eatom.p;
    }
    if (h->keep_on) {
      h->keep_u.reserve(2 * size_t(h->d.nuf) * n, c.stream);
      h->keep_z.reserve(2 * size_t(h->d.njobs) * n, c.stream);
      A.keep_u = reinterpret_cast<Cplx<double>*>(h->keep_u.p);
      A.keep_z = reinterpret_cast<Cplx<double>*>(h->keep_z.p);
    }
    auto k = k_snap<double, 0>;
    EMD_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    TimedLaunch t(c, fused ? "snap_fp64_energy" : "snap_fp64");
    k<<<n, SNAP_THREADS, smem, c.stream>>>(A);
    if (fused) {
      c.snap_pe_fused_valid = true;
      c.snap_pe_fused_version = c.x_version;
    }
    if (h->keep_on) {
      h->keep_valid = true;
      h->keep_xver = c.x_version;
      h->keep_builds = c.neigh_builds;
      h->keep_n = n;
    }
  } else {
    TimedLaunch t(c, "snap_mixed");
    snap_mixed_launch(A, smem, c.stream);
  }
  EMD_CHECK_LAUNCH();
}

// d/dbeta of (dL_dE * E + sum_i dL_dF_i . F_i) for a loss L(E, F) of the
// total SNAP energy and the owned atoms' forces (host arrays)
static void snap_adjoint(Ctx& c, const double* dL_dF, double dL_dE, double* grad) {
  SnapHost* h = static_cast<SnapHost*>(c.snap);
  require(h != nullptr, EMD_ERR_STATE, "SNAP not initialised");
  require(c.neigh_ready && c.neigh_rows == c.N_local && !c.half_neigh && !c.neigh_packed, EMD_ERR_STATE,
          "emd_snap_adjoint needs a current full neighbour list");
  const SnapDev& S = h->d;
  const int n = c.N_local, nelem = S.nelem, ncols = 2 * S.nfull + 1;
  std::vector<double> sums(size_t(nelem) * ncols, 0.0);
  if (n > 0) {
    h->adj_g.reserve(3 * size_t(n), c.stream);
    EMD_CUDA(cudaMemcpyAsync(h->adj_g.p, dL_dF, sizeof(double) * 3 * size_t(n), cudaMemcpyHostToDevice, c.stream));
    h->adj.reserve(size_t(ncols) * n, c.stream);
    h->adj_sum.reserve(size_t(nelem) * ncols, c.stream);
    SnapArgs A;
    A.S = S;
    A.x4 = c.x4.p;
    A.type = c.type.p;
    A.f = nullptr;
    A.L = list_view(c);
    A.n_local = n;
    A.cap = snap_cap(c, h);
    A.status = c.d_status;
    A.eatom = nullptr;
    A.g = h->adj_g.p;
    A.ghost_owner = c.ghost_owner.p;
    A.newton = c.comm_newton;
    A.adj = h->adj.p;
    A.work_bytes = snap_work_bytes(S, 8);
    // B and C from the last FP64 force pass, when it ran on these positions and this list
    if (h->keep_on && h->keep_valid && h->keep_xver == c.x_version && h->keep_builds == c.neigh_builds &&
        h->keep_n == n) {
      A.keep_u = reinterpret_cast<Cplx<double>*>(h->keep_u.p);
      A.keep_z = reinterpret_cast<Cplx<double>*>(h->keep_z.p);
    }
    const size_t smem = snap_smem_bytes(S, A.cap, 8) + snap_adjoint_bytes(S);
    require(smem <= 227 * 1024, EMD_ERR_ARG, "SNAP adjoint: neighbour rows too long for shared memory");
    auto k = k_snap<double, 2>;
    EMD_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    {
      TimedLaunch t(c, "snap_adjoint");
      k<<<n, SNAP_THREADS, smem, c.stream>>>(A);
      EMD_CHECK_LAUNCH();
    }
    {
      TimedLaunch t(c, "snap_adjoint_reduce");
      k_adj_reduce<<<dim3(ncols, nelem), 256, 0, c.stream>>>(h->adj.p, n, ncols, c.type.p, S.map, h->adj_sum.p);
      EMD_CHECK_LAUNCH();
    }
    EMD_CUDA(cudaMemcpyAsync(sums.data(), h->adj_sum.p, sizeof(double) * sums.size(), cudaMemcpyDeviceToHost,
                             c.stream));
    EMD_CUDA(cudaStreamSynchronize(c.stream));
  }
  for (int e = 0; e < nelem; ++e) {
    const double* P = &sums[size_t(e) * ncols];
    const double* Q = P + S.nfull;
    double* g = grad + size_t(e) * S.ncoeffall;
    g[0] = dL_dE * P[2 * S.nfull];  // E = sum_i (beta_0 + ...)
    for (int k = 0; k < S.ncoeff; ++k)
      g[k + 1] = dL_dE * P[h->k_t1[k]] + Q[h->k_t1[k]] + h->k_f2[k] * Q[h->k_t2[k]] + h->k_f3[k] * Q[h->k_t3[k]];
  }
}

}  // namespace emd

using namespace emd;

extern "C" {

emd_status emd_snap_adjoint(emd_ctx* ctx, const double* dL_dF, double dL_dE, double* grad_beta) {
  EMD_API_BEGIN
  require(grad_beta != nullptr && (dL_dF != nullptr || c.N_local == 0), EMD_ERR_ARG, "emd_snap_adjoint: null array");
  snap_adjoint(c, dL_dF, dL_dE, grad_beta);
  EMD_API_END
}

emd_status emd_snap_init(emd_ctx* ctx, int twojmax, double rfac0, double rmin0, int switchflag, double rcutfac,
                         int nelem, const double* radelem, const double* wjelem, const double* beta, int ncoeffall,
                         int ntypes, const int* map, int precision) {
  EMD_API_BEGIN
  require(twojmax >= 0 && twojmax <= 14, EMD_ERR_ARG, "emd_snap_init: twojmax must be in [0, 14]");
  require(nelem >= 1 && radelem && wjelem && beta && map && ntypes >= 1, EMD_ERR_ARG, "emd_snap_init: arguments");
  require(precision == EMD_PREC_FP64 || precision == EMD_PREC_MIXED, EMD_ERR_ARG, "emd_snap_init: precision");
  require(switchflag == 0 || switchflag == 1, EMD_ERR_ARG, "emd_snap_init: switchflag");
  for (int t = 0; t < ntypes; ++t)
    require(map[t] >= 0 && map[t] < nelem, EMD_ERR_ARG, "emd_snap_init: every type must map to an element");
  free_snap(c);
  SnapHost* h = new SnapHost();
  c.snap = h;
  h->precision = precision;
  SnapDev& S = h->d;
  S.twojmax = twojmax;
  S.L = twojmax + 1;
  const int L = S.L;
  // index lists (SNA::build_indexlist, sna_impl.hpp:88-139, diagonalstyle 3)
  std::vector<int> trip;
  std::vector<int> idxj;  // positions of the idxj triples (j >= j1) in the full list
  std::vector<int> idx3;
  for (int j1 = 0; j1 <= twojmax; j1++)
    for (int j2 = 0; j2 <= j1; j2++)
      for (int j = std::abs(j1 - j2); j <= std::min(twojmax, j1 + j2); j += 2) {
        trip.push_back(j1);
        trip.push_back(j2);
        trip.push_back(j);
        if (j >= j1) {
          idx3.push_back(j1);
          idx3.push_back(j2);
          idx3.push_back(j);
        }
      }
  S.nfull = int(trip.size() / 3);
  S.ncoeff = int(idx3.size() / 3);
  require(ncoeffall == S.ncoeff + 1, EMD_ERR_ARG, "emd_snap_init: ncoeffall does not match twojmax");
  S.ncoeffall = ncoeffall;
  auto find_full = [&](int a, int b, int cc) {
    for (int t = 0; t < S.nfull; ++t)
      if (trip[3 * t] == a && trip[3 * t + 1] == b && trip[3 * t + 2] == cc) return t;
    throw Error(EMD_ERR_ARG, "SNAP: triple not found");
  };
  // compact CG blocks
  std::vector<int> cg_off(static_cast<size_t>(S.nfull));
  std::vector<double> cg;
  for (int t = 0; t < S.nfull; ++t) {
    const int a = trip[3 * t], b = trip[3 * t + 1], cc = trip[3 * t + 2];
    cg_off[size_t(t)] = int(cg.size());
    for (int m1 = 0; m1 <= a; ++m1)
      for (int m2 = 0; m2 <= b; ++m2) cg.push_back(clebsch_gordan(a, b, cc, m1, m2));
  }
  // Z jobs over the half grid of every triple, grouped by Y element
  auto yoff_h = [](int j) {
    int s = 0;
    for (int k = 0; k < j; ++k) s += (k + 1) * (k / 2 + 1);
    return s;
  };
  S.nyh = yoff_h(L);
  S.nuf = L * (L + 1) * (2 * L + 1) / 6;
  std::vector<std::vector<int>> by_y(static_cast<size_t>(S.nyh));
  std::vector<int> jobs, tjob_off;
  for (int t = 0; t < S.nfull; ++t) {
    const int cc = trip[3 * t + 2];
    tjob_off.push_back(int(jobs.size()));
    for (int mb = 0; 2 * mb <= cc; ++mb)
      for (int ma = 0; ma <= cc; ++ma) {
        by_y[size_t(yoff_h(cc) + mb * (cc + 1) + ma)].push_back(int(jobs.size()));
        jobs.push_back((t << 8) | (ma << 4) | mb);
      }
  }
  S.njobs = int(jobs.size());
  tjob_off.push_back(S.njobs);
  const std::vector<int4> zord = zjob_order(trip, cg_off, jobs);
  std::vector<int> yred_off(size_t(S.nyh) + 1, 0), yred_job;
  for (int e = 0; e < S.nyh; ++e) {
    yred_off[size_t(e)] = int(yred_job.size());
    for (int jb : by_y[size_t(e)]) yred_job.push_back(jb);
  }
  yred_off[size_t(S.nyh)] = int(yred_job.size());
  for (int k = 0; k < S.ncoeff; ++k) {
    const int j1 = idx3[3 * k], j2 = idx3[3 * k + 1], j = idx3[3 * k + 2];
    h->k_t1.push_back(find_full(j1, j2, j));
    h->k_t2.push_back(find_full(std::max(j, j2), std::min(j, j2), j1));
    h->k_t3.push_back(find_full(std::max(j1, j), std::min(j1, j), j2));
    h->k_f2.push_back((j + 1) / (j1 + 1.0));
    h->k_f3.push_back((j + 1) / (j2 + 1.0));
    h->k_j.insert(h->k_j.end(), {j1, j2, j});
  }
  std::vector<double> cY, beta0;
  snap_fold_beta(*h, S.nfull, nelem, ncoeffall, beta, cY, beta0);
  // over the half grid: 1 / f_j(ma, mb) of the rescaled recursion and the
  // D contraction's Y scale (twice the half-grid weight over f); the largest
  // half layer of even and odd j
  std::vector<double> invf(static_cast<size_t>(S.nyh));
  std::vector<double> yscale(static_cast<size_t>(S.nyh));
  S.bh_even = S.bh_odd = 1;
  for (int j = 0; j <= twojmax; ++j) {
    const int nh = (j + 1) * (j / 2 + 1);
    (j & 1 ? S.bh_odd : S.bh_even) = std::max(j & 1 ? S.bh_odd : S.bh_even, nh);
    for (int mb = 0; 2 * mb <= j; ++mb)
      for (int ma = 0; ma <= j; ++ma) {
        const size_t e = size_t(yoff_h(j) + mb * (j + 1) + ma);
        invf[e] = std::sqrt(factorial(j - ma) * factorial(ma) / (factorial(j - mb) * factorial(mb)));
        // twice the half-grid contraction weight (sna_impl.hpp:384-413)
        const double w2 = (2 * mb < j || 2 * ma < j) ? 2.0 : (2 * ma == j ? 1.0 : 0.0);
        yscale[e] = w2 * invf[e];
      }
  }
  double rcutmax = 0.0;
  for (int e = 0; e < nelem; e++) rcutmax = std::max(2.0 * radelem[e] * rcutfac, rcutmax);
  S.rfac0 = rfac0;
  S.rmin0 = rmin0;
  S.rcutfac = rcutfac;
  S.cutsq = rcutmax * rcutmax;
  S.wself = 1.0;
  S.switchflag = switchflag;
  S.nelem = nelem;
  S.ntypes = ntypes;
  upload_i(c, h->trip, trip);
  upload_i(c, h->cg_off, cg_off);
  upload(c, h->cg, cg);
  std::vector<float> cgf(cg.begin(), cg.end()), cYf(cY.begin(), cY.end());
  upload(c, h->cg_f, cgf);
  upload_i(c, h->jobs, jobs);
  h->zord.reserve(zord.size(), c.stream);
  EMD_CUDA(cudaMemcpyAsync(h->zord.p, zord.data(), sizeof(int4) * zord.size(), cudaMemcpyHostToDevice, c.stream));
  S.nzo = int(zord.size());
  upload_i(c, h->tjob_off, tjob_off);
  upload_i(c, h->yred_off, yred_off);
  upload_i(c, h->yred_job, yred_job);
  upload(c, h->cY, cY);
  upload(c, h->cY_f, cYf);
  upload(c, h->invf, invf);
  upload(c, h->yscale, yscale);
  upload(c, h->yscale_f, std::vector<float>(yscale.begin(), yscale.end()));
  upload(c, h->beta0, beta0);
  upload(c, h->radelem, std::vector<double>(radelem, radelem + nelem));
  upload(c, h->wjelem, std::vector<double>(wjelem, wjelem + nelem));
  upload_i(c, h->map, std::vector<int>(map, map + ntypes));
  EMD_CUDA(cudaStreamSynchronize(c.stream));
  S.trip = h->trip.p;
  S.cg_off = h->cg_off.p;
  S.cg = h->cg.p;
  S.cg_f = h->cg_f.p;
  S.jobs = h->jobs.p;
  S.zord = h->zord.p;
  S.tjob_off = h->tjob_off.p;
  S.yred_off = h->yred_off.p;
  S.yred_job = h->yred_job.p;
  S.cY = h->cY.p;
  S.cY_f = h->cY_f.p;
  S.invf = h->invf.p;
  S.yscale = h->yscale.p;
  S.yscale_f = h->yscale_f.p;
  S.beta0 = h->beta0.p;
  S.radelem = h->radelem.p;
  S.wjelem = h->wjelem.p;
  S.map = h->map.p;
  EMD_API_END
}

emd_status emd_snap_keep_for_adjoint(emd_ctx* ctx, int on) {
  EMD_API_BEGIN
  SnapHost* h = static_cast<SnapHost*>(c.snap);
  require(h != nullptr, EMD_ERR_STATE, "emd_snap_keep_for_adjoint: SNAP not initialised");
  h->keep_on = on != 0;
  h->keep_valid = false;
  if (!h->keep_on) {
    h->keep_u.release();
    h->keep_z.release();
  }
  EMD_API_END
}

emd_status emd_snap_info(emd_ctx* ctx, int* nelem, int* ncoeffall) {
  EMD_API_BEGIN
  const SnapHost* h = static_cast<const SnapHost*>(c.snap);
  require(h != nullptr, EMD_ERR_STATE, "emd_snap_info: SNAP not initialised");
  if (nelem) *nelem = h->d.nelem;
  if (ncoeffall) *ncoeffall = h->d.ncoeffall;
  EMD_API_END
}

emd_status emd_snap_set_beta(emd_ctx* ctx, const double* beta) {
  EMD_API_BEGIN
  SnapHost* h = static_cast<SnapHost*>(c.snap);
  require(h != nullptr, EMD_ERR_STATE, "emd_snap_set_beta: SNAP not initialised");
  require(beta != nullptr, EMD_ERR_ARG, "emd_snap_set_beta: null beta");
  std::vector<double> cY, beta0;
  snap_fold_beta(*h, h->d.nfull, h->d.nelem, h->d.ncoeffall, beta, cY, beta0);
  std::vector<float> cYf(cY.begin(), cY.end());
  EMD_CUDA(cudaMemcpyAsync(h->cY.p, cY.data(), sizeof(double) * cY.size(), cudaMemcpyHostToDevice, c.stream));
  EMD_CUDA(cudaMemcpyAsync(h->cY_f.p, cYf.data(), sizeof(float) * cYf.size(), cudaMemcpyHostToDevice, c.stream));
  EMD_CUDA(cudaMemcpyAsync(h->beta0.p, beta0.data(), sizeof(double) * beta0.size(), cudaMemcpyHostToDevice,
                           c.stream));
  EMD_CUDA(cudaStreamSynchronize(c.stream));
  EMD_API_END
}

emd_status emd_snap_compute(emd_ctx* ctx) {
  EMD_API_BEGIN
  struct EndRequest {  // a request serves this compute only
    Ctx& c;
    ~EndRequest() { c.snap_energy_request = false; }
  } end_request{c};
  c.snap_pe_fused_valid = false;
  snap_launch(c, false);
  EMD_API_END
}

emd_status emd_snap_request_energy(emd_ctx* ctx) {
  EMD_API_BEGIN
  require(c.snap != nullptr, EMD_ERR_STATE, "emd_snap_request_energy: SNAP not initialised");
  c.snap_energy_request = true;
  EMD_API_END
}

emd_status emd_snap_force_energy(emd_ctx* ctx, double* pe, int* available) {
  EMD_API_BEGIN
  require(pe && available, EMD_ERR_ARG, "emd_snap_force_energy: null output");
  *available = (c.snap_pe_fused_valid && c.snap_pe_fused_version == c.x_version) ? 1 : 0;
  *pe = 0.0;
  if (*available && c.N_local > 0) *pe = device_sum(c, static_cast<SnapHost*>(c.snap)->eatom.p, c.N_local);
  EMD_API_END
}

emd_status emd_snap_energy(emd_ctx* ctx, double* pe) {
  EMD_API_BEGIN
  require(pe != nullptr, EMD_ERR_ARG, "emd_snap_energy: null output");
  if (c.N_local == 0) {
    *pe = 0.0;
    return EMD_OK;
  }
  snap_launch(c, true);
  *pe = device_sum(c, static_cast<SnapHost*>(c.snap)->eatom.p, c.N_local);
  EMD_API_END
}

emd_status emd_snap_ncoeff(emd_ctx* ctx, int* ncoeff) {
  EMD_API_BEGIN
  require(c.snap != nullptr && ncoeff != nullptr, EMD_ERR_STATE, "emd_snap_ncoeff: SNAP not initialised");
  *ncoeff = static_cast<SnapHost*>(c.snap)->d.ncoeff;
  EMD_API_END
}

}  // extern "C"
