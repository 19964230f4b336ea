// Oracle (test infrastructure only): the Fock-build driver of the CPU
// restatement -- Schwarz bounds, shell density, the OpenMP quartet loop,
// storeints, the RHF/UROHF digestion and the response (TDHF, MRSF, UMRSF)
// digestions -- and the C entry points the tests and the CPU-baseline leg of
// bench.py call through ctypes.
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <memory>
#include <omp.h>

#include "oracle_basis.h"

using namespace orc;

using OrcHandle = orc::Handle;

struct OrcStats {
  double t_init, t_schwarz, t_twoei, t_total;
  long long quartets, screened, prim_quartets, stored;
};

// int2_run_cam (int2.F90:538-584): pass 1 regular integrals with
// scale_coulomb = alpha_c (1 by default), scale_exchange = alpha; pass 2
// erf-attenuated integrals (own Schwarz bounds) with scale_coulomb = beta_c
// (0 by default), scale_exchange = beta.
struct Cam {
  double alpha, beta, mu, alpha_c, beta_c;
};

// ints_exchange (int2.F90:1582-1737): Q(i,j) = sqrt(max |(ij|ij)|) with the
// very tight cutoffs 1e-15 / 1e-17 / 1e-17 / 50 (attenuated integrals when
// inv_mu2 != 0, int2.F90:675-681).
static void schwarz(const Basis& B, std::vector<double>& Q, int nthreads, double inv_mu2 = 0.0) {
  const Cutoffs cut = Cutoffs::make(1e-15, 1e-17, 1e-17, 50.0, inv_mu2);
  PairStore PS;
  PS.build(B, cut);
  const int ns = B.nshell;
  Q.assign((size_t)ns * ns, 0.0);
#pragma omp parallel num_threads(nthreads)
  {
    QuartetWork W;
    std::vector<double> blk(10 * 10 * 10 * 10);
#pragma omp for schedule(dynamic, 4)
    for (int i = 0; i < ns; ++i) {
      for (int j = 0; j <= i; ++j) {
        int ids[4] = {i, j, i, j}, s[4], fl[4];
        flip_quartet(B, ids, s, fl);
        double vmax = 0.0;
        if (rys_quartet(B, PS, cut, s, blk.data(), W) > 0) {
          int n = 1;
          for (int t = 0; t < 4; ++t) n *= B.sh[s[t]].nao;
          for (int e = 0; e < n; ++e) vmax = std::max(vmax, std::fabs(blk[e]));
        }
        Q[(size_t)i * ns + j] = Q[(size_t)j * ns + i] = std::sqrt(vmax);
      }
    }
  }
}

// shlden (int2.F90:999-1047): max |D| over the AO block of every shell pair
// and over the density matrices.
static void shlden(const Basis& B, const double* d, int nfocks, std::vector<double>& dsh) {
  const int ns = B.nshell;
  const size_t ntri = (size_t)B.nbf * (B.nbf + 1) / 2;
  dsh.assign((size_t)ns * ns, 0.0);
  for (int f = 0; f < nfocks; ++f) {
    const double* df = d + f * ntri;
    for (int si = 0; si < ns; ++si) {
      const int mini = B.sh[si].aoff, maxi = mini + B.sh[si].nao - 1;
      for (int sj = 0; sj <= si; ++sj) {
        const int minj = B.sh[sj].aoff;
        int maxj = minj + B.sh[sj].nao - 1;
        double dmax = 0;
        for (int i = mini; i <= maxi; ++i) {
          if (si == sj) maxj = i;
          for (int j = minj; j <= maxj; ++j) {
            const size_t ij = (size_t)i * (i + 1) / 2 + j;
            dmax = std::max(std::fabs(df[ij]), dmax);
          }
        }
        double& t = dsh[(size_t)si * ns + sj];
        t = std::max(dmax, t);
      }
    }
  }
  for (int si = 0; si < ns; ++si)
    for (int sj = si + 1; sj < ns; ++sj) dsh[(size_t)si * ns + sj] = dsh[(size_t)sj * ns + si];
}

// int2_build_shell_pair_map (int2.F90:864-921): pairs in descending estimated
// cost (counting sort over log2 classes), i descending as the secondary key.
static void pair_map(const Basis& B, const std::vector<double>& Q, std::vector<int>& pi, std::vector<int>& pj) {
  const int ns = B.nshell, NCLASS = 64, OFFS = 42;
  const int np = ns * (ns + 1) / 2;
  pi.assign(np, 0); pj.assign(np, 0);
  std::vector<int> cnt(NCLASS + 1, 0), off(NCLASS + 1, 0);
  auto cls_of = [&](int i, int j) {
    // shell numbers are 1-based in the cost formula
    const int nbfi = ncart(B.sh[i].am), nbfj = ncart(B.sh[j].am);
    const double sw = std::max(Q[(size_t)i * ns + j], 1e-30);
    const double cost = sw * (double)(nbfi * nbfj) * (double)(i + 1);
    const int lg = (int)(std::log(cost) / std::log(2.0));
    return NCLASS - std::max(0, std::min(NCLASS, lg + OFFS));
  };
  for (int i = ns - 1; i >= 0; --i)
    for (int j = 0; j <= i; ++j) cnt[cls_of(i, j)]++;
  off[0] = 0;
  for (int c = 1; c <= NCLASS; ++c) off[c] = off[c - 1] + cnt[c - 1];
  for (int i = ns - 1; i >= 0; --i)
    for (int j = 0; j <= i; ++j) {
      const int c = cls_of(i, j);
      const int p = off[c]++;
      pi[p] = i; pj[p] = j;
    }
}

struct Store {
  std::vector<int> ids;     // 4 per element, 0-based AO indices
  std::vector<double> val;
  int n = 0;
  explicit Store(int cap) : ids(4 * (size_t)cap), val(cap) {}
};

// int2_rhf_data_t_update / int2_urohf_data_t_update (int2.F90:1414-1578)
static void update(Store& st, const double* d, double* f, int nfocks, size_t ntri, bool urohf, double se,
                   double sc) {
  for (int n = 0; n < st.n; ++n) {
    const long ii = st.ids[4 * n] + 1, jj = st.ids[4 * n + 1] + 1, kk = st.ids[4 * n + 2] + 1,
               ll = st.ids[4 * n + 3] + 1;
    const double val = st.val[n];
    const long ii2 = ii * (ii - 1) / 2, jj2 = jj * (jj - 1) / 2, kk2 = kk * (kk - 1) / 2;
    const long ij = ii2 + jj - 1, ik = ii2 + kk - 1, il = ii2 + ll - 1, kl = kk2 + ll - 1;
    long jk = jj2 + kk - 1, jl = jj2 + ll - 1;
    if (jj < kk) jk = kk2 + jj - 1;
    if (jj < ll) jl = ll * (ll - 1) / 2 + jj - 1;
    if (!urohf) {
      const double val1 = val * se, val4 = val * 4 * sc;
      for (int q = 0; q < nfocks; ++q) {
        const double* dq = d + q * ntri;
        double* fq = f + q * ntri;
        fq[ij] += val4 * dq[kl];
        fq[kl] += val4 * dq[ij];
        fq[ik] -= val1 * dq[jl];
        fq[jl] -= val1 * dq[ik];
        fq[il] -= val1 * dq[jk];
        fq[jk] -= val1 * dq[il];
      }
    } else {
      const double val1 = val * 2 * se, val4 = val * 4 * sc;
      const double* da = d;
      const double* db = d + ntri;
      const double cij = val4 * (da[ij] + db[ij]);
      const double ckl = val4 * (da[kl] + db[kl]);
      for (int q = 0; q < 2; ++q) {
        const double* dq = d + q * ntri;
        double* fq = f + q * ntri;
        fq[ij] += ckl;
        fq[kl] += cij;
        fq[ik] -= val1 * dq[jl];
        fq[jl] -= val1 * dq[ik];
        fq[il] -= val1 * dq[jk];
        fq[jk] -= val1 * dq[il];
      }
    }
  }
  st.n = 0;
}

// int2_compute_data_t_storeints (int2.F90:1741-1865)
// flush(st) digests the buffered elements and empties the buffer (the
// reference's update call when the 50 000-element buffer is full).
template <class Flush>
static long storeints(const Basis& B, const int ids[4], const double* blk, double cutoff, Store& st, Flush& flush) {
  const int n1 = B.sh[ids[0]].nao, n2 = B.sh[ids[1]].nao, n3 = B.sh[ids[2]].nao, n4 = B.sh[ids[3]].nao;
  const bool same = ids[0] == ids[2] && ids[1] == ids[3];
  const bool iandj = ids[0] == ids[1];
  const bool kandl = ids[2] == ids[3];
  const int loci = B.sh[ids[0]].aoff, locj = B.sh[ids[1]].aoff, lock = B.sh[ids[2]].aoff,
            locl = B.sh[ids[3]].aoff;
  long nint = 0;
  int nij = 0;
  int maxj = n2;
  for (int i = 0; i < n1; ++i) {
    if (iandj) maxj = i + 1;
    for (int j = 0; j < maxj; ++j) {
      ++nij;
      int nkl = nij;
      int maxl = n4;
      bool next_j = false;
      for (int k = 0; k < n3 && !next_j; ++k) {
        if (kandl) maxl = k + 1;
        if (same) {
          const int itmp = std::min(maxl, nkl);
          if (itmp == 0) { next_j = true; break; }
          maxl = itmp;
          nkl -= itmp;
        }
        for (int l = 0; l < maxl; ++l) {
          double val = blk[((i * n2 + j) * n3 + k) * n4 + l];
          if (std::fabs(val) < cutoff) continue;
          ++nint;
          int i1 = i + loci, j1 = j + locj, k1 = k + lock, l1 = l + locl;
          if (i1 < j1) std::swap(i1, j1);
          if (k1 < l1) std::swap(k1, l1);
          int ii = i1, jj = j1, kk = k1, ll = l1;
          if (ii < kk) { ii = k1; jj = l1; kk = i1; ll = j1; }
          else if (ii == kk && jj < ll) { ii = i1; jj = l1; kk = k1; ll = j1; }
          if (ii == jj) val *= 0.5;
          if (kk == ll) val *= 0.5;
          if (ii == kk && jj == ll) val *= 0.5;
          int* p = &st.ids[4 * (size_t)st.n];
          p[0] = ii; p[1] = jj; p[2] = kk; p[3] = ll;
          st.val[st.n++] = val;
          if (st.n == (int)st.val.size()) flush(st);
        }
      }
    }
  }
  return nint;
}

struct TwoeiCounts {
  long long nq = 0, nsk = 0, npq = 0, nst = 0;
};

// int2_twoei (int2.F90:589-923): the OpenMP loop over the cost-sorted bra
// pairs with the pair screen Q_ij max_den < tau and the quartet screen
// Q_ij Q_kl max(4 Dsh_ij, 4 Dsh_kl, Dsh_jl, Dsh_jk, Dsh_il, Dsh_ik) < tau
// (int2.F90:963-986); every surviving quartet is evaluated and stored, and
// make(tid) gives the digestion of thread tid (the data type's update).
// stride/offset > 1 keep only the bra pairs p with p mod stride == offset.
template <class MakeFlush>
static TwoeiCounts twoei(const Basis& B, const PairStore& PS, const Cutoffs& cutoffs, double cut,
                         const std::vector<double>& Q, const std::vector<double>& dsh, int nthreads, int stride,
                         int offset, MakeFlush&& make) {
  double max_den = 0;
  for (double v : dsh) max_den = std::max(max_den, std::fabs(v));
  std::vector<int> pi, pj;
  pair_map(B, Q, pi, pj);
  const int ns = B.nshell;
  const int np = ns * (ns + 1) / 2;
  long long nq = 0, nsk = 0, npq = 0, nst = 0;
#pragma omp parallel num_threads(nthreads) reduction(+ : nq, nsk, npq, nst)
  {
    const int tid = omp_get_thread_num();
    auto flush = make(tid);
    QuartetWork W;
    std::vector<double> blk(10 * 10 * 10 * 10);
    Store st(50000);
#pragma omp for schedule(dynamic, 1)
    for (int p = 0; p < np; ++p) {
      if (stride > 1 && p % stride != offset) continue;
      const int i = pi[p], j = pj[p];
      const double qij = Q[(size_t)i * ns + j];
      if (qij * max_den < cut) { nsk += (long long)(i + 1) * i / 2 + j + 1; continue; }
      for (int k = 0; k <= i; ++k) {
        const int jork = (k == i) ? j : k;
        for (int l = 0; l <= jork; ++l) {
          double test = qij * Q[(size_t)k * ns + l];
          const double* D = dsh.data();
          test *= std::max({4 * D[(size_t)i * ns + j], 4 * D[(size_t)k * ns + l], D[(size_t)j * ns + l],
                            D[(size_t)j * ns + k], D[(size_t)i * ns + l], D[(size_t)i * ns + k]});
          if (test < cut) { ++nsk; continue; }
          ++nq;
          const int ids0[4] = {i, j, k, l};
          int s[4], fl[4];
          flip_quartet(B, ids0, s, fl);
          const long pq = rys_quartet(B, PS, cutoffs, s, blk.data(), W);
          if (pq == 0) continue;
          npq += pq;
          nst += storeints(B, s, blk.data(), cut, st, flush);
        }
      }
    }
    flush(st);
  }
  TwoeiCounts c;
  c.nq = nq; c.nsk = nsk; c.npq = npq; c.nst = nst;
  return c;
}

static double now() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// fock_jk (scf_addons.F90:1063-1214) with int2_twoei (int2.F90:589-923).
// stride/offset > 1 keep only the shell pairs p of the cost-sorted list with
// p mod stride == offset: the reference's own MPI work split
// (int2.F90:759-761), used to time a bounded sample of a large build.
static int fock_jk(OrcHandle* H, const double* d, double* fout, int nfocks, double se, double sc, int urohf,
                   int nthreads, const double* qext, OrcStats* stats, int stride = 1, int offset = 0,
                   const Cam* cam = nullptr) {
  const Basis& B = H->B;
  const double t0 = now();
  const double cut = H->cutoff;
  const Cutoffs cutoffs = Cutoffs::make(cut, 1e-2 * cut, 1e-4 * cut, 25.0 * std::log(10.0));
  PairStore PS;
  PS.build(B, cutoffs);
  const double t1 = now();
  std::vector<double> Q;
  if (qext) Q.assign(qext, qext + (size_t)B.nshell * B.nshell);
  else schwarz(B, Q, nthreads);
  const double t2 = now();
  std::vector<double> dsh;
  shlden(B, d, nfocks, dsh);
  const size_t ntri = (size_t)B.nbf * (B.nbf + 1) / 2;
  const int nf = urohf ? 2 : nfocks;
  std::vector<double> facc((size_t)nthreads * nf * ntri, 0.0);
  const double se1 = cam ? cam->alpha : se, sc1 = cam ? cam->alpha_c : sc;
  TwoeiCounts cnt = twoei(B, PS, cutoffs, cut, Q, dsh, nthreads, stride, offset, [&](int tid) {
    double* f = facc.data() + (size_t)tid * nf * ntri;
    return [=](Store& st) { update(st, d, f, nfocks, ntri, urohf, se1, sc1); };
  });
  if (cam) {
    const double inv_mu2 = 1.0 / (cam->mu * cam->mu);
    const Cutoffs ca = Cutoffs::make(cut, 1e-2 * cut, 1e-4 * cut, 25.0 * std::log(10.0), inv_mu2);
    std::vector<double> Qa;
    schwarz(B, Qa, nthreads, inv_mu2);
    const double se2 = cam->beta, sc2 = cam->beta_c;
    const TwoeiCounts c2 = twoei(B, PS, ca, cut, Qa, dsh, nthreads, stride, offset, [&](int tid) {
      double* f = facc.data() + (size_t)tid * nf * ntri;
      return [=](Store& st) { update(st, d, f, nfocks, ntri, urohf, se2, sc2); };
    });
    cnt.nq += c2.nq; cnt.nsk += c2.nsk; cnt.npq += c2.npq; cnt.nst += c2.nst;
  }
  // parallel_stop: reduce the replicated copies
  for (int t = 1; t < nthreads; ++t)
    for (size_t e = 0; e < (size_t)nf * ntri; ++e) facc[e] += facc[(size_t)t * nf * ntri + e];
  // scaling: f = 0.5 f, diagonal doubled
  for (int q = 0; q < nf; ++q) {
    for (size_t e = 0; e < ntri; ++e) fout[q * ntri + e] = 0.5 * facc[q * ntri + e];
    size_t ii = 0;
    for (int i = 0; i < B.nbf; ++i) { ii += i + 1; fout[q * ntri + ii - 1] *= 2; }
  }
  const double t3 = now();
  if (stats) {
    stats->t_init = t1 - t0; stats->t_schwarz = t2 - t1; stats->t_twoei = t3 - t2; stats->t_total = t3 - t0;
    stats->quartets = cnt.nq; stats->screened = cnt.nsk; stats->prim_quartets = cnt.npq; stats->stored = cnt.nst;
  }
  return 0;
}

// ---------------------------------------------------------------------------
// Response-type consumers of the same quartet loop (int2_td_data_t,
// int2_mrsf_data_t, int2_umrsf_data_t): general square densities, one digestion
// per data type.  Matrices are Fortran column-major; M(r, c) of an (n, n)
// matrix is m[c * n + r].

// shltd (tdhf_lib.F90:300-325) and shell_den_screen_mrsf
// (tdhf_mrsf_lib.F90:189-214): for shells ish >= jsh, the maximum of |X(r, c)|
// over r in jsh, c in ish (that one orientation of the block) and over the
// matrices q at x + q mstep; element (r, c) of a matrix is at r rstep + c cstep.
static void shell_den_general(const Basis& B, const double* x, int nmat, size_t mstep, size_t rstep, size_t cstep,
                              std::vector<double>& dsh) {
  const int ns = B.nshell;
  dsh.assign((size_t)ns * ns, 0.0);
  for (int si = 0; si < ns; ++si) {
    const int mini = B.sh[si].aoff, maxi = mini + B.sh[si].nao;
    for (int sj = 0; sj <= si; ++sj) {
      const int minj = B.sh[sj].aoff, maxj = minj + B.sh[sj].nao;
      double m = 0;
      for (int q = 0; q < nmat; ++q)
        for (int c = mini; c < maxi; ++c)
          for (int r = minj; r < maxj; ++r) m = std::max(m, std::fabs(x[q * mstep + r * rstep + c * cstep]));
      dsh[(size_t)si * ns + sj] = m;
      dsh[(size_t)sj * ns + si] = m;
    }
  }
}

enum { TD_APB = 1, TD_AMB = 2, TD_TDA = 4, TD_TDA_COUL = 8 };

// int2_td_data_t_update (tdhf_lib.F90:140-224)
static void td_update(Store& st, const double* d2, double* apb, double* amb, int n, int nvec, int flags,
                      double se, double sc) {
  const size_t n2 = (size_t)n * n;
  const double xval1 = se, cval2 = 2 * sc, cval4 = 4 * sc;
  for (int v = 0; v < nvec; ++v) {
    const double* d = d2 + v * n2;
    double* P = apb + v * n2;
    double* M = amb + v * n2;
    auto D = [&](int r, int c) { return d[(size_t)c * n + r]; };
    auto A = [&](double* m, int r, int c) -> double& { return m[(size_t)c * n + r]; };
    for (int e = 0; e < st.n; ++e) {
      const int i = st.ids[4 * e], j = st.ids[4 * e + 1], k = st.ids[4 * e + 2], l = st.ids[4 * e + 3];
      const double val = st.val[e];
      if (flags & TD_TDA) {
        const double val1 = val * xval1, val2c = val * cval2;
        A(M, i, k) -= val1 * D(j, l);
        A(M, k, i) -= val1 * D(l, j);
        A(M, i, l) -= val1 * D(j, k);
        A(M, l, i) -= val1 * D(k, j);
        A(M, j, k) -= val1 * D(i, l);
        A(M, k, j) -= val1 * D(l, i);
        A(M, j, l) -= val1 * D(i, k);
        A(M, l, j) -= val1 * D(k, i);
        if (flags & TD_TDA_COUL) {
          A(M, i, j) += val2c * (D(k, l) + D(l, k));
          A(M, j, i) += val2c * (D(k, l) + D(l, k));
          A(M, k, l) += val2c * (D(i, j) + D(j, i));
          A(M, l, k) += val2c * (D(i, j) + D(j, i));
        }
      } else {
        const double val1 = val * xval1, val4c = val * cval4;
        if (flags & TD_APB) {
          A(P, i, j) += val4c * (D(k, l) + D(l, k));
          A(P, k, l) += val4c * (D(i, j) + D(j, i));
          A(P, i, k) -= val1 * (D(j, l) + D(l, j));
          A(P, i, l) -= val1 * (D(j, k) + D(k, j));
          A(P, j, k) -= val1 * (D(i, l) + D(l, i));
          A(P, j, l) -= val1 * (D(i, k) + D(k, i));
        }
        if (flags & TD_AMB) {
          A(M, i, k) += val1 * (D(l, j) - D(j, l));
          A(M, i, l) += val1 * (D(k, j) - D(j, k));
          A(M, j, k) += val1 * (D(l, i) - D(i, l));
          A(M, j, l) += val1 * (D(k, i) - D(i, k));
          A(M, k, i) -= val1 * (D(l, j) - D(j, l));
          A(M, l, i) -= val1 * (D(k, j) - D(j, k));
          A(M, k, j) -= val1 * (D(l, i) - D(i, l));
          A(M, l, j) -= val1 * (D(k, i) - D(i, k));
        }
      }
    }
  }
  st.n = 0;
}

// int2_tdgrd_data_t_update (tdhf_lib.F90:228-295): two spin densities,
// Coulomb of their sum into both A+B matrices, exchange of each spin into its
// own, A-B of the first only.
static void tdgrd_update(Store& st, const double* d2, double* apb, double* amb, int n, int flags, double se,
                         double sc) {
  const size_t n2 = (size_t)n * n;
  const double xval1 = se, xval2 = 2 * sc;
  auto D = [&](int r, int c, int s) { return d2[s * n2 + (size_t)c * n + r]; };
  auto A = [&](double* m, int r, int c, int s) -> double& { return m[s * n2 + (size_t)c * n + r]; };
  for (int e = 0; e < st.n; ++e) {
    const int i = st.ids[4 * e], j = st.ids[4 * e + 1], k = st.ids[4 * e + 2], l = st.ids[4 * e + 3];
    const double val = st.val[e];
    const double val1 = val * xval1, val2 = val * xval2;
    if (flags & TD_APB) {
      const double ckl = D(k, l, 0) + D(l, k, 0) + D(k, l, 1) + D(l, k, 1);
      const double cij = D(i, j, 0) + D(j, i, 0) + D(i, j, 1) + D(j, i, 1);
      for (int s = 0; s < 2; ++s) {
        A(apb, i, j, s) += val2 * ckl;
        A(apb, k, l, s) += val2 * cij;
        A(apb, i, k, s) -= val1 * (D(j, l, s) + D(l, j, s));
        A(apb, i, l, s) -= val1 * (D(j, k, s) + D(k, j, s));
        A(apb, j, k, s) -= val1 * (D(i, l, s) + D(l, i, s));
        A(apb, j, l, s) -= val1 * (D(i, k, s) + D(k, i, s));
      }
    }
    if (flags & TD_AMB) {
      A(amb, i, k, 0) += val1 * (D(l, j, 0) - D(j, l, 0));
      A(amb, i, l, 0) += val1 * (D(k, j, 0) - D(j, k, 0));
      A(amb, j, k, 0) += val1 * (D(l, i, 0) - D(i, l, 0));
      A(amb, j, l, 0) += val1 * (D(k, i, 0) - D(i, k, 0));
      A(amb, k, i, 0) -= val1 * (D(l, j, 0) - D(j, l, 0));
      A(amb, l, i, 0) -= val1 * (D(k, j, 0) - D(j, k, 0));
      A(amb, k, j, 0) -= val1 * (D(l, i, 0) - D(i, l, 0));
      A(amb, l, j, 0) -= val1 * (D(k, i, 0) - D(i, k, 0));
    }
  }
  st.n = 0;
}

// int2_mrsf_data_t_update (tdhf_mrsf_lib.F90:218-333, the FP64 pass-1 branch)
// and int2_umrsf_data_t_update (tdhf_mrsf_lib.F90:337-426, pass 1).
// d3 / f3 are (nvec, nmat, n, n): element (v, c, r, col) at ((col n + r) nmat + c) nvec + v.
static void mrsf_update(Store& st, const double* d3, const double* ds, double* f3, int n, int nvec, int nmat,
                        bool umrsf, double se, double sc) {
  auto at = [&](int v, int c, int r, int col) { return (((size_t)col * n + r) * nmat + c) * nvec + v; };
  for (int e = 0; e < st.n; ++e) {
    const int i = st.ids[4 * e], j = st.ids[4 * e + 1], k = st.ids[4 * e + 2], l = st.ids[4 * e + 3];
    const double val = st.val[e];
    const double xval = val * se, cval = val * sc;
    auto K8 = [&](int c, int v) {
      f3[at(v, c, i, k)] -= xval * d3[at(v, c, j, l)];
      f3[at(v, c, k, i)] -= xval * d3[at(v, c, l, j)];
      f3[at(v, c, i, l)] -= xval * d3[at(v, c, j, k)];
      f3[at(v, c, l, i)] -= xval * d3[at(v, c, k, j)];
      f3[at(v, c, j, k)] -= xval * d3[at(v, c, i, l)];
      f3[at(v, c, k, j)] -= xval * d3[at(v, c, l, i)];
      f3[at(v, c, j, l)] -= xval * d3[at(v, c, i, k)];
      f3[at(v, c, l, j)] -= xval * d3[at(v, c, k, i)];
    };
    if (!umrsf) {
      for (int c = 0; c < 4; ++c)
        for (int v = 0; v < nvec; ++v) {
          const size_t dkl = (((size_t)l * n + k) * 4 + c) * nvec + v, dij = (((size_t)j * n + i) * 4 + c) * nvec + v;
          f3[at(v, c, i, j)] += cval * ds[dkl];
          f3[at(v, c, j, i)] += cval * ds[dkl];
          f3[at(v, c, k, l)] += cval * ds[dij];
          f3[at(v, c, l, k)] += cval * ds[dij];
        }
      for (int c = 0; c < 7; ++c)
        for (int v = 0; v < nvec; ++v) K8(c, v);
    } else {
      for (int c = 0; c < 8; ++c)
        for (int v = 0; v < nvec; ++v) {
          f3[at(v, c, i, j)] += cval * d3[at(v, c, k, l)];
          f3[at(v, c, k, l)] += cval * d3[at(v, c, i, j)];
          f3[at(v, c, i, j)] += cval * d3[at(v, c, l, k)];
          f3[at(v, c, l, k)] += cval * d3[at(v, c, i, j)];
          f3[at(v, c, j, i)] += cval * d3[at(v, c, k, l)];
          f3[at(v, c, k, l)] += cval * d3[at(v, c, j, i)];
          f3[at(v, c, j, i)] += cval * d3[at(v, c, l, k)];
          f3[at(v, c, l, k)] += cval * d3[at(v, c, j, i)];
          K8(c, v);
        }
      for (int c = 8; c < 10; ++c)
        for (int v = 0; v < nvec; ++v) {
          f3[at(v, c, i, l)] -= xval * d3[at(v, c, k, j)];
          f3[at(v, c, l, i)] -= xval * d3[at(v, c, j, k)];
          f3[at(v, c, k, j)] -= xval * d3[at(v, c, i, l)];
          f3[at(v, c, j, k)] -= xval * d3[at(v, c, l, i)];
          f3[at(v, c, i, k)] -= xval * d3[at(v, c, l, j)];
          f3[at(v, c, k, i)] -= xval * d3[at(v, c, j, l)];
          f3[at(v, c, l, j)] -= xval * d3[at(v, c, i, k)];
          f3[at(v, c, j, l)] -= xval * d3[at(v, c, k, i)];
        }
      for (int v = 0; v < nvec; ++v) K8(10, v);
    }
  }
  st.n = 0;
}

// int2_mrsf_data_t_update / int2_umrsf_data_t_update, pass 2 (CAM): only the
// last component (agdlr), exchange with scale_exchange = beta
// (tdhf_mrsf_lib.F90:314-328, 409-420).
static void mrsf_update_pass2(Store& st, const double* d3, double* f3, int n, int nvec, int nmat, double se) {
  auto at = [&](int v, int c, int r, int col) { return (((size_t)col * n + r) * nmat + c) * nvec + v; };
  const int c = nmat - 1;
  for (int e = 0; e < st.n; ++e) {
    const int i = st.ids[4 * e], j = st.ids[4 * e + 1], k = st.ids[4 * e + 2], l = st.ids[4 * e + 3];
    const double xval = st.val[e] * se;
    for (int v = 0; v < nvec; ++v) {
      f3[at(v, c, i, k)] -= xval * d3[at(v, c, j, l)];
      f3[at(v, c, k, i)] -= xval * d3[at(v, c, l, j)];
      f3[at(v, c, i, l)] -= xval * d3[at(v, c, j, k)];
      f3[at(v, c, l, i)] -= xval * d3[at(v, c, k, j)];
      f3[at(v, c, j, k)] -= xval * d3[at(v, c, i, l)];
      f3[at(v, c, k, j)] -= xval * d3[at(v, c, l, i)];
      f3[at(v, c, j, l)] -= xval * d3[at(v, c, i, k)];
      f3[at(v, c, l, j)] -= xval * d3[at(v, c, k, i)];
    }
  }
  st.n = 0;
}

struct Prepared {
  PairStore PS;
  Cutoffs cutoffs;
  std::vector<double> Q;
};

static void prepare(OrcHandle* H, int nthreads, Prepared& P) {
  const double cut = H->cutoff;
  P.cutoffs = Cutoffs::make(cut, 1e-2 * cut, 1e-4 * cut, 25.0 * std::log(10.0));
  P.PS.build(H->B, P.cutoffs);
  schwarz(H->B, P.Q, nthreads);
}

// TDHF-type build: d2 (n, n, nvec) -> apb, amb (n, n, nvec), both overwritten;
// int2_td_data_t_parallel_start/stop (tdhf_lib.F90:59-111): the replicated
// copies are summed and every apb matrix symmetrised (mathlib.F90:134-143).
// stride/offset > 1 restrict the bra pairs as in fock_jk (a timed sample);
// stats: [0] seconds outside the quartet loop (pairs, Schwarz, shell
// density, replicated copies and their reduction), [1] quartet-loop seconds,
// [2] quartets evaluated.
static int fock_td(OrcHandle* H, const double* d2, double* apb, double* amb, int nvec, int flags, double se,
                   double sc, int nthreads, int stride = 1, int offset = 0, double* stats = nullptr,
                   const Cam* cam = nullptr) {
  const Basis& B = H->B;
  const int n = B.nbf;
  const size_t n2 = (size_t)n * n, tot = n2 * nvec;
  const double t0 = now();
  Prepared P;
  prepare(H, nthreads, P);
  std::vector<double> dsh;
  shell_den_general(B, d2, nvec, n2, 1, n, dsh);
  std::vector<double> acc((size_t)nthreads * 2 * tot, 0.0);
  const double t1 = now();
  const double se1 = cam ? cam->alpha : se, sc1 = cam ? cam->alpha_c : sc;
  TwoeiCounts cnt = twoei(B, P.PS, P.cutoffs, H->cutoff, P.Q, dsh, nthreads, stride, offset, [&](int tid) {
    double* a = acc.data() + (size_t)tid * 2 * tot;
    return [=](Store& st) { td_update(st, d2, a, a + tot, n, nvec, flags, se1, sc1); };
  });
  if (cam) {
    const double inv_mu2 = 1.0 / (cam->mu * cam->mu), cut = H->cutoff;
    const Cutoffs ca = Cutoffs::make(cut, 1e-2 * cut, 1e-4 * cut, 25.0 * std::log(10.0), inv_mu2);
    std::vector<double> Qa;
    schwarz(B, Qa, nthreads, inv_mu2);
    const double se2 = cam->beta, sc2 = cam->beta_c;
    cnt.nq += twoei(B, P.PS, ca, cut, Qa, dsh, nthreads, stride, offset, [&](int tid) {
      double* a = acc.data() + (size_t)tid * 2 * tot;
      return [=](Store& st) { td_update(st, d2, a, a + tot, n, nvec, flags, se2, sc2); };
    }).nq;
  }
  const double t2 = now();
  for (int t = 1; t < nthreads; ++t)
    for (size_t e = 0; e < 2 * tot; ++e) acc[e] += acc[(size_t)t * 2 * tot + e];
  for (int v = 0; v < nvec; ++v) {
    double* a = acc.data() + v * n2;
    for (int i = 0; i < n; ++i) {
      for (int r = i; r < n; ++r) a[(size_t)i * n + r] += a[(size_t)r * n + i];
      for (int r = 0; r < i; ++r) a[(size_t)i * n + r] = a[(size_t)r * n + i];
    }
  }
  std::memcpy(apb, acc.data(), sizeof(double) * tot);
  std::memcpy(amb, acc.data() + tot, sizeof(double) * tot);
  if (stats) {
    stats[0] = (t1 - t0) + (now() - t2);  // everything but the quartet loop
    stats[1] = t2 - t1;
    stats[2] = (double)cnt.nq;
  }
  return 0;
}

// TD-gradient build of int2_tdgrd_data_t: d2 (n, n, 2) -> apb, amb (n, n, 2),
// overwritten; parallel_stop of int2_td_data_t symmetrises both apb matrices.
static int fock_tdgrd(OrcHandle* H, const double* d2, double* apb, double* amb, int flags, double se, double sc,
                      int nthreads, const Cam* cam = nullptr) {
  const Basis& B = H->B;
  const int n = B.nbf;
  const size_t n2 = (size_t)n * n, tot = 2 * n2;
  Prepared P;
  prepare(H, nthreads, P);
  std::vector<double> dsh;
  shell_den_general(B, d2, 2, n2, 1, n, dsh);
  std::vector<double> acc((size_t)nthreads * 2 * tot, 0.0);
  const double se1 = cam ? cam->alpha : se, sc1 = cam ? cam->alpha_c : sc;
  twoei(B, P.PS, P.cutoffs, H->cutoff, P.Q, dsh, nthreads, 1, 0, [&](int tid) {
    double* a = acc.data() + (size_t)tid * 2 * tot;
    return [=](Store& st) { tdgrd_update(st, d2, a, a + tot, n, flags, se1, sc1); };
  });
  if (cam) {
    const double inv_mu2 = 1.0 / (cam->mu * cam->mu), cut = H->cutoff;
    const Cutoffs ca = Cutoffs::make(cut, 1e-2 * cut, 1e-4 * cut, 25.0 * std::log(10.0), inv_mu2);
    std::vector<double> Qa;
    schwarz(B, Qa, nthreads, inv_mu2);
    const double se2 = cam->beta, sc2 = cam->beta_c;
    twoei(B, P.PS, ca, cut, Qa, dsh, nthreads, 1, 0, [&](int tid) {
      double* a = acc.data() + (size_t)tid * 2 * tot;
      return [=](Store& st) { tdgrd_update(st, d2, a, a + tot, n, flags, se2, sc2); };
    });
  }
  for (int t = 1; t < nthreads; ++t)
    for (size_t e = 0; e < 2 * tot; ++e) acc[e] += acc[(size_t)t * 2 * tot + e];
  for (int v = 0; v < 2; ++v) {
    double* a = acc.data() + v * n2;
    for (int i = 0; i < n; ++i) {
      for (int r = i; r < n; ++r) a[(size_t)i * n + r] += a[(size_t)r * n + i];
      for (int r = 0; r < i; ++r) a[(size_t)i * n + r] = a[(size_t)r * n + i];
    }
  }
  std::memcpy(apb, acc.data(), sizeof(double) * tot);
  std::memcpy(amb, acc.data() + tot, sizeof(double) * tot);
  return 0;
}

// int2_rpagrd_data_t_update_hplus (tdhf_lib.F90:1208-1284): H+[V] of one
// vector v (n, n, ld), spin components 0..nspin-1 of hp (n, n, nspin).
static void rpagrd_hplus(const Store& st, const double* v, size_t ld_step, double* hp, int n, int nspin, double se,
                         double sc) {
  const size_t n2 = (size_t)n * n;
  auto V = [&](int r, int c, int s) { return v[s * ld_step + (size_t)c * n + r]; };
  auto H = [&](int r, int c, int s) -> double& { return hp[s * n2 + (size_t)c * n + r]; };
  if (nspin == 1) {
    const double xfact = 2 * se, cfact = 8 * sc;
    for (int e = 0; e < st.n; ++e) {
      const int i = st.ids[4 * e], j = st.ids[4 * e + 1], k = st.ids[4 * e + 2], l = st.ids[4 * e + 3];
      const double xval = st.val[e] * xfact, cval = st.val[e] * cfact;
      H(i, j, 0) += cval * V(l, k, 0);
      H(k, l, 0) += cval * V(j, i, 0);
      H(i, k, 0) -= xval * V(l, j, 0);
      H(i, l, 0) -= xval * V(k, j, 0);
      H(j, k, 0) -= xval * V(l, i, 0);
      H(j, l, 0) -= xval * V(k, i, 0);
    }
  } else {
    const double xfact = se, cfact = 2 * sc;
    for (int e = 0; e < st.n; ++e) {
      const int i = st.ids[4 * e], j = st.ids[4 * e + 1], k = st.ids[4 * e + 2], l = st.ids[4 * e + 3];
      const double xval = st.val[e] * xfact, cval = st.val[e] * cfact;
      const double ckl = V(k, l, 0) + V(l, k, 0) + V(k, l, 1) + V(l, k, 1);
      const double cij = V(i, j, 0) + V(j, i, 0) + V(i, j, 1) + V(j, i, 1);
      for (int s = 0; s < 2; ++s) {
        H(i, j, s) += cval * ckl;
        H(k, l, s) += cval * cij;
        H(i, k, s) -= xval * (V(j, l, s) + V(l, j, s));
        H(i, l, s) -= xval * (V(j, k, s) + V(k, j, s));
        H(j, k, s) -= xval * (V(i, l, s) + V(l, i, s));
        H(j, l, s) -= xval * (V(i, k, s) + V(k, i, s));
      }
    }
  }
}

// int2_rpagrd_data_t_update_hminus (tdhf_lib.F90:1286-1322): spin component 0 only.
static void rpagrd_hminus(const Store& st, const double* v, double* hm, int n, double se) {
  auto V = [&](int r, int c) { return v[(size_t)c * n + r]; };
  auto H = [&](int r, int c) -> double& { return hm[(size_t)c * n + r]; };
  for (int e = 0; e < st.n; ++e) {
    const int i = st.ids[4 * e], j = st.ids[4 * e + 1], k = st.ids[4 * e + 2], l = st.ids[4 * e + 3];
    const double xval = st.val[e] * se;
    H(i, k) += xval * (V(l, j) - V(j, l));
    H(i, l) += xval * (V(k, j) - V(j, k));
    H(j, k) += xval * (V(l, i) - V(i, l));
    H(j, l) += xval * (V(k, i) - V(i, k));
    H(k, i) -= xval * (V(l, j) - V(j, l));
    H(l, i) -= xval * (V(k, j) - V(j, k));
    H(k, j) -= xval * (V(l, i) - V(i, l));
    H(l, j) -= xval * (V(k, i) - V(i, k));
  }
}

// int2_rpagrd_data_t (tdhf_lib.F90:1068-1322): xpy (n, n, ldp, np), xmy
// (n, n, ldm, nm), t (n, n, ldt, nt) -> hpp (n, n, nspin, np), hpt
// (n, n, nspin, nt), hmm (n, n, nspin, nm), overwritten.  The shell density
// is the maximum over every component of xpy and xmy (both only when np > 0)
// and of t (init_screen, :1161-1173); parallel_stop symmetrises hpp and hpt.
static int fock_rpagrd(OrcHandle* H, const double* xpy, int ldp, int np, const double* xmy, int ldm, int nm,
                       const double* t, int ldt, int nt, int nspin, double* hpp, double* hpt, double* hmm, double se,
                       double sc, int nthreads, const Cam* cam = nullptr) {
  const Basis& B = H->B;
  const int n = B.nbf;
  const size_t n2 = (size_t)n * n, blk = n2 * nspin;
  const size_t tp = blk * np, tt = blk * nt, tm = blk * nm, tot = tp + tt + tm;
  Prepared P;
  prepare(H, nthreads, P);
  std::vector<double> dsh((size_t)B.nshell * B.nshell, 0.0), part;
  auto screen = [&](const double* x, int nmat) {
    shell_den_general(B, x, nmat, n2, 1, n, part);
    for (size_t e = 0; e < dsh.size(); ++e) dsh[e] = std::max(dsh[e], part[e]);
  };
  if (np > 0) screen(xpy, ldp * np);
  if (np > 0 && nm > 0) screen(xmy, ldm * nm);
  if (nt > 0) screen(t, ldt * nt);
  std::vector<double> acc((size_t)nthreads * tot, 0.0);
  auto pass = [&](const Cutoffs& cuts, const std::vector<double>& Q, double sx, double scl) {
    twoei(B, P.PS, cuts, H->cutoff, Q, dsh, nthreads, 1, 0, [&](int tid) {
      double* a = acc.data() + (size_t)tid * tot;
      return [=](Store& st) {
        for (int v = 0; v < np; ++v) rpagrd_hplus(st, xpy + v * ldp * n2, n2, a + v * blk, n, nspin, sx, scl);
        for (int v = 0; v < nt; ++v) rpagrd_hplus(st, t + v * ldt * n2, n2, a + tp + v * blk, n, nspin, sx, scl);
        for (int v = 0; v < nm; ++v) rpagrd_hminus(st, xmy + v * ldm * n2, a + tp + tt + v * blk, n, sx);
        st.n = 0;
      };
    });
  };
  pass(P.cutoffs, P.Q, cam ? cam->alpha : se, cam ? cam->alpha_c : sc);
  if (cam) {
    const double inv_mu2 = 1.0 / (cam->mu * cam->mu), cut = H->cutoff;
    const Cutoffs ca = Cutoffs::make(cut, 1e-2 * cut, 1e-4 * cut, 25.0 * std::log(10.0), inv_mu2);
    std::vector<double> Qa;
    schwarz(B, Qa, nthreads, inv_mu2);
    pass(ca, Qa, cam->beta, cam->beta_c);
  }
  for (int th = 1; th < nthreads; ++th)
    for (size_t e = 0; e < tot; ++e) acc[e] += acc[(size_t)th * tot + e];
  for (size_t v = 0; v < (size_t)(np + nt) * nspin; ++v) {
    double* a = acc.data() + v * n2;
    for (int i = 0; i < n; ++i) {
      for (int r = i; r < n; ++r) a[(size_t)i * n + r] += a[(size_t)r * n + i];
      for (int r = 0; r < i; ++r) a[(size_t)i * n + r] = a[(size_t)r * n + i];
    }
  }
  if (np) std::memcpy(hpp, acc.data(), sizeof(double) * tp);
  if (nt) std::memcpy(hpt, acc.data() + tp, sizeof(double) * tt);
  if (nm) std::memcpy(hmm, acc.data() + tp + tt, sizeof(double) * tm);
  return 0;
}

// MRSF (nmat = 7) / UMRSF (nmat = 11) response build: d3 -> f3 (overwritten),
// int2_mrsf_data_t_parallel_start/stop (tdhf_mrsf_lib.F90:58-149); the
// screening density is the last component (tdhf_mrsf_lib.F90:171-185).
static int fock_mrsf(OrcHandle* H, const double* d3, double* f3, int nvec, int nmat, double se, double sc,
                     int nthreads, const Cam* cam = nullptr, int stride = 1, int offset = 0,
                     double* stats = nullptr) {
  const double t0 = now();
  const Basis& B = H->B;
  const int n = B.nbf;
  const bool umrsf = nmat == 11;
  if (nmat != 7 && nmat != 11) return 3;
  const size_t tot = (size_t)n * n * nmat * nvec;
  Prepared P;
  prepare(H, nthreads, P);
  std::vector<double> dsh;
  shell_den_general(B, d3 + (size_t)(nmat - 1) * nvec, nvec, 1, (size_t)nmat * nvec, (size_t)n * nmat * nvec, dsh);
  // symmetrised Coulomb components ds(v, c, r, col) = d3(v, c, r, col) + d3(v, c, col, r), c < 4
  std::vector<double> ds;
  if (!umrsf) {
    ds.assign((size_t)n * n * 4 * nvec, 0.0);
    for (int col = 0; col < n; ++col)
      for (int r = 0; r < n; ++r)
        for (int c = 0; c < 4; ++c)
          for (int v = 0; v < nvec; ++v)
            ds[(((size_t)col * n + r) * 4 + c) * nvec + v] =
                d3[(((size_t)col * n + r) * nmat + c) * nvec + v] + d3[(((size_t)r * n + col) * nmat + c) * nvec + v];
  }
  std::vector<double> acc((size_t)nthreads * tot, 0.0);
  const double* dsp = ds.data();
  const double se1 = cam ? cam->alpha : se, sc1 = cam ? cam->alpha_c : sc;
  const double t1 = now();
  const TwoeiCounts cnt = twoei(B, P.PS, P.cutoffs, H->cutoff, P.Q, dsh, nthreads, stride, offset, [&](int tid) {
    double* a = acc.data() + (size_t)tid * tot;
    return [=](Store& st) { mrsf_update(st, d3, dsp, a, n, nvec, nmat, umrsf, se1, sc1); };
  });
  const double t2 = now();
  if (cam) {
    const double inv_mu2 = 1.0 / (cam->mu * cam->mu), cut = H->cutoff;
    const Cutoffs ca = Cutoffs::make(cut, 1e-2 * cut, 1e-4 * cut, 25.0 * std::log(10.0), inv_mu2);
    std::vector<double> Qa;
    schwarz(B, Qa, nthreads, inv_mu2);
    const double se2 = cam->beta;
    twoei(B, P.PS, ca, cut, Qa, dsh, nthreads, 1, 0, [&](int tid) {
      double* a = acc.data() + (size_t)tid * tot;
      return [=](Store& st) { mrsf_update_pass2(st, d3, a, n, nvec, nmat, se2); };
    });
  }
  for (int t = 1; t < nthreads; ++t)
    for (size_t e = 0; e < tot; ++e) acc[e] += acc[(size_t)t * tot + e];
  std::memcpy(f3, acc.data(), sizeof(double) * tot);
  if (stats) {
    stats[0] = (t1 - t0) + (now() - t2);  // everything but the (first) quartet loop
    stats[1] = t2 - t1;
    stats[2] = (double)cnt.nq;
  }
  return 0;
}

extern "C" {

// Basis registration in OpenQP's basis_set layout (basis_tools.F90:32-84):
// per shell am, ncontr, origin (1-based atom), harmonic; ex/cc concatenated
// (cc primitive-normalised); xyz(3, natom) in Bohr.
void* orc_create(int nshell, const int* am, const int* ncontr, const int* origin, const double* ex,
                 const double* cc, const int* harmonic, int natom, const double* xyz, double cutoff) {
  auto* H = new OrcHandle;
  Basis& B = H->B;
  B.nshell = nshell; B.natom = natom;
  B.xyz.assign(xyz, xyz + 3 * natom);
  int poff = 0, aoff = 0;
  for (int s = 0; s < nshell; ++s) {
    Shell S;
    S.am = am[s]; S.nprim = ncontr[s]; S.atom = origin[s] - 1; S.harm = harmonic ? harmonic[s] : 0;
    S.poff = poff; S.aoff = aoff;
    S.nao = (S.harm && S.am >= 2) ? 2 * S.am + 1 : ncart(S.am);
    for (int d = 0; d < 3; ++d) S.c[d] = xyz[3 * S.atom + d];
    poff += S.nprim; aoff += S.nao;
    B.maxam = std::max(B.maxam, S.am);
    B.sh.push_back(S);
  }
  B.nbf = aoff;
  B.ex.assign(ex, ex + poff);
  B.cc.assign(cc, cc + poff);
  H->cutoff = cutoff;
  return H;
}

void orc_destroy(void* h) { delete (OrcHandle*)h; }
int orc_nbf(void* h) { return ((OrcHandle*)h)->B.nbf; }

int orc_fock_jk(void* h, const double* d, double* f, int nfocks, double se, double sc, int urohf, int nthreads,
                const double* schwarz_in, double* stats6) {
  OrcStats st;
  const int rc = fock_jk((OrcHandle*)h, d, f, nfocks, se, sc, urohf, nthreads, schwarz_in, &st);
  if (stats6) {
    stats6[0] = st.t_init; stats6[1] = st.t_schwarz; stats6[2] = st.t_twoei; stats6[3] = st.t_total;
    stats6[4] = (double)st.quartets; stats6[5] = (double)st.screened; stats6[6] = (double)st.prim_quartets;
    stats6[7] = (double)st.stored;
  }
  return rc;
}

// Same build restricted to the shell pairs p with p mod stride == offset.
int orc_fock_jk_sample(void* h, const double* d, double* f, int nfocks, double se, double sc, int urohf,
                       int nthreads, const double* schwarz_in, int stride, int offset, double* stats6) {
  OrcStats st;
  const int rc = fock_jk((OrcHandle*)h, d, f, nfocks, se, sc, urohf, nthreads, schwarz_in, &st, stride, offset);
  if (stats6) {
    stats6[0] = st.t_init; stats6[1] = st.t_schwarz; stats6[2] = st.t_twoei; stats6[3] = st.t_total;
    stats6[4] = (double)st.quartets; stats6[5] = (double)st.screened; stats6[6] = (double)st.prim_quartets;
    stats6[7] = (double)st.stored;
  }
  return rc;
}

// flags: 1 A+B, 2 A-B, 4 Tamm-Dancoff, 8 Tamm-Dancoff with Coulomb terms.
int orc_fock_td(void* h, const double* d2, double* apb, double* amb, int nvec, int flags, double se, double sc,
                int nthreads) {
  return fock_td((OrcHandle*)h, d2, apb, amb, nvec, flags, se, sc, nthreads);
}

// The same build over the bra pairs p with p mod stride == offset; stats3 as fock_td.
int orc_fock_td_sample(void* h, const double* d2, double* apb, double* amb, int nvec, int flags, double se,
                       double sc, int nthreads, int stride, int offset, double* stats3) {
  return fock_td((OrcHandle*)h, d2, apb, amb, nvec, flags, se, sc, nthreads, stride, offset, stats3);
}

int orc_fock_mrsf(void* h, const double* d3, double* f3, int nvec, int nmat, double se, double sc, int nthreads) {
  return fock_mrsf((OrcHandle*)h, d3, f3, nvec, nmat, se, sc, nthreads);
}

// fock_mrsf over the bra pairs p (cost-sorted) with p % stride == offset;
// stats3 = {seconds outside the quartet loop, loop seconds, quartets}.
int orc_fock_mrsf_sample(void* h, const double* d3, double* f3, int nvec, int nmat, double se, double sc,
                         int nthreads, int stride, int offset, double* stats3) {
  return fock_mrsf((OrcHandle*)h, d3, f3, nvec, nmat, se, sc, nthreads, nullptr, stride, offset, stats3);
}

int orc_fock_tdgrd(void* h, const double* d2, double* apb, double* amb, int flags, double se, double sc,
                   int nthreads) {
  return fock_tdgrd((OrcHandle*)h, d2, apb, amb, flags, se, sc, nthreads);
}

int orc_fock_rpagrd(void* h, const double* xpy, int ldp, int np, const double* xmy, int ldm, int nm, const double* t,
                    int ldt, int nt, int nspin, double* hpp, double* hpt, double* hmm, double se, double sc,
                    const double* cam5, int nthreads) {
  if (cam5) {
    const Cam cam{cam5[0], cam5[1], cam5[2], cam5[3], cam5[4]};
    return fock_rpagrd((OrcHandle*)h, xpy, ldp, np, xmy, ldm, nm, t, ldt, nt, nspin, hpp, hpt, hmm, se, sc,
                       nthreads, &cam);
  }
  return fock_rpagrd((OrcHandle*)h, xpy, ldp, np, xmy, ldm, nm, t, ldt, nt, nspin, hpp, hpt, hmm, se, sc, nthreads);
}

int orc_fock_tdgrd_cam(void* h, const double* d2, double* apb, double* amb, int flags, const double* cam5,
                       int nthreads) {
  const Cam cam{cam5[0], cam5[1], cam5[2], cam5[3], cam5[4]};
  return fock_tdgrd((OrcHandle*)h, d2, apb, amb, flags, 1.0, 1.0, nthreads, &cam);
}

// CAM (two-pass) forms: cam5 = {alpha, beta, mu, alpha_coulomb, beta_coulomb}.
int orc_fock_jk_cam(void* h, const double* d, double* f, int nfocks, int urohf, const double* cam5, int nthreads) {
  const Cam cam{cam5[0], cam5[1], cam5[2], cam5[3], cam5[4]};
  return fock_jk((OrcHandle*)h, d, f, nfocks, 0.0, 0.0, urohf, nthreads, nullptr, nullptr, 1, 0, &cam);
}
// CAM build over the bra pairs p with p mod stride == offset (both passes); stats6 as orc_fock_jk.
int orc_fock_jk_cam_sample(void* h, const double* d, double* f, int nfocks, int urohf, const double* cam5,
                           int nthreads, int stride, int offset, double* stats6) {
  const Cam cam{cam5[0], cam5[1], cam5[2], cam5[3], cam5[4]};
  OrcStats st;
  const int rc = fock_jk((OrcHandle*)h, d, f, nfocks, 0.0, 0.0, urohf, nthreads, nullptr, &st, stride, offset, &cam);
  if (stats6) {
    stats6[0] = st.t_init; stats6[1] = st.t_schwarz; stats6[2] = st.t_twoei; stats6[3] = st.t_total;
    stats6[4] = (double)st.quartets; stats6[5] = (double)st.screened; stats6[6] = (double)st.prim_quartets;
    stats6[7] = (double)st.stored;
  }
  return rc;
}
int orc_fock_td_cam(void* h, const double* d2, double* apb, double* amb, int nvec, int flags, const double* cam5,
                    int nthreads) {
  const Cam cam{cam5[0], cam5[1], cam5[2], cam5[3], cam5[4]};
  return fock_td((OrcHandle*)h, d2, apb, amb, nvec, flags, 0.0, 0.0, nthreads, 1, 0, nullptr, &cam);
}
int orc_fock_mrsf_cam(void* h, const double* d3, double* f3, int nvec, int nmat, const double* cam5, int nthreads) {
  const Cam cam{cam5[0], cam5[1], cam5[2], cam5[3], cam5[4]};
  return fock_mrsf((OrcHandle*)h, d3, f3, nvec, nmat, 0.0, 0.0, nthreads, &cam);
}

// Schwarz bounds of the erf-attenuated operator (mu > 0).
void orc_schwarz_att(void* h, double* q, int nthreads, double mu) {
  std::vector<double> Q;
  schwarz(((OrcHandle*)h)->B, Q, nthreads, 1.0 / (mu * mu));
  std::memcpy(q, Q.data(), sizeof(double) * Q.size());
}

void orc_schwarz(void* h, double* q, int nthreads) {
  std::vector<double> Q;
  schwarz(((OrcHandle*)h)->B, Q, nthreads);
  std::memcpy(q, Q.data(), sizeof(double) * Q.size());
}

void orc_shlden(void* h, const double* d, int nfocks, double* dsh) {
  std::vector<double> v;
  shlden(((OrcHandle*)h)->B, d, nfocks, v);
  std::memcpy(dsh, v.data(), sizeof(double) * v.size());
}

// Normalised (pure) shell-quartet block in the caller's (i,j,k,l) order,
// out[a][b][c][d]; screening cutoffs of a Fock build with the handle's cutoff.
int orc_eri_quartet_att(void* h, int i, int j, int k, int l, double mu, double* out);
int orc_eri_quartet(void* h, int i, int j, int k, int l, double* out) {
  return orc_eri_quartet_att(h, i, j, k, l, 0.0, out);
}

// The same with the erf(mu r)/r operator (mu <= 0: regular 1/r).
int orc_eri_quartet_att(void* h, int i, int j, int k, int l, double mu, double* out) {
  const Basis& B = ((OrcHandle*)h)->B;
  const double cut = ((OrcHandle*)h)->cutoff;
  const Cutoffs cutoffs =
      Cutoffs::make(cut, 1e-2 * cut, 1e-4 * cut, 25.0 * std::log(10.0), mu > 0 ? 1.0 / (mu * mu) : 0.0);
  PairStore PS;
  PS.build(B, cutoffs);
  const int ids[4] = {i, j, k, l};
  int s[4], fl[4];
  flip_quartet(B, ids, s, fl);
  QuartetWork W;
  std::vector<double> blk(10 * 10 * 10 * 10, 0.0);
  rys_quartet(B, PS, cutoffs, s, blk.data(), W);
  int n[4], nf[4];
  for (int t = 0; t < 4; ++t) { n[t] = B.sh[ids[t]].nao; nf[t] = B.sh[s[t]].nao; }
  // blk is in flipped order; position t of the flipped block holds ids[fl[t]]
  int inv[4];
  for (int t = 0; t < 4; ++t) inv[fl[t]] = t;
  int idx[4];
  for (idx[0] = 0; idx[0] < n[0]; ++idx[0])
    for (idx[1] = 0; idx[1] < n[1]; ++idx[1])
      for (idx[2] = 0; idx[2] < n[2]; ++idx[2])
        for (idx[3] = 0; idx[3] < n[3]; ++idx[3]) {
          int fi[4];
          for (int t = 0; t < 4; ++t) fi[inv[t]] = idx[t];
          out[((idx[0] * n[1] + idx[1]) * n[2] + idx[2]) * n[3] + idx[3]] =
              blk[((fi[0] * nf[1] + fi[1]) * nf[2] + fi[2]) * nf[3] + fi[3]];
        }
  return 0;
}

// Dense (nbf^4) ERI tensor through the same engine without any screening
// (tests of the J/K semantics on small systems).
int orc_eri_dense_att(void* h, double mu, double* eri);
int orc_eri_dense(void* h, double* eri) { return orc_eri_dense_att(h, 0.0, eri); }

// mu > 0: the erf(mu r)/r operator.
int orc_eri_dense_att(void* h, double mu, double* eri) {
  const Basis& B = ((OrcHandle*)h)->B;
  const int nb = B.nbf, ns = B.nshell;
  const Cutoffs cutoffs = Cutoffs::make(0.0, 0.0, 0.0, 1e300, mu > 0 ? 1.0 / (mu * mu) : 0.0);
  PairStore PS;
  PS.build(B, cutoffs);
  QuartetWork W;
  std::vector<double> blk(10 * 10 * 10 * 10, 0.0);
  for (int i = 0; i < ns; ++i)
    for (int j = 0; j < ns; ++j)
      for (int k = 0; k < ns; ++k)
        for (int l = 0; l < ns; ++l) {
          const int ids[4] = {i, j, k, l};
          int s[4], fl[4];
          flip_quartet(B, ids, s, fl);
          rys_quartet(B, PS, cutoffs, s, blk.data(), W);
          int nf[4], inv[4];
          for (int t = 0; t < 4; ++t) { nf[t] = B.sh[s[t]].nao; inv[fl[t]] = t; }
          const Shell* S[4] = {&B.sh[i], &B.sh[j], &B.sh[k], &B.sh[l]};
          int idx[4];
          for (idx[0] = 0; idx[0] < S[0]->nao; ++idx[0])
            for (idx[1] = 0; idx[1] < S[1]->nao; ++idx[1])
              for (idx[2] = 0; idx[2] < S[2]->nao; ++idx[2])
                for (idx[3] = 0; idx[3] < S[3]->nao; ++idx[3]) {
                  int fi[4];
                  for (int t = 0; t < 4; ++t) fi[inv[t]] = idx[t];
                  const size_t o = (((size_t)(S[0]->aoff + idx[0]) * nb + S[1]->aoff + idx[1]) * nb +
                                    S[2]->aoff + idx[2]) * nb + S[3]->aoff + idx[3];
                  eri[o] = blk[((fi[0] * nf[1] + fi[1]) * nf[2] + fi[2]) * nf[3] + fi[3]];
                }
        }
  return 0;
}

void orc_rys(int n, double X, double* x, double* w) { rys_eval(n, X, x, w); }
void orc_boys(int m, double T, double* F) { boys(m, T, F); }

}  // extern "C"
