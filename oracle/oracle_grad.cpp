// Oracle (test infrastructure only): CPU restatement of OpenQP's analytic HF
// gradient pieces that the GPU gradient is checked against.  Never linked
// into the product.
//
//   orc_grad2e  two-electron part, restating grd2_driver_gen
//               (source/integrals/grd2.F90:145-391): Schwarz screen
//               Q_ij Q_kl < cutoff, two-particle density of get_density
//               (source/modules/hf_gradient.F90:427-575)
//                 G_ijkl = 4 cs D_ij D_kl - hf (D_ik D_jl + D_il D_jk [+ spin])
//               with its max as the density screen dabmax Q_ij Q_kl < cutoff/2,
//               the primitive screens of grd2_rys_compute
//               (source/integrals/grd2_rys.F90:303-420), the shell-identity
//               halving of apply_translation_invariance (grd2_rys.F90:1333-1346)
//               and the pair table cutoffs of grd2 (dabcut 1e-11, 10^-20,
//               20 ln 10).  Derivative integrals come from the Gaussian
//               derivative rule d/dA_x phi_a = 2 alpha phi_{a+1x} - a_x phi_{a-1x}
//               (grd2_rys.F90:848-868) applied to McMurchie-Davidson primitive
//               integrals of the raised / lowered shells, for all four centres
//               (no translational-invariance shortcut, so it also checks that).
//   orc_grad1e  one-electron part: sum D dH/dR - W dS/dR including the
//               Hellmann-Feynman term of the nuclear attraction (the
//               derivative with respect to each nucleus follows from
//               translational invariance of the three-centre integral).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <omp.h>
#include <vector>

#include "oracle_basis.h"

using namespace orc;

extern "C" void orc_schwarz(void* h, double* q, int nthreads);
extern "C" void orc_schwarz_att(void* h, double* q, int nthreads, double mu);

namespace {

// Cartesian components of l <= 4 in a fixed order; for l <= 3 it is OpenQP's
// order (source/constants.F90:33-60), l = 4 (raised f shells) is internal to
// this file.
struct CartList {
  int n[5];
  int e[5][15][3];
  CartList() {
    for (int l = 0; l <= 4; ++l) {
      int k = 0;
      if (l <= 3) {
        for (int c = 0; c < ncart(l); ++c) cart_exps(l, c, e[l][c]);
        k = ncart(l);
      } else {
        for (int x = l; x >= 0; --x)
          for (int y = l - x; y >= 0; --y) {
            e[l][k][0] = x; e[l][k][1] = y; e[l][k][2] = l - x - y;
            ++k;
          }
      }
      n[l] = k;
    }
  }
  int index(int l, const int* x) const {
    for (int c = 0; c < n[l]; ++c)
      if (e[l][c][0] == x[0] && e[l][c][1] == x[1] && e[l][c][2] == x[2]) return c;
    return -1;
  }
};
const CartList CL;

// 1D Hermite expansion coefficients E[i][j][t], i <= 4, j <= 6
struct Herm {
  double E[5][7][12];
  void build(int imax, int jmax, double p, double PA, double PB) {
    std::memset(E, 0, sizeof(E));
    E[0][0][0] = 1.0;
    const double o = 0.5 / p;
    for (int i = 0; i <= imax; ++i)
      for (int j = 0; j <= jmax; ++j) {
        if (i == 0 && j == 0) continue;
        for (int t = 0; t <= i + j; ++t) {
          double v;
          if (i > 0) {
            v = PA * E[i - 1][j][t] + (t + 1 < 12 ? (t + 1) * E[i - 1][j][t + 1] : 0.0);
            if (t > 0) v += o * E[i - 1][j][t - 1];
          } else {
            v = PB * E[i][j - 1][t] + (t + 1 < 12 ? (t + 1) * E[i][j - 1][t + 1] : 0.0);
            if (t > 0) v += o * E[i][j - 1][t - 1];
          }
          E[i][j][t] = v;
        }
      }
  }
};

// Hermite Coulomb integrals R_tuv(alpha, PC), t + u + v <= L <= 11
struct HermR {
  int L = 0;
  std::vector<double> R;
  double at(int t, int u, int v) const { return R[((size_t)t * (L + 1) + u) * (L + 1) + v]; }
  void build(int L_, double alpha, double X, double Y, double Z) {
    L = L_;
    const int n1 = L + 1;
    std::vector<double> F(L + 1);
    boys(L, alpha * (X * X + Y * Y + Z * Z), F.data());
    std::vector<double> Rn((size_t)n1 * n1 * n1 * n1, 0.0);
    auto A = [&](int n, int t, int u, int v) -> double& { return Rn[(((size_t)n * n1 + t) * n1 + u) * n1 + v]; };
    double f = 1.0;
    for (int n = 0; n <= L; ++n) { A(n, 0, 0, 0) = f * F[n]; f *= -2.0 * alpha; }
    for (int tot = 1; tot <= L; ++tot)
      for (int n = 0; n <= L - tot; ++n)
        for (int t = 0; t <= tot; ++t)
          for (int u = 0; u <= tot - t; ++u) {
            const int v = tot - t - u;
            double val;
            if (t > 0) {
              val = X * A(n + 1, t - 1, u, v);
              if (t > 1) val += (t - 1) * A(n + 1, t - 2, u, v);
            } else if (u > 0) {
              val = Y * A(n + 1, t, u - 1, v);
              if (u > 1) val += (u - 1) * A(n + 1, t, u - 2, v);
            } else {
              val = Z * A(n + 1, t, u, v - 1);
              if (v > 1) val += (v - 1) * A(n + 1, t, u, v - 2);
            }
            A(n, t, u, v) = val;
          }
    R.assign((size_t)n1 * n1 * n1, 0.0);
    for (int t = 0; t <= L; ++t)
      for (int u = 0; u <= L - t; ++u)
        for (int v = 0; v <= L - t - u; ++v) R[((size_t)t * n1 + u) * n1 + v] = A(0, t, u, v);
  }
};

// Primitive ERI block over unnormalised Cartesian components (l <= 4 each),
// out[((a*nb + b)*nc + c)*nd + d], without contraction coefficients.
// inv_mu2 > 0: the erf(mu r)/r operator (Hermite exponent alpha -> alpha mu^2 /
// (alpha + mu^2), prefactor x sqrt(mu^2 / (alpha + mu^2))).
void prim_eri(const int l[4], const double* C[4], const double ex[4], std::vector<double>& out,
              double inv_mu2 = 0.0) {
  const double a = ex[0], b = ex[1], c = ex[2], d = ex[3];
  const double p = a + b, q = c + d;
  double P[3], Q[3], ab2 = 0, cd2 = 0;
  for (int k = 0; k < 3; ++k) {
    P[k] = (a * C[0][k] + b * C[1][k]) / p;
    Q[k] = (c * C[2][k] + d * C[3][k]) / q;
    ab2 += (C[0][k] - C[1][k]) * (C[0][k] - C[1][k]);
    cd2 += (C[2][k] - C[3][k]) * (C[2][k] - C[3][k]);
  }
  Herm Eab[3], Ecd[3];
  for (int k = 0; k < 3; ++k) {
    Eab[k].build(l[0], l[1], p, P[k] - C[0][k], P[k] - C[1][k]);
    Ecd[k].build(l[2], l[3], q, Q[k] - C[2][k], Q[k] - C[3][k]);
  }
  HermR R;
  double alpha = p * q / (p + q), att = 1.0;
  if (inv_mu2 > 0.0) {
    att = 1.0 / (1.0 + alpha * inv_mu2);   // mu^2 / (alpha + mu^2)
    alpha *= att;
  }
  R.build(l[0] + l[1] + l[2] + l[3], alpha, P[0] - Q[0], P[1] - Q[1], P[2] - Q[2]);
  const double pref = 2.0 * std::pow(PI, 2.5) / (p * q * std::sqrt(p + q)) * std::sqrt(att) *
                      std::exp(-a * b / p * ab2) * std::exp(-c * d / q * cd2);
  const int n[4] = {CL.n[l[0]], CL.n[l[1]], CL.n[l[2]], CL.n[l[3]]};
  out.assign((size_t)n[0] * n[1] * n[2] * n[3], 0.0);
  size_t idx = 0;
  for (int ia = 0; ia < n[0]; ++ia)
    for (int ib = 0; ib < n[1]; ++ib)
      for (int ic = 0; ic < n[2]; ++ic)
        for (int id = 0; id < n[3]; ++id, ++idx) {
          const int* xa = CL.e[l[0]][ia];
          const int* xb = CL.e[l[1]][ib];
          const int* xc = CL.e[l[2]][ic];
          const int* xd = CL.e[l[3]][id];
          double v = 0;
          for (int t = 0; t <= xa[0] + xb[0]; ++t)
            for (int u = 0; u <= xa[1] + xb[1]; ++u)
              for (int w = 0; w <= xa[2] + xb[2]; ++w) {
                const double e1 = Eab[0].E[xa[0]][xb[0]][t] * Eab[1].E[xa[1]][xb[1]][u] * Eab[2].E[xa[2]][xb[2]][w];
                if (e1 == 0.0) continue;
                for (int tt = 0; tt <= xc[0] + xd[0]; ++tt)
                  for (int uu = 0; uu <= xc[1] + xd[1]; ++uu)
                    for (int ww = 0; ww <= xc[2] + xd[2]; ++ww) {
                      const double e2 =
                          Ecd[0].E[xc[0]][xd[0]][tt] * Ecd[1].E[xc[1]][xd[1]][uu] * Ecd[2].E[xc[2]][xd[2]][ww];
                      const double sgn = ((tt + uu + ww) & 1) ? -1.0 : 1.0;
                      v += e1 * sgn * e2 * R.at(t + tt, u + uu, w + ww);
                    }
              }
          out[idx] = pref * v;
        }
}

// Cartesian-effective density of one AO matrix: Dc = N T^T D T N per shell
// block (T = pure d / f projection for pure shells, N = Cartesian norms), in the
// Cartesian layout of the basis (offsets coff).
void cart_density(const Basis& B, const double* D, const std::vector<int>& coff, int ncart_tot,
                  std::vector<double>& Dc) {
  Dc.assign((size_t)ncart_tot * ncart_tot, 0.0);
  for (int si = 0; si < B.nshell; ++si)
    for (int sj = 0; sj < B.nshell; ++sj) {
      const Shell& A = B.sh[si];
      const Shell& C = B.sh[sj];
      const int na = ncart(A.am), nc = ncart(C.am);
      for (int x = 0; x < na; ++x)
        for (int y = 0; y < nc; ++y) {
          double v = 0;
          const bool pa = A.harm && A.am >= 2, pc = C.harm && C.am >= 2;
          const int ma = pa ? 2 * A.am + 1 : na, mc = pc ? 2 * C.am + 1 : nc;
          auto pure = [](int l, int m, int c) { return l == 2 ? PURE_D[m][c] : PURE_F[m][c]; };
          for (int p = 0; p < ma; ++p) {
            const double tp = pa ? pure(A.am, p, x) : (p == x ? 1.0 : 0.0);
            if (tp == 0.0) continue;
            for (int r = 0; r < mc; ++r) {
              const double tr = pc ? pure(C.am, r, y) : (r == y ? 1.0 : 0.0);
              if (tr == 0.0) continue;
              v += tp * tr * D[(size_t)(A.aoff + p) * B.nbf + C.aoff + r];
            }
          }
          Dc[(size_t)(coff[si] + x) * ncart_tot + coff[sj] + y] = v * cart_norm(A.am, x) * cart_norm(C.am, y);
        }
    }
}

}  // namespace

extern "C" {

// Two-electron gradient (accumulated into de[3*natom]).  Dt: total density,
// Ds: spin density (UHF/ROHF; null for RHF), both full nbf x nbf AO matrices.
// Two-particle density G = cj Dt_ij Dt_kl - ck (Dt_ik Dt_jl + Dt_il Dt_jk
// [+ Ds_ik Ds_jl + Ds_il Ds_jk]); OpenQP's HF values are cj = 4 coulscale,
// ck = hfscale.  stride > 1 evaluates only the bra pairs ij with
// ij % stride == offset (a bounded sample for timing).  Returns the number of
// shell quartets evaluated.
}  // extern "C"

namespace {

// Cartesian layout of the basis: offset of every shell, total count, pure flag.
struct CartLayout {
  std::vector<int> coff;
  int nct = 0;
  bool pure = false;
  explicit CartLayout(const Basis& B) : coff(B.nshell) {
    for (int s = 0; s < B.nshell; ++s) {
      coff[s] = nct;
      nct += ncart(B.sh[s].am);
      if (B.sh[s].harm && B.sh[s].am >= 2) pure = true;
    }
  }
};

// grd2_driver_gen over the canonical shell quartets with the two-particle
// density gamma_fn(ra, rb, rc, rd) of Cartesian-effective indices.
// inv_mu2 > 0: the erf-attenuated pass of grd2_driver's CAM branch
// (grd2.F90:117-128): attenuated Schwarz bounds (grd2.F90:247-248) and
// ab = p + q + pq / mu^2 in the primitive screens (grd2_rys.F90:368-373).
template <class GammaFn>
long long grad2e_impl(void* h, const CartLayout& CLy, GammaFn gamma_fn, double cutoff, int nthreads, int stride,
                      int offset, double* de, double inv_mu2 = 0.0) {
  const Basis& B = ((Handle*)h)->B;
  const int ns = B.nshell;
  // grd2 pair cutoffs (grd2.F90:238-260): dabcut, 10^-20, 10^-20, 20 ln 10
  double zbig = 0;
  for (double e : B.ex) zbig = std::max(zbig, e);
  double dabcut = 1e-11;
  if (zbig > 1e6) dabcut /= 10;
  if (zbig > 1e7) dabcut /= 10;
  const double dtol = 1e-20, rtol = std::log(10.0) * 20.0;
  const Cutoffs cut = Cutoffs::make(dabcut, dtol, dtol, rtol);
  PairStore PS;
  PS.build(B, cut);
  std::vector<double> Q((size_t)ns * ns);
  if (inv_mu2 > 0.0) orc_schwarz_att(h, Q.data(), nthreads, 1.0 / std::sqrt(inv_mu2));
  else orc_schwarz(h, Q.data(), nthreads);
  const std::vector<int>& coff = CLy.coff;
  const bool pure = CLy.pure;
  const double dtol2 = dtol * dtol;
  const double cutoff2 = cutoff / 2.0;
  long long numint = 0;
  const int natom = B.natom;
  std::vector<double> de_all((size_t)nthreads * 3 * natom, 0.0);
#pragma omp parallel num_threads(nthreads) reduction(+ : numint)
  {
    double* my = de_all.data() + (size_t)omp_get_thread_num() * 3 * natom;
    std::vector<double> gam, blk, bp, bm;
#pragma omp for schedule(dynamic, 1)
    for (int i = 0; i < ns; ++i)
      for (int j = 0; j <= i; ++j) {
        const int ij = pair_id(i, j);
        if (PS.cnt[ij] == 0) continue;
        if (stride > 1 && ij % stride != offset) continue;
        for (int k = 0; k <= i; ++k)
          for (int l = 0; l <= (k == i ? j : k); ++l) {
            const int kl = pair_id(k, l);
            if (PS.cnt[kl] == 0) continue;
            const double gmax = Q[(size_t)i * ns + j] * Q[(size_t)k * ns + l];
            if (gmax < cutoff) continue;
            const int at[4] = {B.sh[i].atom, B.sh[j].atom, B.sh[k].atom, B.sh[l].atom};
            if (at[0] == at[1] && at[0] == at[2] && at[0] == at[3]) continue;  // invariance: no contribution
            const Shell* S[4] = {&B.sh[i], &B.sh[j], &B.sh[k], &B.sh[l]};
            int lv[4], n[4];
            for (int t = 0; t < 4; ++t) { lv[t] = S[t]->am; n[t] = ncart(lv[t]); }
            const size_t ne = (size_t)n[0] * n[1] * n[2] * n[3];
            // two-particle density over Cartesian components (with norms) and its screening max
            gam.assign(ne, 0.0);
            double dabmax = 0;
            size_t e = 0;
            for (int a = 0; a < n[0]; ++a)
              for (int b = 0; b < n[1]; ++b)
                for (int c = 0; c < n[2]; ++c)
                  for (int d = 0; d < n[3]; ++d, ++e) {
                    const size_t ra = coff[i] + a, rb = coff[j] + b, rc = coff[k] + c, rd = coff[l] + d;
                    const double g = gamma_fn(ra, rb, rc, rd);
                    gam[e] = g;
                    const double nrm = pure ? 1.0
                                            : cart_norm(lv[0], a) * cart_norm(lv[1], b) * cart_norm(lv[2], c) *
                                                  cart_norm(lv[3], d);
                    dabmax = std::max(dabmax, std::fabs(g / nrm));
                  }
            if (dabmax * gmax < cutoff2) continue;
            ++numint;
            double fd[4][3] = {{0}};
            // primitive quartets (grd2_rys.F90:361-372 screens; dtol and dabcut
            // enter squared, grd2.F90:301 and grd2_rys.F90:146)
            const int pij = PS.off[ij], pkl = PS.off[kl];
            for (int u = 0; u < PS.cnt[kl]; ++u)
              for (int v = 0; v < PS.cnt[ij]; ++v) {
                const double da = PS.k[pij + v] * PS.ginv[pij + v], db = PS.k[pkl + u] * PS.ginv[pkl + u];
                const double aa = PS.g[pij + v], bb = PS.g[pkl + u];
                const double pfac = da * db, test = pfac * pfac, s = aa + bb + aa * bb * inv_mu2;
                if (test < dtol2 * s) continue;
                if (test * dabmax * dabmax < dabcut * dabcut * s) continue;  // gdat_init squares dabcut
                // exponents of the four primitives, per caller shell (the pair store
                // orients each pair with am(sha) <= am(shb))
                double xe[4];
                const bool fij = PS.sha[ij] == i, fkl = PS.sha[kl] == k;
                xe[0] = fij ? PS.aa[pij + v] : PS.ab[pij + v];
                xe[1] = fij ? PS.ab[pij + v] : PS.aa[pij + v];
                xe[2] = fkl ? PS.aa[pkl + u] : PS.ab[pkl + u];
                xe[3] = fkl ? PS.ab[pkl + u] : PS.aa[pkl + u];
                // contraction coefficients of those primitives
                auto coef = [&](const Shell* sh, double x) {
                  for (int q = 0; q < sh->nprim; ++q)
                    if (B.ex[sh->poff + q] == x) return B.cc[sh->poff + q];
                  return 0.0;
                };
                const double cc4 = coef(S[0], xe[0]) * coef(S[1], xe[1]) * coef(S[2], xe[2]) * coef(S[3], xe[3]);
                const double* Cn[4] = {S[0]->c, S[1]->c, S[2]->c, S[3]->c};
                for (int ctr = 0; ctr < 4; ++ctr) {
                  int lp[4] = {lv[0], lv[1], lv[2], lv[3]}, lm[4] = {lv[0], lv[1], lv[2], lv[3]};
                  lp[ctr] += 1;
                  lm[ctr] -= 1;
                  prim_eri(lp, Cn, xe, bp, inv_mu2);
                  if (lm[ctr] >= 0) prim_eri(lm, Cn, xe, bm, inv_mu2);
                  int np[4] = {CL.n[lp[0]], CL.n[lp[1]], CL.n[lp[2]], CL.n[lp[3]]};
                  int nm[4] = {lm[0] >= 0 ? CL.n[lm[0]] : 0, lm[1] >= 0 ? CL.n[lm[1]] : 0,
                               lm[2] >= 0 ? CL.n[lm[2]] : 0, lm[3] >= 0 ? CL.n[lm[3]] : 0};
                  size_t ee = 0;
                  int cidx[4];
                  for (cidx[0] = 0; cidx[0] < n[0]; ++cidx[0])
                    for (cidx[1] = 0; cidx[1] < n[1]; ++cidx[1])
                      for (cidx[2] = 0; cidx[2] < n[2]; ++cidx[2])
                        for (cidx[3] = 0; cidx[3] < n[3]; ++cidx[3], ++ee) {
                          if (gam[ee] == 0.0) continue;
                          for (int x = 0; x < 3; ++x) {
                            int ep[4], em[4];
                            for (int t = 0; t < 4; ++t) { ep[t] = cidx[t]; em[t] = cidx[t]; }
                            int xp[3], xm[3];
                            const int* x0 = CL.e[lv[ctr]][cidx[ctr]];
                            for (int d = 0; d < 3; ++d) { xp[d] = x0[d]; xm[d] = x0[d]; }
                            xp[x] += 1;
                            ep[ctr] = CL.index(lp[ctr], xp);
                            double val = 2.0 * xe[ctr] *
                                         bp[((size_t)(ep[0] * np[1] + ep[1]) * np[2] + ep[2]) * np[3] + ep[3]];
                            if (x0[x] > 0) {
                              xm[x] -= 1;
                              em[ctr] = CL.index(lm[ctr], xm);
                              val -= x0[x] * bm[((size_t)(em[0] * nm[1] + em[1]) * nm[2] + em[2]) * nm[3] + em[3]];
                            }
                            fd[ctr][x] += cc4 * gam[ee] * val;
                          }
                        }
                }
              }
            double f = 1.0;
            if (i == j) f *= 0.5;
            if (k == l) f *= 0.5;
            if (i == k && j == l) f *= 0.5;
            for (int t = 0; t < 4; ++t)
              for (int x = 0; x < 3; ++x) my[3 * at[t] + x] += f * fd[t][x];
          }
      }
  }
  for (int t = 0; t < nthreads; ++t)
    for (int x = 0; x < 3 * natom; ++x) de[x] += de_all[(size_t)t * 3 * natom + x];
  return numint;
}

// The MRSF two-particle density of grd2_mrsf_compute_data_t_get_density
// (modules/tdhf_mrsf_gradient.F90:404-601), literally, over the
// Cartesian-effective matrices M[0..10] = d2a, d2b, p2a, p2b (after the init
// sum / difference, :341-355), ball, bo2v, bo1v, bco1, bco2, o21v, co12.
struct MrsfGamma {
  const std::vector<double>* M;
  int n;
  double coulfact, xcfact, xcfact2, q1, q2, q3, sgnk;
  double operator()(size_t i1, size_t j1, size_t k1, size_t l1) const {
    auto E = [&](int m, size_t r, size_t c) { return M[m][r * n + c]; };
    auto d2a = [&](size_t r, size_t c) { return E(0, r, c); };
    auto d2b = [&](size_t r, size_t c) { return E(1, r, c); };
    auto p2a = [&](size_t r, size_t c) { return E(2, r, c); };
    auto p2b = [&](size_t r, size_t c) { return E(3, r, c); };
    auto ball = [&](size_t r, size_t c) { return E(4, r, c); };
    auto bo2v = [&](size_t r, size_t c) { return E(5, r, c); };
    auto bo1v = [&](size_t r, size_t c) { return E(6, r, c); };
    auto bco1 = [&](size_t r, size_t c) { return E(7, r, c); };
    auto bco2 = [&](size_t r, size_t c) { return E(8, r, c); };
    auto o21v = [&](size_t r, size_t c) { return E(9, r, c); };
    auto co12 = [&](size_t r, size_t c) { return E(10, r, c); };
    double df1 = (d2a(i1, j1) + p2a(i1, j1)) * d2a(k1, l1) + d2a(i1, j1) * p2a(k1, l1);
    df1 = df1 * coulfact;
    if (xcfact != 0.0 || xcfact2 != 0.0) {
      const double dq1 = (d2a(i1, k1) + p2a(i1, k1)) * d2a(j1, l1) + d2a(i1, k1) * p2a(j1, l1) +
                         (d2a(i1, l1) + p2a(i1, l1)) * d2a(j1, k1) + d2a(i1, l1) * p2a(j1, k1) +
                         (d2b(i1, k1) + p2b(i1, k1)) * d2b(j1, l1) + d2b(i1, k1) * p2b(j1, l1) +
                         (d2b(i1, l1) + p2b(i1, l1)) * d2b(j1, k1) + d2b(i1, l1) * p2b(j1, k1);
      const double dt2 = ball(i1, k1) * ball(j1, l1) + ball(k1, i1) * ball(l1, j1) + ball(i1, l1) * ball(j1, k1) +
                         ball(l1, i1) * ball(k1, j1);
      df1 = df1 - xcfact * dq1 - xcfact2 * 2.0 * dt2;
    }
    auto eight = [&](auto X) {   // db1 / db2 pattern
      return X(i1, k1) * X(l1, j1) + X(i1, l1) * X(k1, j1) + X(j1, k1) * X(l1, i1) + X(j1, l1) * X(k1, i1) +
             X(l1, j1) * X(i1, k1) + X(k1, j1) * X(i1, l1) + X(l1, i1) * X(j1, k1) + X(k1, i1) * X(j1, l1);
    };
    if (q1 != 0.0) df1 = df1 + sgnk * q1 * eight(co12);
    if (q2 != 0.0) df1 = df1 + sgnk * q2 * eight(o21v);
    if (q3 != 0.0) {
      auto dc = [&](auto X, auto Y) {
        return X(i1, k1) * Y(j1, l1) + X(i1, l1) * Y(j1, k1) + X(j1, k1) * Y(i1, l1) + X(j1, l1) * Y(i1, k1) +
               X(l1, j1) * Y(k1, i1) + X(k1, j1) * Y(l1, i1) + X(l1, i1) * Y(k1, j1) + X(k1, i1) * Y(l1, j1);
      };
      auto dd = [&](auto X, auto Y) {
        return X(i1, j1) * Y(l1, k1) + X(i1, j1) * Y(k1, l1) + X(j1, i1) * Y(l1, k1) + X(j1, i1) * Y(k1, l1) +
               X(l1, k1) * Y(i1, j1) + X(k1, l1) * Y(i1, j1) + X(l1, k1) * Y(j1, i1) + X(k1, l1) * Y(j1, i1);
      };
      const double dc1 = dc(bco1, bo2v), dc2 = dc(bco2, bo1v), dc3 = dc(bo2v, bco1), dc4 = dc(bo1v, bco2);
      const double dd1 = dd(bco1, bo2v), dd2 = dd(bco2, bo1v), dd3 = dd(bo2v, bco1), dd4 = dd(bo1v, bco2);
      df1 = df1 + sgnk * q3 * (-dc1 - dc2 - dc3 - dc4 + dd1 + dd2 + dd3 + dd4);
    }
    return df1;
  }
};

}  // namespace

extern "C" {

long long orc_grad2e(void* h, const double* Dt, const double* Ds, double cj, double ck, double cutoff, int nthreads,
                     int stride, int offset, double* de) {
  const Basis& B = ((Handle*)h)->B;
  const CartLayout CLy(B);
  const int nct = CLy.nct;
  std::vector<double> Dtc, Dsc;
  cart_density(B, Dt, CLy.coff, nct, Dtc);
  if (Ds) cart_density(B, Ds, CLy.coff, nct, Dsc);
  const bool spin = Ds != nullptr;
  auto gam = [&](size_t ra, size_t rb, size_t rc, size_t rd) {
    auto M = [&](const std::vector<double>& X, size_t r, size_t s) { return X[r * nct + s]; };
    double g = cj * M(Dtc, ra, rb) * M(Dtc, rc, rd) -
               ck * (M(Dtc, ra, rc) * M(Dtc, rb, rd) + M(Dtc, ra, rd) * M(Dtc, rb, rc));
    if (spin) g -= ck * (M(Dsc, ra, rc) * M(Dsc, rb, rd) + M(Dsc, ra, rd) * M(Dsc, rb, rc));
    return g;
  };
  return grad2e_impl(h, CLy, gam, cutoff, nthreads, stride, offset, de);
}

// CAM form of orc_grad2e (grd2_driver, grd2.F90:104-128): pass 1 regular
// integrals with coulscale 1 and hfscale alpha, pass 2 erf(mu r)/r with
// coulscale 0 and hfscale beta, accumulated into de.
long long orc_grad2e_cam(void* h, const double* Dt, const double* Ds, double alpha, double beta, double mu,
                         double cutoff, int nthreads, double* de) {
  const Basis& B = ((Handle*)h)->B;
  const CartLayout CLy(B);
  const int nct = CLy.nct;
  std::vector<double> Dtc, Dsc;
  cart_density(B, Dt, CLy.coff, nct, Dtc);
  if (Ds) cart_density(B, Ds, CLy.coff, nct, Dsc);
  const bool spin = Ds != nullptr;
  long long nq = 0;
  for (int pass = 0; pass < 2; ++pass) {
    const double cj = pass ? 0.0 : 4.0, ck = pass ? beta : alpha;
    auto gam = [&](size_t ra, size_t rb, size_t rc, size_t rd) {
      auto M = [&](const std::vector<double>& X, size_t r, size_t s) { return X[r * nct + s]; };
      double g = cj * M(Dtc, ra, rb) * M(Dtc, rc, rd) -
                 ck * (M(Dtc, ra, rc) * M(Dtc, rb, rd) + M(Dtc, ra, rd) * M(Dtc, rb, rc));
      if (spin) g -= ck * (M(Dsc, ra, rc) * M(Dsc, rb, rd) + M(Dsc, ra, rd) * M(Dsc, rb, rc));
      return g;
    };
    nq += grad2e_impl(h, CLy, gam, cutoff, nthreads, 1, 0, de, pass ? 1.0 / (mu * mu) : 0.0);
  }
  return nq;
}

// MRSF two-electron gradient (accumulated into de[3*natom]): d, p (nbf, nbf, 2)
// the raw alpha / beta SCF and relaxed difference densities, spc (7, nbf, nbf)
// the response densities, all Fortran column-major (the routec_grad2_mrsf
// layout); spcscale = {spc_coco, spc_ovov, spc_coov}; mrst 1 or 3; stride /
// offset as in orc_grad2e.  cam5 (or null) = {reference alpha, reference beta,
// response alpha, response beta, mu}: the two passes of grd2_driver's CAM
// branch (the hfscale / hfscale2 / coulscale arguments are then unused).
long long orc_grad2e_mrsf(void* h, const double* d, const double* p, const double* spc, double hfscale,
                          double hfscale2, double coulscale, const double* spcscale, int mrst, double cutoff,
                          int nthreads, int stride, int offset, double* de, const double* cam5) {
  const Basis& B = ((Handle*)h)->B;
  const int n = B.nbf;
  const size_t n2 = (size_t)n * n;
  const CartLayout CLy(B);
  std::vector<double> raw(n2);
  std::vector<double> M[11];
  auto fort = [&](const double* F, size_t r, size_t c) { return F[r + n * c]; };
  auto make = [&](int m, auto elem) {
    for (int r = 0; r < n; ++r)
      for (int c = 0; c < n; ++c) raw[(size_t)r * n + c] = elem(r, c);
    cart_density(B, raw.data(), CLy.coff, CLy.nct, M[m]);
  };
  make(0, [&](int r, int c) { return fort(d, r, c) + fort(d + n2, r, c); });
  make(1, [&](int r, int c) { return fort(d, r, c) - fort(d + n2, r, c); });
  make(2, [&](int r, int c) { return fort(p, r, c) + fort(p + n2, r, c); });
  make(3, [&](int r, int c) { return fort(p, r, c) - fort(p + n2, r, c); });
  // spc(7, nbf, nbf): ball is component 7, then bo2v, bo1v, bco1, bco2, o21v, co12 = 1..6
  const int comp[7] = {6, 0, 1, 2, 3, 4, 5};
  for (int q = 0; q < 7; ++q)
    make(4 + q, [&](int r, int c) { return spc[comp[q] + 7 * ((size_t)r + (size_t)n * c)]; });
  MrsfGamma G{M, CLy.nct, 4.0 * coulscale, hfscale, hfscale2, spcscale[0], spcscale[1], spcscale[2],
              mrst == 3 ? -1.0 : 1.0};
  if (cam5) {   // grd2_driver's CAM branch: pass 1 with the alphas, pass 2 attenuated with the betas
    G.coulfact = 4.0;
    G.xcfact = cam5[0];
    G.xcfact2 = cam5[2];
    long long nq = grad2e_impl(h, CLy, G, cutoff, nthreads, stride, offset, de);
    G.coulfact = 0.0;
    G.xcfact = cam5[1];
    G.xcfact2 = cam5[3];
    return nq + grad2e_impl(h, CLy, G, cutoff, nthreads, stride, offset, de, 1.0 / (cam5[4] * cam5[4]));
  }
  return grad2e_impl(h, CLy, G, cutoff, nthreads, stride, offset, de);
}

// One-electron gradient (accumulated into de[3*natom]): sum_uv D_uv dH_uv/dR
// - W_uv dS_uv/dR with H = T + V (point charges zq at the atoms).  D, W: full
// nbf x nbf AO matrices (total density, energy-weighted density).
int orc_grad1e(void* h, const double* D, const double* W, const double* zq, double* de) {
  const Basis& B = ((Handle*)h)->B;
  const int nb = B.nbf;
  std::vector<double> Dc, Wc;
  std::vector<int> coff(B.nshell);
  int nct = 0;
  for (int s = 0; s < B.nshell; ++s) { coff[s] = nct; nct += ncart(B.sh[s].am); }
  cart_density(B, D, coff, nct, Dc);
  cart_density(B, W, coff, nct, Wc);
  (void)nb;
  for (int si = 0; si < B.nshell; ++si)
    for (int sj = 0; sj < B.nshell; ++sj) {
      const Shell& A = B.sh[si];
      const Shell& C = B.sh[sj];
      const int la = A.am, lb = C.am;
      for (int p1 = 0; p1 < A.nprim; ++p1)
        for (int p2 = 0; p2 < C.nprim; ++p2) {
          const double a = B.ex[A.poff + p1], b = B.ex[C.poff + p2], p = a + b;
          const double cab = B.cc[A.poff + p1] * B.cc[C.poff + p2];
          double P[3], ab2 = 0;
          for (int d = 0; d < 3; ++d) {
            P[d] = (a * A.c[d] + b * C.c[d]) / p;
            ab2 += (A.c[d] - C.c[d]) * (A.c[d] - C.c[d]);
          }
          const double K = cab * std::exp(-a * b / p * ab2);
          Herm E[3];
          for (int d = 0; d < 3; ++d) E[d].build(la + 1, lb + 3, p, P[d] - A.c[d], P[d] - C.c[d]);
          const double s1 = std::sqrt(PI / p);
          // 1D overlap / kinetic pieces for exponents i (bra) j (ket)
          auto S1 = [&](int d, int i, int j) { return E[d].E[i][j][0] * s1; };
          auto T1 = [&](int d, int i, int j) {
            double t = -2.0 * b * b * E[d].E[i][j + 2][0] + b * (2 * j + 1) * E[d].E[i][j][0];
            if (j >= 2) t -= 0.5 * j * (j - 1) * E[d].E[i][j - 2][0];
            return t * s1;
          };
          // S and T of bra exponents xa, ket exponents xb
          auto ST = [&](const int* xa, const int* xb, double& s, double& t) {
            const double sx = S1(0, xa[0], xb[0]), sy = S1(1, xa[1], xb[1]), sz = S1(2, xa[2], xb[2]);
            s = sx * sy * sz;
            t = T1(0, xa[0], xb[0]) * sy * sz + sx * T1(1, xa[1], xb[1]) * sz + sx * sy * T1(2, xa[2], xb[2]);
          };
          for (int ia = 0; ia < ncart(la); ++ia)
            for (int ib = 0; ib < ncart(lb); ++ib) {
              const double dw = Dc[(size_t)(coff[si] + ia) * nct + coff[sj] + ib];
              const double ww = Wc[(size_t)(coff[si] + ia) * nct + coff[sj] + ib];
              if (dw == 0.0 && ww == 0.0) continue;
              int xa[3], xb[3];
              cart_exps(la, ia, xa);
              cart_exps(lb, ib, xb);
              // derivative with respect to the bra centre A (the ket centre follows
              // from d/dB = -d/dA for these two-centre integrals)
              for (int x = 0; x < 3; ++x) {
                int xp[3] = {xa[0], xa[1], xa[2]}, xm[3] = {xa[0], xa[1], xa[2]};
                xp[x] += 1;
                double sp, tp, sm = 0, tm = 0;
                ST(xp, xb, sp, tp);
                if (xa[x] > 0) { xm[x] -= 1; ST(xm, xb, sm, tm); }
                const double dS = K * (2.0 * a * sp - xa[x] * sm);
                const double dT = K * (2.0 * a * tp - xa[x] * tm);
                const double g = dw * dT - ww * dS;
                de[3 * A.atom + x] += g;
                de[3 * C.atom + x] -= g;
              }
              // nuclear attraction: d/dA and d/dB of each nucleus term, the
              // nucleus gets -(d/dA + d/dB)
              for (int at = 0; at < B.natom; ++at) {
                if (zq[at] == 0.0) continue;
                HermR R;
                R.build(la + lb + 1, p, P[0] - B.xyz[3 * at], P[1] - B.xyz[3 * at + 1], P[2] - B.xyz[3 * at + 2]);
                const double pref = -zq[at] * 2.0 * PI / p * K;
                auto V1 = [&](const int* ya, const int* yb) {
                  double v = 0;
                  for (int t = 0; t <= ya[0] + yb[0]; ++t)
                    for (int u = 0; u <= ya[1] + yb[1]; ++u)
                      for (int w = 0; w <= ya[2] + yb[2]; ++w)
                        v += E[0].E[ya[0]][yb[0]][t] * E[1].E[ya[1]][yb[1]][u] * E[2].E[ya[2]][yb[2]][w] * R.at(t, u, w);
                  return pref * v;
                };
                for (int x = 0; x < 3; ++x) {
                  int ap[3] = {xa[0], xa[1], xa[2]}, am[3] = {xa[0], xa[1], xa[2]};
                  int bp[3] = {xb[0], xb[1], xb[2]}, bm[3] = {xb[0], xb[1], xb[2]};
                  ap[x] += 1;
                  bp[x] += 1;
                  double dA = 2.0 * a * V1(ap, xb), dB = 2.0 * b * V1(xa, bp);
                  if (xa[x] > 0) { am[x] -= 1; dA -= xa[x] * V1(am, xb); }
                  if (xb[x] > 0) { bm[x] -= 1; dB -= xb[x] * V1(xa, bm); }
                  de[3 * A.atom + x] += dw * dA;
                  de[3 * C.atom + x] += dw * dB;
                  de[3 * at + x] -= dw * (dA + dB);
                }
              }
            }
        }
    }
  return 0;
}

}  // extern "C"
