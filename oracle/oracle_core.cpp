// Oracle (test infrastructure only): CPU restatement of OpenQP's direct
// two-electron Fock build, used by the tests, the smoke check and the CPU
// baseline leg of bench.py as the checker.  Never linked into the product.
//
// Restates, function by function (paths relative to the OpenQP checkout):
//   primitive pairs         source/integrals/int2_pairs.F90:74-266
//   cutoffs                 source/integrals/int2.F90:245-272, int2_pairs.F90:285-294
//   Schwarz bounds          source/integrals/int2.F90:1582-1737 (ints_exchange)
//   shell density           source/integrals/int2.F90:999-1047 (shlden)
//   quartet loop + screens  source/integrals/int2.F90:589-923, 963-986
//   cost-sorted pair list   source/integrals/int2.F90:864-921
//   element store           source/integrals/int2.F90:1741-1865 (storeints)
//   RHF / UROHF digestion   source/integrals/int2.F90:1414-1578
//   final scaling           source/scf_addons.F90:1177-1185, 1207-1210
//   ERI engine              Rys quadrature as in source/integrals/int_rys.F90:156-713
//                           (VRR on the first centre of each pair, HRR to the
//                           second), with the primitive screening of the
//                           rotated-axis engine that OpenQP runs for s-d
//                           quartets (source/integrals/int_rotaxis.F90:292-306,629)
//   normalisation / pure    source/integrals/int2.F90:1186-1208 (normalize_ints),
//                           source/constants.F90:33-60,110-140,
//                           source/integrals/int2_pure_generated.F90:119-149 (d and f)
// Rys nodes/weights come from our generated interpolation tables
// (openqp_gb300/csrc/rys_tables.inc), not from OpenQP's rys.F90 fits.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <omp.h>

#include "oracle_basis.h"
#include "../openqp_gb300/csrc/rys_tables.inc"

namespace orc {

const double PURE_D[5][6] = {
    {0, 0, 0, 1, 0, 0},                                  // xy
    {0, 0, 0, 0, 0, 1},                                  // yz
    {-0.5, -0.5, 1, 0, 0, 0},                            // 3z^2 - r^2
    {0, 0, 0, 0, 1, 0},                                  // xz
    {0.86602540378443865, -0.86602540378443865, 0, 0, 0, 0},  // x^2 - y^2
};

// Pure f (m = -3 .. 3) from the normalised Cartesians xxx yyy zzz xxy xxz xyy
// yyz xzz yzz xyz: the real solid harmonics, e.g. m = 0: z^3 - 3/(2 sqrt 5)
// (xxz + yyz) in normalised components.
const double PURE_F[7][10] = {
    {0, -0.79056941504209483, 0, 1.0606601717798213, 0, 0, 0, 0, 0, 0},   // y(3x^2 - y^2)
    {0, 0, 0, 0, 0, 0, 0, 0, 0, 1},                                         // xyz
    {0, -0.61237243569579452, 0, -0.27386127875258306, 0, 0, 0, 0, 1.0954451150103321, 0},  // y(4z^2 - r^2)
    {0, 0, 1, 0, -0.67082039324993691, 0, -0.67082039324993691, 0, 0, 0},  // z(2z^2 - 3r^2)
    {-0.61237243569579452, 0, 0, 0, 0, -0.27386127875258306, 0, 1.0954451150103321, 0, 0},  // x(4z^2 - r^2)
    {0, 0, 0, 0, 0.86602540378443865, 0, -0.86602540378443865, 0, 0, 0},  // z(x^2 - y^2)
    {0.79056941504209483, 0, 0, 0, 0, -1.0606601717798213, 0, 0, 0, 0},   // x(x^2 - 3y^2)
};

void cart_exps(int l, int idx, int* e) {
  static const int T[4][10][3] = {
      {{0, 0, 0}},
      {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}},
      {{2, 0, 0}, {0, 2, 0}, {0, 0, 2}, {1, 1, 0}, {1, 0, 1}, {0, 1, 1}},
      {{3, 0, 0}, {0, 3, 0}, {0, 0, 3}, {2, 1, 0}, {2, 0, 1}, {1, 2, 0}, {0, 2, 1}, {1, 0, 2}, {0, 1, 2},
       {1, 1, 1}}};
  e[0] = T[l][idx][0]; e[1] = T[l][idx][1]; e[2] = T[l][idx][2];
}

double cart_norm(int l, int idx) {
  if (l == 2 && idx >= 3) return 1.7320508075688772;
  if (l == 3 && idx >= 3) return idx == 9 ? 3.8729833462074170 : 2.2360679774997897;
  return 1.0;
}

void rys_eval(int n, double X, double* x, double* w) {
  if (X >= RYS_XMAX[n]) {
    const int o = n * (n - 1) / 2;
    const double rx = 1.0 / X, rs = 1.0 / std::sqrt(X);
    for (int i = 0; i < n; ++i) { x[i] = RYS_HERM_R2[o + i] * rx; w[i] = RYS_HERM_W[o + i] * rs; }
    return;
  }
  int k;
  double a, h;
  const int k0 = RYS_X_SPLIT * RYS_LO_PER_UNIT;
  if (X < RYS_X_SPLIT) { k = (int)(X * RYS_LO_PER_UNIT); h = 1.0 / RYS_LO_PER_UNIT; a = k * h; }
  else { k = k0 + (int)((X - RYS_X_SPLIT) / RYS_W_HI); a = RYS_X_SPLIT + (k - k0) * RYS_W_HI; h = RYS_W_HI; }
  const double s = 2.0 * (X - a) / h - 1.0;
  const double* t = RYS_TABLE + RYS_OFFSET[n - 1] + (size_t)k * 2 * n * RYS_NCOEF;
  for (int i = 0; i < n; ++i) {
    const double* cx = t + (2 * i) * RYS_NCOEF;
    const double* cw = t + (2 * i + 1) * RYS_NCOEF;
    double vx = cx[RYS_NCOEF - 1], vw = cw[RYS_NCOEF - 1];
    for (int c = RYS_NCOEF - 2; c >= 0; --c) { vx = vx * s + cx[c]; vw = vw * s + cw[c]; }
    x[i] = vx; w[i] = vw;
  }
}

void boys(int m, double T, double* F) {
  if (T < 30.0) {
    double s = 0, term = 1.0 / (2 * m + 1);
    for (int i = 1; i < 400; ++i) {
      s += term;
      term *= 2 * T / (2 * m + 2 * i + 1);
      if (term < 1e-18 * s) break;
    }
    const double e = std::exp(-T);
    F[m] = e * s;
    for (int k = m - 1; k >= 0; --k) F[k] = (2 * T * F[k + 1] + e) / (2 * k + 1);
  } else {
    const double e = std::exp(-T);
    F[0] = 0.5 * std::sqrt(PI / T) * std::erf(std::sqrt(T));
    for (int k = 0; k < m; ++k) F[k + 1] = ((2 * k + 1) * F[k] - e) / (2 * T);
  }
}

// int2_prepare_pair_storage + int2_prepare_pair (int2_pairs.F90:74-266)
void PairStore::build(const Basis& b, const Cutoffs& cut) {
  const int ns = b.nshell, np = ns * (ns + 1) / 2;
  cnt.assign(np, 0); off.assign(np, 0); sha.assign(np, 0); shb.assign(np, 0);
  aa.clear(); ab.clear(); g.clear(); ginv.clear(); k.clear(); px.clear(); py.clear(); pz.clear();
  const double sqrtpito52 = std::sqrt(2.0) * std::pow(PI, 1.25);
  for (int i = 0; i < ns; ++i) {
    for (int j = 0; j <= i; ++j) {
      const int id = pair_id(i, j);
      int s1 = i, s2 = j;
      if (b.sh[s1].am > b.sh[s2].am) std::swap(s1, s2);
      sha[id] = s1; shb[id] = s2;
      const Shell& A = b.sh[s1];
      const Shell& B = b.sh[s2];
      double ab2 = 0;
      for (int d = 0; d < 3; ++d) ab2 += (A.c[d] - B.c[d]) * (A.c[d] - B.c[d]);
      off[id] = (int)aa.size();
      for (int p1 = 0; p1 < A.nprim; ++p1) {
        for (int p2 = 0; p2 < B.nprim; ++p2) {
          const double a1 = b.ex[A.poff + p1], a2 = b.ex[B.poff + p2];
          const double gp = a1 + a2;
          double e12 = a1 * a2 * ab2;
          if (e12 > gp * cut.exponent) continue;
          const double gi = 1.0 / gp;
          e12 *= gi;
          const double k1 = b.cc[A.poff + p1] * b.cc[B.poff + p2] * std::exp(-e12);
          if (std::fabs(k1) < cut.quartet) continue;
          aa.push_back(a1); ab.push_back(a2); g.push_back(gp); ginv.push_back(gi);
          k.push_back(sqrtpito52 * k1);
          px.push_back((a1 * A.c[0] + a2 * B.c[0]) * gi);
          py.push_back((a1 * A.c[1] + a2 * B.c[1]) * gi);
          pz.push_back((a1 * A.c[2] + a2 * B.c[2]) * gi);
        }
      }
      cnt[id] = (int)aa.size() - off[id];
    }
  }
}

// ---------------------------------------------------------------------------
// Rys shell-quartet block.  s[] is already in the flipped order of
// gdat_set_ids (int_rys.F90:127-154): am0 <= am1, am2 <= am3, am0+am1 <= am2+am3.
// Output: normalised, pure-projected block out[a][b][c][d] (AO dims of the
// flipped shells).  Returns the number of primitive quartets evaluated.
static void project_index(double* blk, int dims[4], int pos, int l, int harm, double* tmp) {
  // normalise Cartesian components along index pos, then pure-project if needed
  int pre = 1, post = 1;
  for (int i = 0; i < pos; ++i) pre *= dims[i];
  for (int i = pos + 1; i < 4; ++i) post *= dims[i];
  const int n = dims[pos];
  for (int a = 0; a < pre; ++a)
    for (int c = 0; c < n; ++c) {
      const double f = cart_norm(l, c);
      if (f != 1.0)
        for (int p = 0; p < post; ++p) blk[(a * n + c) * post + p] *= f;
    }
  if (!harm || l < 2) return;
  const int nc = ncart(l), np = 2 * l + 1;
  for (int a = 0; a < pre; ++a)
    for (int m = 0; m < np; ++m)
      for (int p = 0; p < post; ++p) {
        double v = 0;
        for (int c = 0; c < nc; ++c) v += (l == 2 ? PURE_D[m][c] : PURE_F[m][c]) * blk[(a * nc + c) * post + p];
        tmp[(a * np + m) * post + p] = v;
      }
  dims[pos] = np;
  std::memcpy(blk, tmp, sizeof(double) * pre * np * post);
}

long rys_quartet(const Basis& B, const PairStore& PS, const Cutoffs& cut, const int s[4], double* out,
                 QuartetWork& W) {
  const Shell* S[4] = {&B.sh[s[0]], &B.sh[s[1]], &B.sh[s[2]], &B.sh[s[3]]};
  const int la = S[0]->am, lb = S[1]->am, lc = S[2]->am, ld = S[3]->am;
  const int na = ncart(la), nb = ncart(lb), nc = ncart(lc), nd = ncart(ld);
  const int nroots = (la + lb + lc + ld) / 2 + 1;
  const int nmax = la + lb, mmax = lc + ld;
  const int idP = pair_id(s[0], s[1]), idQ = pair_id(s[2], s[3]);
  const int nP = PS.cnt[idP], nQ = PS.cnt[idQ], oP = PS.off[idP], oQ = PS.off[idQ];
  const int nel = na * nb * nc * nd;
  std::fill(W.acc, W.acc + nel, 0.0);
  long nprimq = 0;
  const double AB[3] = {S[0]->c[0] - S[1]->c[0], S[0]->c[1] - S[1]->c[1], S[0]->c[2] - S[1]->c[2]};
  const double CD[3] = {S[2]->c[0] - S[3]->c[0], S[2]->c[1] - S[3]->c[1], S[2]->c[2] - S[3]->c[2]};
  int ea[10][3], eb[10][3], ec[10][3], ed[10][3];
  for (int i = 0; i < na; ++i) cart_exps(la, i, ea[i]);
  for (int i = 0; i < nb; ++i) cart_exps(lb, i, eb[i]);
  for (int i = 0; i < nc; ++i) cart_exps(lc, i, ec[i]);
  for (int i = 0; i < nd; ++i) cart_exps(ld, i, ed[i]);
  // 2D integrals I[root][dim][i][j][k][l], i<=la, j<=lb, k<=lc, l<=ld
  static thread_local double I2[7][3][4][4][4][4];
  double G[7][7];
  for (int q = 0; q < nQ; ++q) {
    const double sq = PS.k[oQ + q] * PS.ginv[oQ + q];
    if (std::fabs(sq) < cut.quartet) continue;
    const double qq = PS.g[oQ + q];
    const double Q[3] = {PS.px[oQ + q], PS.py[oQ + q], PS.pz[oQ + q]};
    const double QC[3] = {Q[0] - S[2]->c[0], Q[1] - S[2]->c[1], Q[2] - S[2]->c[2]};
    for (int p = 0; p < nP; ++p) {
      const double sp = PS.k[oP + p] * PS.ginv[oP + p];
      if (std::fabs(sp) < cut.quartet) continue;
      const double pp = PS.g[oP + p];
      const double fqz = sp * sq;
      const double x41 = pp + qq;
      if (fqz * fqz < cut.quartet2 * x41) continue;
      ++nprimq;
      // erf-attenuated: rho -> rho mu^2 / (mu^2 + rho), prefactor x sqrt(mu^2 / (mu^2 + rho))
      // (int_rotaxis.F90:634-638), i.e. p + q -> p + q + p q / mu^2 (int_rys.F90:225-227)
      const double inv = 1.0 / (cut.inv_mu2 != 0.0 ? x41 + pp * qq * cut.inv_mu2 : x41);
      const double rho = pp * qq * inv;
      const double P[3] = {PS.px[oP + p], PS.py[oP + p], PS.pz[oP + p]};
      const double PA[3] = {P[0] - S[0]->c[0], P[1] - S[0]->c[1], P[2] - S[0]->c[2]};
      const double PQ[3] = {P[0] - Q[0], P[1] - Q[1], P[2] - Q[2]};
      const double X = rho * (PQ[0] * PQ[0] + PQ[1] * PQ[1] + PQ[2] * PQ[2]);
      const double pref = fqz * std::sqrt(inv);
      double rx[7], rw[7];
      rys_eval(nroots, X, rx, rw);
      for (int r = 0; r < nroots; ++r) {
        const double u = rx[r];
        const double b00 = 0.5 * u * inv;
        const double b10 = 0.5 / pp * (1.0 - u * qq * inv);
        const double b01 = 0.5 / qq * (1.0 - u * pp * inv);
        for (int d = 0; d < 3; ++d) {
          const double c00 = PA[d] - u * qq * inv * PQ[d];
          const double d00 = QC[d] + u * pp * inv * PQ[d];
          // VRR (int_rys.F90:529-617 in structure)
          G[0][0] = (d == 2) ? rw[r] * pref : 1.0;
          if (nmax > 0) G[1][0] = c00 * G[0][0];
          for (int n = 1; n < nmax; ++n) G[n + 1][0] = c00 * G[n][0] + n * b10 * G[n - 1][0];
          for (int m = 0; m < mmax; ++m) {
            for (int n = 0; n <= nmax; ++n) {
              double v = d00 * G[n][m];
              if (m > 0) v += m * b01 * G[n][m - 1];
              if (n > 0) v += n * b00 * G[n - 1][m];
              G[n][m + 1] = v;
            }
          }
          // HRR bra then ket (int_rys.F90:619-661 in structure)
          double H[7][4][7];  // H[i][j][m]
          for (int m = 0; m <= mmax; ++m) {
            for (int i = 0; i <= nmax; ++i) H[i][0][m] = G[i][m];
            for (int j = 1; j <= lb; ++j)
              for (int i = 0; i <= nmax - j; ++i) H[i][j][m] = H[i + 1][j - 1][m] + AB[d] * H[i][j - 1][m];
          }
          for (int i = 0; i <= la; ++i)
            for (int j = 0; j <= lb; ++j) {
              double K2[7][4];
              for (int k = 0; k <= mmax; ++k) K2[k][0] = H[i][j][k];
              for (int l = 1; l <= ld; ++l)
                for (int k = 0; k <= mmax - l; ++k) K2[k][l] = K2[k + 1][l - 1] + CD[d] * K2[k][l - 1];
              for (int k = 0; k <= lc; ++k)
                for (int l = 0; l <= ld; ++l) I2[r][d][i][j][k][l] = K2[k][l];
            }
        }
      }
      int e = 0;
      for (int a = 0; a < na; ++a)
        for (int b = 0; b < nb; ++b)
          for (int c = 0; c < nc; ++c)
            for (int dd = 0; dd < nd; ++dd, ++e) {
              double v = 0;
              for (int r = 0; r < nroots; ++r)
                v += I2[r][0][ea[a][0]][eb[b][0]][ec[c][0]][ed[dd][0]] *
                     I2[r][1][ea[a][1]][eb[b][1]][ec[c][1]][ed[dd][1]] *
                     I2[r][2][ea[a][2]][eb[b][2]][ec[c][2]][ed[dd][2]];
              W.acc[e] += v;
            }
    }
  }
  int dims[4] = {na, nb, nc, nd};
  for (int pos = 0; pos < 4; ++pos) project_index(W.acc, dims, pos, S[pos]->am, S[pos]->harm, W.tmp);
  std::memcpy(out, W.acc, sizeof(double) * dims[0] * dims[1] * dims[2] * dims[3]);
  return nprimq;
}

// flips of gdat_set_ids (int_rys.F90:127-154)
void flip_quartet(const Basis& B, const int ids[4], int s[4], int fl[4]) {
  int am[4];
  for (int i = 0; i < 4; ++i) { fl[i] = i; am[i] = B.sh[ids[i]].am; }
  if (am[0] > am[1]) { std::swap(fl[0], fl[1]); std::swap(am[0], am[1]); }
  if (am[2] > am[3]) { std::swap(fl[2], fl[3]); std::swap(am[2], am[3]); }
  if (am[0] + am[1] > am[2] + am[3]) {
    std::swap(fl[0], fl[2]); std::swap(fl[1], fl[3]);
    std::swap(am[0], am[2]); std::swap(am[1], am[3]);
  }
  for (int i = 0; i < 4; ++i) s[i] = ids[fl[i]];
}

}  // namespace orc
