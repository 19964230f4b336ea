// One-electron integrals on the host (overlap, kinetic, nuclear attraction)
// for the SCF driver around the Fock build.  They are O(nbf^2 natom) set-up
// work per geometry, not part of the GPU hot path.
//
// McMurchie-Davidson Hermite expansion (J. Comput. Phys. 26, 218 (1978)):
// per Cartesian direction E^{ij}_t by the two-term recursions, overlaps from
// E^{ij}_0, kinetic energy from overlaps with the ket raised/lowered by two,
// and nuclear attraction V = -Z 2 pi / p sum_tuv E_t E_u E_v R_tuv(p, P - C)
// with the Hermite Coulomb integrals R from the Boys function (series below
// T = 30, erf and upward recursion above).  AO conventions match the Fock
// build: individually normalised Cartesians (xx yy zz xy xz yz) and pure d
// (xy, yz, z^2, xz, x^2-y^2).  Shell pairs are spread over host threads.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <thread>
#include <vector>

#include "../../include/openqp_gb300.h"

namespace {

constexpr double kPi = 3.14159265358979323846;

struct Sh {
  int l, n, off, harm, nao, aoff;
  double c[3];
};

int ncart1(int l) { return (l + 1) * (l + 2) / 2; }

// Cartesian exponents in OpenQP order (constants.F90:33-60): s; x y z;
// xx yy zz xy xz yz; xxx yyy zzz xxy xxz xyy yyz xzz yzz xyz.
void exps_of(int l, int idx, int* e) {
  static const int T[4][10][3] = {
      {{0, 0, 0}},
      {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}},
      {{2, 0, 0}, {0, 2, 0}, {0, 0, 2}, {1, 1, 0}, {1, 0, 1}, {0, 1, 1}},
      {{3, 0, 0}, {0, 3, 0}, {0, 0, 3}, {2, 1, 0}, {2, 0, 1}, {1, 2, 0}, {0, 2, 1}, {1, 0, 2}, {0, 1, 2}, {1, 1, 1}}};
  e[0] = T[l][idx][0]; e[1] = T[l][idx][1]; e[2] = T[l][idx][2];
}

// F_0..F_m(T)
void boys_f(int m, double T, double* F) {
  if (T < 30.0) {
    double s = 0, term = 1.0 / (2 * m + 1);
    for (int i = 1; i < 500; ++i) {
      s += term;
      term *= 2 * T / (2 * m + 2 * i + 1);
      if (term < 1e-18 * s) break;
    }
    const double e = std::exp(-T);
    F[m] = e * s;
    for (int k = m - 1; k >= 0; --k) F[k] = (2 * T * F[k + 1] + e) / (2 * k + 1);
  } else {
    const double e = std::exp(-T);
    F[0] = 0.5 * std::sqrt(kPi / T) * std::erf(std::sqrt(T));
    for (int k = 0; k < m; ++k) F[k + 1] = ((2 * k + 1) * F[k] - e) / (2 * T);
  }
}

// Hermite expansion coefficients E[i][j][t], i <= 3, j <= 5, t <= 8
struct Herm {
  double E[4][6][9];
  void build(int imax, int jmax, double p, double PA, double PB) {
    std::memset(E, 0, sizeof(E));
    E[0][0][0] = 1.0;
    const double o = 0.5 / p;
    for (int i = 0; i <= imax; ++i)
      for (int j = 0; j <= jmax; ++j) {
        if (i == 0 && j == 0) continue;
        for (int t = 0; t <= i + j; ++t) {
          const double(*src)[9] = (i > 0) ? E[i - 1] : E[i];
          const int jj = (i > 0) ? j : j - 1;
          const double X = (i > 0) ? PA : PB;
          double v = X * src[jj][t];
          if (t + 1 <= 8) v += (t + 1) * src[jj][t + 1];
          if (t > 0) v += o * src[jj][t - 1];
          E[i][j][t] = v;
        }
      }
  }
};

// Hermite Coulomb integrals R[t][u][v] for t+u+v <= L <= 6
void hermite_r(int L, double alpha, double X, double Y, double Z, double R[7][7][7]) {
  double F[9];
  boys_f(L, alpha * (X * X + Y * Y + Z * Z), F);
  double Rn[7][7][7][7];  // [n][t][u][v]
  double f = 1.0;
  for (int n = 0; n <= L; ++n) { Rn[n][0][0][0] = f * F[n]; f *= -2.0 * alpha; }
  for (int tot = 1; tot <= L; ++tot)
    for (int n = 0; n <= L - tot; ++n)
      for (int t = 0; t <= tot; ++t)
        for (int u = 0; u <= tot - t; ++u) {
          const int v = tot - t - u;
          double val;
          if (t > 0) {
            val = X * Rn[n + 1][t - 1][u][v];
            if (t > 1) val += (t - 1) * Rn[n + 1][t - 2][u][v];
          } else if (u > 0) {
            val = Y * Rn[n + 1][t][u - 1][v];
            if (u > 1) val += (u - 1) * Rn[n + 1][t][u - 2][v];
          } else {
            val = Z * Rn[n + 1][t][u][v - 1];
            if (v > 1) val += (v - 1) * Rn[n + 1][t][u][v - 2];
          }
          Rn[n][t][u][v] = val;
        }
  for (int t = 0; t <= L; ++t)
    for (int u = 0; u <= L - t; ++u)
      for (int v = 0; v <= L - t - u; ++v) R[t][u][v] = Rn[0][t][u][v];
}

// shells_pnrm2 (constants.F90:110-140)
double cnorm(int l, int idx) {
  if (l == 2 && idx >= 3) return 1.7320508075688772;
  if (l == 3 && idx >= 3) return idx == 9 ? 3.8729833462074170 : 2.2360679774997897;
  return 1.0;
}

// pure d and f (m = -l .. l) from normalised Cartesians (int2_pure_generated.F90:119-149)
const double* pure_row(int l, int m) {
  static const double D[5][10] = {{0, 0, 0, 1, 0, 0}, {0, 0, 0, 0, 0, 1}, {-0.5, -0.5, 1, 0, 0, 0},
                                  {0, 0, 0, 0, 1, 0}, {0.86602540378443865, -0.86602540378443865, 0, 0, 0, 0}};
  static const double F[7][10] = {
      {0, -0.79056941504209483, 0, 1.0606601717798213, 0, 0, 0, 0, 0, 0},
      {0, 0, 0, 0, 0, 0, 0, 0, 0, 1},
      {0, -0.61237243569579452, 0, -0.27386127875258306, 0, 0, 0, 0, 1.0954451150103321, 0},
      {0, 0, 1, 0, -0.67082039324993691, 0, -0.67082039324993691, 0, 0, 0},
      {-0.61237243569579452, 0, 0, 0, 0, -0.27386127875258306, 0, 1.0954451150103321, 0, 0},
      {0, 0, 0, 0, 0.86602540378443865, 0, -0.86602540378443865, 0, 0, 0},
      {0.79056941504209483, 0, 0, 0, 0, -1.0606601717798213, 0, 0, 0, 0}};
  return l == 2 ? D[m] : F[m];
}

// normalise and pure-project a (na x nb) Cartesian block in place; returns dims
void finish(double* blk, int la, int lb, int ha, int hb, int& da, int& db) {
  const int na = ncart1(la), nb = ncart1(lb);
  for (int i = 0; i < na; ++i)
    for (int j = 0; j < nb; ++j) blk[i * nb + j] *= cnorm(la, i) * cnorm(lb, j);
  double tmp[100];
  da = na; db = nb;
  if (ha && la >= 2) {
    const int np = 2 * la + 1;
    for (int m = 0; m < np; ++m)
      for (int j = 0; j < nb; ++j) {
        const double* T = pure_row(la, m);
        double v = 0;
        for (int c = 0; c < na; ++c) v += T[c] * blk[c * nb + j];
        tmp[m * nb + j] = v;
      }
    da = np;
    std::memcpy(blk, tmp, sizeof(double) * da * nb);
  }
  if (hb && lb >= 2) {
    const int np = 2 * lb + 1;
    for (int i = 0; i < da; ++i)
      for (int m = 0; m < np; ++m) {
        const double* T = pure_row(lb, m);
        double v = 0;
        for (int c = 0; c < nb; ++c) v += T[c] * blk[i * nb + c];
        tmp[i * np + m] = v;
      }
    db = np;
    std::memcpy(blk, tmp, sizeof(double) * da * db);
  }
}

}  // namespace

extern "C" int oqpg_one_electron(int nshell, const int* am, const int* ncontr, const int* origin, const double* ex,
                                 const double* cc, const int* harmonic, int natom, const double* xyz,
                                 const double* charges, int which, double* out) {
  if (nshell <= 0 || which < 0 || which > 2 || !out) return 3;
  std::vector<Sh> sh(nshell);
  int off = 0, aoff = 0;
  for (int s = 0; s < nshell; ++s) {
    if (am[s] < 0 || am[s] > 3 || origin[s] < 1 || origin[s] > natom) return 3;
    Sh& S = sh[s];
    S.l = am[s]; S.n = ncontr[s]; S.off = off; S.harm = harmonic ? harmonic[s] : 0;
    S.nao = (S.harm && S.l >= 2) ? 2 * S.l + 1 : ncart1(S.l);
    S.aoff = aoff;
    for (int d = 0; d < 3; ++d) S.c[d] = xyz[3 * (origin[s] - 1) + d];
    off += S.n; aoff += S.nao;
  }
  const int nb = aoff;
  std::memset(out, 0, sizeof(double) * nb * nb);
  auto pair_block = [&](int si, int sj) {
    const Sh& A = sh[si];
    const Sh& B = sh[sj];
    const int na = ncart1(A.l), nbb = ncart1(B.l);
    int ea[10][3], eb[10][3];
    for (int i = 0; i < na; ++i) exps_of(A.l, i, ea[i]);
    for (int i = 0; i < nbb; ++i) exps_of(B.l, i, eb[i]);
    double blk[100] = {0};
    double ab2 = 0;
    for (int d = 0; d < 3; ++d) ab2 += (A.c[d] - B.c[d]) * (A.c[d] - B.c[d]);
    for (int p1 = 0; p1 < A.n; ++p1)
      for (int p2 = 0; p2 < B.n; ++p2) {
        const double a = ex[A.off + p1], b = ex[B.off + p2], p = a + b;
        const double K = cc[A.off + p1] * cc[B.off + p2] * std::exp(-a * b / p * ab2);
        double P[3];
        for (int d = 0; d < 3; ++d) P[d] = (a * A.c[d] + b * B.c[d]) / p;
        Herm E[3];
        for (int d = 0; d < 3; ++d) E[d].build(A.l, B.l + 2, p, P[d] - A.c[d], P[d] - B.c[d]);
        const double s1 = std::sqrt(kPi / p);
        if (which < 2) {
          for (int i = 0; i < na; ++i)
            for (int j = 0; j < nbb; ++j) {
              double S1[3], T1[3];
              for (int d = 0; d < 3; ++d) {
                const int x = ea[i][d], y = eb[j][d];
                S1[d] = E[d].E[x][y][0] * s1;
                double t = -2.0 * b * b * E[d].E[x][y + 2][0] + b * (2 * y + 1) * E[d].E[x][y][0];
                if (y >= 2) t -= 0.5 * y * (y - 1) * E[d].E[x][y - 2][0];
                T1[d] = t * s1;
              }
              const double v = (which == 0) ? S1[0] * S1[1] * S1[2]
                                            : T1[0] * S1[1] * S1[2] + S1[0] * T1[1] * S1[2] + S1[0] * S1[1] * T1[2];
              blk[i * nbb + j] += K * v;
            }
        } else {
          for (int at = 0; at < natom; ++at) {
            const double Z = charges[at];
            if (Z == 0.0) continue;
            double R[7][7][7];
            hermite_r(A.l + B.l, p, P[0] - xyz[3 * at], P[1] - xyz[3 * at + 1], P[2] - xyz[3 * at + 2], R);
            const double pref = -Z * 2.0 * kPi / p * K;
            for (int i = 0; i < na; ++i)
              for (int j = 0; j < nbb; ++j) {
                double v = 0;
                for (int t = 0; t <= ea[i][0] + eb[j][0]; ++t)
                  for (int u = 0; u <= ea[i][1] + eb[j][1]; ++u)
                    for (int w = 0; w <= ea[i][2] + eb[j][2]; ++w)
                      v += E[0].E[ea[i][0]][eb[j][0]][t] * E[1].E[ea[i][1]][eb[j][1]][u] *
                           E[2].E[ea[i][2]][eb[j][2]][w] * R[t][u][w];
                blk[i * nbb + j] += pref * v;
              }
          }
        }
      }
    int da, db;
    finish(blk, A.l, B.l, A.harm, B.harm, da, db);
    for (int i = 0; i < da; ++i)
      for (int j = 0; j < db; ++j) {
        out[(size_t)(A.aoff + i) * nb + B.aoff + j] = blk[i * db + j];
        out[(size_t)(B.aoff + j) * nb + A.aoff + i] = blk[i * db + j];
      }
  };
  unsigned nt = std::max(1u, std::min(64u, std::thread::hardware_concurrency()));
  std::vector<std::thread> pool;
  for (unsigned t = 0; t < nt; ++t)
    pool.emplace_back([&, t]() {
      for (int si = (int)t; si < nshell; si += (int)nt)
        for (int sj = 0; sj <= si; ++sj) pair_block(si, sj);
    });
  for (auto& th : pool) th.join();
  return 0;
}
