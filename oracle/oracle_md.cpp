// Oracle (test infrastructure only): an independent McMurchie-Davidson
// integral code (Hermite expansion + Boys function, McMurchie & Davidson,
// J. Comput. Phys. 26, 218 (1978)).  It shares nothing with the Rys engine
// except the basis data model, so it cross-checks the Rys ERIs, and it
// provides the one-electron integrals (S, T, V) that the golden-energy pins
// need (OpenQP: source/integrals/int1.F90).
#include <cstring>
#include <vector>

#include "oracle_basis.h"

using namespace orc;

using OrcHandleView = orc::Handle;

namespace {

// 1D Hermite coefficients E[i][j][t] for i<=imax, j<=jmax (pair prefactor excluded)
struct Herm1D {
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

// Hermite Coulomb integrals R_{tuv}(alpha, PC), t+u+v <= L
struct HermR {
  int L;
  std::vector<double> R;  // R[t][u][v] with stride (L+1)
  double& at(int t, int u, int v) { return R[((size_t)t * (L + 1) + u) * (L + 1) + v]; }
  void build(int L_, double alpha, double X, double Y, double Z) {
    L = L_;
    const int n1 = L + 1;
    std::vector<double> F(L + 1);
    boys(L, alpha * (X * X + Y * Y + Z * Z), F.data());
    // Rn[n][t][u][v]
    std::vector<double> Rn((size_t)n1 * n1 * n1 * n1, 0.0);
    auto A = [&](int n, int t, int u, int v) -> double& {
      return Rn[(((size_t)n * n1 + t) * n1 + u) * n1 + v];
    };
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
        for (int v = 0; v <= L - t - u; ++v) at(t, u, v) = A(0, t, u, v);
  }
};

// normalise + pure-project a block along every index (dims updated)
void finish_block(const Basis& B, const int* sh, int nidx, std::vector<double>& blk, int* dims) {
  for (int pos = 0; pos < nidx; ++pos) {
    int pre = 1, post = 1;
    for (int i = 0; i < pos; ++i) pre *= dims[i];
    for (int i = pos + 1; i < nidx; ++i) post *= dims[i];
    const int l = B.sh[sh[pos]].am, n = dims[pos];
    for (int a = 0; a < pre; ++a)
      for (int c = 0; c < n; ++c)
        for (int p = 0; p < post; ++p) blk[((size_t)a * n + c) * post + p] *= cart_norm(l, c);
    if (B.sh[sh[pos]].harm && l >= 2) {
      const int nc = ncart(l), np = 2 * l + 1;
      std::vector<double> t((size_t)pre * np * post);
      for (int a = 0; a < pre; ++a)
        for (int m = 0; m < np; ++m)
          for (int p = 0; p < post; ++p) {
            double v = 0;
            for (int c = 0; c < nc; ++c)
              v += (l == 2 ? PURE_D[m][c] : PURE_F[m][c]) * blk[((size_t)a * nc + c) * post + p];
            t[((size_t)a * np + m) * post + p] = v;
          }
      dims[pos] = np;
      blk.swap(t);
    }
  }
}

}  // namespace

extern "C" {

// Cartesian-normalised (pure-projected) ERI block in the caller's order, by
// McMurchie-Davidson, no screening.
int orc_md_quartet_att(void* h, int i, int j, int k, int l, double mu, double* out);
int orc_md_quartet(void* h, int i, int j, int k, int l, double* out) {
  return orc_md_quartet_att(h, i, j, k, l, 0.0, out);
}

// erf(mu r)/r (mu > 0): the operator's Fourier transform 4 pi k^-2 exp(-k^2 / 4 mu^2)
// turns the Hermite Coulomb exponent alpha = pq/(p+q) into alpha mu^2 / (alpha + mu^2)
// and scales the prefactor by sqrt(mu^2 / (alpha + mu^2)).
int orc_md_quartet_att(void* h, int i, int j, int k, int l, double mu, double* out) {
  const Basis& B = ((OrcHandleView*)h)->B;
  const int sh[4] = {i, j, k, l};
  const Shell* S[4] = {&B.sh[i], &B.sh[j], &B.sh[k], &B.sh[l]};
  int n[4], e[4][10][3];
  for (int t = 0; t < 4; ++t) {
    n[t] = ncart(S[t]->am);
    for (int c = 0; c < n[t]; ++c) cart_exps(S[t]->am, c, e[t][c]);
  }
  const int ntot = n[0] * n[1] * n[2] * n[3];
  std::vector<double> blk(ntot, 0.0);
  const int Lab = S[0]->am + S[1]->am, Lcd = S[2]->am + S[3]->am;
  for (int pa = 0; pa < S[0]->nprim; ++pa)
    for (int pb = 0; pb < S[1]->nprim; ++pb) {
      const double a = B.ex[S[0]->poff + pa], b = B.ex[S[1]->poff + pb];
      const double p = a + b;
      double P[3], ab2 = 0;
      for (int d = 0; d < 3; ++d) {
        P[d] = (a * S[0]->c[d] + b * S[1]->c[d]) / p;
        ab2 += (S[0]->c[d] - S[1]->c[d]) * (S[0]->c[d] - S[1]->c[d]);
      }
      const double Kab = B.cc[S[0]->poff + pa] * B.cc[S[1]->poff + pb] * std::exp(-a * b / p * ab2);
      Herm1D Eab[3];
      for (int d = 0; d < 3; ++d) Eab[d].build(S[0]->am, S[1]->am, p, P[d] - S[0]->c[d], P[d] - S[1]->c[d]);
      for (int pc = 0; pc < S[2]->nprim; ++pc)
        for (int pd = 0; pd < S[3]->nprim; ++pd) {
          const double c = B.ex[S[2]->poff + pc], dd = B.ex[S[3]->poff + pd];
          const double q = c + dd;
          double Q[3], cd2 = 0;
          for (int d = 0; d < 3; ++d) {
            Q[d] = (c * S[2]->c[d] + dd * S[3]->c[d]) / q;
            cd2 += (S[2]->c[d] - S[3]->c[d]) * (S[2]->c[d] - S[3]->c[d]);
          }
          const double Kcd = B.cc[S[2]->poff + pc] * B.cc[S[3]->poff + pd] * std::exp(-c * dd / q * cd2);
          Herm1D Ecd[3];
          for (int d = 0; d < 3; ++d) Ecd[d].build(S[2]->am, S[3]->am, q, Q[d] - S[2]->c[d], Q[d] - S[3]->c[d]);
          double alpha = p * q / (p + q);
          double att = 1.0;
          if (mu > 0) {
            att = mu * mu / (alpha + mu * mu);
            alpha *= att;
          }
          HermR R;
          R.build(Lab + Lcd, alpha, P[0] - Q[0], P[1] - Q[1], P[2] - Q[2]);
          const double pref = 2.0 * std::pow(PI, 2.5) / (p * q * std::sqrt(p + q)) * std::sqrt(att) * Kab * Kcd;
          int idx = 0;
          for (int ia = 0; ia < n[0]; ++ia)
            for (int ib = 0; ib < n[1]; ++ib)
              for (int ic = 0; ic < n[2]; ++ic)
                for (int id = 0; id < n[3]; ++id, ++idx) {
                  const int* xa = e[0][ia]; const int* xb = e[1][ib];
                  const int* xc = e[2][ic]; const int* xd = e[3][id];
                  double v = 0;
                  for (int t = 0; t <= xa[0] + xb[0]; ++t)
                    for (int u = 0; u <= xa[1] + xb[1]; ++u)
                      for (int w = 0; w <= xa[2] + xb[2]; ++w) {
                        const double e1 = Eab[0].E[xa[0]][xb[0]][t] * Eab[1].E[xa[1]][xb[1]][u] *
                                          Eab[2].E[xa[2]][xb[2]][w];
                        if (e1 == 0.0) continue;
                        for (int tt = 0; tt <= xc[0] + xd[0]; ++tt)
                          for (int uu = 0; uu <= xc[1] + xd[1]; ++uu)
                            for (int ww = 0; ww <= xc[2] + xd[2]; ++ww) {
                              const double e2 = Ecd[0].E[xc[0]][xd[0]][tt] * Ecd[1].E[xc[1]][xd[1]][uu] *
                                                Ecd[2].E[xc[2]][xd[2]][ww];
                              const double sgn = ((tt + uu + ww) & 1) ? -1.0 : 1.0;
                              v += e1 * sgn * e2 * R.at(t + tt, u + uu, w + ww);
                            }
                      }
                  blk[idx] += pref * v;
                }
        }
    }
  int dims[4] = {n[0], n[1], n[2], n[3]};
  finish_block(B, sh, 4, blk, dims);
  std::memcpy(out, blk.data(), sizeof(double) * blk.size());
  return 0;
}

// One-electron matrices (nbf x nbf, AO basis incl. pure d): which = 0 overlap,
// 1 kinetic, 2 nuclear attraction with point charges zq[natom] at the atoms.
int orc_one_electron(void* h, int which, const double* zq, double* M) {
  const Basis& B = ((OrcHandleView*)h)->B;
  const int nb = B.nbf;
  std::memset(M, 0, sizeof(double) * nb * nb);
  for (int si = 0; si < B.nshell; ++si)
    for (int sj = 0; sj < B.nshell; ++sj) {
      const Shell& A = B.sh[si];
      const Shell& C = B.sh[sj];
      const int na = ncart(A.am), nc = ncart(C.am);
      int ea[10][3], ec[10][3];
      for (int c = 0; c < na; ++c) cart_exps(A.am, c, ea[c]);
      for (int c = 0; c < nc; ++c) cart_exps(C.am, c, ec[c]);
      std::vector<double> blk((size_t)na * nc, 0.0);
      for (int p1 = 0; p1 < A.nprim; ++p1)
        for (int p2 = 0; p2 < C.nprim; ++p2) {
          const double a = B.ex[A.poff + p1], b = B.ex[C.poff + p2];
          const double p = a + b;
          double P[3], ab2 = 0;
          for (int d = 0; d < 3; ++d) {
            P[d] = (a * A.c[d] + b * C.c[d]) / p;
            ab2 += (A.c[d] - C.c[d]) * (A.c[d] - C.c[d]);
          }
          const double K = B.cc[A.poff + p1] * B.cc[C.poff + p2] * std::exp(-a * b / p * ab2);
          Herm1D E[3];
          for (int d = 0; d < 3; ++d) E[d].build(A.am, C.am + 2, p, P[d] - A.c[d], P[d] - C.c[d]);
          const double s1 = std::sqrt(PI / p);
          if (which == 0 || which == 1) {
            for (int ia = 0; ia < na; ++ia)
              for (int ic = 0; ic < nc; ++ic) {
                double S1[3], T1[3];
                for (int d = 0; d < 3; ++d) {
                  const int i = ea[ia][d], j = ec[ic][d];
                  S1[d] = E[d].E[i][j][0] * s1;
                  double t = -2.0 * b * b * E[d].E[i][j + 2][0] + b * (2 * j + 1) * E[d].E[i][j][0];
                  if (j >= 2) t -= 0.5 * j * (j - 1) * E[d].E[i][j - 2][0];
                  T1[d] = t * s1;
                }
                double v;
                if (which == 0) v = S1[0] * S1[1] * S1[2];
                else v = T1[0] * S1[1] * S1[2] + S1[0] * T1[1] * S1[2] + S1[0] * S1[1] * T1[2];
                blk[(size_t)ia * nc + ic] += K * v;
              }
          } else {
            for (int at = 0; at < B.natom; ++at) {
              if (zq[at] == 0.0) continue;
              HermR R;
              R.build(A.am + C.am, p, P[0] - B.xyz[3 * at], P[1] - B.xyz[3 * at + 1], P[2] - B.xyz[3 * at + 2]);
              const double pref = -zq[at] * 2.0 * PI / p * K;
              for (int ia = 0; ia < na; ++ia)
                for (int ic = 0; ic < nc; ++ic) {
                  double v = 0;
                  for (int t = 0; t <= ea[ia][0] + ec[ic][0]; ++t)
                    for (int u = 0; u <= ea[ia][1] + ec[ic][1]; ++u)
                      for (int w = 0; w <= ea[ia][2] + ec[ic][2]; ++w)
                        v += E[0].E[ea[ia][0]][ec[ic][0]][t] * E[1].E[ea[ia][1]][ec[ic][1]][u] *
                             E[2].E[ea[ia][2]][ec[ic][2]][w] * R.at(t, u, w);
                  blk[(size_t)ia * nc + ic] += pref * v;
                }
            }
          }
        }
      const int shp[2] = {si, sj};
      int dims[2] = {na, nc};
      finish_block(B, shp, 2, blk, dims);
      for (int ia = 0; ia < dims[0]; ++ia)
        for (int ic = 0; ic < dims[1]; ++ic)
          M[(size_t)(A.aoff + ia) * nb + C.aoff + ic] = blk[(size_t)ia * dims[1] + ic];
    }
  return 0;
}

}  // extern "C"
