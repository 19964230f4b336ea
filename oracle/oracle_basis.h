// Oracle (test infrastructure only): CPU restatement of OpenQP's direct
// two-electron Fock build.  Nothing in the product links this code; the tests,
// the smoke check and the CPU-baseline leg of bench.py use it as the checker.
//
// Data model shared by the oracle translation units.
#pragma once
#include <cmath>
#include <cstdint>
#include <vector>

namespace orc {

constexpr double PI = 3.14159265358979323846;

inline int ncart(int l) { return (l + 1) * (l + 2) / 2; }

struct Shell {
  int am = 0;        // angular momentum
  int harm = 0;      // 1 = pure spherical (only acts for am >= 2)
  int nprim = 0;     // contraction degree
  int atom = 0;      // 0-based atom index
  int poff = 0;      // offset into ex / cc
  int aoff = 0;      // 0-based AO offset
  int nao = 0;       // AOs in the shell (2l+1 for pure, else Cartesian count)
  double c[3] = {0, 0, 0};
};

struct Basis {
  int nshell = 0, nbf = 0, natom = 0;
  std::vector<Shell> sh;
  std::vector<double> ex, cc;   // cc: primitive-normalised coefficients
  std::vector<double> xyz;      // 3*natom, Bohr
  int maxam = 0;
};

// int2_cutoffs_t (source/integrals/int2_pairs.F90:27-35,285-294)
// inv_mu2 = 1/mu^2 selects the erf-attenuated operator erf(mu r)/r of the
// second CAM pass (int2.F90:538-584); 0 is the regular 1/r.
struct Cutoffs {
  double integral, pair, quartet, exponent, pair2, quartet2;
  double inv_mu2 = 0.0;
  static Cutoffs make(double cut, double pc, double qc, double ec, double inv_mu2 = 0.0) {
    Cutoffs c;
    c.integral = cut; c.pair = pc; c.quartet = qc; c.exponent = ec;
    c.pair2 = pc * pc; c.quartet2 = qc * qc;
    c.inv_mu2 = inv_mu2;
    return c;
  }
};

// int2_pair_storage (source/integrals/int2_pairs.F90:14-25): primitive pairs
// of every shell pair i >= j (0-based pair id i(i+1)/2 + j).  The pair is
// stored oriented so that am(sha) <= am(shb) (int2_pairs.F90:202-212).
struct PairStore {
  std::vector<int> cnt, off, sha, shb;
  std::vector<double> aa, ab, g, ginv, k, px, py, pz;
  void build(const Basis& b, const Cutoffs& cut);
};

inline int pair_id(int i, int j) { return i >= j ? i * (i + 1) / 2 + j : j * (j + 1) / 2 + i; }

// Handle behind the oracle's C entry points.
struct Handle {
  Basis B;
  double cutoff = 1e-10;
};

// Rys nodes/weights from the generated tables (x = t^2).
void rys_eval(int n, double X, double* x, double* w);

// Boys function F_0..F_m(T), accurate to ~1e-15 (series / recursion).
void boys(int m, double T, double* F);

// Cartesian component exponents in OpenQP order (source/constants.F90:33-60):
// s; x y z; xx yy zz xy xz yz.
void cart_exps(int l, int idx, int* e);
// shells_pnrm2 (source/constants.F90:110-140) for l <= 3
double cart_norm(int l, int idx);
// Pure d / f projections of normalised Cartesians (source/integrals/int2_pure_generated.F90:119-149)
extern const double PURE_D[5][6];
extern const double PURE_F[7][10];

struct QuartetWork {
  double acc[10 * 10 * 10 * 10];
  double tmp[10 * 10 * 10 * 10];
};

// Normalised, pure-projected block of the flipped quartet s[]; returns the
// number of primitive quartets evaluated (0: every primitive was screened).
long rys_quartet(const Basis& B, const PairStore& PS, const Cutoffs& cut, const int s[4], double* out,
                 QuartetWork& W);
// Shell order of gdat_set_ids (source/integrals/int_rys.F90:127-154).
void flip_quartet(const Basis& B, const int ids[4], int s[4], int fl[4]);

}  // namespace orc
