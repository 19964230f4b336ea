// Device-side building blocks of the GB300 direct J/K Fock build: shell and
// pair tables, Cartesian component tables, Rys root evaluation and the
// per-primitive-quartet Rys coefficients.
//
// FP64 is the binding resource on GB300 (about 2 FP64 FMA lanes per clock per
// SM, 64x below FP32), so everything here is written to minimise FP64
// instructions: integer/FP32 work is effectively free next to it.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace oqpg {

// ---------------------------------------------------------------------------
// Tables resident in device memory (one set per registered molecule).
struct ShellDev {
  double x, y, z;
  int am, nao, aoff, harm;  // aoff: first AO within the shell's molecule (matrix column)
  int mrow;                 // first row of the shell's molecule in the stacked matrices
};

// One primitive pair of a shell pair (bra or ket), 80 bytes.
struct PrimPair {
  double p;      // exponent sum
  double hp;     // 0.5 / p
  double px, py, pz;     // Gaussian product centre
  double ax, ay, az;     // P - A (A: first shell of the pair in kernel orientation); in the
                         // Fock tables P - B when A is an s shell (the recursion then runs on B)
  double sp;     // K / p with K = sqrt(2) pi^(5/4) c_a c_b exp(-a b |AB|^2 / p)
  float spf, pf; // FP32 copies of sp and p for the primitive-quartet pre-screen
};

// FP32 copy of a primitive pair for the small-bound quartets of the
// precision-split build, 40 bytes: p, 0.5/p, P, P - A, K/p, pad.
struct PrimPairF {
  float p, hp, px, py, pz, ax, ay, az, sp, pad;
};

// Double-float copy of a primitive pair (the "df" precision mode), defined with
// the double-float type in oqpg_df.cuh.
struct PrimPairDF;
struct dfl;

struct PairDev {
  int sha, shb;    // kernel orientation: am(sha) <= am(shb)
  int poff, pcnt;  // primitive-pair range
};

// A quartet-list entry is (bra pair, ket pair).  With the petite list the two
// top bits of the bra pair index carry log2 of the quartet's orbit weight
// (1, 2, 4 or 8 symmetry-equivalent quartets); pair indices stay below 2^30.
constexpr unsigned PAIR_MASK = 0x3fffffffu;
__host__ __device__ inline unsigned entry_pair(unsigned x) { return x & PAIR_MASK; }
__host__ __device__ inline int entry_wlog2(unsigned x) { return (int)(x >> 30); }

// Shell families: two s shells on one atom whose primitive exponents are the
// same, or one's among the other's (the generally contracted shells of
// correlation-consistent sets, e.g. the 1s and 2s of O in cc-pVDZ).  A family pair
// (two families, or a family and another shell) has up to FAM_MAX member
// shell pairs that share every primitive pair's geometry and differ only in
// the contraction coefficients, so one primitive integral serves them all.
// Its primitive pairs are the union of the members' (PrimPair, with sp the
// largest member |K/p|, for the screens); FamCoef holds each member's own K/p,
// zero where the member's primitive-pair screen drops the pair.
constexpr int FAM_MAX = 4;
struct FamMem {
  int n;             // member shell pairs (1..FAM_MAX)
  int m[FAM_MAX];    // their indices in the canonical pair table
};
struct FamCoef {
  double sp[FAM_MAX];
  float spf[FAM_MAX];
};
// the members' K/p as double-float pairs (hi, lo), for the df family kernels
struct FamCoefDF {
  float2 sp[FAM_MAX];
};
// Family-quartet list entries: family pair indices in the low 24 bits of x
// and y, and the member combinations (m of x, n of y) that pass the quartet
// screen as bit 4m + n of a 16-bit mask, bits 0-7 in the top byte of x and
// bits 8-15 in the top byte of y.
constexpr unsigned FAM_IDX_MASK = 0xffffffu;
__host__ __device__ inline uint2 fam_entry(unsigned fx, unsigned fy, unsigned mask) {
  return make_uint2(fx | ((mask & 0xffu) << 24), fy | ((mask >> 8) << 24));
}
__host__ __device__ inline unsigned fam_mask(uint2 e) { return (e.x >> 24) | ((e.y >> 24) << 8); }

// Parameters of one Fock build (or Schwarz pass) shared by the class kernels.
struct BuildArgs {
  const ShellDev* shells;
  const PairDev* pairs;
  const PrimPair* prims;
  const PrimPairF* primsf; // FP32 copy (precision-split builds)
  const PrimPairDF* primsdf;  // double-float copy (df mode)
  const float2* rysdf;        // Rys table and large-X constants as FP32 pairs (df mode)
  const uint2* quartets;   // (bra pair, ket pair) per quartet of this class
  long long nquartets;     // quartets (or, with range, the capacity that sizes the grid)
  const unsigned long long* range;  // optional device [begin, end) into quartets, read at kernel start
  int nbf;                 // row stride of the stacked matrices (largest nbf of the batch)
  size_t kstride;          // elements between consecutive densities / accumulators (J or K)
  int nj;                  // number of Coulomb densities (1 for the SCF builds)
  int nk;                  // number of exchange densities (1 RHF, 2 UHF/ROHF)
  double prim_cut;         // |K/p| pre-screen of a primitive pair
  double prim_cut2;        // (sp sq)^2 < prim_cut2 (p + q) skips a primitive quartet
  float prim_cut_lo;       // FP32 decision band of that test: |sp sq| / sqrt(p+q) below lo
  float prim_cut_hi;       // skips, above hi keeps, in between FP64 decides
  double elem_cut;         // element cutoff on |(ab|cd)|
  double inv_mu2;          // 1/mu^2 of the erf(mu r)/r operator (CAM pass 2); 0: 1/r
  const double* dj;        // nj full nbf x nbf densities for Coulomb
  const double* dk;        // nk full densities for exchange
  const float* djf;        // FP32 copies of dj / dk for the FP32 quartets
  const float* dkf;
  const struct dfl* djdf;  // double-float copies (df mode)
  const struct dfl* dkdf;
  double* gj;              // nj x nbf x nbf Coulomb accumulators
  double* gk;              // nk x nbf x nbf exchange accumulators
  double* schwarz_out;     // Schwarz mode: per pair sqrt(max |(ab|ab)|)
  unsigned long long* counters;  // [0] primitive quartets evaluated by this launch
  unsigned long long* work;      // work-distribution counter of this launch (zeroed before it)
  int roots_f32;                 // FP32 quartets: evaluate Rys roots/weights in FP32 too
  int chunk;                     // thread-per-quartet kernels: quartets per warp grab (multiple of 32)
  int team;                      // a class with both kernel families: 1 = warp per quartet
  int ctas_per_sm;               // launch: grid cap per SM (0: as many as fit)
  // shell-family builds (quartets are family quartets; pairs stays the
  // canonical pair table, for the members' digestion)
  const PairDev* fpairs;         // family pairs: representative shells, union primitive range
  const FamMem* fmem;
  const PrimPair* fprims;        // union primitive pairs
  const PrimPairF* fprimsf;      // FP32 copy (the FP32 family quartets of the precision split)
  const PrimPairDF* fprimsdf;    // double-float copy (the double-float modes)
  const FamCoef* fcoef;          // per union primitive pair: the members' K/p
  const FamCoefDF* fcoefdf;      // and as double-float pairs
};

// ---------------------------------------------------------------------------
__host__ __device__ constexpr int ncart(int l) { return (l + 1) * (l + 2) / 2; }

// Cartesian exponents in OpenQP order (constants.F90:33-60): s; x y z;
// xx yy zz xy xz yz; xxx yyy zzz xxy xxz xyy yyz xzz yzz xyz.
__host__ __device__ constexpr int cart_e3(int idx, int dim) {
  // packed exponents (x | y << 2 | z << 4) of the ten f components
  return ((idx == 0 ? 3 : idx == 1 ? 12 : idx == 2 ? 48 : idx == 3 ? 6 : idx == 4 ? 18 : idx == 5 ? 9
           : idx == 6 ? 24 : idx == 7 ? 33 : idx == 8 ? 36 : 21) >> (2 * dim)) & 3;
}
__host__ __device__ constexpr int cart_e(int l, int idx, int dim) {
  return l == 0 ? 0
       : l == 1 ? (idx == dim ? 1 : 0)
       : l == 3 ? cart_e3(idx, dim)
       : (idx < 3 ? (idx == dim ? 2 : 0)
          : idx == 3 ? (dim < 2 ? 1 : 0)
          : idx == 4 ? (dim != 1 ? 1 : 0)
                     : (dim > 0 ? 1 : 0));
}
// shells_pnrm2 for l <= 3 (individually normalised Cartesians)
__host__ __device__ constexpr double cart_norm(int l, int idx) {
  return (l == 2 && idx >= 3) ? 1.7320508075688772
       : (l == 3 && idx >= 3) ? (idx == 9 ? 3.8729833462074170 : 2.2360679774997897)
                              : 1.0;
}

// FP64 reciprocal: the hardware approximation rcp.approx.ftz.f64 refined by
// two Newton-Raphson steps for f(r) = 1/r - x (r <- r + r (1 - x r)), each
// doubling the correct bits; 4 FP64 FMA, about 1 ulp.
__device__ __forceinline__ double rcp64(double x) {
  double r;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
  double e = fma(-x, r, 1.0);
  r = fma(r, e, r);
  e = fma(-x, r, 1.0);
  return fma(r, e, r);
}

// FP64 1/sqrt(x) for a positive normal x with 2^-126 <= x < 2^128 (every
// argument of the integral kernels: exponent sums p + q and Rys arguments X).
// Seed: y0 = rsqrtf(x'), x' = x truncated to FP32 (same exponent, leading 23
// mantissa bits), so y0 is within 2^-21 of 1/sqrt(x) (rsqrtf: at most 2 ulp).
// One third-order step of the binomial series
//   1/sqrt(x) = y0 (1 - t)^(-1/2) = y0 (1 + t/2 + 3 t^2 / 8 + 5 t^3 / 16 + ...),
//   t = 1 - x y0^2
// (Householder's method of order 3 for x^(-1/2)), truncated after t^2: the
// dropped terms are below 2^-60 relative, so the result is within about one
// ulp.  The FP64 <-> FP32 conversions are integer bit operations, so the
// whole evaluation costs 5 FP64 instructions (2 DMUL, 3 DFMA).
__device__ __forceinline__ double rsqrt64(double x) {
  const int hi = __double2hiint(x);
  const unsigned lo = (unsigned)__double2loint(x);
  // FP32 bits: exponent rebased by 1023 - 127 = 896, mantissa truncated
  const float xf = __uint_as_float(((unsigned)(hi - (896 << 20)) << 3) | (lo >> 29));
  const unsigned yb = __float_as_uint(rsqrtf(xf));
  // back to FP64 bits (y0 is a positive normal FP32 number)
  const double y0 = __hiloint2double((int)((((yb >> 23) + 896u) << 20) | ((yb & 0x7fffffu) >> 3)),
                                     (int)((yb & 7u) << 29));
  const double xy = x * y0;
  const double t = fma(-xy, y0, 1.0);
  const double a = fma(t, 0.375, 0.5);
  return fma(t * y0, a, y0);
}

}  // namespace oqpg
