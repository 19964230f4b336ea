// Class-specialised shell-quartet kernels: Rys quadrature ERIs contracted on
// the fly into Coulomb / exchange accumulators.
//
// One instantiation per (la lb | lc ld) class (la <= lb, lc <= ld, bra pair
// type <= ket pair type), per AO convention of the d shells (Cartesian or
// pure), per mode (Fock build or Schwarz bound) and per arithmetic type T:
// double for the plain path and the large-bound quartets of the precision
// split, float for its small-bound quartets.  FP32 quartets keep the Rys
// root/weight evaluation in FP64 (degree-4 tables, ~1e-8 relative) and add
// their digested blocks into the same FP64 accumulators.
//
//   k_small : one thread per quartet, everything in registers (classes with at
//             most 54 Cartesian elements, 27 with an f shell).
//   k_prim  : heavily contracted small-class quartets, one warp per quartet,
//             lanes split the primitive loop.
//   k_team  : one warp per quartet.  Lanes share the primitive loop: Rys
//             roots/weights (one quantity per lane), the 2D integrals (one
//             root x dimension per lane) go to shared memory, each lane
//             accumulates its own subset of the Cartesian elements; the
//             digestion distributes the J/K target elements over the lanes.
//
// The integral algebra follows Rys, Dupuis & King (J. Comput. Chem. 4, 154
// (1983)): per root t^2 = u, with s = p + q,
//   B00 = u / 2s, B10 = (1 - u q/s) / 2p, B01 = (1 - u p/s) / 2q,
//   C00 = (P - A) - u (q/s) (P - Q),   D00 = (Q - C) + u (p/s) (P - Q),
//   I(n+1,0) = C00 I(n,0) + n B10 I(n-1,0)
//   I(n,m+1) = D00 I(n,m) + m B01 I(n,m-1) + n B00 I(n-1,m)
// followed by the horizontal transfers I(i,j+1) = I(i+1,j) + (A-B) I(i,j)
// on each pair (the structure of OpenQP's int_rys.F90:529-661).  Screening
// thresholds and the element cutoff follow OpenQP's s-d path
// (int_rotaxis.F90:292-306,629; int2.F90:1806-1812).
#pragma once
#include <type_traits>

#include "oqpg_common.cuh"
#include "oqpg_df.cuh"

namespace oqpg {

#define RYS_STORAGE static __device__ const
#include "rys_tables.inc"
#include "rys_tables_df.inc"
#include "rys_tables_fine.inc"
#undef RYS_STORAGE

__host__ __device__ constexpr int rys_xmax(int n) { return 32 + 8 * n; }
__host__ __device__ constexpr int rys_nint(int n) { return RYS_X_SPLIT * RYS_LO_PER_UNIT + (rys_xmax(n) - RYS_X_SPLIT); }
__host__ __device__ constexpr int rys_offset(int n, int ncoef) {  // start of the n-root table
  return n <= 1 ? 0 : rys_offset(n - 1, ncoef) + rys_nint(n - 1) * 2 * (n - 1) * ncoef;
}
// The finer grid of the one- and two-root FP64 tables (rys_tables_fine.inc)
__host__ __device__ constexpr int rys_nint_fine(int n) {
  return RYS_X_SPLIT * RYS_FINE_LO_PER_UNIT + (rys_xmax(n) - RYS_X_SPLIT) * RYS_FINE_HI_PER_UNIT;
}
__host__ __device__ constexpr int rys_offset_fine(int n) {
  return n <= 1 ? 0 : rys_offset_fine(n - 1) + rys_nint_fine(n - 1) * 2 * (n - 1) * RYS_FINE_NCOEF;
}
static_assert(rys_offset_fine(RYS_FINE_NMAX + 1) == RYS_TABLE_FINE_SIZE, "fine Rys table layout");

// Interval k of a table at X >= 0 and the Chebyshev variable s in [-1, 1],
// for intervals of width 2^-LL below 32 and 2^-LH from 32 up: with
// f = floor(X 2^L) (L = LL or LH), k = f below 32 and
// 32 2^LL + (f - 32 2^LH) above, s = 2^(L+1) X - (2f+1).  The floors and the
// constant 2f+1 come from the bits of X with integer instructions, so the
// only FP64 instruction is the FMA that forms s.  The standard tables use
// LL = 2, LH = 0; the fine one- and two-root tables LL = 3, LH = 1.
template <int LL, int LH>
__device__ __forceinline__ int rys_interval(long long xb, double X, double& s) {
  const bool lo = xb < __double_as_longlong((double)RYS_X_SPLIT);
  // floor(X 2^L) (X < 2^30)
  const int e = (int)(xb >> 52) - 1023 + (lo ? LL : LH);
  const long long m = (xb & 0xfffffffffffffll) | 0x10000000000000ll;
  const int f = (int)(m >> (e < 0 ? 63 : 52 - e));
  // -(2f + 1) as a double: odd integer v < 2^21, exponent from its leading bit
  const unsigned v = 2u * (unsigned)f + 1u;
  const int ev = 31 - __clz(v);
  const double c = __longlong_as_double((long long)((1ull << 63) | ((unsigned long long)(1023 + ev) << 52) |
                                                    (((unsigned long long)v << (52 - ev)) & 0xfffffffffffffull)));
  s = fma(lo ? (double)(2 << LL) : (double)(2 << LH), X, c);
  return lo ? f : (RYS_X_SPLIT << LL) + (f - (RYS_X_SPLIT << LH));
}
static_assert(RYS_LO_PER_UNIT == 4 && RYS_FINE_LO_PER_UNIT == 8 && RYS_FINE_HI_PER_UNIT == 2,
              "rys_interval grids: 1/4 and 1 (standard), 1/8 and 1/2 (fine)");

// Above the table (X >= 32 + 8N) the nodes and weights are R2/X and W/sqrt(X):
// polynomials of degree 2 and 1 in y = X^-1/2 (y from one reciprocal square
// root).  A warp whose lanes all lie above the table evaluates them directly;
// a warp whose lanes all lie in the table runs the interpolant; a warp with
// lanes on both sides runs ONE Horner chain, in the interval variable s for
// table lanes and in y for the others with the coefficients (0, 0, R2, 0, ...)
// and (0, W, 0, ...), so the two kinds of lanes share every FMA of the chain
// (a divergent branch would issue both evaluations for the whole warp).  The
// zero coefficients make the chain exact: R2 y y and W y.

// Quantity q of the N-root rule at X (FP64): q even -> node x_{q/2}, q odd ->
// weight w_{q/2}.  X >= 0, so the range tests compare bit patterns as
// integers (no FP64 instruction).
template <int N, int NCOEF, bool FINE = false>
__device__ __forceinline__ double rys_eval(const double* table, double X, int q) {
  const long long xb = __double_as_longlong(X);
  const bool asym = xb >= __double_as_longlong((double)rys_xmax(N));
  const unsigned act = __activemask();
  const unsigned ba = __ballot_sync(act, asym);
  const int r = (N * (N - 1)) / 2 + (q >> 1);
  if (ba == act) {
    // nodes R2 / X and weights W / sqrt(X) from one reciprocal square root, so
    // lanes that evaluate nodes and lanes that evaluate weights take one path
    const double y = rsqrt64(X);
    return (q & 1) ? RYS_HERM_W[r] * y : RYS_HERM_R2[r] * (y * y);
  }
  double s, a = 0.0;
  const double* c = table;
  if (asym) {
    s = rsqrt64(X);
    a = (q & 1) ? RYS_HERM_W[r] : RYS_HERM_R2[r];
  } else {
    const int k = FINE ? rys_interval<3, 1>(xb, X, s) : rys_interval<2, 0>(xb, X, s);
    c = table + (FINE ? rys_offset_fine(N) : rys_offset(N, NCOEF)) + (k * 2 * N + q) * NCOEF;
  }
  // the single nonzero coefficient of the large-X form: degree 1 (weight) or 2 (node)
  const int ia = (q & 1) ? 1 : 2;
  double v = asym ? 0.0 : __ldg(c + NCOEF - 1);
#pragma unroll
  for (int i = NCOEF - 2; i >= 0; --i) v = fma(v, s, asym ? (i == ia ? a : 0.0) : __ldg(c + i));
  return v;
}

// Node u and weight w of root r together (FP64): one range test for both, and
// above the table both come from one reciprocal square root y = X^-1/2
// (u = R2_r y^2, w = W_r y) instead of a reciprocal and a reciprocal square root.
// FINE: the one- and two-root fine tables (degree 6, rys_tables_fine.inc).
template <int N, int NCOEF, bool FINE = false>
__device__ __forceinline__ void rys_eval_uw(const double* table, double X, int r, double& u, double& w) {
  const long long xb = __double_as_longlong(X);
  const bool asym = xb >= __double_as_longlong((double)rys_xmax(N));
  const unsigned act = __activemask();
  const unsigned ba = __ballot_sync(act, asym);
  const int i0 = (N * (N - 1)) / 2 + r;
  if (ba == act) {
    const double y = rsqrt64(X);
    u = RYS_HERM_R2[i0] * (y * y);
    w = RYS_HERM_W[i0] * y;
    return;
  }
  double s, r2 = 0.0, wh = 0.0;
  const double* c = table;
  if (asym) {
    s = rsqrt64(X);
    r2 = RYS_HERM_R2[i0];
    wh = RYS_HERM_W[i0];
  } else {
    const int k = FINE ? rys_interval<3, 1>(xb, X, s) : rys_interval<2, 0>(xb, X, s);
    // node coefficients at c, weight coefficients at c + NCOEF
    c = table + (FINE ? rys_offset_fine(N) : rys_offset(N, NCOEF)) + (k * 2 * N + 2 * r) * NCOEF;
  }
  double vu = asym ? 0.0 : __ldg(c + NCOEF - 1), vw = asym ? 0.0 : __ldg(c + 2 * NCOEF - 1);
#pragma unroll
  for (int i = NCOEF - 2; i >= 0; --i) {
    vu = fma(vu, s, asym ? (i == 2 ? r2 : 0.0) : __ldg(c + i));
    vw = fma(vw, s, asym ? (i == 1 ? wh : 0.0) : __ldg(c + NCOEF + i));
  }
  u = vu;
  w = vw;
}

// FP32 variant of the same evaluation (the degree-4 table rounded to FP32),
// for the FP32 quartets when the split is asked to keep no FP64 at all.
template <int N>
__device__ __forceinline__ float rys_eval_f32(float X, int q) {
  if (X >= (float)rys_xmax(N)) {
    const int r = (N * (N - 1)) / 2 + (q >> 1);
    return (q & 1) ? (float)RYS_HERM_W[r] * rsqrtf(X) : (float)RYS_HERM_R2[r] / X;
  }
  int k;
  float s;
  if (X < (float)RYS_X_SPLIT) {
    k = min(__float2int_rz(X * (float)RYS_LO_PER_UNIT), RYS_X_SPLIT * RYS_LO_PER_UNIT - 1);
    s = fmaf(2.0f * RYS_LO_PER_UNIT, X, -(float)(2 * k + 1));
  } else {
    const int f = min(__float2int_rz(X), rys_xmax(N) - 1);
    k = RYS_X_SPLIT * RYS_LO_PER_UNIT + (f - RYS_X_SPLIT);
    s = fmaf(2.0f, X, -(float)(2 * f + 1));
  }
  const float* c = RYS_TABLE_F32F + rys_offset(N, RYS_NCOEF_F32) + (k * 2 * N + q) * RYS_NCOEF_F32;
  float v = __ldg(c + RYS_NCOEF_F32 - 1);
#pragma unroll
  for (int i = RYS_NCOEF_F32 - 2; i >= 0; --i) v = fmaf(v, s, __ldg(c + i));
  return v;
}

// Double-float evaluation of the degree-7 FP64 table (coefficients as FP32
// pairs), interval selection on the leading FP32 word.
// Double-float Horner chains start in plain FP32: the interpolants'
// coefficients of degree >= 5 are below 2e-7 of the leading one (all root
// counts, every interval), so the FP32 rounding of c7 s^2 + c6 s + c5 stays
// below 2e-14 of the result, under the double-float resolution; degrees 4..0
// run in double-float (5 of the 7 FMAs of the chain).
constexpr int RYS_DF_TAIL = 5;

template <int N>
__device__ __forceinline__ dfl rys_eval_df(dfl X, int q) {
  if (X.hi >= (float)rys_xmax(N)) {
    const int r = (N * (N - 1)) / 2 + (q >> 1);
    const float2 c = RYS_HERM_W_DF[r], c2 = RYS_HERM_R2_DF[r];
    // one reciprocal square root for nodes and weights (one path for all lanes)
    const dfl y = df_rsqrt(X);
    return (q & 1) ? dfl(c.x, c.y) * y : dfl(c2.x, c2.y) * (y * y);
  }
  int k;
  dfl s;
  if (X.hi < (float)RYS_X_SPLIT) {
    k = min(__float2int_rz(X.hi * (float)RYS_LO_PER_UNIT), RYS_X_SPLIT * RYS_LO_PER_UNIT - 1);
    s = dfl(X.hi * (2.0f * RYS_LO_PER_UNIT), X.lo * (2.0f * RYS_LO_PER_UNIT)) + dfl(-(2 * k + 1));
  } else {
    const int f = min(__float2int_rz(X.hi), rys_xmax(N) - 1);
    k = RYS_X_SPLIT * RYS_LO_PER_UNIT + (f - RYS_X_SPLIT);
    s = dfl(X.hi * 2.0f, X.lo * 2.0f) + dfl(-(2 * f + 1));
  }
  const float2* c = RYS_TABLE_DF + rys_offset(N, RYS_NCOEF) + (k * 2 * N + q) * RYS_NCOEF;
  // the top of the chain in FP32 (see RYS_DF_TAIL), the rest in double-float
  float f = __ldg(c + RYS_NCOEF - 1).x;
#pragma unroll
  for (int i = RYS_NCOEF - 2; i >= RYS_DF_TAIL; --i) f = fmaf(f, s.hi, __ldg(c + i).x);
  dfl v(f, 0.0f);
#pragma unroll
  for (int i = RYS_DF_TAIL - 1; i >= 0; --i) {
    const float2 t = __ldg(c + i);
    v = fma(v, s, dfl(t.x, t.y));
  }
  return v;
}

// Node u and weight w of root r together in double-float (the FP64 joint
// evaluation's structure: one range test, one reciprocal square root above the table).
template <int N>
__device__ __forceinline__ void rys_eval_uw_df(dfl X, int r, dfl& u, dfl& w) {
  if (X.hi >= (float)rys_xmax(N)) {
    const int i = (N * (N - 1)) / 2 + r;
    const float2 c = RYS_HERM_W_DF[i], c2 = RYS_HERM_R2_DF[i];
    const dfl y = df_rsqrt(X);
    u = dfl(c2.x, c2.y) * (y * y);
    w = dfl(c.x, c.y) * y;
    return;
  }
  int k;
  dfl s;
  if (X.hi < (float)RYS_X_SPLIT) {
    k = min(__float2int_rz(X.hi * (float)RYS_LO_PER_UNIT), RYS_X_SPLIT * RYS_LO_PER_UNIT - 1);
    s = dfl(X.hi * (2.0f * RYS_LO_PER_UNIT), X.lo * (2.0f * RYS_LO_PER_UNIT)) + dfl(-(2 * k + 1));
  } else {
    const int f = min(__float2int_rz(X.hi), rys_xmax(N) - 1);
    k = RYS_X_SPLIT * RYS_LO_PER_UNIT + (f - RYS_X_SPLIT);
    s = dfl(X.hi * 2.0f, X.lo * 2.0f) + dfl(-(2 * f + 1));
  }
  const float2* c = RYS_TABLE_DF + rys_offset(N, RYS_NCOEF) + (k * 2 * N + 2 * r) * RYS_NCOEF;
  float fu = __ldg(c + RYS_NCOEF - 1).x, fw = __ldg(c + 2 * RYS_NCOEF - 1).x;
#pragma unroll
  for (int i = RYS_NCOEF - 2; i >= RYS_DF_TAIL; --i) {
    fu = fmaf(fu, s.hi, __ldg(c + i).x);
    fw = fmaf(fw, s.hi, __ldg(c + RYS_NCOEF + i).x);
  }
  dfl vu(fu, 0.0f), vw(fw, 0.0f);
#pragma unroll
  for (int i = RYS_DF_TAIL - 1; i >= 0; --i) {
    const float2 tu = __ldg(c + i), tw = __ldg(c + RYS_NCOEF + i);
    vu = fma(vu, s, dfl(tu.x, tu.y));
    vw = fma(vw, s, dfl(tw.x, tw.y));
  }
  u = vu;
  w = vw;
}

// FP64 kernels: the degree-7 FP64 tables (degree 6 on the finer grid for one
// and two roots).  FP32 kernels: the degree-4 tables, evaluated in FP64
// (default) or, with roots_f32, in FP32.  Double-float kernels: the degree-7
// table in double-float.
template <int N, typename T>
__device__ __forceinline__ T rys_quantity(T X, int q, bool roots_f32 = false) {
  if constexpr (std::is_same<T, double>::value) {
    if constexpr (N <= RYS_FINE_NMAX) return rys_eval<N, RYS_FINE_NCOEF, true>(RYS_TABLE_FINE, X, q);
    else return rys_eval<N, RYS_NCOEF>(RYS_TABLE, X, q);
  }
  else if constexpr (std::is_same<T, dfl>::value) return rys_eval_df<N>(X, q);
  else {
    if (roots_f32) return rys_eval_f32<N>(X, q);
    return (float)rys_eval<N, RYS_NCOEF_F32>(RYS_TABLE_F32, (double)X, q);
  }
}

// Node and weight of root r (the pair that a thread-per-quartet loop needs).
template <int N, typename T>
__device__ __forceinline__ void rys_node_weight(T X, int r, bool roots_f32, T& u, T& w) {
  if constexpr (std::is_same<T, double>::value) {
    if constexpr (N <= RYS_FINE_NMAX) rys_eval_uw<N, RYS_FINE_NCOEF, true>(RYS_TABLE_FINE, X, r, u, w);
    else rys_eval_uw<N, RYS_NCOEF>(RYS_TABLE, X, r, u, w);
  } else if constexpr (std::is_same<T, dfl>::value) {
    rys_eval_uw_df<N>(X, r, u, w);
  } else {
    u = rys_quantity<N, T>(X, 2 * r, roots_f32);
    w = rys_quantity<N, T>(X, 2 * r + 1, roots_f32);
  }
}

__host__ __device__ constexpr int naos(int l, bool pure) { return (pure && l >= 2) ? 2 * l + 1 : ncart(l); }
__host__ __device__ constexpr int cmax(int a, int b) { return a > b ? a : b; }
__host__ __device__ constexpr int cmin(int a, int b) { return a < b ? a : b; }

// Pure-d projection row m, Cartesian component c (m = -2..2: xy, yz, z^2, xz, x^2-y^2)
__host__ __device__ constexpr double pure_d(int m, int c) {
  return m == 0 ? (c == 3 ? 1.0 : 0.0)
       : m == 1 ? (c == 5 ? 1.0 : 0.0)
       : m == 2 ? (c == 2 ? 1.0 : (c < 2 ? -0.5 : 0.0))
       : m == 3 ? (c == 4 ? 1.0 : 0.0)
                : (c == 0 ? 0.86602540378443865 : (c == 1 ? -0.86602540378443865 : 0.0));
}

// Pure-f projection row m (m = -3..3), Cartesian component c of the normalised
// Cartesians xxx yyy zzz xxy xxz xyy yyz xzz yzz xyz: the real solid harmonics
// (coefficients sqrt(10)/4, 3/(2 sqrt 2), sqrt(6)/4, sqrt(30)/20, sqrt(6/5),
// 3/(2 sqrt 5), sqrt(3)/2; OpenQP int2_pure_generated.F90:134-149)
__host__ __device__ constexpr double pure_f(int m, int c) {
  constexpr double A = 0.79056941504209483, B = 1.0606601717798213, C = 0.61237243569579452,
                   D = 0.27386127875258306, E = 1.0954451150103321, G = 0.67082039324993691,
                   H = 0.86602540378443865;
  return m == 0 ? (c == 1 ? -A : c == 3 ? B : 0.0)
       : m == 1 ? (c == 9 ? 1.0 : 0.0)
       : m == 2 ? (c == 1 ? -C : c == 3 ? -D : c == 8 ? E : 0.0)
       : m == 3 ? (c == 2 ? 1.0 : (c == 4 || c == 6) ? -G : 0.0)
       : m == 4 ? (c == 0 ? -C : c == 5 ? -D : c == 7 ? E : 0.0)
       : m == 5 ? (c == 4 ? H : c == 6 ? -H : 0.0)
                : (c == 0 ? A : c == 5 ? -B : 0.0);
}
__host__ __device__ constexpr double pure_coef(int l, int m, int c) { return l == 2 ? pure_d(m, c) : pure_f(m, c); }

// ---------------------------------------------------------------------------
// Primitive pairs in the arithmetic type of the kernel.
template <typename T> struct PrimT;
template <> struct PrimT<double> { using type = PrimPair; };
template <> struct PrimT<float> { using type = PrimPairF; };
template <> struct PrimT<dfl> { using type = PrimPairDF; };

template <typename T> __device__ __forceinline__ const typename PrimT<T>::type* prims_of(const BuildArgs& a);
template <> __device__ __forceinline__ const PrimPair* prims_of<double>(const BuildArgs& a) { return a.prims; }
template <> __device__ __forceinline__ const PrimPairF* prims_of<float>(const BuildArgs& a) { return a.primsf; }
template <> __device__ __forceinline__ const PrimPairDF* prims_of<dfl>(const BuildArgs& a) { return a.primsdf; }

template <typename T> __device__ __forceinline__ const T* dj_of(const BuildArgs& a);
template <> __device__ __forceinline__ const double* dj_of<double>(const BuildArgs& a) { return a.dj; }
template <> __device__ __forceinline__ const float* dj_of<float>(const BuildArgs& a) { return a.djf; }
template <> __device__ __forceinline__ const dfl* dj_of<dfl>(const BuildArgs& a) { return a.djdf; }
template <typename T> __device__ __forceinline__ const T* dk_of(const BuildArgs& a);
template <> __device__ __forceinline__ const double* dk_of<double>(const BuildArgs& a) { return a.dk; }
template <> __device__ __forceinline__ const float* dk_of<float>(const BuildArgs& a) { return a.dkf; }
template <> __device__ __forceinline__ const dfl* dk_of<dfl>(const BuildArgs& a) { return a.dkdf; }

__device__ __forceinline__ void prim_load(const PrimPair* __restrict__ src, PrimPair& d) {
  const double2* s = reinterpret_cast<const double2*>(src);
  double2 v0 = __ldg(s), v1 = __ldg(s + 1), v2 = __ldg(s + 2), v3 = __ldg(s + 3), v4 = __ldg(s + 4);
  d.p = v0.x; d.hp = v0.y; d.px = v1.x; d.py = v1.y; d.pz = v2.x; d.ax = v2.y; d.ay = v3.x; d.az = v3.y;
  d.sp = v4.x;
  const long long bits = __double_as_longlong(v4.y);
  d.spf = __int_as_float((int)(bits & 0xffffffffll));
  d.pf = __int_as_float((int)(bits >> 32));
}
__device__ __forceinline__ void prim_load(const PrimPairF* __restrict__ src, PrimPairF& d) {
  const float2* s = reinterpret_cast<const float2*>(src);
  float2 v0 = __ldg(s), v1 = __ldg(s + 1), v2 = __ldg(s + 2), v3 = __ldg(s + 3), v4 = __ldg(s + 4);
  d.p = v0.x; d.hp = v0.y; d.px = v1.x; d.py = v1.y; d.pz = v2.x; d.ax = v2.y; d.ay = v3.x; d.az = v3.y;
  d.sp = v4.x; d.pad = v4.y;
}

__device__ __forceinline__ void prim_load(const PrimPairDF* __restrict__ src, PrimPairDF& d) {
  const float4* s = reinterpret_cast<const float4*>(src);
  const float4 v0 = __ldg(s), v1 = __ldg(s + 1), v2 = __ldg(s + 2), v3 = __ldg(s + 3), v4 = __ldg(s + 4);
  d.p = dfl(v0.x, v0.y); d.hp = dfl(v0.z, v0.w); d.px = dfl(v1.x, v1.y); d.py = dfl(v1.z, v1.w);
  d.pz = dfl(v2.x, v2.y); d.ax = dfl(v2.z, v2.w); d.ay = dfl(v3.x, v3.y); d.az = dfl(v3.z, v3.w);
  d.sp = dfl(v4.x, v4.y); d.spf = v4.z; d.pf = v4.w;
}

// FP32 screening data (K/p, p) of a primitive pair.
__device__ __forceinline__ float2 prim_screen(const PrimPair* p) {
  const long long bits = __double_as_longlong(__ldg(reinterpret_cast<const double*>(p) + 9));
  return make_float2(__int_as_float((int)(bits & 0xffffffffll)), __int_as_float((int)(bits >> 32)));
}
__device__ __forceinline__ float2 prim_screen(const PrimPairDF* p) {
  const float* f = reinterpret_cast<const float*>(p);
  return make_float2(__ldg(f + 18), __ldg(f + 19));
}
__device__ __forceinline__ float2 prim_screen(const PrimPairF* p) {
  const float* f = reinterpret_cast<const float*>(p);
  return make_float2(__ldg(f + 8), __ldg(f));
}

// Primitive-quartet screen (sp sq)^2 < cut2 (p + q) of the rotated-axis engine
// (int_rotaxis.F90:629), decided in FP32 unless |sp sq| / sqrt(p + q) falls in
// the narrow band [lo, hi] around the cutoff, where FP64 decides (FP64 pairs).
__device__ __forceinline__ bool screen_keep(const PrimPair* bp, float2 bs, const PrimPair* kp, float2 ks,
                                            const BuildArgs& a) {
  const float r = fabsf(bs.x * ks.x) * rsqrtf(bs.y + ks.y);
  if (r < a.prim_cut_lo) return false;
  if (r > a.prim_cut_hi) return true;
  const double* b = reinterpret_cast<const double*>(bp);
  const double* k = reinterpret_cast<const double*>(kp);
  const double fqz = __ldg(b + 8) * __ldg(k + 8);
  return !(fqz * fqz < a.prim_cut2 * (__ldg(b) + __ldg(k)));
}
// Double-float pairs: the same band; inside it the test in double-float.
__device__ __forceinline__ bool screen_keep(const PrimPairDF* bp, float2 bs, const PrimPairDF* kp, float2 ks,
                                            const BuildArgs& a) {
  const float r = fabsf(bs.x * ks.x) * rsqrtf(bs.y + ks.y);
  if (r < a.prim_cut_lo) return false;
  if (r > a.prim_cut_hi) return true;
  const dfl fqz = df_ld(&bp->sp) * df_ld(&kp->sp);
  const dfl lhs = fqz * fqz, rhs = dfl(a.prim_cut2) * (df_ld(&bp->p) + df_ld(&kp->p));
  return !((lhs - rhs).hi < 0.0f);
}
__device__ __forceinline__ bool screen_keep(const PrimPairF*, float2 bs, const PrimPairF*, float2 ks,
                                            const BuildArgs& a) {
  const float r = fabsf(bs.x * ks.x) * rsqrtf(bs.y + ks.y);
  return !(r < 0.5f * (a.prim_cut_lo + a.prim_cut_hi));
}

// Per-primitive-quartet scalars shared by all roots.
template <typename T>
struct PrimQuartet {
  T inv, qi, pi, pref, X;
  T PQ[3];
};

__device__ __forceinline__ double rsqrt_t(double x) { return rsqrt64(x); }
__device__ __forceinline__ float rsqrt_t(float x) { return rsqrtf(x); }
__device__ __forceinline__ dfl rsqrt_t(dfl x) { return df_rsqrt(x); }

// ATT, att = 1/mu^2: the erf(mu r)/r operator of the CAM pass: p + q
// becomes p + q + pq/mu^2 in rho, in the prefactor and in the recurrence
// coefficients (int_rys.F90:225-240; int_rotaxis.F90:634-638 writes the same
// as rho mu^2/(mu^2 + rho)).  The primitive screen keeps the plain p + q.
// XPI: X = q (p/s) |PQ|^2 instead of p (q/s) |PQ|^2 (same value), for callers
// that never use q/s (a bra pair of two s shells): one multiply fewer.
template <typename T, bool ATT = false, bool XPI = false, typename PP>
__device__ __forceinline__ void prim_setup(const PP& bp, const PP& kp, PrimQuartet<T>& o, T att = T(0)) {
  const T fqz = bp.sp * kp.sp;
  T s = bp.p + kp.p;
  if constexpr (ATT) s = fma(bp.p * kp.p, att, s);
  const T y = rsqrt_t(s);
  o.inv = y * y;
  o.qi = kp.p * o.inv;
  o.pi = bp.p * o.inv;
  o.PQ[0] = bp.px - kp.px;
  o.PQ[1] = bp.py - kp.py;
  o.PQ[2] = bp.pz - kp.pz;
  const T r2 = fma(o.PQ[0], o.PQ[0], fma(o.PQ[1], o.PQ[1], o.PQ[2] * o.PQ[2]));
  o.X = XPI ? kp.p * o.pi * r2 : bp.p * o.qi * r2;
  o.pref = fqz * y;
}

// 2D integrals of one root and one Cartesian dimension:
// out[((i*(LB+1)+j)*(LC+1)+k)*(LD+1)+l], i<=LA, j<=LB, k<=LC, l<=LD.
// A pair whose first shell is an s shell (LA = 0, LC = 0) runs the recursion
// on its second centre and needs no transfer: the caller's c00 (d00) is then
// formed from P - B (Q - D), which the Fock pair tables store for such pairs.
template <int LA, int LB, int LC, int LD, typename T, typename Out>
__device__ __forceinline__ void twod(T g00, T c00, T d00, T b00, T b10, T b01, T ab, T cd, Out&& out) {
  constexpr int NMAX = LA + LB, MMAX = LC + LD;
  T G[NMAX + 1][MMAX + 1];
  G[0][0] = g00;
  if (NMAX > 0) G[1][0] = c00 * g00;
#pragma unroll
  for (int n = 1; n < NMAX; ++n) G[n + 1][0] = fma(c00, G[n][0], (T)n * b10 * G[n - 1][0]);
#pragma unroll
  for (int m = 0; m < MMAX; ++m) {
#pragma unroll
    for (int n = 0; n <= NMAX; ++n) {
      T v = d00 * G[n][m];
      if (m > 0) v = fma((T)m * b01, G[n][m - 1], v);
      if (n > 0) v = fma((T)n * b00, G[n - 1][m], v);
      G[n][m + 1] = v;
    }
  }
  // bra transfer: H[i][j][m]
  T H[LA + 1][LB + 1][MMAX + 1];
#pragma unroll
  for (int m = 0; m <= MMAX; ++m) {
    if constexpr (LA == 0) {
#pragma unroll
      for (int j = 0; j <= LB; ++j) H[0][j][m] = G[j][m];
    } else {
      T col[NMAX + 1];
#pragma unroll
      for (int i = 0; i <= NMAX; ++i) col[i] = G[i][m];
#pragma unroll
      for (int i = 0; i <= LA; ++i) H[i][0][m] = col[i];
#pragma unroll
      for (int j = 1; j <= LB; ++j) {
#pragma unroll
        for (int i = 0; i <= NMAX - j; ++i) col[i] = fma(ab, col[i], col[i + 1]);
#pragma unroll
        for (int i = 0; i <= LA; ++i) H[i][j][m] = col[i];
      }
    }
  }
  // ket transfer
#pragma unroll
  for (int i = 0; i <= LA; ++i)
#pragma unroll
    for (int j = 0; j <= LB; ++j) {
      if constexpr (LC == 0) {
#pragma unroll
        for (int l = 0; l <= LD; ++l) out((i * (LB + 1) + j) * (LD + 1) + l, H[i][j][l]);
      } else {
        T col[MMAX + 1];
#pragma unroll
        for (int k = 0; k <= MMAX; ++k) col[k] = H[i][j][k];
#pragma unroll
        for (int k = 0; k <= LC; ++k) out(((i * (LB + 1) + j) * (LC + 1) + k) * (LD + 1) + 0, col[k]);
#pragma unroll
        for (int l = 1; l <= LD; ++l) {
#pragma unroll
          for (int k = 0; k <= MMAX - l; ++k) col[k] = fma(cd, col[k], col[k + 1]);
#pragma unroll
          for (int k = 0; k <= LC; ++k) out(((i * (LB + 1) + j) * (LC + 1) + k) * (LD + 1) + l, col[k]);
        }
      }
    }
}

template <int LA, int LB, int LC, int LD>
struct Cls {
  static constexpr int NA = ncart(LA), NB = ncart(LB), NC = ncart(LC), ND = ncart(LD);
  static constexpr int NE = NA * NB * NC * ND;
  static constexpr int NR = (LA + LB + LC + LD) / 2 + 1;
  static constexpr int N2D = (LA + 1) * (LB + 1) * (LC + 1) * (LD + 1);
  // 2D-table offset of Cartesian element e along dimension dim
  __host__ __device__ static constexpr int off2d(int e, int dim) {
    return ((cart_e(LA, e / (NB * NC * ND), dim) * (LB + 1) + cart_e(LB, (e / (NC * ND)) % NB, dim)) * (LC + 1) +
            cart_e(LC, (e / ND) % NC, dim)) * (LD + 1) + cart_e(LD, e % ND, dim);
  }
  __host__ __device__ static constexpr double norm(int e) {
    return cart_norm(LA, e / (NB * NC * ND)) * cart_norm(LB, (e / (NC * ND)) % NB) * cart_norm(LC, (e / ND) % NC) *
           cart_norm(LD, e % ND);
  }
};

template <typename T>
__device__ __forceinline__ T pick3(int d, T a, T b, T c) { return d == 0 ? a : (d == 1 ? b : c); }

template <int LA, int LB, int LC, int LD, bool PURE>
struct Epi {
  static constexpr int A = naos(LA, PURE), B = naos(LB, PURE), C = naos(LC, PURE), D = naos(LD, PURE);
  static constexpr int NEP = A * B * C * D;
};

// In-register pure projection of one index of angular momentum L (compile-time
// dims; L < 2: copy); the Cartesian norms of the projected components are
// folded into the coefficients, so projected indices need no separate
// normalisation.
template <int D0, int D1, int D2, int D3, int POS, int L, typename T>
__device__ __forceinline__ void project_regs(const T* in, T* out) {
  constexpr int DIMS[4] = {D0, D1, D2, D3};
  constexpr int PRE = POS == 0 ? 1 : (POS == 1 ? D0 : (POS == 2 ? D0 * D1 : D0 * D1 * D2));
  constexpr int N = DIMS[POS];
  constexpr int POST = POS == 3 ? 1 : (POS == 2 ? D3 : (POS == 1 ? D2 * D3 : D1 * D2 * D3));
  if constexpr (L < 2) {
#pragma unroll
    for (int i = 0; i < PRE * N * POST; ++i) out[i] = in[i];
  } else {
    constexpr int NP = 2 * L + 1;
#pragma unroll
    for (int a = 0; a < PRE; ++a)
#pragma unroll
      for (int m = 0; m < NP; ++m)
#pragma unroll
        for (int p = 0; p < POST; ++p) {
          T v = 0;
#pragma unroll
          for (int c = 0; c < N; ++c)
            if (pure_coef(L, m, c) != 0.0)
              v = fma((T)(pure_coef(L, m, c) * cart_norm(L, c)), in[(a * N + c) * POST + p], v);
          out[(a * NP + m) * POST + p] = v;
        }
  }
}

__device__ __constant__ const double SQRT3_POW[5] = {1.0, 1.7320508075688772, 3.0, 5.196152422706632, 9.0};
__device__ __constant__ const float SQRT3_POWF[5] = {1.0f, 1.7320508075688772f, 3.0f, 5.196152422706632f, 9.0f};
template <typename T> __device__ __forceinline__ T sqrt3_pow(int n);
template <> __device__ __forceinline__ double sqrt3_pow<double>(int n) { return SQRT3_POW[n]; }
template <> __device__ __forceinline__ float sqrt3_pow<float>(int n) { return SQRT3_POWF[n]; }
// sqrt(3)^n as FP32 pairs (hi = round(v), lo = round(v - hi))
__device__ __constant__ const float2 SQRT3_POW_DF[5] = {{1.0f, 0.0f},
                                                       {1.7320507764816284f, 3.1087250107475484e-08f},
                                                       {3.0f, 0.0f},
                                                       {5.196152210235596f, 2.1247103632049402e-07f},
                                                       {9.0f, 0.0f}};
template <> __device__ __forceinline__ dfl sqrt3_pow<dfl>(int n) { return dfl(SQRT3_POW_DF[n].x, SQRT3_POW_DF[n].y); }

// sqrt(3)^n / 2^k, n <= 4, |k| <= 3: the component norms of a Cartesian element
// times the shell-identity factor and the petite-list weight, 2^-k.  FP64: a select of the constant and an
// integer subtraction from its exponent (exact), so the element pays one FP64
// multiply for both factors.
template <typename T> __device__ __forceinline__ T norm_pow(int n, int k) {
  return sqrt3_pow<T>(n) * (T)__int_as_float((127 - k) << 23);   // 2^-k, |k| <= 3
}
template <> __device__ __forceinline__ double norm_pow<double>(int n, int k) {
  const double c = n == 0 ? 1.0 : n == 1 ? 1.7320508075688772 : n == 2 ? 3.0 : n == 3 ? 5.196152422706632 : 9.0;
  return __longlong_as_double(__double_as_longlong(c) - ((long long)k << 52));
}
// sqrt(5)^n, n <= 4
template <typename T> __device__ __forceinline__ T sqrt5_pow(int n) {
  return (T)(n == 0 ? 1.0f : n == 1 ? 2.23606798f : n == 2 ? 5.0f : n == 3 ? 11.1803399f : 25.0f);
}
template <> __device__ __forceinline__ double sqrt5_pow<double>(int n) {
  return n == 0 ? 1.0 : n == 1 ? 2.2360679774997897 : n == 2 ? 5.0 : n == 3 ? 11.180339887498949 : 25.0;
}
template <> __device__ __forceinline__ dfl sqrt5_pow<dfl>(int n) {
  return dfl(n == 0 ? 1.0 : n == 1 ? 2.2360679774997897 : n == 2 ? 5.0 : n == 3 ? 11.180339887498949 : 25.0);
}

// Element cutoff |v| < cut -> 0 (cut > 0), decided on the bit patterns: for
// non-negative IEEE values the order of the magnitudes is the integer order of
// their bits, so no FP64 compare is spent.
__device__ __forceinline__ double cut_elem(double v, double cut) {
  const long long m = __double_as_longlong(v) & 0x7fffffffffffffffll;
  return m < __double_as_longlong(cut) ? 0.0 : v;
}
__device__ __forceinline__ float cut_elem(float v, float cut) {
  const int m = __float_as_int(v) & 0x7fffffff;
  return m < __float_as_int(cut) ? 0.0f : v;
}

// Persistent-warp work distribution: warps take chunks of the (sorted) class
// list from a global counter, heaviest quartets first.
__device__ __forceinline__ long long grab(unsigned long long* counter, unsigned chunk, int lane) {
  unsigned long long base = 0;
  if (lane == 0) base = atomicAdd(counter, (unsigned long long)chunk);
  return (long long)__shfl_sync(0xffffffffu, base, 0);
}

// The quartets this launch works on: [0, nquartets) of a.quartets, or the
// device-resident range [range[0], range[1]) when the launch was issued before
// the list lengths were known (device-driven builds, graph replay).
__device__ __forceinline__ void work_range(const BuildArgs& a, const uint2*& q, long long& n) {
  if (a.range) {
    const unsigned long long b = a.range[0], e = a.range[1];
    q = a.quartets + b;
    n = e > b ? (long long)(e - b) : 0;
  } else {
    q = a.quartets;
    n = a.nquartets;
  }
}

template <typename T>
__device__ __forceinline__ void quartet_geometry(const BuildArgs& a, uint2 qd, PairDev& P, PairDev& Q, T AB[3],
                                                 T CD[3]) {
  P = a.pairs[entry_pair(qd.x)];
  Q = a.pairs[qd.y];
  const ShellDev SA = a.shells[P.sha], SB = a.shells[P.shb], SC = a.shells[Q.sha], SD = a.shells[Q.shb];
  AB[0] = (T)(SA.x - SB.x); AB[1] = (T)(SA.y - SB.y); AB[2] = (T)(SA.z - SB.z);
  CD[0] = (T)(SC.x - SD.x); CD[1] = (T)(SC.y - SD.y); CD[2] = (T)(SC.z - SD.z);
}

// ===========================================================================
// Small classes (at most 108 Cartesian elements, 27 with an f shell):
// everything in registers.
//
// small_prims accumulates the primitive quartets c = first, first + step, ...
// (c = kq * nP + kb) of one contracted quartet.  Each iteration of the
// arithmetic body computes one surviving candidate of this lane: the cheap
// FP32 scan skips screened candidates without holding the warp in the body.
// The arithmetic body: primitive quartet (bra pair cb, ket pair cq) of one
// contracted quartet added into acc.  UNIT: with unit pair factors K/p (the
// shell-family kernels apply each member's factors afterwards).
template <int LA, int LB, int LC, int LD, typename T, bool ATT, bool UNIT = false>
__device__ __forceinline__ void prim_body(const BuildArgs& a, const typename PrimT<T>::type* bpp,
                                          const typename PrimT<T>::type* kpp, int cb, int cq, const T AB[3],
                                          const T CD[3], T* acc) {
  using K = Cls<LA, LB, LC, LD>;
  using PP = typename PrimT<T>::type;
  constexpr int NE = K::NE, NR = K::NR, N2D = K::N2D;
  PP bp, kp;
  prim_load(bpp + cb, bp);
  prim_load(kpp + cq, kp);
  if constexpr (UNIT) {
    bp.sp = (T)1;
    kp.sp = (T)1;
  }
  PrimQuartet<T> pq;
  prim_setup<T, ATT, LA + LB == 0>(bp, kp, pq, (T)a.inv_mu2);
#pragma unroll
  for (int r = 0; r < NR; ++r) {
    T u, w;
    rys_node_weight<NR, T>(pq.X, r, a.roots_f32 != 0, u, w);
    w *= pq.pref;
    const T uq = u * pq.qi, up = u * pq.pi;
    const T b00 = (T)0.5 * pq.inv * u;
    const T b10 = fma(-bp.hp, uq, bp.hp);
    const T b01 = fma(-kp.hp, up, kp.hp);
    T I[3][N2D];
    const T PA[3] = {bp.ax, bp.ay, bp.az}, QC[3] = {kp.ax, kp.ay, kp.az};
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const T c00 = fma(-uq, pq.PQ[d], PA[d]);
      const T d00 = fma(up, pq.PQ[d], QC[d]);
      twod<LA, LB, LC, LD, T>(d == 2 ? w : (T)1, c00, d00, b00, b10, b01, AB[d], CD[d],
                              [&](int i, T v) { I[d][i] = v; });
    }
#pragma unroll
    for (int e = 0; e < NE; ++e)
      acc[e] = fma(I[0][K::off2d(e, 0)] * I[1][K::off2d(e, 1)], I[2][K::off2d(e, 2)], acc[e]);
  }
}

// The screened primitive quartets c = first, first + step, ... (c = kq nP + kb)
// of one contracted quartet: body(kb, kq) for each that passes the screen.
template <typename PP, typename Body>
__device__ __forceinline__ void prim_loop_lane(const BuildArgs& a, const PP* bpp, const PP* kpp, int nP, int nQ,
                                               int first, int step, unsigned long long& nprim, Body&& body) {
  if (nP == 0 || nQ == 0) return;
  int kq = first / nP, kb = first - kq * nP;
  int kq_loaded = -1;
  float2 ks = make_float2(0.f, 1.f);
  for (;;) {
    int cb = -1, cq = -1;
    while (kq < nQ) {
      if (kq != kq_loaded) { ks = prim_screen(kpp + kq); kq_loaded = kq; }
      const int b = kb, q = kq;
      kb += step;
      while (kb >= nP) { kb -= nP; ++kq; }
      if (screen_keep(bpp + b, prim_screen(bpp + b), kpp + q, ks, a)) { cb = b; cq = q; break; }
    }
    if (cb < 0) break;
    ++nprim;
    body(cb, cq);
  }
}

template <int LA, int LB, int LC, int LD, typename T, bool ATT>
__device__ __forceinline__ void small_prims_impl(const BuildArgs& a, const PairDev& P, const PairDev& Q,
                                                 const T AB[3], const T CD[3], int first, int step, T* acc,
                                                 unsigned long long& nprim) {
  using PP = typename PrimT<T>::type;
  const PP* bpp = prims_of<T>(a) + P.poff;
  const PP* kpp = prims_of<T>(a) + Q.poff;
  prim_loop_lane(a, bpp, kpp, P.pcnt, Q.pcnt, first, step, nprim,
                 [&](int cb, int cq) { prim_body<LA, LB, LC, LD, T, ATT>(a, bpp, kpp, cb, cq, AB, CD, acc); });
}

// The attenuated (CAM) operator is a separate instance of the primitive
// loop, chosen once per quartet, so the plain loop carries no extra work.
template <int LA, int LB, int LC, int LD, typename T>
__device__ __forceinline__ void small_prims(const BuildArgs& a, const PairDev& P, const PairDev& Q, const T AB[3],
                                            const T CD[3], int first, int step, T* acc, unsigned long long& nprim) {
  if (a.inv_mu2 != 0.0) small_prims_impl<LA, LB, LC, LD, T, true>(a, P, Q, AB, CD, first, step, acc, nprim);
  else small_prims_impl<LA, LB, LC, LD, T, false>(a, P, Q, AB, CD, first, step, acc, nprim);
}

// All 32 lanes of a warp on the primitive quartets of ONE contracted quartet
// (the primitive-parallel kernels).  The lanes screen a window of 32
// candidates (one each, FP32), and the survivors are dealt to the lanes that
// hold none, in order; the arithmetic body runs only when every lane holds a
// survivor (or the candidates are exhausted), so its FP64 instructions issue
// on 32 lanes instead of on the lanes whose stride-32 slice happened to keep
// a candidate.  Each lane accumulates its survivors into its own acc; the
// caller reduces over the warp.
template <typename PP, typename Body>
__device__ __forceinline__ void prim_loop_warp(const BuildArgs& a, const PP* bpp, const PP* kpp, int nP, int nQ,
                                               int lane, unsigned long long& nprim, Body&& body) {
  const int total = nP * nQ;
  int hb = 0, hq = 0;   // the survivor this lane holds
  int held = 0;         // lanes [0, held) hold one (uniform over the warp)
  for (int w = 0; w < total; w += 32) {
    const int c = w + lane;
    bool keep = false;
    int cb = 0, cq = 0;
    if (c < total) {
      cq = c / nP;
      cb = c - cq * nP;
      keep = screen_keep(bpp + cb, prim_screen(bpp + cb), kpp + cq, prim_screen(kpp + cq), a);
    }
    unsigned m = __ballot_sync(0xffffffffu, keep);
    while (m) {
      const int s = __popc(m);
      const int take = s < 32 - held ? s : 32 - held;
      // lane held + j receives the (j+1)-th surviving candidate of the window
      const int j = lane - held;
      const bool mine = j >= 0 && j < take;
      const int src = mine ? (int)__fns(m, 0, j + 1) : 0;
      const int sb = __shfl_sync(0xffffffffu, cb, src), sq = __shfl_sync(0xffffffffu, cq, src);
      if (mine) { hb = sb; hq = sq; }
      const unsigned last = __fns(m, 0, take);   // position of the last survivor taken
      m = last >= 31u ? 0u : (m & ~((2u << last) - 1u));
      held += take;
      if (held == 32) {
        nprim += 1;
        body(hb, hq);
        held = 0;
      }
    }
  }
  if (lane < held) {
    nprim += 1;
    body(hb, hq);
  }
}

template <int LA, int LB, int LC, int LD, typename T, bool ATT>
__device__ __forceinline__ void warp_prims_impl(const BuildArgs& a, const PairDev& P, const PairDev& Q,
                                                const T AB[3], const T CD[3], int lane, T* acc,
                                                unsigned long long& nprim) {
  using PP = typename PrimT<T>::type;
  const PP* bpp = prims_of<T>(a) + P.poff;
  const PP* kpp = prims_of<T>(a) + Q.poff;
  prim_loop_warp(a, bpp, kpp, P.pcnt, Q.pcnt, lane, nprim,
                 [&](int cb, int cq) { prim_body<LA, LB, LC, LD, T, ATT>(a, bpp, kpp, cb, cq, AB, CD, acc); });
}

template <int LA, int LB, int LC, int LD, typename T>
__device__ __forceinline__ void warp_prims(const BuildArgs& a, const PairDev& P, const PairDev& Q, const T AB[3],
                                           const T CD[3], int lane, T* acc, unsigned long long& nprim) {
  if (a.inv_mu2 != 0.0) warp_prims_impl<LA, LB, LC, LD, T, true>(a, P, Q, AB, CD, lane, acc, nprim);
  else warp_prims_impl<LA, LB, LC, LD, T, false>(a, P, Q, AB, CD, lane, acc, nprim);
}

// Normalisation, pure projection, element cutoff and digestion of one
// contracted small-class quartet (single lane).
template <int LA, int LB, int LC, int LD, bool PURE, bool SCH, typename T>
__device__ __forceinline__ void small_epilogue(const BuildArgs& a, uint2 qd, const PairDev& P, const PairDev& Q,
                                               T* acc) {
  using K = Cls<LA, LB, LC, LD>;
  using E = Epi<LA, LB, LC, LD, PURE>;
  constexpr int NE = K::NE;
  const ShellDev SA = a.shells[P.sha], SB = a.shells[P.shb], SC = a.shells[Q.sha], SD = a.shells[Q.shb];
  // Cartesian d components carry their norms; projected (pure) indices get
  // them inside project_regs
#pragma unroll
  for (int e = 0; e < NE; ++e) acc[e] *= (T)(PURE ? 1.0 : K::norm(e));
  constexpr int DA = K::NA, DB = K::NB, DC = K::NC, DD = K::ND;
  T t1[NE], t2[NE];
  project_regs<DA, DB, DC, DD, 0, PURE ? LA : 0>(acc, t1);
  project_regs<E::A, DB, DC, DD, 1, PURE ? LB : 0>(t1, t2);
  project_regs<E::A, E::B, DC, DD, 2, PURE ? LC : 0>(t2, t1);
  project_regs<E::A, E::B, E::C, DD, 3, PURE ? LD : 0>(t1, t2);
  T* V = t2;
  if constexpr (SCH) {
    T m = 0;
#pragma unroll
    for (int e = 0; e < E::NEP; ++e) m = fmax(m, fabs(V[e]));
    a.schwarz_out[qd.x] = sqrt((double)m);
    return;
  }
  const T cut = (T)a.elem_cut;
  // the shell-identity factor f (a power of two) scales the block once, not
  // every digested target: exact, and NEP multiplies instead of one per atomic
  // times the petite-list orbit weight 2^w (w = 0 without symmetry)
  const int kf = (P.sha == P.shb) + (Q.sha == Q.shb) + (entry_pair(qd.x) == qd.y) - entry_wlog2(qd.x);
  const double f = __longlong_as_double((long long)(1023 - kf) << 52);   // 2^-kf, exact
  const T fT = (T)f;
#pragma unroll
  for (int e = 0; e < E::NEP; ++e) V[e] = cut_elem(V[e], cut) * fT;
  const int n = a.nbf;
  // columns within the molecule, rows in the stacked matrices
  const int oa = SA.aoff, ob = SB.aoff, oc = SC.aoff, od = SD.aoff;
  const int ra = SA.mrow + oa, rb = SB.mrow + ob, rc = SC.mrow + oc;
  // Coulomb: G_J[ab] += 2f sum_cd V D_cd ; G_J[cd] += 2f sum_ab V D_ab
  for (int jj = 0; jj < a.nj; ++jj) {
    const T* djt = dj_of<T>(a) + (size_t)jj * a.kstride;
    double* gj = a.gj + (size_t)jj * a.kstride;
    T dab[E::A * E::B], dcd[E::C * E::D];
#pragma unroll
    for (int i = 0; i < E::A; ++i)
#pragma unroll
      for (int j = 0; j < E::B; ++j) dab[i * E::B + j] = __ldg(djt + (size_t)(ra + i) * n + ob + j);
#pragma unroll
    for (int i = 0; i < E::C; ++i)
#pragma unroll
      for (int j = 0; j < E::D; ++j) dcd[i * E::D + j] = __ldg(djt + (size_t)(rc + i) * n + od + j);
    T jab[E::A * E::B], jcd[E::C * E::D];
#pragma unroll
    for (int i = 0; i < E::A * E::B; ++i) jab[i] = 0;
#pragma unroll
    for (int i = 0; i < E::C * E::D; ++i) jcd[i] = 0;
#pragma unroll
    for (int ab = 0; ab < E::A * E::B; ++ab)
#pragma unroll
      for (int cd = 0; cd < E::C * E::D; ++cd) {
        const T v = V[ab * E::C * E::D + cd];
        jab[ab] = fma(v, dcd[cd], jab[ab]);
        jcd[cd] = fma(v, dab[ab], jcd[cd]);
      }
#pragma unroll
    for (int i = 0; i < E::A; ++i)
#pragma unroll
      for (int j = 0; j < E::B; ++j)
        atomicAdd(gj + (size_t)(ra + i) * n + ob + j, (double)(jab[i * E::B + j] + jab[i * E::B + j]));
#pragma unroll
    for (int i = 0; i < E::C; ++i)
#pragma unroll
      for (int j = 0; j < E::D; ++j)
        atomicAdd(gj + (size_t)(rc + i) * n + od + j, (double)(jcd[i * E::D + j] + jcd[i * E::D + j]));
  }
  // Exchange: G_K[ac] += f sum V D_bd ; [ad] += f V D_bc ; [bc] += f V D_ad ; [bd] += f V D_ac
  for (int kk = 0; kk < a.nk; ++kk) {
    const T* dk = dk_of<T>(a) + (size_t)kk * a.kstride;
    double* gk = a.gk + (size_t)kk * a.kstride;
    T dac[E::A * E::C], dad[E::A * E::D], dbc[E::B * E::C], dbd[E::B * E::D];
#pragma unroll
    for (int i = 0; i < E::A; ++i) {
#pragma unroll
      for (int j = 0; j < E::C; ++j) dac[i * E::C + j] = __ldg(dk + (size_t)(ra + i) * n + oc + j);
#pragma unroll
      for (int j = 0; j < E::D; ++j) dad[i * E::D + j] = __ldg(dk + (size_t)(ra + i) * n + od + j);
    }
#pragma unroll
    for (int i = 0; i < E::B; ++i) {
#pragma unroll
      for (int j = 0; j < E::C; ++j) dbc[i * E::C + j] = __ldg(dk + (size_t)(rb + i) * n + oc + j);
#pragma unroll
      for (int j = 0; j < E::D; ++j) dbd[i * E::D + j] = __ldg(dk + (size_t)(rb + i) * n + od + j);
    }
    T kac[E::A * E::C], kad[E::A * E::D], kbc[E::B * E::C], kbd[E::B * E::D];
#pragma unroll
    for (int i = 0; i < E::A * E::C; ++i) kac[i] = 0;
#pragma unroll
    for (int i = 0; i < E::A * E::D; ++i) kad[i] = 0;
#pragma unroll
    for (int i = 0; i < E::B * E::C; ++i) kbc[i] = 0;
#pragma unroll
    for (int i = 0; i < E::B * E::D; ++i) kbd[i] = 0;
#pragma unroll
    for (int i = 0; i < E::A; ++i)
#pragma unroll
      for (int j = 0; j < E::B; ++j)
#pragma unroll
        for (int k = 0; k < E::C; ++k)
#pragma unroll
          for (int l = 0; l < E::D; ++l) {
            const T v = V[((i * E::B + j) * E::C + k) * E::D + l];
            kac[i * E::C + k] = fma(v, dbd[j * E::D + l], kac[i * E::C + k]);
            kad[i * E::D + l] = fma(v, dbc[j * E::C + k], kad[i * E::D + l]);
            kbc[j * E::C + k] = fma(v, dad[i * E::D + l], kbc[j * E::C + k]);
            kbd[j * E::D + l] = fma(v, dac[i * E::C + k], kbd[j * E::D + l]);
          }
#pragma unroll
    for (int i = 0; i < E::A; ++i) {
#pragma unroll
      for (int j = 0; j < E::C; ++j) atomicAdd(gk + (size_t)(ra + i) * n + oc + j, (double)kac[i * E::C + j]);
#pragma unroll
      for (int j = 0; j < E::D; ++j) atomicAdd(gk + (size_t)(ra + i) * n + od + j, (double)kad[i * E::D + j]);
    }
#pragma unroll
    for (int i = 0; i < E::B; ++i) {
#pragma unroll
      for (int j = 0; j < E::C; ++j) atomicAdd(gk + (size_t)(rb + i) * n + oc + j, (double)kbc[i * E::C + j]);
#pragma unroll
      for (int j = 0; j < E::D; ++j) atomicAdd(gk + (size_t)(rb + i) * n + od + j, (double)kbd[i * E::D + j]);
    }
  }
}

// One thread per quartet; warps take chunks of a.chunk (32 by default)
// consecutive quartets of the sorted list (similar primitive counts on all lanes).
template <int LA, int LB, int LC, int LD, bool PURE, bool SCH, typename T>
__global__ void __launch_bounds__(128) k_small(const BuildArgs a) {
  constexpr int NE = Cls<LA, LB, LC, LD>::NE;
  const int lane = threadIdx.x & 31;
  const uint2* quartets;
  long long nquartets;
  work_range(a, quartets, nquartets);
  unsigned long long nprim = 0;
  const unsigned chunk = a.chunk >= 32 ? (unsigned)a.chunk : 32u;
  for (;;) {
    const long long base = grab(a.work, chunk, lane);
    if (base >= nquartets) break;
    const long long end = base + chunk < nquartets ? base + chunk : nquartets;
    for (long long t = base + lane; t < end; t += 32) {
      const uint2 qd = quartets[t];
      PairDev P, Q;
      T AB[3], CD[3];
      quartet_geometry<T>(a, qd, P, Q, AB, CD);
      T acc[NE];
#pragma unroll
      for (int e = 0; e < NE; ++e) acc[e] = 0;
      small_prims<LA, LB, LC, LD, T>(a, P, Q, AB, CD, 0, 1, acc, nprim);
      small_epilogue<LA, LB, LC, LD, PURE, SCH, T>(a, qd, P, Q, acc);
    }
  }
  if (a.counters && nprim) atomicAdd(a.counters, nprim);
}

// Heavily contracted small-class quartets: one warp per quartet, the lanes
// split its primitive quartets, the partial blocks are summed across the warp.
template <int LA, int LB, int LC, int LD, bool PURE, typename T>
__global__ void __launch_bounds__(128) k_prim(const BuildArgs a) {
  constexpr int NE = Cls<LA, LB, LC, LD>::NE;
  const int lane = threadIdx.x & 31;
  const uint2* quartets;
  long long nquartets;
  work_range(a, quartets, nquartets);
  unsigned long long nprim = 0;
  for (;;) {
    const long long t = grab(a.work, 1u, lane);
    if (t >= nquartets) break;
    const uint2 qd = quartets[t];
    PairDev P, Q;
    T AB[3], CD[3];
    quartet_geometry<T>(a, qd, P, Q, AB, CD);
    T acc[NE];
#pragma unroll
    for (int e = 0; e < NE; ++e) acc[e] = 0;
    warp_prims<LA, LB, LC, LD, T>(a, P, Q, AB, CD, lane, acc, nprim);
#pragma unroll
    for (int e = 0; e < NE; ++e) {
      T v = acc[e];
#pragma unroll
      for (int s = 16; s > 0; s >>= 1) v += __shfl_xor_sync(0xffffffffu, v, s);
      acc[e] = v;
    }
    if (lane == 0) small_epilogue<LA, LB, LC, LD, PURE, false, T>(a, qd, P, Q, acc);
    __syncwarp();
  }
  if (a.counters && nprim) atomicAdd(a.counters, nprim);
}

// ===========================================================================
// Large classes: one warp per quartet.
// Order of the six digestion target kinds by decreasing dot-product length
// (stable: equal lengths keep their index order).
struct KindOrder {
  int k[6];
};
__host__ __device__ constexpr KindOrder kind_order(const int (&nt)[6]) {
  KindOrder o{{0, 1, 2, 3, 4, 5}};
  for (int i = 1; i < 6; ++i)
    for (int j = i; j > 0 && nt[o.k[j]] > nt[o.k[j - 1]]; --j) {
      const int t = o.k[j];
      o.k[j] = o.k[j - 1];
      o.k[j - 1] = t;
    }
  return o;
}

template <int LA, int LB, int LC, int LD, bool PURE>
struct TeamSmem {
  using K = Cls<LA, LB, LC, LD>;
  using E = Epi<LA, LB, LC, LD, PURE>;
  // primitive quartets that k_team evaluates side by side: each takes 3 NR
  // lanes in the 2D-table phase (one per root and dimension); the largest
  // classes, whose element phase dominates, keep one
  static constexpr int G = (K::NE > 400 || 32 / (3 * K::NR) < 1) ? 1 : 32 / (3 * K::NR);
  static constexpr int PH1 = G * (2 * K::NR + K::NR * 3 * K::N2D);
  static constexpr int DJ = E::A * E::B + E::C * E::D;
  static constexpr int DK = E::A * E::C + E::A * E::D + E::B * E::C + E::B * E::D;
  // [0, NE): the quartet's accumulators (lane-owned elements), then the
  // region shared by the primitive loop (roots, 2D tables), the pure
  // projection (NE) and the digestion (density blocks)
  static constexpr int REST = cmax(PH1, cmax(K::NE, DJ + 2 * DK));
  static constexpr int PER_WARP = K::NE + REST;   // elements of the kernel's type
  // exchange / Coulomb densities digested per pass: as many as the shared
  // region holds (at least 2 and 1), at most 8 each
  static constexpr int PK = cmin(8, (REST - DJ) / DK);
  static constexpr int PJ = cmax(1, cmin(8, (REST - PK * DK) / DJ));
};

// Epilogue of a warp-owned contracted quartet whose raw Cartesian block is in
// V = W[0, NE) (shared memory of the warp): normalisation, pure projection,
// element cutoff and the J/K digestion (or the Schwarz bound), the lanes
// splitting elements and targets.
template <int LA, int LB, int LC, int LD, bool PURE, bool SCH, typename T>
__device__ __forceinline__ void team_epilogue(const BuildArgs& a, uint2 qd, const PairDev& P, const PairDev& Q,
                                              T* W, int lane) {
  using K = Cls<LA, LB, LC, LD>;
  using E = Epi<LA, LB, LC, LD, PURE>;
  using SM = TeamSmem<LA, LB, LC, LD, PURE>;
  constexpr int NE = K::NE, KE = (NE + 31) / 32;
  T* V = W;
  const ShellDev SA = a.shells[P.sha], SB = a.shells[P.shb], SC = a.shells[Q.sha], SD = a.shells[Q.shb];
  // the shell-identity factor f = 1/2^k of the digestion (a power of two).  A
  // Cartesian block takes it in the same multiply as the component norms,
  // which is exact (V N f == (V N) f bit for bit), and its element cutoff
  // |V N| < tau becomes |V N f| < tau f; a block without norms is scaled only
  // when f != 1 (uniform over the warp).  Pure blocks are scaled after the
  // projection, the Schwarz pass not at all.
  // f = 2^-kf; the petite-list orbit weight 2^w of the entry enters as -w (w = 0 without symmetry)
  const int kf = (P.sha == P.shb) + (Q.sha == Q.shb) + (entry_pair(qd.x) == qd.y) - entry_wlog2(qd.x);
  const double f = __longlong_as_double((long long)(1023 - kf) << 52);   // 2^-kf, exact
  const T fT = (T)f;
  const int kn = (PURE || SCH) ? 0 : kf;   // the halvings the norm multiply carries
  constexpr bool NORMS = LA >= 2 || LB >= 2 || LC >= 2 || LD >= 2;
  // ---- epilogue: V = normalised block in smem, pure projection in place
  T* Tm = W + NE;
  if (NORMS || (!PURE && !SCH && f != 1.0)) {
#pragma unroll (KE <= 8 ? KE : 4)
    for (int k = 0; k < KE; ++k) {
      const int e = lane + 32 * k;
      if (e < NE) {
        const int ia = e / (K::NB * K::NC * K::ND), ib = (e / (K::NC * K::ND)) % K::NB, ic = (e / K::ND) % K::NC,
                  id = e % K::ND;
        // product of the component norms: sqrt(3)^n for n off-diagonal d components,
        // looked up rather than multiplied out (one FP64 multiply per element)
        if constexpr (NORMS) {
          // sqrt(3) per off-diagonal d component, sqrt(5) per f component xxy..yzz,
          // sqrt(15) = sqrt(3) sqrt(5) for xyz (shells_pnrm2)
          auto c3 = [](int l, int i) { return (l == 2 && i >= 3) || (l == 3 && i == 9); };
          auto c5 = [](int l, int i) { return l == 3 && i >= 3; };
          const int n3 = c3(LA, ia) + c3(LB, ib) + c3(LC, ic) + c3(LD, id);
          if constexpr (LA == 3 || LB == 3 || LC == 3 || LD == 3) {
            const int n5 = c5(LA, ia) + c5(LB, ib) + c5(LC, ic) + c5(LD, id);
            V[e] *= norm_pow<T>(n3, kn) * sqrt5_pow<T>(n5);
          } else {
            V[e] *= norm_pow<T>(n3, kn);
          }
        } else {
          V[e] *= fT;
        }
      }
    }
  }
  __syncwarp();
  int dims[4] = {K::NA, K::NB, K::NC, K::ND};
  if (PURE) {
    const int ls[4] = {LA, LB, LC, LD};
#pragma unroll
    for (int pos = 0; pos < 4; ++pos) {
      if (ls[pos] < 2) continue;
      int pre = 1, post = 1;
      for (int i = 0; i < pos; ++i) pre *= dims[i];
      for (int i = pos + 1; i < 4; ++i) post *= dims[i];
      if (ls[pos] == 2) {
        const int nout = pre * 5 * post;
        for (int o = lane; o < nout; o += 32) {
          const int p = o % post, m = (o / post) % 5, q = o / (5 * post);
          const T* src = V + (size_t)q * 6 * post + p;
          T v;
          if (m == 0) v = src[3 * post];
          else if (m == 1) v = src[5 * post];
          else if (m == 2) v = src[2 * post] - (T)0.5 * (src[0] + src[post]);
          else if (m == 3) v = src[4 * post];
          else v = (T)0.86602540378443865 * (src[0] - src[post]);
          Tm[o] = v;
        }
        __syncwarp();
        for (int o = lane; o < nout; o += 32) V[o] = Tm[o];
        __syncwarp();
        dims[pos] = 5;
      } else {  // f: 10 normalised Cartesians -> 7
        const int nout = pre * 7 * post;
        for (int o = lane; o < nout; o += 32) {
          const int p = o % post, m = (o / post) % 7, q = o / (7 * post);
          const T* src = V + (size_t)q * 10 * post + p;
          T v = 0;
#pragma unroll
          for (int c = 0; c < 10; ++c) {
            const double w = pure_f(m, c);
            if (w != 0.0) v = fma((T)w, src[c * post], v);
          }
          Tm[o] = v;
        }
        __syncwarp();
        for (int o = lane; o < nout; o += 32) V[o] = Tm[o];
        __syncwarp();
        dims[pos] = 7;
      }
    }
  }
  constexpr int NEP = E::NEP;
  if constexpr (SCH) {
    T m = 0;
    for (int e = lane; e < NEP; e += 32) m = fmax(m, fabs(V[e]));
#pragma unroll
    for (int s = 16; s > 0; s >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, s));
    if (lane == 0) a.schwarz_out[qd.x] = sqrt((double)m);
    __syncwarp();
    return;
  }
  const T cut = (T)a.elem_cut;
  if constexpr (PURE) {
    for (int e = lane; e < NEP; e += 32) V[e] = cut_elem(V[e], cut) * fT;
  } else {
    const T cutf = cut * fT;   // the block already carries f (exact)
    for (int e = lane; e < NEP; e += 32) V[e] = cut_elem(V[e], cutf);
  }
  // density blocks: up to PJ Coulomb and PK exchange densities per pass (one
  // pass for the SCF builds)
  const int n = a.nbf;
  const int oa = SA.aoff, ob = SB.aoff, oc = SC.aoff, od = SD.aoff;
  const int ra = SA.mrow + oa, rb = SB.mrow + ob, rc = SC.mrow + oc;
  constexpr int PJ = SM::PJ, PK = SM::PK, DJS = SM::DJ, DKS = SM::DK;
  T* Dj = W + NE;                  // after V (NE >= NEP); per Coulomb density: ab, cd
  T* Dk = Dj + PJ * DJS;           // per exchange density: ac, ad, bc, bd
  constexpr int NAB = E::A * E::B, NCD = E::C * E::D;
  constexpr int NAC = E::A * E::C, NAD = E::A * E::D, NBC = E::B * E::C, NBD = E::B * E::D;
  constexpr int BCD = E::B * E::C * E::D, CD_ = E::C * E::D;
  // target kinds 0..5 = J[ab], J[cd], K[ac], K[ad], K[bc], K[bd]; targets per
  // density and dot-product lengths
  constexpr int CNT[6] = {NAB, NCD, NAC, NAD, NBC, NBD};
  constexpr int NT[6] = {NCD, NAB, NBD, NBC, NAD, NAC};
  // kinds in order of decreasing dot length, so that the long dot products
  // share rounds of 32 lanes with each other rather than with short ones
  constexpr auto ORD = kind_order(NT);
  const int npj = (a.nj + PJ - 1) / PJ, npk = (a.nk + PK - 1) / PK;
  const int npass = npj > npk ? npj : npk;
  for (int pass = 0; pass < npass; ++pass) {
    const int j0 = pass * PJ, k0 = pass * PK;
    const int pj = a.nj - j0 >= PJ ? PJ : (a.nj - j0 > 0 ? a.nj - j0 : 0);
    const int pk = a.nk - k0 >= PK ? PK : (a.nk - k0 > 0 ? a.nk - k0 : 0);
    if (pass) __syncwarp();  // the previous pass has read its blocks
    for (int jj = 0; jj < pj; ++jj) {
      const T* djt = dj_of<T>(a) + (size_t)(j0 + jj) * a.kstride;
      T* dab = Dj + jj * DJS;
      for (int i = lane; i < NAB; i += 32) dab[i] = __ldg(djt + (size_t)(ra + i / E::B) * n + ob + i % E::B);
      for (int i = lane; i < NCD; i += 32) dab[NAB + i] = __ldg(djt + (size_t)(rc + i / E::D) * n + od + i % E::D);
    }
    for (int kk = 0; kk < pk; ++kk) {
      const T* dk = dk_of<T>(a) + (size_t)(k0 + kk) * a.kstride;
      T* base = Dk + kk * DKS;
      for (int i = lane; i < NAC; i += 32) base[i] = __ldg(dk + (size_t)(ra + i / E::C) * n + oc + i % E::C);
      base += NAC;
      for (int i = lane; i < NAD; i += 32) base[i] = __ldg(dk + (size_t)(ra + i / E::D) * n + od + i % E::D);
      base += NAD;
      for (int i = lane; i < NBC; i += 32) base[i] = __ldg(dk + (size_t)(rb + i / E::C) * n + oc + i % E::C);
      base += NBC;
      for (int i = lane; i < NBD; i += 32) base[i] = __ldg(dk + (size_t)(rb + i / E::D) * n + od + i % E::D);
    }
    __syncwarp();
    const int ntarget = (NAB + NCD) * pj + (NAC + NAD + NBC + NBD) * pk;
    // Every target element is a strided dot product of V with a density block:
    //   s = sum_{u < n1, v < n2} V[vb + u s1 + v s2] Dv[u n2 + v].
    // Only the (integer) descriptor depends on the target kind, so the lanes of
    // a round share one FP64 instruction stream whatever kinds they hold.
    for (int o = lane; o < ntarget; o += 32) {
      int r = o, kind = 0;
#pragma unroll
      for (int q = 0, found = 0; q < 6; ++q) {
        const int kd = ORD.k[q];
        const int cnt = CNT[kd] * (kd < 2 ? pj : pk);
        if (!found) {
          if (r < cnt) { kind = kd; found = 1; } else { r -= cnt; }
        }
      }
      const int di = r / CNT[kind], e = r - di * CNT[kind];
      int vb, s1, s2, n1, n2;
      const T* dv;
      double* dst;
      if (kind == 0) {  // J[a][b] += sum_cd V D[c][d]
        const int i = e / E::B, j = e % E::B;
        vb = e * NCD; s1 = 0; s2 = 1; n1 = 1; n2 = NCD; dv = Dj + di * DJS + NAB;
        dst = a.gj + (size_t)(j0 + di) * a.kstride + (size_t)(ra + i) * n + ob + j;
      } else if (kind == 1) {  // J[c][d] += sum_ab V D[a][b]
        const int k = e / E::D, l = e % E::D;
        vb = e; s1 = NCD; s2 = 0; n1 = NAB; n2 = 1; dv = Dj + di * DJS;
        dst = a.gj + (size_t)(j0 + di) * a.kstride + (size_t)(rc + k) * n + od + l;
      } else {
        const T* dk = Dk + di * DKS;
        double* gk = a.gk + (size_t)(k0 + di) * a.kstride;
        if (kind == 2) {  // K[a][c] += sum_bd V[a b c d] D[b][d]
          const int i = e / E::C, k = e % E::C;
          vb = i * BCD + k * E::D; s1 = CD_; s2 = 1; n1 = E::B; n2 = E::D; dv = dk + NAC + NAD + NBC;
          dst = gk + (size_t)(ra + i) * n + oc + k;
        } else if (kind == 3) {  // K[a][d] += sum_bc V D[b][c]
          const int i = e / E::D, l = e % E::D;
          vb = i * BCD + l; s1 = CD_; s2 = E::D; n1 = E::B; n2 = E::C; dv = dk + NAC + NAD;
          dst = gk + (size_t)(ra + i) * n + od + l;
        } else if (kind == 4) {  // K[b][c] += sum_ad V D[a][d]
          const int j = e / E::C, k = e % E::C;
          vb = j * CD_ + k * E::D; s1 = BCD; s2 = 1; n1 = E::A; n2 = E::D; dv = dk + NAC;
          dst = gk + (size_t)(rb + j) * n + oc + k;
        } else {  // K[b][d] += sum_ac V D[a][c]
          const int j = e / E::D, l = e % E::D;
          vb = j * CD_ + l; s1 = BCD; s2 = E::D; n1 = E::A; n2 = E::C; dv = dk;
          dst = gk + (size_t)(rb + j) * n + od + l;
        }
      }
      T s = 0;
      const int nt = n1 * n2;
      int u = 0, v = 0;
      for (int t = 0; t < nt; ++t) {
        s = fma(V[vb + u * s1 + v * s2], dv[t], s);
        if (++v == n2) { v = 0; ++u; }
      }
      atomicAdd(dst, (double)(kind < 2 ? s + s : s));   // Coulomb targets carry the factor 2
    }
  }
}

template <int LA, int LB, int LC, int LD, bool PURE, bool SCH, typename T>
__global__ void __launch_bounds__(128) k_team(const BuildArgs a) {
  using K = Cls<LA, LB, LC, LD>;
  using E = Epi<LA, LB, LC, LD, PURE>;
  using SM = TeamSmem<LA, LB, LC, LD, PURE>;
  using PP = typename PrimT<T>::type;
  constexpr int NE = K::NE, NR = K::NR, N2D = K::N2D, KE = (NE + 31) / 32;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  // packed 2D offsets (10 bits per dimension) of every Cartesian element,
  // shared by the CTA: keeping them out of registers leaves room for twod
  __shared__ int s_offs[NE];
  T* smem = reinterpret_cast<T*>(smem_raw);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  T* W = smem + warp * SM::PER_WARP;
  constexpr int G = SM::G;
  T* V = W;                // [NE] accumulators, then the normalised block
  T* RT = W + NE;          // [g][2 NR]: x_r, w_r * pref of group g
  T* I2 = RT + G * 2 * NR; // [g][r][d][N2D]
  // lane groups of 3 NR lanes, one primitive quartet each (lanes >= 3 NR G idle)
  const int grp = lane / (3 * NR), gl = lane - grp * (3 * NR);
  for (int e = threadIdx.x; e < NE; e += blockDim.x) {
    const int ia = e / (K::NB * K::NC * K::ND), ib = (e / (K::NC * K::ND)) % K::NB, ic = (e / K::ND) % K::NC,
              id = e % K::ND;
    int ox[3];
#pragma unroll
    for (int d = 0; d < 3; ++d)
      ox[d] = ((cart_e(LA, ia, d) * (LB + 1) + cart_e(LB, ib, d)) * (LC + 1) + cart_e(LC, ic, d)) * (LD + 1) +
              cart_e(LD, id, d);
    s_offs[e] = ox[0] | (ox[1] << 10) | (ox[2] << 20);
  }
  __syncthreads();
  const uint2* quartets;
  long long nquartets;
  work_range(a, quartets, nquartets);
  unsigned long long nprim = 0;
  for (;;) {
    const long long t = grab(a.work, 1u, lane);
    if (t >= nquartets) break;
    const uint2 qd = quartets[t];
    PairDev P, Q;
    T AB[3], CD[3];
    quartet_geometry<T>(a, qd, P, Q, AB, CD);
#pragma unroll (KE <= 8 ? KE : 4)
    for (int k = 0; k < KE; ++k)
      if (lane + 32 * k < NE) V[lane + 32 * k] = 0;
    const PP* bpp = prims_of<T>(a) + P.poff;
    const PP* kpp = prims_of<T>(a) + Q.poff;
    const int nP = P.pcnt, total = P.pcnt * Q.pcnt;
    // candidates c = kq nP + kb in windows of 32: each lane screens one, the
    // survivors are dealt to the lane groups G at a time (one instance of
    // the loop per operator: plain 1/r or the CAM pass's erf(mu r)/r)
    auto prim_loop = [&](auto att_tag) {
    constexpr bool ATT = decltype(att_tag)::value;
    for (int c0 = 0; c0 < total; c0 += 32) {
      bool keep = false;
      {
        const int c = c0 + lane;
        if (c < total) {
          const int kq = c / nP, kb = c - kq * nP;
          keep = screen_keep(bpp + kb, prim_screen(bpp + kb), kpp + kq, prim_screen(kpp + kq), a);
        }
      }
      unsigned mask = __ballot_sync(0xffffffffu, keep);
      while (mask) {
        const int avail = __popc(mask);
        const int ng = avail < G ? avail : G;
        // this group's candidate: the grp-th surviving one of the window
        unsigned m = mask;
        for (int i = 0; i < grp && i < ng; ++i) m &= m - 1;
        const int myc = c0 + __ffs(m) - 1;
        for (int i = 0; i < ng; ++i) mask &= mask - 1;
        nprim += ng;
        const bool active = grp < ng;
        PP bp, kp;
        PrimQuartet<T> pq;
        if (active) {
          const int kq = myc / nP, kb = myc - kq * nP;
          prim_load(bpp + kb, bp);
          prim_load(kpp + kq, kp);
          prim_setup<T, ATT>(bp, kp, pq, (T)a.inv_mu2);
          if (gl < 2 * NR) {
            const T v = rys_quantity<NR, T>(pq.X, gl, a.roots_f32 != 0);
            RT[grp * 2 * NR + gl] = (gl & 1) ? v * pq.pref : v;
          }
        }
        __syncwarp();
        if (active) {
          const int r = gl / 3, d = gl - 3 * r;
          const T u = RT[grp * 2 * NR + 2 * r], w = RT[grp * 2 * NR + 2 * r + 1];
          const T uq = u * pq.qi, up = u * pq.pi;
          const T b00 = (T)0.5 * pq.inv * u;
          const T b10 = fma(-bp.hp, uq, bp.hp);
          const T b01 = fma(-kp.hp, up, kp.hp);
          const T pqd = pick3(d, pq.PQ[0], pq.PQ[1], pq.PQ[2]);
          const T c00 = fma(-uq, pqd, pick3(d, bp.ax, bp.ay, bp.az));
          const T d00 = fma(up, pqd, pick3(d, kp.ax, kp.ay, kp.az));
          T* dst = I2 + ((grp * NR + r) * 3 + d) * N2D;
          twod<LA, LB, LC, LD, T>(d == 2 ? w : (T)1, c00, d00, b00, b10, b01, pick3(d, AB[0], AB[1], AB[2]),
                                  pick3(d, CD[0], CD[1], CD[2]), [&](int i, T v) { dst[i] = v; });
        }
        __syncwarp();
#pragma unroll (KE <= 8 ? KE : 4)
        for (int k = 0; k < KE; ++k) {
          const int e = lane + 32 * k;
          if (e < NE) {
            const int o = s_offs[e];
            const int ox = o & 1023, oy = (o >> 10) & 1023, oz = o >> 20;
            T v = V[e];
            for (int g = 0; g < ng; ++g) {
#pragma unroll
              for (int r = 0; r < NR; ++r) {
                const T* gt = I2 + (g * NR + r) * 3 * N2D;
                v = fma(gt[ox] * gt[N2D + oy], gt[2 * N2D + oz], v);
              }
            }
            V[e] = v;
          }
        }
        __syncwarp();
      }
    }
    };
    if (a.inv_mu2 != 0.0) prim_loop(std::true_type{});
    else prim_loop(std::false_type{});
    team_epilogue<LA, LB, LC, LD, PURE, SCH, T>(a, qd, P, Q, W, lane);
    __syncwarp();
  }
  if (a.counters && lane == 0 && nprim) atomicAdd(a.counters, nprim);
}

// Heavily contracted quartets of the warp-per-quartet classes whose Cartesian
// block and one root's 2D tables fit in registers: one warp per quartet, the
// lanes split the primitive quartets as in k_prim; a recursive-halving
// reduce-scatter sums the lanes' blocks (lane l ends with elements
// [KE l, KE l + KE)), which go to shared memory for the team epilogue.
template <int LA, int LB, int LC, int LD, bool PURE, typename T>
__global__ void __launch_bounds__(128) k_prim_team(const BuildArgs a) {
  using K = Cls<LA, LB, LC, LD>;
  using SM = TeamSmem<LA, LB, LC, LD, PURE>;
  constexpr int NE = K::NE, KE = (NE + 31) / 32, MP = 32 * KE;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* smem = reinterpret_cast<T*>(smem_raw);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  T* W = smem + warp * SM::PER_WARP;
  const uint2* quartets;
  long long nquartets;
  work_range(a, quartets, nquartets);
  unsigned long long nprim = 0;
  for (;;) {
    const long long t = grab(a.work, 1u, lane);
    if (t >= nquartets) break;
    const uint2 qd = quartets[t];
    PairDev P, Q;
    T AB[3], CD[3];
    quartet_geometry<T>(a, qd, P, Q, AB, CD);
    T acc[MP];
#pragma unroll
    for (int e = 0; e < MP; ++e) acc[e] = 0;
    warp_prims<LA, LB, LC, LD, T>(a, P, Q, AB, CD, lane, acc, nprim);
    // reduce-scatter over the 32 lanes: at each level keep the half selected
    // by the lane bit, add the partner's copy of it
#pragma unroll
    for (int lvl = 0; lvl < 5; ++lvl) {
      const int off = 16 >> lvl;
      const int m = MP >> (lvl + 1);
      const bool up = (lane & off) != 0;
#pragma unroll
      for (int j = 0; j < (MP >> 1); ++j) {
        if (j < m) {
          const T keep = up ? acc[m + j] : acc[j];
          const T send = up ? acc[j] : acc[m + j];
          acc[j] = keep + shfl_xor_t(send, off);
        }
      }
    }
#pragma unroll
    for (int j = 0; j < KE; ++j)
      if (KE * lane + j < NE) W[KE * lane + j] = acc[j];
    __syncwarp();
    team_epilogue<LA, LB, LC, LD, PURE, false, T>(a, qd, P, Q, W, lane);
    __syncwarp();
  }
  if (a.counters && nprim) atomicAdd(a.counters, nprim);
}

// Double-float ("df") variants of the thread-per-quartet and primitive-
// parallel kernels: the primitive loop (pair set-up, Rys roots and weights,
// 2D integrals, accumulation) runs in double-float on the FP32 pipe; the
// contracted block is converted to FP64 once per quartet and digested by the
// FP64 epilogue (measured: a double-float digestion is 3 % slower at C2).
template <int LA, int LB, int LC, int LD, bool PURE>
__global__ void __launch_bounds__(128) k_small_df(const BuildArgs a) {
  constexpr int NE = Cls<LA, LB, LC, LD>::NE;
  const int lane = threadIdx.x & 31;
  const uint2* quartets;
  long long nquartets;
  work_range(a, quartets, nquartets);
  unsigned long long nprim = 0;
  const unsigned chunk = a.chunk >= 32 ? (unsigned)a.chunk : 32u;
  for (;;) {
    const long long base = grab(a.work, chunk, lane);
    if (base >= nquartets) break;
    const long long end = base + chunk < nquartets ? base + chunk : nquartets;
    for (long long t = base + lane; t < end; t += 32) {
      const uint2 qd = quartets[t];
      PairDev P, Q;
      dfl AB[3], CD[3];
      quartet_geometry<dfl>(a, qd, P, Q, AB, CD);
      dfl acc[NE];
#pragma unroll
      for (int e = 0; e < NE; ++e) acc[e] = dfl();
      small_prims<LA, LB, LC, LD, dfl>(a, P, Q, AB, CD, 0, 1, acc, nprim);
      double accd[NE];
#pragma unroll
      for (int e = 0; e < NE; ++e) accd[e] = df_to_double(acc[e]);
      small_epilogue<LA, LB, LC, LD, PURE, false, double>(a, qd, P, Q, accd);
    }
  }
  if (a.counters && nprim) atomicAdd(a.counters, nprim);
}

template <int LA, int LB, int LC, int LD, bool PURE>
__global__ void __launch_bounds__(128) k_prim_df(const BuildArgs a) {
  constexpr int NE = Cls<LA, LB, LC, LD>::NE;
  const int lane = threadIdx.x & 31;
  const uint2* quartets;
  long long nquartets;
  work_range(a, quartets, nquartets);
  unsigned long long nprim = 0;
  for (;;) {
    const long long t = grab(a.work, 1u, lane);
    if (t >= nquartets) break;
    const uint2 qd = quartets[t];
    PairDev P, Q;
    dfl AB[3], CD[3];
    quartet_geometry<dfl>(a, qd, P, Q, AB, CD);
    dfl acc[NE];
#pragma unroll
    for (int e = 0; e < NE; ++e) acc[e] = dfl();
    warp_prims<LA, LB, LC, LD, dfl>(a, P, Q, AB, CD, lane, acc, nprim);
    double accd[NE];
#pragma unroll
    for (int e = 0; e < NE; ++e) {
      dfl v = acc[e];
#pragma unroll
      for (int s = 16; s > 0; s >>= 1)
        v = v + dfl(__shfl_xor_sync(0xffffffffu, v.hi, s), __shfl_xor_sync(0xffffffffu, v.lo, s));
      accd[e] = df_to_double(v);
    }
    if (lane == 0) small_epilogue<LA, LB, LC, LD, PURE, false, double>(a, qd, P, Q, accd);
    __syncwarp();
  }
  if (a.counters && nprim) atomicAdd(a.counters, nprim);
}

}  // namespace oqpg
