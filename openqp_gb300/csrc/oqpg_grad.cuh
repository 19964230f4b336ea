// Derivative-ERI kernels of the two-electron HF gradient, contracted on the
// fly with the two-particle density (nothing is stored).
//
// For a canonical shell quartet (ab|cd) in kernel orientation the kernels
// accumulate dE/dR for the centres A, B and C,
//   g_X = f sum_e Gamma_e d(ab|cd)_e / dX,
// and D follows from translational invariance, g_D = -(g_A + g_B + g_C).
// f halves for A = B, C = D and AB = CD (OpenQP grd2_rys.F90:1333-1346).
// The derivatives use the Gaussian rule d/dA_x phi_a = 2 alpha phi_{a+1x} -
// a_x phi_{a-1x} (grd2_rys.F90:848-868) on one Rys 2D table per root and
// dimension in which A and C are raised by one:
//   dA = 2 a I(a+1,b,c,d) - a_x I(a-1,b,c,d)
//   dB = 2 b [I(a+1,b,c,d) + (A-B) I(a,b,c,d)] - b_x I(a,b-1,c,d)   (HRR)
//   dC = 2 c I(a,b,c+1,d) - c_x I(a,b,c-1,d)
// The entries with both A and C raised are never used, so the root count of
// one raised shell suffices: NR = (la+lb+lc+ld+1)/2 + 1.
//
// The two-particle density is the symmetric bilinear form of OpenQP's
// get_density (source/modules/hf_gradient.F90:427-575),
//   Gamma = cj sym(X_ab Y_cd) - ckt sym(X_ac Y_bd + X_ad Y_bc) - cks (same with the spin pair)
// over Cartesian-effective matrices (AO density projected to Cartesian
// components with their norms folded in); X = Y = D gives the energy
// gradient, X != Y the geometry part of the adjoint of a Fock build.
//
//   k_grad_lane : small classes; one warp per quartet, the lanes split the
//                 primitive quartets, each lane keeps its 2D tables in registers.
//   k_grad_small: the same classes, one thread per quartet (the light
//                 quartets of a list sorted by primitive-pair product).
//   k_grad_team : larger classes; one warp per quartet, the tables of each
//                 primitive quartet go to shared memory (one root x dimension
//                 per lane), derivative tables are built by all lanes, each
//                 lane contracts its own Cartesian elements.
#pragma once
#include "oqpg_eri.cuh"

namespace oqpg {

struct GradArgs {
  const ShellDev* shells;
  const PairDev* pairs;     // same pair order as the Fock tables
  const PrimPair* prims;    // primitive pairs with OpenQP's gradient cutoffs
  const double* alpha;      // exponent of the pair's first shell, per primitive pair
  const PrimPairF* primsf;  // FP32 copies for the small-bound quartets of the precision split
  const float* alphaf;
  const float* xtf;         // FP32 copies of the Cartesian-effective matrices
  const float* ytf;
  const float* xsf;
  const float* ysf;
  int roots_f32;            // FP32 quartets: Rys roots/weights in FP32 too
  const uint2* quartets;
  long long nquartets;
  unsigned long long* work;
  const double* xt;         // Cartesian-effective matrices, ncart x ncart
  const double* yt;
  const double* xs;         // spin pair (null: none)
  const double* ys;
  int ncart;
  const int* coff;          // Cartesian offset of each shell
  const int* atom;          // atom of each shell
  double cj, ckt, cks;
  int pure;                 // screening value from the Cartesian-effective (pure) or AO (Cartesian) density
  const double* q;          // Schwarz bound per pair
  double cutoff2;           // quartet skipped if dabmax Q_P Q_Q < cutoff / 2
  double dtol2;             // (sp sq)^2 < dtol2 (p + q): primitive quartet skipped
  double dabcut2;           // (sp sq)^2 dabmax^2 < dabcut2 (p + q): skipped
  float sdtol, sdab;        // sqrt(dtol2), sqrt(dabcut2) for the FP32 pre-screen
  // MRSF form (mrsf != 0): eleven Cartesian-effective matrices d2a, d2b, p2a,
  // p2b, ball, bo2v, bo1v, bco1, bco2, o21v, co12 at mm + m ncart^2 and the
  // coefficients of grd2_mrsf_compute_data_t_get_density (mq with sgnk)
  int mrsf;
  const double* mm;
  double mcoul, mx, mx2, mq1, mq2, mq3;
  double inv_mu2;           // erf(mu r)/r pass of the CAM gradient: 1/mu^2 (0: 1/r)
  double* de;               // 3 x natom, accumulated
  unsigned long long* counters;  // [0] primitive quartets evaluated, [1] quartets evaluated
  int ctas_per_sm;
  int small;                // lane classes: one thread per quartet (k_grad_small)
};

template <typename T> struct GAcc;
template <> struct GAcc<double> {
  static __device__ __forceinline__ const PrimPair* prims(const GradArgs& g) { return g.prims; }
  static __device__ __forceinline__ double alpha(const GradArgs& g, int i) { return __ldg(g.alpha + i); }
  static __device__ __forceinline__ const double* xt(const GradArgs& g) { return g.xt; }
  static __device__ __forceinline__ const double* yt(const GradArgs& g) { return g.yt; }
  static __device__ __forceinline__ const double* xs(const GradArgs& g) { return g.xs; }
  static __device__ __forceinline__ const double* ys(const GradArgs& g) { return g.ys; }
};
template <> struct GAcc<float> {
  static __device__ __forceinline__ const PrimPairF* prims(const GradArgs& g) { return g.primsf; }
  static __device__ __forceinline__ float alpha(const GradArgs& g, int i) { return __ldg(g.alphaf + i); }
  static __device__ __forceinline__ const float* xt(const GradArgs& g) { return g.xtf; }
  static __device__ __forceinline__ const float* yt(const GradArgs& g) { return g.ytf; }
  static __device__ __forceinline__ const float* xs(const GradArgs& g) { return g.xsf; }
  static __device__ __forceinline__ const float* ys(const GradArgs& g) { return g.ysf; }
};

template <int LA, int LB, int LC, int LD>
struct GCls {
  using K = Cls<LA, LB, LC, LD>;
  static constexpr int NR = (LA + LB + LC + LD + 1) / 2 + 1;
  static constexpr int N2D = K::N2D;
  static constexpr int N2DX = (LA + 2) * (LB + 1) * (LC + 2) * (LD + 1);
  static constexpr int SA = (LB + 1) * (LC + 2) * (LD + 1), SB = (LC + 2) * (LD + 1), SC = LD + 1;
  __host__ __device__ static constexpr int ia(int e) { return e / (K::NB * K::NC * K::ND); }
  __host__ __device__ static constexpr int ib(int e) { return (e / (K::NC * K::ND)) % K::NB; }
  __host__ __device__ static constexpr int ic(int e) { return (e / K::ND) % K::NC; }
  __host__ __device__ static constexpr int id(int e) { return e % K::ND; }
  // offset of element e along dim in the extended (A, C raised) table
  __host__ __device__ static constexpr int xoff(int e, int dim) {
    return ((cart_e(LA, ia(e), dim) * (LB + 1) + cart_e(LB, ib(e), dim)) * (LC + 2) + cart_e(LC, ic(e), dim)) *
               (LD + 1) + cart_e(LD, id(e), dim);
  }
};

// MRSF two-particle density of grd2_mrsf_compute_data_t_get_density
// (modules/tdhf_mrsf_gradient.F90:404-601) at Cartesian-effective indices
// (i, j, k, l).  The reference's eight-term sums are regrouped: the
// co12 / o21v sums are twice four products, and its dc / dd sums pair up as
// dc(X, Y) = dc(Y, X), dd(X, Y) = dd(Y, X).
static __device__ __noinline__ double gamma_mrsf(const GradArgs& g, int i, int j, int k, int l) {
  const size_t n = (size_t)g.ncart, n2 = n * n;
  auto X = [&](int m, int r, int c) { return __ldg(g.mm + m * n2 + (size_t)r * n + c); };
  enum { A = 0, B = 1, P = 2, Q = 3, L = 4, V2 = 5, V1 = 6, K1 = 7, K2 = 8, O = 9, C = 10 };
  const double aij = X(A, i, j), pij = X(P, i, j);
  double df1 = g.mcoul * ((aij + pij) * X(A, k, l) + aij * X(P, k, l));
  if (g.mx != 0.0 || g.mx2 != 0.0) {
    const double aik = X(A, i, k), ail = X(A, i, l), bik = X(B, i, k), bil = X(B, i, l);
    const double dq1 = (aik + X(P, i, k)) * X(A, j, l) + aik * X(P, j, l) + (ail + X(P, i, l)) * X(A, j, k) +
                       ail * X(P, j, k) + (bik + X(Q, i, k)) * X(B, j, l) + bik * X(Q, j, l) +
                       (bil + X(Q, i, l)) * X(B, j, k) + bil * X(Q, j, k);
    const double dt2 = X(L, i, k) * X(L, j, l) + X(L, k, i) * X(L, l, j) + X(L, i, l) * X(L, j, k) +
                       X(L, l, i) * X(L, k, j);
    df1 -= g.mx * dq1 + 2.0 * g.mx2 * dt2;
  }
  auto four = [&](int m) {
    return X(m, i, k) * X(m, l, j) + X(m, i, l) * X(m, k, j) + X(m, j, k) * X(m, l, i) + X(m, j, l) * X(m, k, i);
  };
  if (g.mq1 != 0.0) df1 += 2.0 * g.mq1 * four(C);
  if (g.mq2 != 0.0) df1 += 2.0 * g.mq2 * four(O);
  if (g.mq3 != 0.0) {
    auto dc = [&](int x, int y) {
      return X(x, i, k) * X(y, j, l) + X(x, i, l) * X(y, j, k) + X(x, j, k) * X(y, i, l) + X(x, j, l) * X(y, i, k) +
             X(x, l, j) * X(y, k, i) + X(x, k, j) * X(y, l, i) + X(x, l, i) * X(y, k, j) + X(x, k, i) * X(y, l, j);
    };
    auto dd = [&](int x, int y) {
      return (X(x, i, j) + X(x, j, i)) * (X(y, k, l) + X(y, l, k)) +
             (X(x, k, l) + X(x, l, k)) * (X(y, i, j) + X(y, j, i));
    };
    df1 += 2.0 * g.mq3 * (dd(K1, V2) + dd(K2, V1) - dc(K1, V2) - dc(K2, V1));
  }
  return df1;
}

// Two-particle density of Cartesian element (ra, rb, rc, rd) (matrix rows /
// columns in the Cartesian layout).
template <typename T>
__device__ __forceinline__ T gamma_elem(const GradArgs& g, int ra, int rb, int rc, int rd) {
  if constexpr (std::is_same<T, double>::value) {
    if (g.mrsf) return gamma_mrsf(g, ra, rb, rc, rd);
  }
  const int n = g.ncart;
  const T* xt = GAcc<T>::xt(g);
  const T* yt = GAcc<T>::yt(g);
  auto X = [&](const T* M, int r, int c) { return __ldg(M + (size_t)r * n + c); };
  T v = (T)(0.5 * g.cj) * (X(xt, ra, rb) * X(yt, rc, rd) + X(yt, ra, rb) * X(xt, rc, rd));
  v -= (T)(0.5 * g.ckt) * (X(xt, ra, rc) * X(yt, rb, rd) + X(yt, ra, rc) * X(xt, rb, rd) +
                           X(xt, ra, rd) * X(yt, rb, rc) + X(yt, ra, rd) * X(xt, rb, rc));
  if (g.xs) {
    const T* xs = GAcc<T>::xs(g);
    const T* ys = GAcc<T>::ys(g);
    v -= (T)(0.5 * g.cks) * (X(xs, ra, rc) * X(ys, rb, rd) + X(ys, ra, rc) * X(xs, rb, rd) +
                             X(xs, ra, rd) * X(ys, rb, rc) + X(ys, ra, rd) * X(xs, rb, rc));
  }
  return v;
}

template <typename T>
__device__ __forceinline__ T warp_max(T v) {
#pragma unroll
  for (int s = 16; s > 0; s >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, s));
  return v;
}
template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int s = 16; s > 0; s >>= 1) v += __shfl_xor_sync(0xffffffffu, v, s);
  return v;
}

// Reduce the lanes' 9 partial sums (A, B, C x xyz), apply f, add to de.
// dE/dR of one quartet (one lane's acc) into de: f = 1/2 for A = B, C = D,
// AB = CD each; D from translational invariance.
template <typename T>
__device__ __forceinline__ void grad_write(const GradArgs& g, const PairDev& P, const PairDev& Q, uint2 qd,
                                           const T* acc) {
  {
    double f = 1.0;
    if (P.sha == P.shb) f *= 0.5;
    if (Q.sha == Q.shb) f *= 0.5;
    if (qd.x == qd.y) f *= 0.5;
    const int at[4] = {__ldg(g.atom + P.sha), __ldg(g.atom + P.shb), __ldg(g.atom + Q.sha), __ldg(g.atom + Q.shb)};
#pragma unroll
    for (int x = 0; x < 3; ++x) {
      const double a = f * (double)acc[x], b = f * (double)acc[3 + x], c = f * (double)acc[6 + x];
      atomicAdd(g.de + 3 * at[0] + x, a);
      atomicAdd(g.de + 3 * at[1] + x, b);
      atomicAdd(g.de + 3 * at[2] + x, c);
      atomicAdd(g.de + 3 * at[3] + x, -(a + b + c));
    }
  }
}

// warp-shared quartet: sum the lanes' acc, lane 0 writes
template <typename T>
__device__ __forceinline__ void grad_store(const GradArgs& g, const PairDev& P, const PairDev& Q, uint2 qd,
                                           T* acc, int lane) {
#pragma unroll
  for (int k = 0; k < 9; ++k) acc[k] = warp_sum(acc[k]);
  if (lane == 0) grad_write(g, P, Q, qd, acc);
}

template <typename T>
__device__ __forceinline__ void quartet_setup(const GradArgs& g, uint2 qd, PairDev& P, PairDev& Q, T AB[3],
                                              T CD[3], int ro[4]) {
  P = g.pairs[qd.x];
  Q = g.pairs[qd.y];
  const ShellDev SA = g.shells[P.sha], SB = g.shells[P.shb], SC = g.shells[Q.sha], SD = g.shells[Q.shb];
  AB[0] = (T)(SA.x - SB.x); AB[1] = (T)(SA.y - SB.y); AB[2] = (T)(SA.z - SB.z);
  CD[0] = (T)(SC.x - SD.x); CD[1] = (T)(SC.y - SD.y); CD[2] = (T)(SC.z - SD.z);
  ro[0] = __ldg(g.coff + P.sha); ro[1] = __ldg(g.coff + P.shb);
  ro[2] = __ldg(g.coff + Q.sha); ro[3] = __ldg(g.coff + Q.shb);
}

// Primitive-quartet screens of grd2_rys_compute (grd2_rys.F90:361-372),
// (sp sq)^2 < dtol2 s and (sp sq)^2 dabmax^2 < dabcut2 s with s = p + q (+ pq /
// mu^2 in the attenuated pass), written without the squares so that FP32
// quartets do not underflow.
template <typename T>
__device__ __forceinline__ bool grad_prim_skip(const GradArgs& g, T pfac, T dabmax, T s) {
  const T a = fabs(pfac), rs = sqrt(s);
  return a < (T)sqrt(g.dtol2) * rs || a * dabmax < (T)sqrt(g.dabcut2) * rs;
}

// grd2's primitive screens for primitive pairs b and k: kept or skipped.  In
// FP64 kernels the tests run in FP32 first (no FP64 square root) and in FP64
// only within 1e-4 of a threshold.
template <typename T>
__device__ __forceinline__ bool grad_prim_keep(const GradArgs& g, const typename PrimT<T>::type* b,
                                               const typename PrimT<T>::type* k, T dabmax) {
  if constexpr (std::is_same<T, double>::value) {
    const float2 bs = prim_screen(b), ks = prim_screen(k);
    const float af = fabsf(bs.x * ks.x);
    const float rsf = sqrtf(fmaf(bs.y * ks.y, (float)g.inv_mu2, bs.y + ks.y));
    const float t1 = g.sdtol * rsf, t2 = g.sdab * rsf, a2 = af * (float)dabmax;
    if (af < t1 * 0.9999f || a2 < t2 * 0.9999f) return false;
    if (af > t1 * 1.0001f && a2 > t2 * 1.0001f) return true;
  }
  const T pb = __ldg(&b->p), pk = __ldg(&k->p);
  return !grad_prim_skip<T>(g, __ldg(&b->sp) * __ldg(&k->sp), dabmax, fma(pb * pk, (T)g.inv_mu2, pb + pk));
}

// One primitive quartet (bra kb, ket kq) of a contracted quartet: skipped by
// grd2's primitive screens (returns false), or its derivative integrals
// contracted with the density block gam into acc (dA, dB, dC per dimension).
template <int LA, int LB, int LC, int LD, typename T>
__device__ __forceinline__ bool grad_prim_body(const GradArgs& g, const typename PrimT<T>::type* prims,
                                               const PairDev& P, const PairDev& Q, int kb, int kq, const T AB[3],
                                               const T CD[3], const T* gam, T dabmax, T* acc) {
  using K = Cls<LA, LB, LC, LD>;
  using G = GCls<LA, LB, LC, LD>;
  using PP = typename PrimT<T>::type;
  constexpr int NE = K::NE, NR = G::NR, N2DX = G::N2DX;
  if (!grad_prim_keep<T>(g, prims + P.poff + kb, prims + Q.poff + kq, dabmax)) return false;
  PP bp, kp;
  prim_load(prims + P.poff + kb, bp);
  prim_load(prims + Q.poff + kq, kp);
  PrimQuartet<T> pqd;
  prim_setup<T, true>(bp, kp, pqd, (T)g.inv_mu2);
  const T a2 = (T)2 * GAcc<T>::alpha(g, P.poff + kb);
  const T b2 = (T)2 * bp.p - a2;
  const T c2 = (T)2 * GAcc<T>::alpha(g, Q.poff + kq);
#pragma unroll
  for (int r = 0; r < NR; ++r) {
    T u, w;
    rys_node_weight<NR, T>(pqd.X, r, g.roots_f32 != 0, u, w);
    w *= pqd.pref;
    const T uq = u * pqd.qi, up = u * pqd.pi;
    const T b00 = (T)0.5 * pqd.inv * u;
    const T b10 = fma(-bp.hp, uq, bp.hp);
    const T b01 = fma(-kp.hp, up, kp.hp);
    T X[3][N2DX];
    const T PA[3] = {bp.ax, bp.ay, bp.az}, QC[3] = {kp.ax, kp.ay, kp.az};
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const T c00 = fma(-uq, pqd.PQ[d], PA[d]);
      const T d00 = fma(up, pqd.PQ[d], QC[d]);
      twod<LA + 1, LB, LC + 1, LD, T>(d == 2 ? w : (T)1, c00, d00, b00, b10, b01, AB[d], CD[d],
                                      [&](int i, T v) { X[d][i] = v; });
    }
#pragma unroll
    for (int e = 0; e < NE; ++e) {
      T I[3], dA[3], dB[3], dC[3];
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        const int o = G::xoff(e, d);
        const int ea = cart_e(LA, G::ia(e), d), eb = cart_e(LB, G::ib(e), d), ec = cart_e(LC, G::ic(e), d);
        I[d] = X[d][o];
        const T up1 = X[d][o + G::SA];
        dA[d] = a2 * up1;
        if (ea > 0) dA[d] = fma(-(T)ea, X[d][o - G::SA], dA[d]);
        dB[d] = b2 * fma(AB[d], I[d], up1);
        if (eb > 0) dB[d] = fma(-(T)eb, X[d][o - G::SB], dB[d]);
        dC[d] = c2 * X[d][o + G::SC];
        if (ec > 0) dC[d] = fma(-(T)ec, X[d][o - G::SC], dC[d]);
      }
      const T ge = gam[e];
      const T tz = ge * I[2];
      const T yz = I[1] * tz, xz = I[0] * tz, xy = I[0] * I[1] * ge;
      acc[0] = fma(dA[0], yz, acc[0]); acc[1] = fma(dA[1], xz, acc[1]); acc[2] = fma(dA[2], xy, acc[2]);
      acc[3] = fma(dB[0], yz, acc[3]); acc[4] = fma(dB[1], xz, acc[4]); acc[5] = fma(dB[2], xy, acc[5]);
      acc[6] = fma(dC[0], yz, acc[6]); acc[7] = fma(dC[1], xz, acc[7]); acc[8] = fma(dC[2], xy, acc[8]);
    }
  }
  return true;
}

// ---------------------------------------------------------------------------
template <int LA, int LB, int LC, int LD, typename T>
__global__ void __launch_bounds__(128) k_grad_lane(const GradArgs g) {
  using K = Cls<LA, LB, LC, LD>;
  using G = GCls<LA, LB, LC, LD>;
  using PP = typename PrimT<T>::type;
  constexpr int NE = K::NE;
  __shared__ T s_gam[4][NE];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  T* gam = s_gam[warp];
  const PP* prims = GAcc<T>::prims(g);
  unsigned long long nprim = 0, nq = 0;
  for (;;) {
    const long long t = grab(g.work, 1u, lane);
    if (t >= g.nquartets) break;
    const uint2 qd = g.quartets[t];
    PairDev P, Q;
    T AB[3], CD[3];
    int ro[4];
    quartet_setup<T>(g, qd, P, Q, AB, CD, ro);
    T dmx = 0;
    for (int e = lane; e < NE; e += 32) {
      const T v = gamma_elem<T>(g, ro[0] + G::ia(e), ro[1] + G::ib(e), ro[2] + G::ic(e), ro[3] + G::id(e));
      gam[e] = v;
      const T nrm = (T)(cart_norm(LA, G::ia(e)) * cart_norm(LB, G::ib(e)) * cart_norm(LC, G::ic(e)) *
                        cart_norm(LD, G::id(e)));
      dmx = fmax(dmx, g.pure ? fabs(v) : fabs(v) / nrm);
    }
    const T dabmax = warp_max(dmx);
    __syncwarp();
    if ((double)dabmax * __ldg(g.q + qd.x) * __ldg(g.q + qd.y) < g.cutoff2) continue;
    ++nq;
    T acc[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) acc[k] = 0;
    const int nP = P.pcnt, nQ = Q.pcnt;
    for (int pq = lane; pq < nP * nQ; pq += 32) {
      const int kq = pq / nP, kb = pq - kq * nP;
      if (grad_prim_body<LA, LB, LC, LD, T>(g, prims, P, Q, kb, kq, AB, CD, gam, dabmax, acc)) ++nprim;
    }
    grad_store<T>(g, P, Q, qd, acc, lane);
    __syncwarp();
  }
  if (g.counters) {
    if (nprim) atomicAdd(g.counters, nprim);
    if (lane == 0 && nq) atomicAdd(g.counters + 1, nq);
  }
}

// Thread per quartet for the same classes (the light quartets of a list
// sorted by primitive-pair product, heaviest first): warps take chunks of
// 32 quartets, each lane runs its quartet's primitive quartets alone, with
// the density block in registers.
template <int LA, int LB, int LC, int LD, typename T>
__global__ void __launch_bounds__(128) k_grad_small(const GradArgs g) {
  using K = Cls<LA, LB, LC, LD>;
  using G = GCls<LA, LB, LC, LD>;
  using PP = typename PrimT<T>::type;
  constexpr int NE = K::NE;
  const int lane = threadIdx.x & 31;
  const PP* prims = GAcc<T>::prims(g);
  unsigned long long nprim = 0, nq = 0;
  for (;;) {
    const long long base = grab(g.work, 32u, lane);
    if (base >= g.nquartets) break;
    const long long t = base + lane;
    if (t >= g.nquartets) continue;
    const uint2 qd = g.quartets[t];
    PairDev P, Q;
    T AB[3], CD[3];
    int ro[4];
    quartet_setup<T>(g, qd, P, Q, AB, CD, ro);
    T gam[NE];
    T dabmax = 0;
#pragma unroll
    for (int e = 0; e < NE; ++e) {
      const T v = gamma_elem<T>(g, ro[0] + G::ia(e), ro[1] + G::ib(e), ro[2] + G::ic(e), ro[3] + G::id(e));
      gam[e] = v;
      const T nrm = (T)(cart_norm(LA, G::ia(e)) * cart_norm(LB, G::ib(e)) * cart_norm(LC, G::ic(e)) *
                        cart_norm(LD, G::id(e)));
      dabmax = fmax(dabmax, g.pure ? fabs(v) : fabs(v) / nrm);
    }
    if ((double)dabmax * __ldg(g.q + qd.x) * __ldg(g.q + qd.y) < g.cutoff2) continue;
    ++nq;
    T acc[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) acc[k] = 0;
    for (int kq = 0; kq < Q.pcnt; ++kq)
      for (int kb = 0; kb < P.pcnt; ++kb)
        if (grad_prim_body<LA, LB, LC, LD, T>(g, prims, P, Q, kb, kq, AB, CD, gam, dabmax, acc)) ++nprim;
    grad_write(g, P, Q, qd, acc);
  }
  if (g.counters) {
    if (nprim) atomicAdd(g.counters, nprim);
    if (nq) atomicAdd(g.counters + 1, nq);
  }
}

// ---------------------------------------------------------------------------
template <int LA, int LB, int LC, int LD>
struct GradTeamSmem {
  using G = GCls<LA, LB, LC, LD>;
  // classes with more than 16 elements per lane keep the two-particle density
  // block in shared memory instead of registers (and loop over it unrolled by 4)
  static constexpr bool BIG = (Cls<LA, LB, LC, LD>::NE + 31) / 32 > 16;
  static constexpr int GM = BIG ? Cls<LA, LB, LC, LD>::NE : 0;
  // roots per pass of the table phases: all of them, or one at a time when
  // the tables of every root would not fit one warp's shared memory (the
  // largest f classes)
  static constexpr bool PR = 8 * (2 * G::NR + 3 * G::NR * G::N2DX + 12 * G::NR * G::N2D + GM) > 200 * 1024;
  static constexpr int RP = PR ? 1 : G::NR;
  // primitive quartets evaluated side by side (lane groups of 3 NR lanes in
  // the table phases), as long as their tables stay small
  static constexpr int NG0 = 32 / (3 * G::NR) > 0 ? 32 / (3 * G::NR) : 1;
  static constexpr int NG = (PR || 8 * NG0 * (3 * G::NR * G::N2DX + 12 * G::NR * G::N2D) > 48 * 1024) ? 1 : NG0;
  static constexpr int RTG = 2 * G::NR + 3;            // per group: x_r, w_r pref, then 2a, 2b, 2c
  static constexpr int RT = NG * RTG;
  static constexpr int XT = NG * 3 * RP * G::N2DX;
  static constexpr int TT = NG * 3 * RP * 4 * G::N2D;  // per group, root x dim: I, dA, dB, dC
  static constexpr int PER_WARP = RT + XT + TT + GM;   // elements of the kernel's type
};

template <int LA, int LB, int LC, int LD, typename T>
__global__ void __launch_bounds__(128) k_grad_team(const GradArgs g) {
  using K = Cls<LA, LB, LC, LD>;
  using G = GCls<LA, LB, LC, LD>;
  using SM = GradTeamSmem<LA, LB, LC, LD>;
  using PP = typename PrimT<T>::type;
  constexpr int NE = K::NE, NR = G::NR, N2D = G::N2D, N2DX = G::N2DX, KE = (NE + 31) / 32;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  T* W = reinterpret_cast<T*>(smem_raw) + (size_t)warp * SM::PER_WARP;
  T* RT = W;
  T* XT = W + SM::RT;
  T* TT = XT + SM::XT;
  const PP* prims = GAcc<T>::prims(g);
  constexpr bool BIG = SM::BIG;
  constexpr int KR = BIG ? 1 : KE;   // register-resident elements per lane
  T* GM = TT + SM::TT;               // BIG: the density block
  // this lane's elements: packed offsets into the per-dim tables
  int offs[KR];
  if constexpr (!BIG) {
#pragma unroll
    for (int k = 0; k < KE; ++k) {
      const int e = lane + 32 * k;
      int o = 0;
      if (e < NE) {
        int ox[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) ox[d] = K::off2d(e, d);
        o = ox[0] | (ox[1] << 10) | (ox[2] << 20);
      }
      offs[k] = o;
    }
  }
  unsigned long long nprim = 0, nq = 0;
  for (;;) {
    const long long t = grab(g.work, 1u, lane);
    if (t >= g.nquartets) break;
    const uint2 qd = g.quartets[t];
    PairDev P, Q;
    T AB[3], CD[3];
    int ro[4];
    quartet_setup<T>(g, qd, P, Q, AB, CD, ro);
    T gam[KR];
    T dmx = 0;
    if constexpr (BIG) {
#pragma unroll 4
      for (int e = lane; e < NE; e += 32) {
        const T v = gamma_elem<T>(g, ro[0] + G::ia(e), ro[1] + G::ib(e), ro[2] + G::ic(e), ro[3] + G::id(e));
        GM[e] = v;
        const T nrm = (T)(cart_norm(LA, G::ia(e)) * cart_norm(LB, G::ib(e)) * cart_norm(LC, G::ic(e)) *
                          cart_norm(LD, G::id(e)));
        dmx = fmax(dmx, g.pure ? fabs(v) : fabs(v) / nrm);
      }
    } else {
#pragma unroll
      for (int k = 0; k < KE; ++k) {
        const int e = lane + 32 * k;
        gam[k] = 0;
        if (e < NE) {
          const T v = gamma_elem<T>(g, ro[0] + G::ia(e), ro[1] + G::ib(e), ro[2] + G::ic(e), ro[3] + G::id(e));
          gam[k] = v;
          const T nrm = (T)(cart_norm(LA, G::ia(e)) * cart_norm(LB, G::ib(e)) * cart_norm(LC, G::ic(e)) *
                            cart_norm(LD, G::id(e)));
          dmx = fmax(dmx, g.pure ? fabs(v) : fabs(v) / nrm);
        }
      }
    }
    const T dabmax = warp_max(dmx);
    if ((double)dabmax * __ldg(g.q + qd.x) * __ldg(g.q + qd.y) < g.cutoff2) continue;
    ++nq;
    T acc[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) acc[k] = 0;
    // candidates c = kq nP + kb in windows of 32: each lane screens one, the
    // survivors are dealt to the NG lane groups of 3 RP lanes
    constexpr int NG = SM::NG, RP = SM::RP, RTG = SM::RTG;
    const int grp = lane / (3 * RP), gl = lane - grp * (3 * RP);
    const int nP = P.pcnt, total = P.pcnt * Q.pcnt;
    for (int c0 = 0; c0 < total; c0 += 32) {
      bool keep = false;
      {
        const int cand = c0 + lane;
        if (cand < total) {
          const int kq = cand / nP, kb = cand - kq * nP;
          keep = grad_prim_keep<T>(g, prims + P.poff + kb, prims + Q.poff + kq, dabmax);
        }
      }
      unsigned mask = __ballot_sync(0xffffffffu, keep);
      while (mask) {
        const int avail = __popc(mask);
        const int ng = avail < NG ? avail : NG;
        unsigned m = mask;
        for (int i = 0; i < grp && i < ng; ++i) m &= m - 1;
        const int myc = c0 + __ffs(m) - 1;
        for (int i = 0; i < ng; ++i) mask &= mask - 1;
        nprim += ng;
        const bool active = grp < ng;
        PP bp, kp;
        PrimQuartet<T> pqd;
        T* RTg = RT + grp * RTG;
        if (active) {
          const int kq = myc / nP, kb = myc - kq * nP;
          prim_load(prims + P.poff + kb, bp);
          prim_load(prims + Q.poff + kq, kp);
          prim_setup<T, true>(bp, kp, pqd, (T)g.inv_mu2);
          for (int q = gl; q < 2 * NR; q += 3 * RP) {  // groups of 3 lanes (one root per pass) loop
            const T v = rys_quantity<NR, T>(pqd.X, q, g.roots_f32 != 0);
            RTg[q] = (q & 1) ? v * pqd.pref : v;
          }
          if (gl == 0) {
            const T a2 = (T)2 * GAcc<T>::alpha(g, P.poff + kb);
            RTg[2 * NR] = a2;
            RTg[2 * NR + 1] = (T)2 * bp.p - a2;
            RTg[2 * NR + 2] = (T)2 * GAcc<T>::alpha(g, Q.poff + kq);
          }
        }
        __syncwarp();
        for (int r0 = 0; r0 < NR; r0 += RP) {
          if (active) {
            const int rl = gl / 3, d = gl - 3 * rl, r = r0 + rl;
            const T u = RTg[2 * r], w = RTg[2 * r + 1];
            const T uq = u * pqd.qi, up = u * pqd.pi;
            const T b00 = (T)0.5 * pqd.inv * u;
            const T b10 = fma(-bp.hp, uq, bp.hp);
            const T b01 = fma(-kp.hp, up, kp.hp);
            const T pqv = pick3(d, pqd.PQ[0], pqd.PQ[1], pqd.PQ[2]);
            const T c00 = fma(-uq, pqv, pick3(d, bp.ax, bp.ay, bp.az));
            const T d00 = fma(up, pqv, pick3(d, kp.ax, kp.ay, kp.az));
            T* dst = XT + ((grp * RP + rl) * 3 + d) * N2DX;
            twod<LA + 1, LB, LC + 1, LD, T>(d == 2 ? w : (T)1, c00, d00, b00, b10, b01,
                                            pick3(d, AB[0], AB[1], AB[2]), pick3(d, CD[0], CD[1], CD[2]),
                                            [&](int i, T v) { dst[i] = v; });
          }
          __syncwarp();
          // derivative tables: per group, root x dim: I, dA, dB, dC over the unraised entries
          for (int idx = lane; idx < ng * 3 * RP * N2D; idx += 32) {
            const int grd = idx / N2D, n = idx - grd * N2D, d = grd % 3, gg = grd / (3 * RP);
            const T* Rg = RT + gg * RTG;
            const T a2 = Rg[2 * NR], b2 = Rg[2 * NR + 1], c2 = Rg[2 * NR + 2];
            const int a = n / ((LB + 1) * (LC + 1) * (LD + 1)), b = (n / ((LC + 1) * (LD + 1))) % (LB + 1),
                      c = (n / (LD + 1)) % (LC + 1), dd = n % (LD + 1);
            const int o = ((a * (LB + 1) + b) * (LC + 2) + c) * (LD + 1) + dd;
            const T* X = XT + grd * N2DX;
            const T i0 = X[o], up1 = X[o + G::SA];
            T vA = a2 * up1, vB = b2 * fma(pick3(d, AB[0], AB[1], AB[2]), i0, up1), vC = c2 * X[o + G::SC];
            if (a > 0) vA = fma(-(T)a, X[o - G::SA], vA);
            if (b > 0) vB = fma(-(T)b, X[o - G::SB], vB);
            if (c > 0) vC = fma(-(T)c, X[o - G::SC], vC);
            T* Tb = TT + grd * 4 * N2D;
            Tb[n] = i0;
            Tb[N2D + n] = vA;
            Tb[2 * N2D + n] = vB;
            Tb[3 * N2D + n] = vC;
          }
          __syncwarp();
          auto contract = [&](int ox, int oy, int oz, T ge) {
            for (int gg = 0; gg < ng; ++gg) {
#pragma unroll
              for (int r = 0; r < RP; ++r) {
                const T* tx = TT + ((gg * RP + r) * 3 + 0) * 4 * N2D;
                const T* ty = TT + ((gg * RP + r) * 3 + 1) * 4 * N2D;
                const T* tz = TT + ((gg * RP + r) * 3 + 2) * 4 * N2D;
                const T ix = tx[ox], iy = ty[oy], iz = tz[oz];
                const T t1 = ge * iz;
                const T yz = iy * t1, xz = ix * t1, xy = ix * iy * ge;
                acc[0] = fma(tx[N2D + ox], yz, acc[0]);
                acc[1] = fma(ty[N2D + oy], xz, acc[1]);
                acc[2] = fma(tz[N2D + oz], xy, acc[2]);
                acc[3] = fma(tx[2 * N2D + ox], yz, acc[3]);
                acc[4] = fma(ty[2 * N2D + oy], xz, acc[4]);
                acc[5] = fma(tz[2 * N2D + oz], xy, acc[5]);
                acc[6] = fma(tx[3 * N2D + ox], yz, acc[6]);
                acc[7] = fma(ty[3 * N2D + oy], xz, acc[7]);
                acc[8] = fma(tz[3 * N2D + oz], xy, acc[8]);
              }
            }
          };
          if constexpr (BIG) {
#pragma unroll 4
            for (int e = lane; e < NE; e += 32) contract(K::off2d(e, 0), K::off2d(e, 1), K::off2d(e, 2), GM[e]);
          } else {
#pragma unroll
            for (int k = 0; k < KE; ++k) {
              if (lane + 32 * k < NE)
                contract(offs[k] & 1023, (offs[k] >> 10) & 1023, offs[k] >> 20, gam[k]);
            }
          }
          __syncwarp();
        }
      }
    }
    grad_store<T>(g, P, Q, qd, acc, lane);
    __syncwarp();
  }
  if (g.counters) {
    if (lane == 0 && nprim) atomicAdd(g.counters, nprim);
    if (lane == 0 && nq) atomicAdd(g.counters + 1, nq);
  }
}

// Classes whose per-lane tables (3 x N2DX doubles per root) stay small run
// lane-parallel over primitive quartets.
template <int LA, int LB, int LC, int LD>
constexpr bool grad_lane_class() { return 3 * GCls<LA, LB, LC, LD>::N2DX <= 48; }

// g.small: the thread-per-quartet kernel (lane classes only)
template <int LA, int LB, int LC, int LD, typename T>
cudaError_t launch_grad_t(const GradArgs& g, int nsm, cudaStream_t st) {
  if (g.nquartets <= 0) return cudaSuccess;
  if constexpr (grad_lane_class<LA, LB, LC, LD>()) {
    if (g.small) {
      auto kern = k_grad_small<LA, LB, LC, LD, T>;
      int per_sm = 1;
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 128, 0);
      if (g.ctas_per_sm > 0 && g.ctas_per_sm < per_sm) per_sm = g.ctas_per_sm;
      if (per_sm < 1) per_sm = 1;
      long long blocks = (g.nquartets + 127) / 128;
      if (blocks > (long long)nsm * per_sm) blocks = (long long)nsm * per_sm;
      kern<<<(unsigned)blocks, 128, 0, st>>>(g);
      return cudaGetLastError();
    }
    auto kern = k_grad_lane<LA, LB, LC, LD, T>;
    int per_sm = 1;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 128, 0);
    if (g.ctas_per_sm > 0 && g.ctas_per_sm < per_sm) per_sm = g.ctas_per_sm;
    if (per_sm < 1) per_sm = 1;
    long long blocks = (g.nquartets + 3) / 4;
    if (blocks > (long long)nsm * per_sm) blocks = (long long)nsm * per_sm;
    kern<<<(unsigned)blocks, 128, 0, st>>>(g);
  } else {
    auto kern = k_grad_team<LA, LB, LC, LD, T>;
    constexpr size_t per_warp = sizeof(T) * GradTeamSmem<LA, LB, LC, LD>::PER_WARP;
    int warps = (int)((200 * 1024) / per_warp);
    if (warps > 4) warps = 4;
    if (warps < 1) warps = 1;
    const size_t smem = per_warp * warps;
    if (smem > 48 * 1024) {
      cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return e;
    }
    int per_sm = 1;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 32 * warps, smem);
    if (g.ctas_per_sm > 0 && g.ctas_per_sm < per_sm) per_sm = g.ctas_per_sm;
    if (per_sm < 1) per_sm = 1;
    long long blocks = (g.nquartets + warps - 1) / warps;
    if (blocks > (long long)nsm * per_sm) blocks = (long long)nsm * per_sm;
    kern<<<(unsigned)blocks, 32 * warps, smem, st>>>(g);
  }
  return cudaGetLastError();
}

// f32: the FP32 quartets of the precision split.
template <int LA, int LB, int LC, int LD>
cudaError_t launch_grad_cls(const GradArgs& g, bool f32, int nsm, cudaStream_t st) {
  return f32 ? launch_grad_t<LA, LB, LC, LD, float>(g, nsm, st) : launch_grad_t<LA, LB, LC, LD, double>(g, nsm, st);
}

}  // namespace oqpg
