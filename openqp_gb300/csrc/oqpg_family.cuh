// Device code of the shell-family quartets (oqpg_family.cu describes the
// scheme): accumulators, the primitive body, the digestion of the member
// quartets and the thread- and warp-per-family-quartet kernels, templated on
// the class and the arithmetic type (FP64, FP32, double-float).
#pragma once
#include "oqpg_launch.cuh"

namespace oqpg {

// ---------------------------------------------------------------------------
// Family-quartet integrals.
template <int LA, int LB, int LC, int LD>
struct FamCls {
  static constexpr int MB = fam_members_max(LA, LB), MK = fam_members_max(LC, LD);
  static constexpr int NE = Cls<LA, LB, LC, LD>::NE;
  static constexpr int NACC = MB * MK * NE;   // member combination (m, n), element e at (m MK + n) NE + e
};

// The primitive-quartet screen of member combination (m, n):
// (K_m/p K_n/q)^2 < prim_cut2 (p + q) drops it (int_rotaxis.F90:629), in FP32
// outside the narrow band around the cutoff, else in FP64; the FP32 family
// quartets decide in FP32 at the middle of the band, as the FP32 shell
// quartets do.
template <typename T>
__device__ __forceinline__ bool fam_keep(const BuildArgs& a, float r, T spm, T sqn, const PrimPair* bp,
                                         const PrimPair* kp) {
  if (r < a.prim_cut_lo) return false;
  if (r > a.prim_cut_hi) return true;
  const double f = (double)spm * (double)sqn;
  return !(f * f < a.prim_cut2 * (__ldg(&bp->p) + __ldg(&kp->p)));
}
template <>
__device__ __forceinline__ bool fam_keep<float>(const BuildArgs& a, float r, float, float, const PrimPair*,
                                                const PrimPair*) {
  return !(r < 0.5f * (a.prim_cut_lo + a.prim_cut_hi));
}
// double-float family quartets: the FP32 decision at the middle of the band
// too (a combination within 1e-4 of the cutoff adds below 1e-14 either way)
template <>
__device__ __forceinline__ bool fam_keep<dfl>(const BuildArgs& a, float r, dfl, dfl, const PrimPair*,
                                              const PrimPair*) {
  return !(r < 0.5f * (a.prim_cut_lo + a.prim_cut_hi));
}

// union primitive pairs and member factors in the kernel's arithmetic type
template <typename T> __device__ __forceinline__ const typename PrimT<T>::type* fprims_of(const BuildArgs& a);
template <> __device__ __forceinline__ const PrimPair* fprims_of<double>(const BuildArgs& a) { return a.fprims; }
template <> __device__ __forceinline__ const PrimPairF* fprims_of<float>(const BuildArgs& a) { return a.fprimsf; }
template <> __device__ __forceinline__ const PrimPairDF* fprims_of<dfl>(const BuildArgs& a) { return a.fprimsdf; }
template <typename T> __device__ __forceinline__ T fam_coef(const FamCoef& c, int m);
template <> __device__ __forceinline__ double fam_coef<double>(const FamCoef& c, int m) { return __ldg(&c.sp[m]); }
template <> __device__ __forceinline__ float fam_coef<float>(const FamCoef& c, int m) { return __ldg(&c.spf[m]); }
// (the double-float factors live in a parallel FamCoefDF array: fam_coef_df)
__device__ __forceinline__ dfl fam_coef_df(const FamCoefDF& c, int m) {
  const float2 v = __ldg(&c.sp[m]);
  return dfl(v.x, v.y);
}

// K/p of member m on union primitive pair i of the pair table starting at co
// (FamCoef; the double-float copy at the same index of a.fcoefdf)
template <typename T>
__device__ __forceinline__ T member_factor(const BuildArgs& a, const FamCoef* co, int i, int m) {
  if constexpr (std::is_same<T, dfl>::value) return fam_coef_df(a.fcoefdf[(co - a.fcoef) + i], m);
  else return fam_coef<T>(co[i], m);
}

// Accumulators of one family quartet in one lane, with the ket factors of
// the current ket primitive (the union primitive quartets arrive in
// increasing c = kq nP + kb, so they are loaded once per ket primitive).
template <int LA, int LB, int LC, int LD, typename T>
struct FamAcc {
  using F = FamCls<LA, LB, LC, LD>;
  T acc[F::NACC];
  T sq[F::MK];
  float sqf[F::MK];
  int kq = -1;
};

template <int LA, int LB, int LC, int LD, typename T>
__device__ __forceinline__ void fam_acc_init(FamAcc<LA, LB, LC, LD, T>& s) {
  using F = FamCls<LA, LB, LC, LD>;
#pragma unroll
  for (int i = 0; i < F::NACC; ++i) s.acc[i] = (T)0;
  s.kq = -1;
}

// One union primitive quartet (bra cb, ket cq): the block with unit pair
// factors, then each member combination's share, K_m/p K_n/q, or nothing
// where the combination's own primitive-quartet screen drops the quartet.
// nb, nk: members of the two family pairs.  (Taking the ket factors out of
// each ket-primitive row instead, NE x nb FMAs per quartet plus a flush per
// row, measured slower: after screening the rows are short.)
template <int LA, int LB, int LC, int LD, typename T>
__device__ __forceinline__ void fam_body(const BuildArgs& a, const typename PrimT<T>::type* bpp,
                                         const typename PrimT<T>::type* kpp, const FamCoef* bco,
                                         const FamCoef* kco, int cb, int cq, const T AB[3], const T CD[3], int nb,
                                         int nk, FamAcc<LA, LB, LC, LD, T>& s) {
  using F = FamCls<LA, LB, LC, LD>;
  constexpr int NE = F::NE, MB = F::MB, MK = F::MK;
  if (cq != s.kq) {
    s.kq = cq;
#pragma unroll
    for (int n = 0; n < MK; ++n) {
      s.sq[n] = member_factor<T>(a, kco, cq, n);
      s.sqf[n] = fabsf(__ldg(&kco[cq].spf[n]));
    }
  }
  T v[NE];
#pragma unroll
  for (int e = 0; e < NE; ++e) v[e] = (T)0;
  prim_body<LA, LB, LC, LD, T, false, true>(a, bpp, kpp, cb, cq, AB, CD, v);
  const float rs = rsqrtf(prim_screen(bpp + cb).y + prim_screen(kpp + cq).y);
  // FP64 band decisions read the FP64 union pairs
  const PrimPair* bp64 = a.fprims + (bpp - fprims_of<T>(a)) + cb;
  const PrimPair* kp64 = a.fprims + (kpp - fprims_of<T>(a)) + cq;
#pragma unroll
  for (int m = 0; m < MB; ++m) {
    if (m >= nb) break;
    const T spm = member_factor<T>(a, bco, cb, m);
    const float spmf = fabsf(__ldg(&bco[cb].spf[m]));
    if constexpr (NE == 1) {
      const T t = spm * v[0];
#pragma unroll
      for (int n = 0; n < MK; ++n) {
        if (n >= nk) break;
        const bool keep = fam_keep<T>(a, spmf * s.sqf[n] * rs, spm, s.sq[n], bp64, kp64);
        s.acc[m * MK + n] = fma(keep ? s.sq[n] : (T)0, t, s.acc[m * MK + n]);
      }
    } else {
#pragma unroll
      for (int n = 0; n < MK; ++n) {
        if (n >= nk) break;
        const bool keep = fam_keep<T>(a, spmf * s.sqf[n] * rs, spm, s.sq[n], bp64, kp64);
        const T f = keep ? spm * s.sq[n] : (T)0;
#pragma unroll
        for (int e = 0; e < NE; ++e) s.acc[(m * MK + n) * NE + e] = fma(f, v[e], s.acc[(m * MK + n) * NE + e]);
      }
    }
  }
}

// Family quartet geometry: representative shells of the two family pairs.
template <typename T>
__device__ __forceinline__ void fam_geometry(const BuildArgs& a, const PairDev& P, const PairDev& Q, T AB[3],
                                             T CD[3]) {
  const ShellDev SA = a.shells[P.sha], SB = a.shells[P.shb], SC = a.shells[Q.sha], SD = a.shells[Q.shb];
  AB[0] = (T)(SA.x - SB.x); AB[1] = (T)(SA.y - SB.y); AB[2] = (T)(SA.z - SB.z);
  CD[0] = (T)(SC.x - SD.x); CD[1] = (T)(SC.y - SD.y); CD[2] = (T)(SC.z - SD.z);
}

// Member combination k = m MK + n of a family quartet digested as the shell
// quartet (member m of the bra family pair | member n of the ket's): its
// block is copied out of acc by compile-time selects (one epilogue instance).
template <int LA, int LB, int LC, int LD, bool PURE, typename T>
__device__ __forceinline__ void fam_digest(const BuildArgs& a, const FamMem& mb, const FamMem& mk, int k,
                                           const T* acc) {
  using F = FamCls<LA, LB, LC, LD>;
  constexpr int NE = F::NE, MB = F::MB, MK = F::MK;
  T blk[NE];
  int P = 0, Q = 0;
#pragma unroll
  for (int e = 0; e < NE; ++e) blk[e] = (T)0;
#pragma unroll
  for (int kk = 0; kk < MB * MK; ++kk)
    if (kk == k) {
#pragma unroll
      for (int e = 0; e < NE; ++e) blk[e] = acc[kk * NE + e];
      P = mb.m[kk / MK];
      Q = mk.m[kk % MK];
    }
  small_epilogue<LA, LB, LC, LD, PURE, false, T>(a, make_uint2((unsigned)P, (unsigned)Q), a.pairs[P], a.pairs[Q],
                                                blk);
}

// Arithmetic of the digestion: the kernel's own, FP64 for double-float.
template <typename T> struct FamEpi {
  using type = T;
  static __device__ __forceinline__ T out(T v) { return v; }
};
template <> struct FamEpi<dfl> {
  using type = double;
  static __device__ __forceinline__ double out(dfl v) { return df_to_double(v); }
};

// Thread per family quartet (the light ones): warps take chunks of the list
// sorted by union primitive quartets, like k_small.
template <int LA, int LB, int LC, int LD, bool PURE, typename T>
__global__ void __launch_bounds__(128) k_fam_small(const BuildArgs a) {
  using F = FamCls<LA, LB, LC, LD>;
  using PP = typename PrimT<T>::type;
  constexpr int MB = F::MB, MK = F::MK;
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
      const uint2 e = quartets[t];
      const unsigned mask = fam_mask(e);
      const PairDev P = a.fpairs[e.x & FAM_IDX_MASK], Q = a.fpairs[e.y & FAM_IDX_MASK];
      const FamMem mb = a.fmem[e.x & FAM_IDX_MASK], mk = a.fmem[e.y & FAM_IDX_MASK];
      T AB[3], CD[3];
      fam_geometry(a, P, Q, AB, CD);
      FamAcc<LA, LB, LC, LD, T> s;
      fam_acc_init(s);
      const PP* bpp = fprims_of<T>(a) + P.poff;
      const PP* kpp = fprims_of<T>(a) + Q.poff;
      const FamCoef* bco = a.fcoef + P.poff;
      const FamCoef* kco = a.fcoef + Q.poff;
      prim_loop_lane(a, bpp, kpp, P.pcnt, Q.pcnt, 0, 1, nprim, [&](int cb, int cq) {
        fam_body<LA, LB, LC, LD, T>(a, bpp, kpp, bco, kco, cb, cq, AB, CD, mb.n, mk.n, s);
      });
      // digestion: FP64 for the double-float kernels (as k_small_df), else in T
      using E = typename FamEpi<T>::type;
      E acc[F::NACC];
#pragma unroll
      for (int i = 0; i < F::NACC; ++i) acc[i] = FamEpi<T>::out(s.acc[i]);
#pragma unroll 1
      for (int k = 0; k < MB * MK; ++k)
        if ((mask >> (4 * (k / MK) + k % MK)) & 1u) fam_digest<LA, LB, LC, LD, PURE, E>(a, mb, mk, k, acc);
    }
  }
  if (a.counters && nprim) atomicAdd(a.counters, nprim);
}

// One warp per heavy family quartet: the lanes share its union primitive
// quartets (dealt as in k_prim), the member blocks are summed over the warp,
// and lane k digests member combination k.
template <int LA, int LB, int LC, int LD, bool PURE, typename T>
__global__ void __launch_bounds__(128) k_fam_warp(const BuildArgs a) {
  using F = FamCls<LA, LB, LC, LD>;
  using PP = typename PrimT<T>::type;
  constexpr int NE = F::NE, MB = F::MB, MK = F::MK;
  const int lane = threadIdx.x & 31;
  const uint2* quartets;
  long long nquartets;
  work_range(a, quartets, nquartets);
  unsigned long long nprim = 0;
  for (;;) {
    const long long t = grab(a.work, 1u, lane);
    if (t >= nquartets) break;
    const uint2 e = quartets[t];
    const unsigned mask = fam_mask(e);
    const PairDev P = a.fpairs[e.x & FAM_IDX_MASK], Q = a.fpairs[e.y & FAM_IDX_MASK];
    const FamMem mb = a.fmem[e.x & FAM_IDX_MASK], mk = a.fmem[e.y & FAM_IDX_MASK];
    T AB[3], CD[3];
    fam_geometry(a, P, Q, AB, CD);
    FamAcc<LA, LB, LC, LD, T> s;
    fam_acc_init(s);
    const PP* bpp = fprims_of<T>(a) + P.poff;
    const PP* kpp = fprims_of<T>(a) + Q.poff;
    const FamCoef* bco = a.fcoef + P.poff;
    const FamCoef* kco = a.fcoef + Q.poff;
    prim_loop_warp(a, bpp, kpp, P.pcnt, Q.pcnt, lane, nprim, [&](int cb, int cq) {
      fam_body<LA, LB, LC, LD, T>(a, bpp, kpp, bco, kco, cb, cq, AB, CD, mb.n, mk.n, s);
    });
    using E = typename FamEpi<T>::type;
    E acc[F::NACC];
#pragma unroll
    for (int i = 0; i < F::NACC; ++i) acc[i] = FamEpi<T>::out(s.acc[i]);
    // warp sums of the listed combinations (the mask is uniform over the warp)
#pragma unroll
    for (int k = 0; k < MB * MK; ++k) {
      if (!((mask >> (4 * (k / MK) + k % MK)) & 1u)) continue;
#pragma unroll
      for (int i = 0; i < NE; ++i) {
        E v = acc[k * NE + i];
#pragma unroll
        for (int s = 16; s > 0; s >>= 1) v += __shfl_xor_sync(0xffffffffu, v, s);
        acc[k * NE + i] = v;
      }
    }
    static_assert(MB * MK <= 32, "one lane per member combination");
    if (lane < MB * MK && ((mask >> (4 * (lane / MK) + lane % MK)) & 1u))
      fam_digest<LA, LB, LC, LD, PURE, E>(a, mb, mk, lane, acc);
  }
  if (a.counters && nprim) atomicAdd(a.counters, nprim);
}

template <int LA, int LB, int LC, int LD, bool PURE, typename T>
cudaError_t launch_fam_t(bool warp, const BuildArgs& a, int nsm, cudaStream_t st) {
  if (warp) return launch_persistent(k_fam_warp<LA, LB, LC, LD, PURE, T>, 0, 4, a, nsm, st);
  return launch_persistent(k_fam_small<LA, LB, LC, LD, PURE, T>, 0, 128, a, nsm, st);
}

}  // namespace oqpg
