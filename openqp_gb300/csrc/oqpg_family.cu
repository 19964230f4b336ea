// Shell families: one primitive integral for every shell pair that shares
// its primitives.
//
// Correlation-consistent basis sets contract several s shells of an atom from
// the same primitives (cc-pVDZ oxygen: the 1s and 2s both from nine
// exponents).  OpenQP stores them as separate shells (segmented form) and its
// Fock build (int2.F90:755-805, the shell-quartet loop) evaluates every shell
// quartet on its own, so a quartet of such shells repeats the same primitive
// integrals with other contraction coefficients.  Here two s shells of one
// atom form a family when one's exponents are all among the other's (equal
// lists, as oxygen's 1s and 2s; or a subset, as hydrogen's uncontracted 2s
// within its 1s contraction in cc-pVDZ), the
// family pairs (two families, or a family and another shell) carry the union
// of their members' primitive pairs, and a family quartet evaluates each
// union primitive quartet once, with unit pair factors, and adds it to every
// member combination with that combination's own factors K_ab/p K_cd/q.
//
// The result is the reference's sum term by term: each member keeps its own
// primitive-pair screen (a dropped pair has factor 0), its own primitive-
// quartet screen (|K/p K/q| / sqrt(p + q) against 1e-4 tau, decided per
// combination), its own quartet screen (the mask k_lists_fam stores per
// combination) and its own element cutoff and digestion (small_epilogue with
// the member's shells).  Only the classes whose members x elements block fits
// in registers are built this way ((ss|ss), (ss|sp), (ss|sd), (ss|pp),
// (ss|pd), (sp|sp), (sp|sd), (sp|pp): fam_class); the other quartets of
// family shells stay shell quartets.  SCF builds in every precision mode
// (fam_on): in the split a family quartet runs in FP32 when every member
// combination it lists would (their bounds below the threshold); the others
// run in FP64, or in double-float in the df modes.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/openqp_gb300.h"
#include "oqpg_family.cuh"
#include "oqpg_internal.h"

namespace oqpg {

// ---------------------------------------------------------------------------
// Family-quartet lists: one CTA per family pair FP, walking the family pairs
// FQ <= FP of its molecule in order of descending bound (the prefix that can
// pass, as k_lists does for shell pairs); a one-member FP walks only the
// family pairs with several members (quartets of two one-member pairs are
// k_lists's).  Each member combination (P, Q) is
// screened exactly as k_lists screens the shell quartet: the pair screen on
// the larger of the two pair indices, then the quartet screen; a family
// quartet is listed when some combination passes, with the passing ones in
// its mask.  For FP == FQ the combinations with Q > P are the same quartets
// as (Q, P) and are skipped.
__device__ __forceinline__ unsigned fam_mask_transpose(unsigned m) {
  unsigned t = 0;
#pragma unroll
  for (int i = 0; i < FAM_MAX; ++i)
#pragma unroll
    for (int j = 0; j < FAM_MAX; ++j) t |= ((m >> (4 * i + j)) & 1u) << (4 * j + i);
  return t;
}

__global__ void __launch_bounds__(256) k_lists_fam(const ListArgs a) {
  // per (precision, class): FP64 family lists, then FP32
  __shared__ unsigned cnt[2 * NCLASS_SD], mcnt[2 * NCLASS_SD];
  __shared__ unsigned long long base[2 * NCLASS_SD];
  __shared__ int s_len;
  const int FP = blockIdx.x;
  const int mi = a.fpair_mol[FP];
  const MolDev M = a.mols[mi];
  const double dmax = __longlong_as_double((long long)a.dmax_bits[mi]);
  const double qFP = a.fq[FP];
  if (qFP * dmax < a.tau) return;
  const FamMem mp = a.fmem[FP];
  const bool single = mp.n == 1;
  const int f0 = single ? a.fmmol0[mi] : a.fmol0[mi];
  const int* sorted_idx = single ? a.fmsorted_idx : a.fsorted_idx;
  if (threadIdx.x == 0) {
    const double thr = a.tau / (4.0 * qFP * dmax) * (1.0 - 1e-9);
    const double* sq = (single ? a.fmsorted_q : a.fsorted_q) + f0;
    int lo = 0, hi = single ? a.fmmoln[mi] : a.fmoln[mi];
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (sq[mid] >= thr) lo = mid + 1;
      else hi = mid;
    }
    s_len = lo;
  }
  __syncthreads();
  const int len = s_len;
  const int ns = M.ns;
  const float* dshf = a.dshf + M.dsh0;
  const double* dshd = a.dsh + M.dsh0;
  const int tFP = a.fpair_type[FP];
  const float tlo = (float)(a.tau * (1.0 - 1e-5)), thi = (float)(a.tau * (1.0 + 1e-5));
  const float mlo = (float)(a.tau_f32 * (1.0 - 1e-5)), mhi = (float)(a.tau_f32 * (1.0 + 1e-5));
  for (int s0 = 0; s0 < len; s0 += blockDim.x) {
    if (threadIdx.x < 2 * NCLASS_SD) cnt[threadIdx.x] = mcnt[threadIdx.x] = 0;
    __syncthreads();
    const int s = s0 + threadIdx.x;
    const int FQ = s < len ? sorted_idx[f0 + s] : 0x7fffffff;
    int cl = -1, li = 0;
    unsigned slot = 0;
    uint2 ent = make_uint2(0u, 0u);
    if (FQ <= FP) {
      const FamMem mq = a.fmem[FQ];
      const int tFQ = a.fpair_type[FQ];
      const int c = tFP <= tFQ ? class_index(tFP, tFQ) : class_index(tFQ, tFP);
      if ((mp.n > 1 || mq.n > 1) && fam_class(c)) {
        unsigned mask = 0;
        bool f32 = a.tau_f32 > 0.0;   // every passing combination below the split threshold
#pragma unroll
        for (int m = 0; m < FAM_MAX; ++m) {
          if (m >= mp.n) break;
          const int P = mp.m[m];
          const int2 ij = a.pair_ij[P];
          const float* di = dshf + (long long)ij.x * ns;
          const float* dj = dshf + (long long)ij.y * ns;
          const float dij4 = 4.0f * di[ij.y];
          const double qP = a.q[P];
          const float qPf = a.qf[P];
#pragma unroll
          for (int n = 0; n < FAM_MAX; ++n) {
            if (n >= mq.n) break;
            const int Q = mq.m[n];
            if (FQ == FP && Q > P) continue;
            if (a.q[P > Q ? P : Q] * dmax < a.tau) continue;   // pair screen of the larger pair index
            const int2 kl = a.pair_ij[Q];
            const float tf = quartet_value_f32(a, ns, dshf, di, dj, dij4, qPf, Q, kl);
            double t = -1.0;  // exact test value, computed only near a threshold
            bool pass;
            if (tf < tlo) pass = false;
            else if (tf > thi) pass = true;
            else {
              t = quartet_value(a, ns, dshd, ij, qP, Q, kl);
              pass = !(t < a.tau);
            }
            if (pass) {
              mask |= 1u << (4 * m + n);
              // the shell-quartet path's split decision for this combination
              if (f32 && !(tf < mlo)) {
                if (tf > mhi) f32 = false;
                else {
                  if (t < 0.0) t = quartet_value(a, ns, dshd, ij, qP, Q, kl);
                  f32 = t < a.tau_f32;
                }
              }
            }
          }
        }
        if (mask) {
          cl = c;
          li = f32 ? 1 : 0;
          ent = tFP <= tFQ ? fam_entry(FP, FQ, mask) : fam_entry(FQ, FP, fam_mask_transpose(mask));
          slot = atomicAdd(&cnt[li * NCLASS_SD + c], 1u);
          atomicAdd(&mcnt[li * NCLASS_SD + c], (unsigned)__popc(mask));
        }
      }
    }
    __syncthreads();
    if (threadIdx.x < 2 * NCLASS_SD && cnt[threadIdx.x]) {
      const int p = threadIdx.x / NCLASS_SD, c = threadIdx.x % NCLASS_SD;
      base[threadIdx.x] = atomicAdd(&a.counts[fam_list_index(c, p)], (unsigned long long)cnt[threadIdx.x]);
      atomicAdd(&a.fam_members[p * NCLASS + c], (unsigned long long)mcnt[threadIdx.x]);
    }
    __syncthreads();
    if (cl >= 0 && a.write) {
      const unsigned long long pos = base[li * NCLASS_SD + cl] + slot;
      const int k = fam_list_index(cl, li);
      if (pos < a.caps[k]) a.lists[k][pos] = ent;
    }
    __syncthreads();
  }
}

// The family kernels (oqpg_family.cuh); the double-float ones are built in
// oqpg_family_df.cu.
template <int LA, int LB, int LC, int LD, bool PURE>
cudaError_t launch_fam_cls(bool warp, int kind, const BuildArgs& a, int nsm, cudaStream_t st) {
  if (kind == FAM_F32) return launch_fam_t<LA, LB, LC, LD, PURE, float>(warp, a, nsm, st);
  return launch_fam_t<LA, LB, LC, LD, PURE, double>(warp, a, nsm, st);
}

cudaError_t launch_family(int c, bool pure, bool warp, int kind, const BuildArgs& a, int nsm, cudaStream_t st) {
  if (kind == FAM_DF) return launch_family_df(c, pure, warp, a, nsm, st);
  switch (c) {
    case 0: return launch_fam_cls<0, 0, 0, 0, false>(warp, kind, a, nsm, st);
    case 1: return launch_fam_cls<0, 0, 0, 1, false>(warp, kind, a, nsm, st);
    case 2: return pure ? launch_fam_cls<0, 0, 0, 2, true>(warp, kind, a, nsm, st)
                        : launch_fam_cls<0, 0, 0, 2, false>(warp, kind, a, nsm, st);
    case 3: return launch_fam_cls<0, 0, 1, 1, false>(warp, kind, a, nsm, st);
    case 4: return pure ? launch_fam_cls<0, 0, 1, 2, true>(warp, kind, a, nsm, st)
                        : launch_fam_cls<0, 0, 1, 2, false>(warp, kind, a, nsm, st);
    case 6: return launch_fam_cls<0, 1, 0, 1, false>(warp, kind, a, nsm, st);
    case 7: return pure ? launch_fam_cls<0, 1, 0, 2, true>(warp, kind, a, nsm, st)
                        : launch_fam_cls<0, 1, 0, 2, false>(warp, kind, a, nsm, st);
    case 8: return launch_fam_cls<0, 1, 1, 1, false>(warp, kind, a, nsm, st);
    default: return cudaErrorInvalidValue;
  }
}

// ---------------------------------------------------------------------------
// Host: the family tables.

// In the double-float modes the family quartets that are not FP32 run in
// double-float (FAM_DF), as the shell quartets there do.
bool fam_on(const oqpg_ctx* c, const Job& job) {
  return c->fam_enabled && c->nfpair > 0 && !job.gen && job.inv_mu2 == 0.0 && !petite_on(c, job);
}

namespace {

// The primitive of shell s with exponent a (bitwise), or -1.
int prim_index(const double* ex, const std::vector<int>& po, const std::vector<int>& nc, int s, double a) {
  for (int i = 0; i < nc[s]; ++i)
    if (std::memcmp(ex + po[s] + i, &a, sizeof(double)) == 0) return i;
  return -1;
}
// Every exponent of shell s is one of shell r's.
bool exps_within(const double* ex, const std::vector<int>& po, const std::vector<int>& nc, int s, int r) {
  for (int i = 0; i < nc[s]; ++i)
    if (prim_index(ex, po, nc, r, ex[po[s] + i]) < 0) return false;
  return true;
}

template <typename T>
cudaError_t upload_vec(DevBuf& b, const std::vector<T>& v, cudaStream_t st) {
  cudaError_t e = b.ensure(std::max<size_t>(sizeof(T) * v.size(), 16));
  if (e != cudaSuccess || v.empty()) return e;
  return cudaMemcpyAsync(b.p, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice, st);
}

}  // namespace

// Families of each molecule (two s shells on one atom, one's exponents all
// among the other's, bitwise; the representative holds every exponent; in
// shell order), and the family pairs of the family
// classes' pair types, molecule by molecule (FA >= FB in family order; the
// representative shells in kernel orientation, the side-A family holding the
// first shell).  Member (x, y), x of side A, y of side B, is the canonical
// shell pair of x and y; its factor on union primitive pair (i, j) (the
// representatives' exponents a_i, a_j; x's and y's primitives with those
// exponents, or factor 0) is
// K/p = sqrt(2) pi^(5/4) c_x,i c_y,j exp(-a_i a_j |AB|^2 / p) / p with the
// reference's pair screens (int2_pairs.F90:179-266 and the rotated-axis
// pre-screen |K|, |K/p| >= 1e-4 tau), evaluated with build_pairs's operation
// order, so each member's nonzero factors are bitwise its own pair table's.
int family_tables(oqpg_ctx* c, double cutoff) {
  c->nfpair = 0;
  c->nfam_multi = 0;
  const double qcut = 1e-4 * cutoff, ecut = 25.0 * std::log(10.0);
  const double sqrtpito52 = std::sqrt(2.0) * std::pow(3.14159265358979323846, 1.25);
  const std::vector<int>& am = c->h_am;
  const std::vector<int>& nc = c->h_ncontr;
  const std::vector<int>& po = c->h_poff;
  const double* ex = c->h_ex.data();
  const double* cc = c->h_cc.data();
  std::vector<PairDev> fpairs;
  std::vector<FamMem> fmem;
  std::vector<PrimPair> fprims;
  std::vector<FamCoef> fcoef;
  std::vector<int> fmol, ftype, fmol0(c->nmol), fmoln(c->nmol);
  std::vector<double> fq;
  std::vector<unsigned char> multi(c->npair, 0);
  for (int mi = 0; mi < c->nmol; ++mi) {
    const MolDev& M = c->mols[mi];
    std::vector<std::vector<int>> fam;
    for (int s = M.shell0; s < M.shell0 + M.ns; ++s) {
      bool placed = false;
      if (am[s] == 0)
        for (auto& f : fam) {
          const int r = f[0];
          if (f.size() < 2 && am[r] == 0 && c->shell_atom[r] == c->shell_atom[s] &&
              (exps_within(ex, po, nc, s, r) || exps_within(ex, po, nc, r, s))) {
            f.push_back(s);
            if (nc[s] > nc[r]) std::swap(f[0], f[1]);   // the representative holds every exponent
            placed = true;
            break;
          }
        }
      if (!placed) fam.push_back({s});
    }
    fmol0[mi] = (int)fpairs.size();
    for (size_t fa = 0; fa < fam.size(); ++fa)
      for (size_t fb = 0; fb <= fa; ++fb) {
        int sa = fam[fa][0], sb = fam[fb][0];
        const bool swap = am[sa] > am[sb];
        if (swap) std::swap(sa, sb);
        const int t = pair_type(am[sa], am[sb]);
        if (!fam_pair_type(t)) continue;
        const std::vector<int>& FA = swap ? fam[fb] : fam[fa];
        const std::vector<int>& FB = swap ? fam[fa] : fam[fb];
        std::vector<std::pair<int, int>> ms;
        if (fa == fb) {
          for (size_t i = 0; i < FA.size(); ++i)
            for (size_t j = 0; j <= i; ++j) ms.push_back({FA[i], FA[j]});
        } else {
          for (int x : FA)
            for (int y : FB) ms.push_back({x, y});
        }
        FamMem fm{};
        fm.n = (int)ms.size();
        double q = 0.0;
        for (int k = 0; k < FAM_MAX; ++k) fm.m[k] = -1;
        for (size_t k = 0; k < ms.size(); ++k) {
          int li = ms[k].first - M.shell0, lj = ms[k].second - M.shell0;
          if (li < lj) std::swap(li, lj);
          fm.m[k] = M.pair0 + li * (li + 1) / 2 + lj;
          q = std::max(q, c->schwarz_pair[fm.m[k]]);
        }
        const ShellDev& A = c->shells[sa];
        const ShellDev& B = c->shells[sb];
        const double ab2 = (A.x - B.x) * (A.x - B.x) + (A.y - B.y) * (A.y - B.y) + (A.z - B.z) * (A.z - B.z);
        PairDev pd;
        pd.sha = sa;
        pd.shb = sb;
        pd.poff = (int)fprims.size();
        for (int i = 0; i < nc[sa]; ++i)
          for (int j = 0; j < nc[sb]; ++j) {
            const double a1 = ex[po[sa] + i], a2 = ex[po[sb] + j];
            const double g = a1 + a2;
            double e12 = a1 * a2 * ab2;
            if (e12 > g * ecut) continue;
            const double gi = 1.0 / g;
            e12 *= gi;
            const double eab = std::exp(-e12);
            FamCoef fc{};
            double mx = 0.0;
            for (size_t k = 0; k < ms.size(); ++k) {
              const int ix = prim_index(ex, po, nc, ms[k].first, a1), iy = prim_index(ex, po, nc, ms[k].second, a2);
              if (ix < 0 || iy < 0) continue;   // the member has no such primitive pair
              const double k1 = cc[po[ms[k].first] + ix] * cc[po[ms[k].second] + iy] * eab;
              if (std::fabs(k1) < qcut) continue;
              const double sp = sqrtpito52 * k1 * gi;
              if (std::fabs(sp) < qcut) continue;
              fc.sp[k] = sp;
              fc.spf[k] = (float)sp;
              mx = std::max(mx, std::fabs(sp));
            }
            if (mx == 0.0) continue;
            PrimPair pp;
            pp.p = g;
            pp.hp = 0.5 * gi;
            pp.px = (a1 * A.x + a2 * B.x) * gi;
            pp.py = (a1 * A.y + a2 * B.y) * gi;
            pp.pz = (a1 * A.z + a2 * B.z) * gi;
            const ShellDev& R = A.am == 0 ? B : A;   // the recursion runs on B when A is an s shell
            pp.ax = pp.px - R.x;
            pp.ay = pp.py - R.y;
            pp.az = pp.pz - R.z;
            pp.sp = mx;
            pp.spf = (float)mx;
            pp.pf = (float)g;
            fprims.push_back(pp);
            fcoef.push_back(fc);
          }
        pd.pcnt = (int)fprims.size() - pd.poff;
        if (ms.size() > 1) {
          ++c->nfam_multi;
          for (size_t k = 0; k < ms.size(); ++k) multi[fm.m[k]] = 1;
        }
        fpairs.push_back(pd);
        fmem.push_back(fm);
        fmol.push_back(mi);
        ftype.push_back(t);
        fq.push_back(q);
      }
    fmoln[mi] = (int)fpairs.size() - fmol0[mi];
  }
  if (c->nfam_multi == 0 || fpairs.size() > FAM_IDX_MASK) {
    c->nfam_multi = 0;
    return OK;   // nothing to share (or too many family pairs for the list entries)
  }
  std::vector<int> order(fpairs.size());
  for (size_t p = 0; p < order.size(); ++p) order[p] = (int)p;
  for (int mi = 0; mi < c->nmol; ++mi)
    std::stable_sort(order.begin() + fmol0[mi], order.begin() + fmol0[mi] + fmoln[mi],
                     [&](int x, int y) { return fq[x] > fq[y]; });
  std::vector<double> sq(order.size());
  for (size_t p = 0; p < order.size(); ++p) sq[p] = fq[order[p]];
  // the same order restricted to the family pairs with several members
  std::vector<int> morder, fmmol0(c->nmol), fmmoln(c->nmol);
  std::vector<double> msq;
  for (int mi = 0; mi < c->nmol; ++mi) {
    fmmol0[mi] = (int)morder.size();
    for (int k = fmol0[mi]; k < fmol0[mi] + fmoln[mi]; ++k)
      if (fmem[order[k]].n > 1) {
        morder.push_back(order[k]);
        msq.push_back(fq[order[k]]);
      }
    fmmoln[mi] = (int)morder.size() - fmmol0[mi];
  }
  cudaStream_t st = c->stream;
  cudaError_t e = cudaSuccess;
  if (e == cudaSuccess) e = upload_vec(c->d_fpairs, fpairs, st);
  if (e == cudaSuccess) e = upload_vec(c->d_fmem, fmem, st);
  if (e == cudaSuccess) e = upload_vec(c->d_fprims, fprims, st);
  std::vector<PrimPairF> fprimsf(fprims.size());   // FP32 copy for the FP32 family quartets
  for (size_t i = 0; i < fprims.size(); ++i) {
    const PrimPair& q = fprims[i];
    fprimsf[i] = PrimPairF{(float)q.p, (float)q.hp, (float)q.px, (float)q.py, (float)q.pz,
                           (float)q.ax, (float)q.ay, (float)q.az, (float)q.sp, 0.0f};
  }
  if (e == cudaSuccess) e = upload_vec(c->d_fprimsf, fprimsf, st);
  // double-float copies for the df modes: every FP64 field as an FP32 pair
  auto split = [](double v) {
    const float h = (float)v;
    return dfl(h, (float)(v - (double)h));
  };
  std::vector<PrimPairDF> fprimsdf(fprims.size());
  for (size_t i = 0; i < fprims.size(); ++i) {
    const PrimPair& q = fprims[i];
    PrimPairDF& o = fprimsdf[i];
    o.p = split(q.p); o.hp = split(q.hp); o.px = split(q.px); o.py = split(q.py); o.pz = split(q.pz);
    o.ax = split(q.ax); o.ay = split(q.ay); o.az = split(q.az); o.sp = split(q.sp);
    o.spf = q.spf; o.pf = q.pf;
  }
  if (e == cudaSuccess) e = upload_vec(c->d_fprimsdf, fprimsdf, st);
  std::vector<FamCoefDF> fcoefdf(fcoef.size());
  for (size_t i = 0; i < fcoef.size(); ++i)
    for (int m = 0; m < FAM_MAX; ++m) {
      const dfl v = split(fcoef[i].sp[m]);
      fcoefdf[i].sp[m] = make_float2(v.hi, v.lo);
    }
  if (e == cudaSuccess) e = upload_vec(c->d_fcoefdf, fcoefdf, st);
  if (e == cudaSuccess) e = upload_vec(c->d_fcoef, fcoef, st);
  if (e == cudaSuccess) e = upload_vec(c->d_fpair_mol, fmol, st);
  if (e == cudaSuccess) e = upload_vec(c->d_fpair_type, ftype, st);
  if (e == cudaSuccess) e = upload_vec(c->d_fq, fq, st);
  if (e == cudaSuccess) e = upload_vec(c->d_fsorted_idx, order, st);
  if (e == cudaSuccess) e = upload_vec(c->d_fsorted_q, sq, st);
  if (e == cudaSuccess) e = upload_vec(c->d_fmol0, fmol0, st);
  if (e == cudaSuccess) e = upload_vec(c->d_fmoln, fmoln, st);
  if (e == cudaSuccess) e = upload_vec(c->d_pair_fam_multi, multi, st);
  if (e == cudaSuccess) e = upload_vec(c->d_fmsorted_idx, morder, st);
  if (e == cudaSuccess) e = upload_vec(c->d_fmsorted_q, msq, st);
  if (e == cudaSuccess) e = upload_vec(c->d_fmmol0, fmmol0, st);
  if (e == cudaSuccess) e = upload_vec(c->d_fmmoln, fmmoln, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return e == cudaErrorMemoryAllocation ? NO_MEM : DEV_ERR;
  c->nfpair = (int)fpairs.size();
  return OK;
}

}  // namespace oqpg

using namespace oqpg;

extern "C" int oqpg_set_shell_families(oqpg_ctx* c, int on) {
  if (!c) return NOT_INIT;
  if (c->gexec) {   // a captured build holds the previous lists
    cudaGraphExecDestroy(c->gexec);
    c->gexec = nullptr;
  }
  c->fam_enabled = on != 0;
  c->hb.sized = false;
  return OK;
}

extern "C" int oqpg_shell_families_info(const oqpg_ctx* c, int* on, int* nshared) {
  if (!c) return NOT_INIT;
  if (on) *on = c->fam_enabled ? 1 : 0;
  if (nshared) *nshared = c->nfpair > 0 ? c->nfam_multi : 0;
  return OK;
}
