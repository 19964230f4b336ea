// Host side of the GB300 Fock build: contexts, shell-pair tables, device
// screening and quartet-list construction, class-kernel dispatch, the final
// symmetrisation into OpenQP's packed layout, and the C ABI.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <vector>

#include "../../include/openqp_gb300.h"
#include "oqpg_internal.h"

namespace oqpg {

static const ClassInfo kClasses[NCLASS] = {
#define C_(a, b, c, d) {{a, b, c, d}, has_small(a, b, c, d), has_team(a, b, c, d), prim_parallel(a, b, c, d)}
    C_(0, 0, 0, 0), C_(0, 0, 0, 1), C_(0, 0, 0, 2), C_(0, 0, 1, 1), C_(0, 0, 1, 2), C_(0, 0, 2, 2),
    C_(0, 1, 0, 1), C_(0, 1, 0, 2), C_(0, 1, 1, 1), C_(0, 1, 1, 2), C_(0, 1, 2, 2),
    C_(0, 2, 0, 2), C_(0, 2, 1, 1), C_(0, 2, 1, 2), C_(0, 2, 2, 2),
    C_(1, 1, 1, 1), C_(1, 1, 1, 2), C_(1, 1, 2, 2),
    C_(1, 2, 1, 2), C_(1, 2, 2, 2),
    C_(2, 2, 2, 2),
    // with an f pair (ket type sf, pf, df, ff; bra type <= ket type)
    C_(0, 0, 0, 3), C_(0, 1, 0, 3), C_(0, 2, 0, 3), C_(1, 1, 0, 3), C_(1, 2, 0, 3), C_(2, 2, 0, 3),
    C_(0, 3, 0, 3), C_(0, 0, 1, 3), C_(0, 1, 1, 3), C_(0, 2, 1, 3), C_(1, 1, 1, 3), C_(1, 2, 1, 3),
    C_(2, 2, 1, 3), C_(0, 3, 1, 3), C_(1, 3, 1, 3), C_(0, 0, 2, 3), C_(0, 1, 2, 3), C_(0, 2, 2, 3),
    C_(1, 1, 2, 3), C_(1, 2, 2, 3), C_(2, 2, 2, 3), C_(0, 3, 2, 3), C_(1, 3, 2, 3), C_(2, 3, 2, 3),
    C_(0, 0, 3, 3), C_(0, 1, 3, 3), C_(0, 2, 3, 3), C_(1, 1, 3, 3), C_(1, 2, 3, 3), C_(2, 2, 3, 3),
    C_(0, 3, 3, 3), C_(1, 3, 3, 3), C_(2, 3, 3, 3), C_(3, 3, 3, 3),
#undef C_
};
static_assert(sizeof(kClasses) / sizeof(kClasses[0]) == NCLASS, "class table");
const ClassInfo& class_info(int c) { return kClasses[c]; }

cudaError_t launch_class(int c, bool pure, int mode, const BuildArgs& a, int nsm, cudaStream_t st) {
  switch (c) {
    case 0: case 1: case 2: case 3:
      return launch_group0(c, pure, mode, a, nsm, st);
    case 4: case 6: case 7: case 8:
      return launch_group1(c, pure, mode, a, nsm, st);
    case 5:
      return launch_group2(c, pure, mode, a, nsm, st);
    case 9:
      return launch_group14(c, pure, mode, a, nsm, st);
    case 10:
      return launch_group15(c, pure, mode, a, nsm, st);
    case 11:
      return launch_group3(c, pure, mode, a, nsm, st);
    case 12:
      return launch_group16(c, pure, mode, a, nsm, st);
    case 15:
      return launch_group17(c, pure, mode, a, nsm, st);
    case 13:
      return launch_group4(c, pure, mode, a, nsm, st);
    case 14: case 16: case 17:
      return launch_group18(c, pure, mode, a, nsm, st);
    case 18:
      return launch_group5(c, pure, mode, a, nsm, st);
    case 19:
      return launch_group6(c, pure, mode, a, nsm, st);
    case 20:
      return launch_group7(c, pure, mode, a, nsm, st);
    case 21: case 22: case 23: case 24: case 25: case 26: case 27:
      return launch_group8(c, pure, mode, a, nsm, st);
    case 28: case 29: case 30: case 31: case 32: case 33: case 34: case 35:
      return launch_group9(c, pure, mode, a, nsm, st);
    case 36: case 37: case 38: case 39: case 40:
      return launch_group10(c, pure, mode, a, nsm, st);
    case 41: case 42: case 43: case 44:
      return launch_group11(c, pure, mode, a, nsm, st);
    case 45: case 46: case 47: case 48: case 49:
      return launch_group12(c, pure, mode, a, nsm, st);
    case 50: case 51: case 52: case 53: case 54:
      return launch_group13(c, pure, mode, a, nsm, st);
    default:
      return cudaErrorInvalidValue;
  }
}

// ---------------------------------------------------------------------------
// Small device kernels



// Packed D -> full symmetric Coulomb density (Da + Db) and exchange densities,
// every molecule of the batch into its rows of the stacked matrices (columns
// beyond a molecule's nbf are zeroed).
__global__ void k_unpack(const double* __restrict__ dp, int nfocks, const MolDev* __restrict__ mols,
                         const int* __restrict__ row_mol, int nrows, int stride, double* dj, double* dk) {
  const long long n2 = (long long)nrows * stride;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n2; t += (long long)gridDim.x * blockDim.x) {
    const int r = (int)(t / stride), j = (int)(t % stride);
    const MolDev m = mols[row_mol[r]];
    const int i = r - m.row0;
    if (j >= m.nbf) {
      dj[t] = 0.0;
      if (nfocks == 2) { dk[t] = 0.0; dk[n2 + t] = 0.0; }
      continue;
    }
    const int hi = i > j ? i : j, lo = i > j ? j : i;
    const long long ntri = (long long)m.nbf * (m.nbf + 1) / 2;
    const double* d = dp + nfocks * m.tri0;
    const long long p = (long long)hi * (hi + 1) / 2 + lo;
    if (nfocks == 1) {
      dj[t] = d[p];
    } else {
      const double a = d[p], b = d[ntri + p];
      dj[t] = a + b;
      dk[t] = a;
      dk[n2 + t] = b;
    }
  }
}

__global__ void k_to_f32(const double* __restrict__ x, long long n, float* y) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x)
    y[t] = (float)x[t];
}

__global__ void k_to_df(const double* __restrict__ x, long long n, dfl* y) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    const double v = x[t];
    const float h = (float)v;
    y[t] = dfl(h, (float)(v - (double)h));
  }
}

// shlden (OpenQP int2.F90:999-1047): max |D| over each shell-pair block and
// over the densities; also each molecule's maximum (max_den).
__global__ void k_dsh(const double* __restrict__ dp, int nfocks, const MolDev* __restrict__ mols,
                      const int* __restrict__ pair_mol, const int2* __restrict__ pair_ij, int npair,
                      const int* __restrict__ aoff, const int* __restrict__ nao, double* dsh, float* dshf,
                      unsigned long long* dmax_bits) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < npair; t += (long long)gridDim.x * blockDim.x) {
    const int mi = pair_mol[t];
    const MolDev M = mols[mi];
    const int2 ij = pair_ij[t];
    const int si = ij.x, sj = ij.y;
    const long long ntri = (long long)M.nbf * (M.nbf + 1) / 2;
    double m = 0.0;
    const int i0 = aoff[M.shell0 + si], i1 = i0 + nao[M.shell0 + si], j0 = aoff[M.shell0 + sj];
    const int j1 = j0 + nao[M.shell0 + sj];
    for (int f = 0; f < nfocks; ++f) {
      const double* d = dp + nfocks * M.tri0 + f * ntri;
      for (int i = i0; i < i1; ++i) {
        const int je = (si == sj) ? i + 1 : j1;
        for (int j = j0; j < je; ++j) m = fmax(m, fabs(d[(long long)i * (i + 1) / 2 + j]));
      }
    }
    dsh[M.dsh0 + (long long)si * M.ns + sj] = m;
    dsh[M.dsh0 + (long long)sj * M.ns + si] = m;
    dshf[M.dsh0 + (long long)si * M.ns + sj] = (float)m;
    dshf[M.dsh0 + (long long)sj * M.ns + si] = (float)m;
    atomicMax(dmax_bits + mi, (unsigned long long)__double_as_longlong(m));
  }
}


// Petite-list weight of the canonical quartet (i, j, k, l) (i >= j, k >= l,
// (i, j) >= (k, l); molecule-local shells) under an abelian group given by the
// shell images map[op ns + s] (petite_quartet_weight, int2.F90:411-469): -1
// when some operation maps it onto a lexicographically larger canonical
// quartet (it is skipped), else log2 of the orbit size nops / |stabiliser|.
__device__ int petite_wlog2(const int* __restrict__ map, int nops, int ns, int i, int j, int k, int l) {
  int nstab = 0;
  for (int op = 0; op < nops; ++op) {
    const int* m = map + op * ns;
    int a1 = __ldg(m + i), a2 = __ldg(m + j), b1 = __ldg(m + k), b2 = __ldg(m + l);
    if (a1 < a2) { const int t = a1; a1 = a2; a2 = t; }
    if (b1 < b2) { const int t = b1; b1 = b2; b2 = t; }
    if (a1 < b1 || (a1 == b1 && a2 < b2)) {
      int t = a1; a1 = b1; b1 = t;
      t = a2; a2 = b2; b2 = t;
    }
    if (a1 != i) { if (a1 > i) return -1; }
    else if (a2 != j) { if (a2 > j) return -1; }
    else if (b1 != k) { if (b1 > k) return -1; }
    else if (b2 != l) { if (b2 > l) return -1; }
    else ++nstab;
  }
  return __ffs(nops / nstab) - 1;   // nops is a power of two, so is the orbit size
}

// Screened quartet lists, one CTA per bra pair P (the larger pair index of the
// canonical quartet, int2.F90:755-805): pair screen Q_P Dmax >= tau, then for
// every Q <= P the quartet screen Q_P Q_Q max(4D_ij, 4D_kl, D_jl, D_jk, D_il, D_ik)
// >= tau (int2.F90:975-986).  Since the max is at most 4 Dmax, only the pairs
// with Q_Q >= tau / (4 Q_P Dmax) can pass: they are a prefix of the pairs
// sorted by Schwarz bound, and only that prefix is walked.  FP32 decides when
// it is clear by a 1e-5 margin, FP64 with the reference's operation order
// otherwise.  With tau_f32 > 0 the surviving quartets whose test value (Schwarz
// bound x shell density) is below tau_f32 go to the FP32 lists.
__global__ void __launch_bounds__(256) k_lists(const ListArgs a) {
  __shared__ unsigned cnt[2 * NCLASS];
  __shared__ unsigned long long base[2 * NCLASS];
  __shared__ int s_len;
  const int P = blockIdx.x;
  const int mi = a.pair_mol[P];
  const MolDev M = a.mols[mi];
  const double dmax = __longlong_as_double((long long)a.dmax_bits[mi]);
  const double qP = a.q[P];
  if (qP * dmax < a.tau) return;
  const int* sorted_idx = a.sorted_idx + M.pair0;
  if (threadIdx.x == 0) {
    // number of the molecule's pairs with q >= thr (q descending), with a rounding margin
    const double thr = a.tau / (4.0 * qP * dmax) * (1.0 - 1e-9);
    const double* sq = a.sorted_q + M.pair0;
    int lo = 0, hi = M.npair;
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
  const int2 ij = a.pair_ij[P];
  const int tP = a.pair_type[P];
  const float qPf = a.qf[P];
  const float* di = dshf + (long long)ij.x * ns;
  const float* dj = dshf + (long long)ij.y * ns;
  const float dij4 = 4.0f * di[ij.y];
  const float tlo = (float)(a.tau * (1.0 - 1e-5)), thi = (float)(a.tau * (1.0 + 1e-5));
  const float mlo = (float)(a.tau_f32 * (1.0 - 1e-5)), mhi = (float)(a.tau_f32 * (1.0 + 1e-5));
  const bool famP = a.fam && a.pair_fam_multi[P];
  // the petite list applies when the density is invariant under the group
  bool petite = false;
  if (a.sym_nops > 1) {
    const double resid = __longlong_as_double((long long)a.sym_bits[0]);
    const double scale = __longlong_as_double((long long)a.sym_bits[1]);
    petite = resid <= 1e-6 * scale;
  }
  for (int s0 = 0; s0 < len; s0 += blockDim.x) {
    if (threadIdx.x < 2 * NCLASS) cnt[threadIdx.x] = 0;
    __syncthreads();
    const int s = s0 + threadIdx.x;
    const int Q = s < len ? sorted_idx[s] : 0x7fffffff;
    int c = -1;
    unsigned slot = 0;
    uint2 ent;
    // quartets of a family class with a member-sharing pair are k_lists_fam's
    const bool fam_skip = Q <= P && a.fam && (famP || a.pair_fam_multi[Q]) &&
                          fam_class(tP <= a.pair_type[Q] ? class_index(tP, a.pair_type[Q])
                                                         : class_index(a.pair_type[Q], tP));
    if (Q <= P && !fam_skip) {
      const int2 kl = a.pair_ij[Q];
      const float tf = quartet_value_f32(a, ns, dshf, di, dj, dij4, qPf, Q, kl);
      double t = -1.0;  // exact test value, computed only near a threshold
      auto exact = [&]() { return quartet_value(a, ns, dshd, ij, qP, Q, kl); };
      bool pass;
      if (tf < tlo) pass = false;
      else if (tf > thi) pass = true;
      else {
        t = exact();
        pass = !(t < a.tau);
      }
      int wl = 0;
      if (pass && petite) {
        wl = petite_wlog2(a.sym_map, a.sym_nops, a.sym_ns, ij.x, ij.y, kl.x, kl.y);
        pass = wl >= 0;
      }
      if (pass) {
        bool f32 = false;
        if (a.tau_f32 > 0.0) {
          if (tf < mlo) f32 = true;
          else if (tf <= mhi) {
            if (t < 0.0) t = exact();
            f32 = t < a.tau_f32;
          }
        }
        const int tQ = a.pair_type[Q];
        if (tP <= tQ) { c = class_index(tP, tQ); ent = make_uint2(P, Q); }
        else { c = class_index(tQ, tP); ent = make_uint2(Q, P); }
        ent.x |= (unsigned)wl << 30;   // orbit weight 2^wl (petite list)
        if (f32 && !class_has_f(c)) c += NCLASS;  // f classes have FP64 kernels only
        slot = atomicAdd(&cnt[c], 1u);
      }
    }
    __syncthreads();
    if (threadIdx.x < 2 * NCLASS && cnt[threadIdx.x])
      base[threadIdx.x] = atomicAdd(&a.counts[threadIdx.x], (unsigned long long)cnt[threadIdx.x]);
    __syncthreads();
    if (c >= 0 && a.write) {
      const unsigned long long pos = base[c] + slot;
      if (pos < a.caps[c]) a.lists[c][pos] = ent;
    }
    __syncthreads();
  }
}

// Counting sort of a class list by primitive-quartet work (descending; exact
// counts below BIN_EXACT, quarter-octave bins above), so that the lanes of a
// warp run loops of equal or similar length.  The work of a quartet is the number of its primitive quartets that
// pass the FP32 pre-screen |sp sq| / sqrt(p + q) >= lo, the loop trip count of
// the FP64 body (without prims: the product of the pair primitive counts).
// k_bin_hist: per-bin counts (and each entry's bin); k_bin_scatter:
// stable-per-CTA scatter into the bin ranges given by the exclusive scan in
// cursors.

__device__ __forceinline__ int work_bin(int n) {
  int b;
  if (n < BIN_EXACT) {
    b = n < 1 ? 0 : n - 1;
  } else {
    // quarter octaves from the leading bit: n = 2^e r, r in [1, 2)
    const int e = 31 - __clz(n);
    const float r = (float)n * __int_as_float((127 - e) << 23);
    b = 4 * e + BIN_EXACT - 25 + (r >= 1.18920712f) + (r >= 1.41421356f) + (r >= 1.68179283f);
  }
  return NBIN - 1 - (b < NBIN - 1 ? b : NBIN - 1);
}

__device__ __forceinline__ int prim_bin(const PairDev* pairs, uint2 q, unsigned xmask, unsigned ymask) {
  return work_bin(pairs[q.x & xmask].pcnt * pairs[q.y & ymask].pcnt);
}

__device__ __forceinline__ int survivor_bin(const PairDev* pairs, const PrimPair* prims, uint2 q, float lo,
                                            unsigned xmask, unsigned ymask) {
  const PairDev P = pairs[q.x & xmask], Q = pairs[q.y & ymask];
  // the heaviest quartets go to the primitive-parallel kernels whatever their
  // exact count: bin them by the product and spare the scan
  if (P.pcnt * Q.pcnt > 512) return work_bin(P.pcnt * Q.pcnt);
  const float lo2 = lo * lo;
  int n = 0;
  for (int j = 0; j < Q.pcnt; ++j) {
    const float ks = __ldg(&prims[Q.poff + j].spf), kp = __ldg(&prims[Q.poff + j].pf);
    for (int i = 0; i < P.pcnt; ++i) {
      // |sp sq| / sqrt(p + q) >= lo, squared (FP32, no reciprocal square root)
      const float t = __ldg(&prims[P.poff + i].spf) * ks;
      n += t * t >= lo2 * (__ldg(&prims[P.poff + i].pf) + kp) ? 1 : 0;
    }
  }
  return work_bin(n);
}

__device__ __forceinline__ long long list_len(long long n, const unsigned long long* n_dev) {
  if (!n_dev) return n;
  const unsigned long long c = *n_dev;
  return c < (unsigned long long)n ? (long long)c : n;
}

__global__ void k_bin_hist(const uint2* __restrict__ list, long long n, const unsigned long long* n_dev,
                           const PairDev* __restrict__ pairs, const PrimPair* __restrict__ prims, float lo,
                           unsigned xmask, unsigned ymask, unsigned char* bins, unsigned long long* hist) {
  __shared__ unsigned h[NBIN];
  n = list_len(n, n_dev);
  for (int i = threadIdx.x; i < NBIN; i += blockDim.x) h[i] = 0;
  __syncthreads();
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    const int b = prims ? survivor_bin(pairs, prims, list[t], lo, xmask, ymask) : prim_bin(pairs, list[t], xmask, ymask);
    if (bins) bins[t] = (unsigned char)b;
    atomicAdd(&h[b], 1u);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < NBIN; i += blockDim.x)
    if (h[i]) atomicAdd(&hist[i], (unsigned long long)h[i]);
}

// Each CTA takes a contiguous chunk, reserves its per-bin ranges once, then
// places its entries (bins: the bins k_bin_hist stored; null: recomputed from
// the primitive counts).  fmem (family lists): within its block of each bin
// the CTA places the family quartets ordered by member pattern (members of
// the bra and of the ket family pair, most first), so that the lanes of a
// warp of the thread-per-family-quartet kernel, which take consecutive
// entries, run member loops and digestions of the same length.
__device__ __forceinline__ int fam_pattern(const FamMem* __restrict__ fmem, uint2 q) {
  const int nb = min(max(__ldg(&fmem[q.x & FAM_IDX_MASK].n), 1), FAM_MAX);
  const int nk = min(max(__ldg(&fmem[q.y & FAM_IDX_MASK].n), 1), FAM_MAX);
  return (FAM_MAX - nb) * FAM_MAX + (FAM_MAX - nk);
}

__global__ void __launch_bounds__(1024) k_bin_scatter(const uint2* __restrict__ list, long long n,
                                                     const unsigned long long* n_dev,
                                                     const PairDev* __restrict__ pairs, unsigned xmask,
                                                     unsigned ymask, const unsigned char* __restrict__ bins,
                                                     unsigned long long* cursors, uint2* out, long long chunk,
                                                     const unsigned* flag, const FamMem* __restrict__ fmem) {
  constexpr int NPAT = FAM_MAX * FAM_MAX;
  __shared__ unsigned h[NBIN];
  __shared__ unsigned long long b[NBIN];
  __shared__ unsigned hp[NBIN * NPAT];
  if (flag && *flag) return;  // a list overflowed: the cursors were not written
  n = list_len(n, n_dev);
  const long long lo = blockIdx.x * chunk;
  if (lo >= n) return;
  const long long hi = lo + chunk < n ? lo + chunk : n;
  for (int i = threadIdx.x; i < NBIN; i += blockDim.x) h[i] = 0;
  if (fmem)
    for (int i = threadIdx.x; i < NBIN * NPAT; i += blockDim.x) hp[i] = 0;
  __syncthreads();
  for (long long t = lo + threadIdx.x; t < hi; t += blockDim.x) {
    const int bin = bins ? bins[t] : prim_bin(pairs, list[t], xmask, ymask);
    atomicAdd(&h[bin], 1u);
    if (fmem) atomicAdd(&hp[bin * NPAT + fam_pattern(fmem, list[t])], 1u);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < NBIN; i += blockDim.x) {
    b[i] = h[i] ? atomicAdd(&cursors[i], (unsigned long long)h[i]) : 0ull;
    h[i] = 0;
    if (fmem) {  // exclusive scan of the bin's pattern counts: each pattern's offset in the bin's block
      unsigned s = 0;
      for (int p = 0; p < NPAT; ++p) {
        const unsigned v = hp[i * NPAT + p];
        hp[i * NPAT + p] = s;
        s += v;
      }
    }
  }
  __syncthreads();
  for (long long t = lo + threadIdx.x; t < hi; t += blockDim.x) {
    const uint2 q = list[t];
    const int bin = bins ? bins[t] : prim_bin(pairs, q, xmask, ymask);
    const unsigned r = fmem ? atomicAdd(&hp[bin * NPAT + fam_pattern(fmem, q)], 1u) : atomicAdd(&h[bin], 1u);
    out[b[bin] + r] = q;
  }
}

// Smallest primitive-quartet count of bin b (work_bin's inverse, lower edge).
__device__ __forceinline__ double bin_count(int b) {
  const int k = NBIN - 1 - b;
  if (k < BIN_EXACT - 1) return (double)(k + 1);
  const int e = (k - (BIN_EXACT - 25)) >> 2, q = (k - (BIN_EXACT - 25)) & 3;
  return ldexp(1.0, e) * (q == 0 ? 1.0 : q == 1 ? 1.18920712 : q == 2 ? 1.41421356 : 1.68179283);
}

// Head of a thread-per-quartet list sized from the list (SPLIT_ADAPTIVE).  A
// thread-per-quartet kernel cannot end before its slowest lane, which runs
// the primitive quartets of its heaviest quartet one after another.  When
// the whole list spread over every lane of the GPU (32 x 4 x nsm) is only a
// few times that chain (short lists, heavy quartets), the heaviest quartets
// dominate the launch: they go to the primitive-parallel kernel, whose 32
// lanes share one quartet.  The head takes the quartets with at least 2^s
// primitive quartets, 2^s the largest power of two up to
// npq / (2 x 32 x 4 x nsm) within [2^6, 2^8] (2^8, the fixed default, for
// lists that fill the GPU many times over; 2^6 keeps two or more primitive
// quartets per lane of the warp kernel).  Measured: (H2O)16 6-31G(d) build
// 20.4 -> 17.2 ms; (H2O)32 cc-pVDZ 0.4 % faster.  (Dividing by a further 4,
// for the four warps that share a sub-partition's FP64 pipe, took more
// quartets of the (H2O)32 cc-pVDZ lists to the warp kernel and was slower:
// (sp|pd) 11.2 -> 11.6 ms, (ss|pd) 4.8 -> 5.3 ms.)  The primitive-parallel
// kernel digests each quartet on one lane, so builds with many densities
// (more than 32 Coulomb and exchange densities: the MRSF sigma build of 8
// vectors digests 88) keep the fixed 2^8: measured on (H2O)16 6-31G(d), the
// MRSF build took 114.4 ms with the adaptive head and 108.2 ms without it,
// the TD build of 8 vectors (24 densities) 28.5 and 31.0 ms.
constexpr int ADAPTIVE_MAX_DENSITIES = 32;
__device__ __forceinline__ int adaptive_head_bins(const unsigned long long* hist, int nsm) {
  double npq = 0.0;
  for (int b = 0; b < NBIN; ++b) npq += (double)hist[b] * bin_count(b);
  const double c = npq / (2.0 * 32.0 * 4.0 * (double)nsm);
  const int s = c >= 256.0 ? 8 : (c >= 128.0 ? 7 : 6);
  return head_bins(s);
}

// Device-side bookkeeping of a device-driven build, one thread per list (one
// CTA of 128 threads): the exclusive scan of its bin counts (scatter cursors)
// and the two work ranges of the sorted list, [0, head) for the
// primitive-parallel kernel and [head, count) for the class kernel, head = the
// entries in the bins of >= 2^split primitive quartets (split_bins[list] bins;
// 0 for none; SPLIT_ADAPTIVE: sized here, adaptive_head_bins, when adaptive
// is set, else 2^PRIM_SPLIT_LOG2).  If any list's
// count exceeded its capacity, overflow is set and every range is empty: the
// scatter and the class kernels then do nothing and the build is redone by
// the host.
__global__ void k_bin_scan(const unsigned long long* counts, const unsigned long long* caps, const int* split_bins,
                           const unsigned long long* hist, unsigned long long* cursors, unsigned long long* ranges,
                           unsigned* overflow, int nsm, int adaptive) {
  __shared__ unsigned s_over;
  const int li = threadIdx.x;
  if (li == 0) s_over = 0;
  __syncthreads();
  const bool mine = li < NLIST;
  const unsigned long long cnt = mine ? counts[li] : 0ull;
  if (mine && cnt > caps[li]) atomicOr(&s_over, 1u);
  __syncthreads();
  if (!mine) return;
  unsigned long long* rg = ranges + 4 * li;
  if (s_over) {
    rg[0] = rg[1] = rg[2] = rg[3] = 0;
    if (li == 0) atomicOr(overflow, 1u);
    return;
  }
  unsigned long long s = 0, head = 0;
  const int nb = split_bins[li] != SPLIT_ADAPTIVE ? split_bins[li]
                 : adaptive                      ? adaptive_head_bins(hist + li * NBIN, nsm)
                                                 : head_bins(PRIM_SPLIT_LOG2);
  for (int b = 0; b < NBIN; ++b) {
    cursors[li * NBIN + b] = s;
    s += hist[li * NBIN + b];
    if (b < nb) head = s;
  }
  if (s != cnt) {  // bookkeeping disagrees with the list: run nothing from it
    atomicOr(overflow, 2u);
    rg[0] = rg[1] = rg[2] = rg[3] = 0;
    return;
  }
  rg[0] = 0; rg[1] = head; rg[2] = head; rg[3] = cnt;
}

// F = sc (GJ + GJ^T) - cK (GK + GK^T) on the packed lower triangles of every
// molecule (+ F_old), molecule-major [molecule][density][triangle].  Skipped
// when a list of this build overflowed (flag set), so that f and f_old stay
// as they were for the rebuild.
__global__ void k_finalize(const double* __restrict__ gj, const double* __restrict__ gk, int nk,
                           const MolDev* __restrict__ mols, int nmol, long long ntri_total, int stride,
                           size_t kstride, double sc, double ck, double* f, double* f_old,
                           const unsigned* __restrict__ flag) {
  if (flag && *flag) return;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < ntri_total;
       t += (long long)gridDim.x * blockDim.x) {
    int lo = 0, hi = nmol - 1;  // last molecule with tri0 <= t
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (mols[mid].tri0 <= t) lo = mid;
      else hi = mid - 1;
    }
    const MolDev M = mols[lo];
    const long long u = t - M.tri0;
    const long long ntri = (long long)M.nbf * (M.nbf + 1) / 2;
    int i = (int)((sqrt(8.0 * (double)u + 1.0) - 1.0) * 0.5);
    while ((long long)i * (i + 1) / 2 > u) --i;
    while ((long long)(i + 1) * (i + 2) / 2 <= u) ++i;
    const int j = (int)(u - (long long)i * (i + 1) / 2);
    const long long ij = (long long)(M.row0 + i) * stride + j, ji = (long long)(M.row0 + j) * stride + i;
    const double J = gj[ij] + gj[ji];
    const long long ob = nk * M.tri0 + u;
    for (int k = 0; k < nk; ++k) {
      const double* g = gk + k * kstride;
      double v = sc * J - ck * (g[ij] + g[ji]);
      if (f_old) {
        v += f_old[ob + k * ntri];
        f_old[ob + k * ntri] = v;
      }
      f[ob + k * ntri] = v;
    }
  }
}


}  // namespace oqpg

using namespace oqpg;

namespace {

std::mutex g_mutex;
oqpg_ctx* g_ctx = nullptr;

}  // namespace

oqpg_ctx* oqpg::routec_context() { return g_ctx; }

namespace {

int to_status(cudaError_t e) {
  if (e == cudaSuccess) return OK;
  if (e == cudaErrorMemoryAllocation) return NO_MEM;
  return DEV_ERR;
}

#define CK(x)                                         \
  do {                                                \
    cudaError_t e_ = (x);                             \
    if (e_ != cudaSuccess) {                          \
      if (std::getenv("OQPG_VERBOSE"))                \
        std::fprintf(stderr, "openqp_gb300: %s at %s:%d\n", cudaGetErrorString(e_), __FILE__, __LINE__); \
      return to_status(e_);                           \
    }                                                 \
  } while (0)

}  // namespace

// OpenQP's int2_prepare_pair (int2_pairs.F90:179-266); with sp_screen also
// the rotated-axis pre-screen |K/p| >= quartet cutoff (int_rotaxis.F90:292-306),
// applied once (the Fock build; the gradient's Rys path has no such screen).
// Pairs are numbered molecule by molecule, canonical (i >= j) within each.
// With sp_screen a primitive pair is kept iff min(|K|, |K/p|) >= qcut; with
// key_order each shell pair's primitive pairs are stored in decreasing order
// of that key, so the pairs a looser cutoff keeps are a prefix of the range
// (the run-time cutoff of oqpg_set_cutoff only shortens the counts).  With
// s_on_b (the tables of the Fock-type kernels) a pair whose first shell is an
// s shell stores P - B in place of P - A: those kernels run the recursion on
// the second centre and skip the horizontal transfer.
void oqpg::build_pairs(const oqpg_ctx& c, const std::vector<int>& am, const std::vector<int>& ncontr,
                       const std::vector<int>& poff, const double* ex, const double* cc, double qcut, double ecut,
                       bool sp_screen, HostPairs& out, bool key_order, bool s_on_b) {
  const double sqrtpito52 = std::sqrt(2.0) * std::pow(3.14159265358979323846, 1.25);
  out.pairs.clear(); out.prims.clear(); out.ij.clear(); out.type.clear(); out.mol.clear(); out.alpha.clear();
  out.key.clear();
  for (int m = 0; m < c.nmol; ++m) {
    const MolDev& M = c.mols[m];
    for (int li = 0; li < M.ns; ++li)
      for (int lj = 0; lj <= li; ++lj) {
        int sa = M.shell0 + li, sb = M.shell0 + lj;
        if (am[sa] > am[sb]) std::swap(sa, sb);
        const ShellDev& A = c.shells[sa];
        const ShellDev& B = c.shells[sb];
        const double ab2 = (A.x - B.x) * (A.x - B.x) + (A.y - B.y) * (A.y - B.y) + (A.z - B.z) * (A.z - B.z);
        PairDev pd;
        pd.sha = sa; pd.shb = sb; pd.poff = (int)out.prims.size();
        const size_t first = out.prims.size();
        for (int p1 = 0; p1 < ncontr[sa]; ++p1)
          for (int p2 = 0; p2 < ncontr[sb]; ++p2) {
            const double a1 = ex[poff[sa] + p1], a2 = ex[poff[sb] + p2];
            const double g = a1 + a2;
            double e12 = a1 * a2 * ab2;
            if (e12 > g * ecut) continue;
            const double gi = 1.0 / g;
            e12 *= gi;
            const double k1 = cc[poff[sa] + p1] * cc[poff[sb] + p2] * std::exp(-e12);
            if (std::fabs(k1) < qcut) continue;
            const double sp = sqrtpito52 * k1 * gi;
            if (sp_screen && std::fabs(sp) < qcut) continue;
            PrimPair pp;
            pp.p = g; pp.hp = 0.5 * gi;
            pp.px = (a1 * A.x + a2 * B.x) * gi;
            pp.py = (a1 * A.y + a2 * B.y) * gi;
            pp.pz = (a1 * A.z + a2 * B.z) * gi;
            // the recursion's centre: A, or B when A is an s shell (no transfer then)
            const ShellDev& R = (s_on_b && A.am == 0) ? B : A;
            pp.ax = pp.px - R.x; pp.ay = pp.py - R.y; pp.az = pp.pz - R.z;
            pp.sp = sp; pp.spf = (float)sp; pp.pf = (float)g;
            out.prims.push_back(pp);
            out.alpha.push_back(a1);
            out.key.push_back(sp_screen ? std::min(std::fabs(k1), std::fabs(sp)) : std::fabs(k1));
          }
        if (key_order) {
          const size_t n = out.prims.size() - first;
          std::vector<int> ord(n);
          for (size_t i = 0; i < n; ++i) ord[i] = (int)i;
          std::stable_sort(ord.begin(), ord.end(),
                           [&](int x, int y) { return out.key[first + x] > out.key[first + y]; });
          std::vector<PrimPair> pp(n);
          std::vector<double> al(n), ky(n);
          for (size_t i = 0; i < n; ++i) {
            pp[i] = out.prims[first + ord[i]];
            al[i] = out.alpha[first + ord[i]];
            ky[i] = out.key[first + ord[i]];
          }
          std::copy(pp.begin(), pp.end(), out.prims.begin() + first);
          std::copy(al.begin(), al.end(), out.alpha.begin() + first);
          std::copy(ky.begin(), ky.end(), out.key.begin() + first);
        }
        pd.pcnt = (int)out.prims.size() - pd.poff;
        out.pairs.push_back(pd);
        out.ij.push_back(make_int2(li, lj));
        out.type.push_back(pair_type(am[sa], am[sb]));
        out.mol.push_back(m);
      }
  }
}

// FP32 decision band of the primitive-quartet screen: |sp sq| / sqrt(p+q)
// against sqrt(prim_cut2).  FP32 products of two screened prefactors stay
// normal down to prim_cut ~ 1e-18; below that every decision goes to FP64.
void oqpg::set_band(BuildArgs& a) {
  const double c = std::sqrt(a.prim_cut2);
  if (c >= 1e-18) {
    a.prim_cut_lo = (float)(c * (1.0 - 1e-4));
    a.prim_cut_hi = (float)(c * (1.0 + 1e-4));
  } else {
    a.prim_cut_lo = 0.0f;
    a.prim_cut_hi = 3.0e38f;
  }
}

namespace {

template <typename T>
int upload(DevBuf& b, const std::vector<T>& v, cudaStream_t st) {
  CK(b.ensure(std::max<size_t>(sizeof(T) * v.size(), 16)));
  if (!v.empty()) CK(cudaMemcpyAsync(b.p, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice, st));
  return OK;
}

void default_tuning(oqpg_tuning& t) {
  for (int k = 0; k < NCLASS; ++k) {
    t.split_log2[k] = -1;   // by the family the list runs (eff_split)
    t.family[k] = 0;        // by list size (list_team)
    t.chunk[k] = 32;
    t.ctas_per_sm[k] = 0;
  }
}

// A batch of nmol molecules: nshell_m[m] shells on natom_m[m] atoms each, the
// shell and atom arrays concatenated molecule by molecule (origin 1-based
// within the molecule).  One molecule is the batch of one.
// Schwarz bounds sqrt(max |(ab|ab)|) per pair (ints_exchange, int2.F90:1582-1737)
// from pair tables built with the very tight cutoffs 1e-17 / 50; inv_mu2 > 0
// gives the bounds of the erf-attenuated operator (int2.F90:675-681).
// Needs the context's shells, AO offsets and molecules on the device.
int schwarz_bounds(oqpg_ctx* c, double inv_mu2, std::vector<double>& out) {
  cudaStream_t st = c->stream;
  int rc;
  HostPairs sp;
  build_pairs(*c, c->h_am, c->h_ncontr, c->h_poff, c->h_ex.data(), c->h_cc.data(), 1e-17, 50.0, true, sp, false,
              true);
  DevBuf d_pairs, d_prims, d_diag, d_q, d_w;
  if ((rc = upload(d_pairs, sp.pairs, st))) return rc;
  if ((rc = upload(d_prims, sp.prims, st))) return rc;
  std::vector<std::vector<uint2>> diag(NCLASS);
  for (int p = 0; p < c->npair; ++p) {
    if (sp.pairs[p].pcnt == 0) continue;
    diag[class_index(sp.type[p], sp.type[p])].push_back(make_uint2(p, p));
  }
  CK(d_q.ensure(sizeof(double) * c->npair));
  CK(d_w.ensure(sizeof(unsigned long long)));
  CK(cudaMemsetAsync(d_q.p, 0, sizeof(double) * c->npair, st));
  for (int cl = 0; cl < NCLASS; ++cl) {
    if (diag[cl].empty()) continue;
    if ((rc = upload(d_diag, diag[cl], st))) return rc;
    BuildArgs a{};
    a.shells = c->d_shells.as<ShellDev>();
    a.pairs = d_pairs.as<PairDev>();
    a.prims = d_prims.as<PrimPair>();
    a.quartets = d_diag.as<uint2>();
    a.nquartets = (long long)diag[cl].size();
    a.nbf = c->stride;
    a.kstride = (size_t)c->nbf * c->stride;
    a.prim_cut = 1e-17;
    a.prim_cut2 = 1e-34;
    a.inv_mu2 = inv_mu2;
    set_band(a);
    a.schwarz_out = d_q.as<double>();
    CK(cudaMemsetAsync(d_w.p, 0, sizeof(unsigned long long), st));
    a.work = d_w.as<unsigned long long>();
    CK(launch_class(cl, c->pure, MODE_SCHWARZ, a, c->nsm, st));
    CK(cudaStreamSynchronize(st));  // d_diag is reused by the next class
  }
  out.resize(c->npair);
  CK(cudaMemcpyAsync(out.data(), d_q.p, sizeof(double) * c->npair, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  return OK;
}

// Device screening tables of one set of Schwarz bounds: the bounds (FP64,
// FP32) and each molecule's pairs by descending bound.
int upload_schwarz(oqpg_ctx* c, const std::vector<double>& q, DevBuf& d_q, DevBuf& d_qf, DevBuf& d_sidx,
                   DevBuf& d_sq) {
  cudaStream_t st = c->stream;
  int rc;
  if ((rc = upload(d_q, q, st))) return rc;
  std::vector<float> qf(c->npair);
  for (int p = 0; p < c->npair; ++p) qf[p] = (float)q[p];
  if ((rc = upload(d_qf, qf, st))) return rc;
  std::vector<int> order(c->npair);
  for (int p = 0; p < c->npair; ++p) order[p] = p;
  for (const MolDev& M : c->mols)
    std::stable_sort(order.begin() + M.pair0, order.begin() + M.pair0 + M.npair,
                     [&](int x, int y) { return q[x] > q[y]; });
  std::vector<double> sq(c->npair);
  for (int p = 0; p < c->npair; ++p) sq[p] = q[order[p]];
  if ((rc = upload(d_sidx, order, st))) return rc;
  if ((rc = upload(d_sq, sq, st))) return rc;
  CK(cudaStreamSynchronize(st));
  return OK;
}

// Pair tables of the Fock-type builds at cutoff (primitive cutoffs 1e-4 tau and
// 25 ln 10, int2.F90:260-272; int2_prepare_pair), key-ordered so that a looser
// run-time cutoff is a prefix of every shell pair's range.
int fock_tables(oqpg_ctx* c, double cutoff) {
  cudaStream_t st = c->stream;
  int rc;
  HostPairs fp;
  build_pairs(*c, c->h_am, c->h_ncontr, c->h_poff, c->h_ex.data(), c->h_cc.data(), 1e-4 * cutoff,
              25.0 * std::log(10.0), true, fp, true, true);
  if ((rc = upload(c->d_pairs, fp.pairs, st))) return rc;
  if ((rc = upload(c->d_prims, fp.prims, st))) return rc;
  std::vector<PrimPairF> pf(fp.prims.size());
  for (size_t i = 0; i < pf.size(); ++i) {
    const PrimPair& q = fp.prims[i];
    pf[i] = PrimPairF{(float)q.p, (float)q.hp, (float)q.px, (float)q.py, (float)q.pz,
                      (float)q.ax, (float)q.ay, (float)q.az, (float)q.sp, 0.0f};
  }
  if ((rc = upload(c->d_primsf, pf, st))) return rc;
  // double-float copy for the df mode: every FP64 field as an FP32 pair
  std::vector<PrimPairDF> pd(fp.prims.size());
  auto split = [](double v) {
    const float h = (float)v;
    return dfl(h, (float)(v - (double)h));
  };
  for (size_t i = 0; i < pd.size(); ++i) {
    const PrimPair& q = fp.prims[i];
    PrimPairDF& o = pd[i];
    o.p = split(q.p); o.hp = split(q.hp); o.px = split(q.px); o.py = split(q.py); o.pz = split(q.pz);
    o.ax = split(q.ax); o.ay = split(q.ay); o.az = split(q.az); o.sp = split(q.sp);
    o.spf = q.spf; o.pf = q.pf;
  }
  if ((rc = upload(c->d_primsdf, pd, st))) return rc;
  if ((rc = upload(c->d_pair_ij, fp.ij, st))) return rc;
  if ((rc = upload(c->d_pair_type, fp.type, st))) return rc;
  if ((rc = upload(c->d_pair_mol, fp.mol, st))) return rc;
  CK(cudaStreamSynchronize(st));
  c->h_fpairs = fp.pairs;
  c->h_fkey = fp.key;
  c->tau_built = cutoff;
  return OK;
}

int ctx_init(oqpg_ctx* c, int nmol, const int* nshell_m, const int* natom_m, const int* am_, const int* ncontr_,
             const int* origin, const double* ex, const double* cc, const int* harmonic, const double* xyz,
             double cutoff) {
  if (nmol <= 0 || !nshell_m || !natom_m || !am_ || !ncontr_ || !origin || !ex || !cc || !xyz) return UNSUPPORTED;
  int nshell = 0, natom = 0;
  for (int m = 0; m < nmol; ++m) {
    if (nshell_m[m] <= 0 || natom_m[m] <= 0) return UNSUPPORTED;
    nshell += nshell_m[m];
    natom += natom_m[m];
  }
  std::vector<int> am(am_, am_ + nshell), ncontr(ncontr_, ncontr_ + nshell), poff(nshell);
  int npure = 0, nd = 0, off = 0;
  c->nmol = nmol; c->nshell = nshell; c->natom = natom; c->tau = cutoff;
  default_tuning(c->tune);
  c->shells.resize(nshell); c->aoff.resize(nshell); c->naos.resize(nshell); c->mols.resize(nmol);
  {
    int s = 0;
    for (int m = 0; m < nmol; ++m)
      for (int k = 0; k < nshell_m[m]; ++k, ++s) {
        if (am[s] < 0 || am[s] > 3 || ncontr[s] <= 0 || origin[s] < 1 || origin[s] > natom_m[m]) return UNSUPPORTED;
        if (am[s] >= 2) { ++nd; if (harmonic && harmonic[s]) ++npure; }
        if (am[s] == 3) c->has_f = true;
        poff[s] = off; off += ncontr[s];
      }
  }
  if (npure != 0 && npure != nd) return UNSUPPORTED;  // mixed Cartesian / pure d, f shells
  c->pure = nd > 0 && npure == nd;
  int s = 0, atom0 = 0, row0 = 0, pair0 = 0, stride = 0;
  long long tri0 = 0, dsh0 = 0;
  std::vector<int> row_mol;
  for (int m = 0; m < nmol; ++m) {
    MolDev& M = c->mols[m];
    M.shell0 = s; M.ns = nshell_m[m]; M.row0 = row0; M.pair0 = pair0;
    M.npair = M.ns * (M.ns + 1) / 2;
    int aoff = 0;
    for (int k = 0; k < M.ns; ++k, ++s) {
      ShellDev& S = c->shells[s];
      const int at = atom0 + origin[s] - 1;
      S.x = xyz[3 * at]; S.y = xyz[3 * at + 1]; S.z = xyz[3 * at + 2];
      S.am = am[s]; S.harm = (c->pure && am[s] >= 2) ? 1 : 0;
      S.nao = (S.harm ? 2 * am[s] + 1 : ncart(am[s]));
      S.aoff = aoff;
      S.mrow = row0;
      c->aoff[s] = aoff; c->naos[s] = S.nao;
      aoff += S.nao;
    }
    M.nbf = aoff;
    M.tri0 = tri0;
    M.dsh0 = dsh0;
    for (int r = 0; r < M.nbf; ++r) row_mol.push_back(m);
    tri0 += (long long)M.nbf * (M.nbf + 1) / 2;
    dsh0 += (long long)M.ns * M.ns;
    row0 += M.nbf;
    pair0 += M.npair;
    atom0 += natom_m[m];
    stride = std::max(stride, M.nbf);
  }
  c->nbf = row0; c->stride = stride; c->ntri = tri0; c->dsh_elems = dsh0; c->npair = pair0;
  if ((unsigned)pair0 > PAIR_MASK) return UNSUPPORTED;   // quartet entries keep two bits of the pair index
  c->h_am = am; c->h_ncontr = ncontr; c->h_poff = poff;
  c->h_ex.assign(ex, ex + off); c->h_cc.assign(cc, cc + off);
  c->shell_atom.resize(nshell);
  {
    int s2 = 0, a0 = 0;
    for (int m = 0; m < nmol; ++m) {
      for (int k = 0; k < nshell_m[m]; ++k, ++s2) c->shell_atom[s2] = a0 + origin[s2] - 1;
      a0 += natom_m[m];
    }
  }
  CK(cudaGetDevice(&c->dev));
  CK(cudaDeviceGetAttribute(&c->nsm, cudaDevAttrMultiProcessorCount, c->dev));
  CK(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
  for (auto& e : c->ev) CK(cudaEventCreate(&e));
  for (auto& p : c->evc) for (auto& e : p) CK(cudaEventCreate(&e));
  cudaStream_t st = c->stream;
  int rc;
  if ((rc = upload(c->d_shells, c->shells, st))) return rc;
  if ((rc = upload(c->d_aoff, c->aoff, st))) return rc;
  if ((rc = upload(c->d_naos, c->naos, st))) return rc;
  if ((rc = upload(c->d_mols, c->mols, st))) return rc;
  if ((rc = upload(c->d_row_mol, row_mol, st))) return rc;

  // --- Schwarz bounds with OpenQP's very tight cutoffs (int2.F90:1600-1604)
  if ((rc = schwarz_bounds(c, 0.0, c->schwarz_pair))) return rc;

  // --- pair tables of the Fock build
  if ((rc = fock_tables(c, cutoff))) return rc;
  CK(cudaStreamSynchronize(st));
  if ((rc = upload_schwarz(c, c->schwarz_pair, c->d_q, c->d_qf, c->d_sorted_idx, c->d_sorted_q))) return rc;
  // --- shell families (shared primitives of generally contracted s shells)
  return family_tables(c, cutoff);
}

}  // namespace

// Screening tables of the erf-attenuated operator for mu (kept until mu changes).
int oqpg::ensure_att(oqpg_ctx* c, double mu) {
  if (!(mu > 0.0)) return UNSUPPORTED;
  if (c->att_mu == mu) return OK;
  c->att_mu = 0.0;
  int rc;
  if ((rc = schwarz_bounds(c, 1.0 / (mu * mu), c->schwarz_pair_att))) return rc;
  if ((rc = upload_schwarz(c, c->schwarz_pair_att, c->d_q_att, c->d_qf_att, c->d_sorted_idx_att,
                           c->d_sorted_q_att)))
    return rc;
  c->att_mu = mu;
  return OK;
}

namespace {

void ctx_free(oqpg_ctx* c) {
  if (!c) return;
  if (c->gexec) cudaGraphExecDestroy(c->gexec);
  DevBuf* bufs[] = {&c->d_shells, &c->d_pairs, &c->d_prims, &c->d_pair_ij, &c->d_pair_type, &c->d_q, &c->d_qf,
                    &c->d_aoff, &c->d_naos, &c->d_mols, &c->d_pair_mol, &c->d_row_mol, &c->d_primsf, &c->d_primsdf,
                    &c->d_sorted_idx, &c->d_sorted_q, &c->d_dp, &c->d_f, &c->d_fold, &c->d_gin, &c->d_gout,
                    &c->d_gpairs, &c->d_gprims, &c->d_galpha, &c->d_gprimsf, &c->d_galphaf, &c->d_coff,
                    &c->d_atom, &c->d_gmat, &c->d_gmatf, &c->d_dshg, &c->d_gcounts, &c->d_gwork, &c->d_de,
                    &c->d_gcnt, &c->d_q_att, &c->d_qf_att, &c->d_sorted_idx_att, &c->d_sorted_q_att,
                    &c->d_fpairs, &c->d_fmem, &c->d_fprims, &c->d_fprimsf, &c->d_fprimsdf, &c->d_fcoef,
                    &c->d_fcoefdf, &c->d_fpair_mol, &c->d_fpair_type,
                    &c->d_fq, &c->d_fsorted_idx, &c->d_fsorted_q, &c->d_fmol0, &c->d_fmoln,
                    &c->d_pair_fam_multi, &c->d_fmsorted_idx, &c->d_fmsorted_q, &c->d_fmmol0, &c->d_fmmoln};
  for (DevBuf* b : bufs) b->release();
  c->hb.release();
  c->gb.release();
  for (auto& b : c->d_glists) b.release();
  for (auto& b : c->d_gslists) b.release();
  c->d_gbins.release();
  c->d_ghist.release();
  c->d_gcur.release();
  if (c->h_in) cudaFreeHost(c->h_in);
  if (c->h_out) cudaFreeHost(c->h_out);
  for (auto& e : c->ev) if (e) cudaEventDestroy(e);
  for (auto& p : c->evc) for (auto& e : p) if (e) cudaEventDestroy(e);
  if (c->gstream) cudaStreamDestroy(c->gstream);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

}  // namespace

namespace oqpg {
bool split_on(const oqpg_ctx* c) {
  return (c->precision_mode == 1 || c->precision_mode == 2 || c->precision_mode == 4) && c->tau_f32 > 0.0;
}
// double-float kernels for the quartets that are not FP32 (modes 3 and 4)
bool df_on(const oqpg_ctx* c) { return c->precision_mode == 3 || c->precision_mode == 4; }
}  // namespace oqpg

namespace {

// Buffers of one pipeline whose sizes follow from the batch and the job.  A
// general job stages all its slices in dk (and its FP32 / double-float copies).
int ensure_bufs(oqpg_ctx* c, BuildBufs& B, const Job& job) {
  const size_t n2 = (size_t)c->nbf * c->stride;
  const size_t nj = (size_t)std::max(job.nj(), 1), nk = (size_t)std::max(job.nk(), 1);
  if (job.gen) {
    const size_t nsl = std::max<size_t>(job.gen->slices.size(), 1);
    CK(B.dk.ensure(sizeof(double) * nsl * n2));
    if (split_on(c)) CK(B.dkf.ensure(sizeof(float) * nsl * n2));
    if (df_on(c)) CK(B.dkdf.ensure(sizeof(dfl) * nsl * n2));
  } else {
    CK(B.dj.ensure(sizeof(double) * n2));
    if (nk == 2) CK(B.dk.ensure(sizeof(double) * 2 * n2));
    if (split_on(c)) {
      CK(B.djf.ensure(sizeof(float) * n2));
      if (nk == 2) CK(B.dkf.ensure(sizeof(float) * 2 * n2));
    }
    if (df_on(c)) {
      CK(B.djdf.ensure(sizeof(dfl) * n2));
      if (nk == 2) CK(B.dkdf.ensure(sizeof(dfl) * 2 * n2));
    }
  }
  CK(B.gj.ensure(sizeof(double) * nj * n2));
  CK(B.gk.ensure(sizeof(double) * nk * n2));
  CK(B.dsh.ensure(sizeof(double) * std::max<long long>(c->dsh_elems, 1)));
  CK(B.dshf.ensure(sizeof(float) * std::max<long long>(c->dsh_elems, 1)));
  CK(B.dmax.ensure(sizeof(unsigned long long) * c->nmol));
  CK(B.counts.ensure(sizeof(unsigned long long) * (NLIST + 2 * NCLASS)));   // + family member quartets
  CK(B.primc.ensure(sizeof(unsigned long long) * NLIST));
  CK(B.hist.ensure(sizeof(unsigned long long) * NLIST * NBIN));
  CK(B.cursor.ensure(sizeof(unsigned long long) * NLIST * NBIN));
  CK(B.work.ensure(sizeof(unsigned long long) * 2 * NLIST));
  CK(B.ranges.ensure(sizeof(unsigned long long) * 4 * NLIST));
  CK(B.caps.ensure(sizeof(unsigned long long) * NLIST));
  CK(B.split.ensure(sizeof(int) * NLIST));
  CK(B.flag.ensure(sizeof(unsigned)));
  if (petite_on(c, job)) {
    CK(B.sym.ensure(sizeof(unsigned long long) * 2));
    CK(B.fsk.ensure(sizeof(double) * (size_t)c->ntri * std::max(job.nfocks, 1)));
  }
  if (!B.h_rb) CK(cudaMallocHost(&B.h_rb, sizeof(unsigned long long) * (1 + 2 * NLIST + 2 * NCLASS)));
  return OK;
}

ListArgs list_args(const oqpg_ctx* c, BuildBufs& B, const Job& job) {
  ListArgs la{};
  la.npair = c->npair;
  la.mols = c->d_mols.as<MolDev>();
  la.pair_mol = c->d_pair_mol.as<int>();
  la.pair_ij = c->d_pair_ij.as<int2>();
  la.pair_type = c->d_pair_type.as<int>();
  const bool att = job.inv_mu2 != 0.0;  // erf-attenuated pass: its own Schwarz bounds
  la.q = (att ? c->d_q_att : c->d_q).as<double>();
  la.qf = (att ? c->d_qf_att : c->d_qf).as<float>();
  la.sorted_idx = (att ? c->d_sorted_idx_att : c->d_sorted_idx).as<int>();
  la.sorted_q = (att ? c->d_sorted_q_att : c->d_sorted_q).as<double>();
  la.dsh = B.dsh.as<double>(); la.dshf = B.dshf.as<float>();
  la.dmax_bits = B.dmax.as<unsigned long long>();
  la.tau = c->tau;
  la.tau_f32 = split_on(c) ? c->tau_f32 : 0.0;
  la.counts = B.counts.as<unsigned long long>();
  for (int k = 0; k < NLIST; ++k) { la.lists[k] = B.lists[k].as<uint2>(); la.caps[k] = B.cap[k]; }
  if (fam_on(c, job)) {
    la.fam = 1;
    la.pair_fam_multi = c->d_pair_fam_multi.as<unsigned char>();
    la.nfpair = c->nfpair;
    la.fpairs = c->d_fpairs.as<PairDev>();
    la.fmem = c->d_fmem.as<FamMem>();
    la.fpair_mol = c->d_fpair_mol.as<int>();
    la.fpair_type = c->d_fpair_type.as<int>();
    la.fq = c->d_fq.as<double>();
    la.fsorted_idx = c->d_fsorted_idx.as<int>();
    la.fsorted_q = c->d_fsorted_q.as<double>();
    la.fmol0 = c->d_fmol0.as<int>();
    la.fmoln = c->d_fmoln.as<int>();
    la.fmsorted_idx = c->d_fmsorted_idx.as<int>();
    la.fmsorted_q = c->d_fmsorted_q.as<double>();
    la.fmmol0 = c->d_fmmol0.as<int>();
    la.fmmoln = c->d_fmmoln.as<int>();
    la.fam_members = B.counts.as<unsigned long long>() + NLIST;
  }
  if (petite_on(c, job)) {
    la.sym_map = c->d_sym_map.as<int>();
    la.sym_nops = c->sym_nops;
    la.sym_ns = c->nshell;
    la.sym_bits = B.sym.as<unsigned long long>();
  }
  return la;
}

// Screening stage shared by the count pass and the build: unpacked densities
// (and FP32 copies), shell densities and their per-molecule maxima.
int issue_densities(oqpg_ctx* c, BuildBufs& B, const Job& job, cudaStream_t st) {
  if (job.gen) return gen_densities(c, B, *job.gen, st);
  const double* dp = job.dp;
  const int nfocks = job.nfocks;
  const size_t n2 = (size_t)c->nbf * c->stride;
  const unsigned g = (unsigned)std::min<long long>((n2 + 255) / 256, c->nsm * 8LL);
  k_unpack<<<g, 256, 0, st>>>(dp, nfocks, c->d_mols.as<MolDev>(), c->d_row_mol.as<int>(), c->nbf, c->stride,
                              B.dj.as<double>(), B.dk.as<double>());
  CK(cudaGetLastError());
  if (split_on(c)) {
    k_to_f32<<<g, 256, 0, st>>>(B.dj.as<double>(), (long long)n2, B.djf.as<float>());
    CK(cudaGetLastError());
    if (nfocks == 2) {
      k_to_f32<<<(unsigned)std::min<long long>((2 * n2 + 255) / 256, c->nsm * 8LL), 256, 0, st>>>(
          B.dk.as<double>(), (long long)(2 * n2), B.dkf.as<float>());
      CK(cudaGetLastError());
    }
  }
  if (df_on(c)) {
    k_to_df<<<g, 256, 0, st>>>(B.dj.as<double>(), (long long)n2, B.djdf.as<dfl>());
    CK(cudaGetLastError());
    if (nfocks == 2) {
      k_to_df<<<(unsigned)std::min<long long>((2 * n2 + 255) / 256, c->nsm * 8LL), 256, 0, st>>>(
          B.dk.as<double>(), (long long)(2 * n2), B.dkdf.as<dfl>());
      CK(cudaGetLastError());
    }
  }
  CK(cudaMemsetAsync(B.dmax.p, 0, sizeof(unsigned long long) * c->nmol, st));
  k_dsh<<<(unsigned)std::min<long long>((c->npair + 127) / 128, c->nsm * 8LL), 128, 0, st>>>(
      dp, nfocks, c->d_mols.as<MolDev>(), c->d_pair_mol.as<int>(), c->d_pair_ij.as<int2>(), c->npair,
      c->d_aoff.as<int>(), c->d_naos.as<int>(), B.dsh.as<double>(), B.dshf.as<float>(),
      B.dmax.as<unsigned long long>());
  CK(cudaGetLastError());
  if (petite_on(c, job)) return petite_check(c, B, job, st);
  return OK;
}

// Whether a list of class cl with capacity cap runs the warp-per-quartet
// kernels: the only family of the class, the tuned one, or by default warp per
// quartet while the list is too short to fill the GPU thread per quartet.
bool list_team(const oqpg_ctx* c, int cl, unsigned long long cap) {
  const ClassInfo& ci = class_info(cl);
  if (!ci.small) return true;
  if (!ci.team) return false;
  if (c->tune.family[cl] == 1) return false;
  if (c->tune.family[cl] == 2) return true;
  return (long long)cap < SMALL_MIN_PER_SM * c->nsm;
}
// The primitive-count split of a list: thread-per-quartet lists hand quartets
// of >= 256 surviving primitive quartets to the primitive-parallel kernel,
// warp-per-quartet lists already those of >= 16, where 32 lanes on the
// primitives beat the team's 2D phase; or the tuned value.
int eff_split(const oqpg_ctx* c, int cl, bool team) {
  const int s = c->tune.split_log2[cl];
  return s >= 0 ? s : (team ? 4 : PRIM_SPLIT_LOG2);
}

// (Re)size the lists of a pipeline for the given per-list counts, with headroom
// for the screening of later densities.
int size_lists(oqpg_ctx* c, BuildBufs& B, const unsigned long long* counts, cudaStream_t st) {
  for (int k = 0; k < NLIST; ++k) {
    if (counts[k] <= B.cap[k] && B.sized) continue;
    const unsigned long long cap = counts[k] ? counts[k] + counts[k] / 4 + 1024 : 0;
    if (cap > B.cap[k]) {
      CK(B.lists[k].ensure(sizeof(uint2) * cap));
      CK(B.slists[k].ensure(sizeof(uint2) * cap));
      CK(B.bins[k].ensure(cap));
      B.cap[k] = cap;
    }
  }
  CK(cudaMemcpyAsync(B.caps.p, B.cap, sizeof(B.cap), cudaMemcpyHostToDevice, st));
  int split[NLIST];
  for (int k = 0; k < NLIST; ++k) {
    const int cl = list_class(k);
    B.team[k] = k < NLIST_SHELL && list_team(c, cl, B.cap[k]) ? 1 : 0;
    // default-tuned thread-per-quartet lists: the head is sized on the device
    split[k] = !class_info(cl).prim                            ? 0
             : (c->tune.split_log2[cl] < 0 && B.team[k] == 0) ? SPLIT_ADAPTIVE
                                                               : head_bins(eff_split(c, cl, B.team[k] != 0));
  }
  CK(cudaMemcpyAsync(B.split.p, split, sizeof(split), cudaMemcpyHostToDevice, st));
  CK(cudaStreamSynchronize(st));  // the host arrays above are stack memory
  B.sized = true;
  return OK;
}

// Count pass: list lengths for the current density without writing the lists.
int count_lists(oqpg_ctx* c, BuildBufs& B, const Job& job, cudaStream_t st, unsigned long long* counts) {
  int rc;
  if ((rc = issue_densities(c, B, job, st))) return rc;
  ListArgs la = list_args(c, B, job);
  la.write = 0;
  CK(cudaMemsetAsync(B.counts.p, 0, sizeof(unsigned long long) * (NLIST + 2 * NCLASS), st));
  k_lists<<<c->npair, 256, 0, st>>>(la);
  CK(cudaGetLastError());
  if (la.fam) {
    k_lists_fam<<<c->nfpair, 256, 0, st>>>(la);
    CK(cudaGetLastError());
  }
  CK(cudaMemcpyAsync(counts, B.counts.p, sizeof(unsigned long long) * NLIST, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  return OK;
}

// Device-driven build: every launch is sized by the pipeline's list
// capacities; list lengths, sort cursors and work ranges stay on the device,
// so the sequence can be captured into a CUDA graph.  A list longer than its
// capacity sets the overflow flag; the finalize kernel then leaves f alone.
int issue_build(oqpg_ctx* c, BuildBufs& B, const Job& job, cudaStream_t st, bool timing, int* nlaunch_out) {
  const int nj = job.nj(), nk = job.nk();
  const size_t n2 = (size_t)c->nbf * c->stride;
  int rc;
  int nlaunch = 0;
  if (timing) CK(cudaEventRecord(c->ev[0], st));
  CK(cudaMemsetAsync(B.flag.p, 0, sizeof(unsigned), st));
  if ((rc = issue_densities(c, B, job, st))) return rc;
  if (job.gen) nlaunch += 2 + (split_on(c) ? 1 : 0) + (df_on(c) ? 1 : 0);
  else nlaunch += 2 + (split_on(c) ? (nk == 2 ? 2 : 1) : 0) + (df_on(c) ? (nk == 2 ? 2 : 1) : 0);
  ListArgs la = list_args(c, B, job);
  la.write = 1;
  B.fam = la.fam != 0;
  CK(cudaMemsetAsync(B.counts.p, 0, sizeof(unsigned long long) * (NLIST + 2 * NCLASS), st));
  k_lists<<<c->npair, 256, 0, st>>>(la);
  CK(cudaGetLastError());
  ++nlaunch;
  if (la.fam) {
    k_lists_fam<<<c->nfpair, 256, 0, st>>>(la);
    CK(cudaGetLastError());
    ++nlaunch;
  }
  // order every list by surviving primitive quartets (counting sort, device-side scan)
  CK(cudaMemsetAsync(B.hist.p, 0, sizeof(unsigned long long) * NLIST * NBIN, st));
  const float lo = (float)(1e-4 * c->tau * (1.0 - 1e-4));
  unsigned long long* counts = B.counts.as<unsigned long long>();
  auto fam_list = [&](int k) { return k >= NLIST_SHELL; };
  for (int k = 0; k < NLIST; ++k) {
    if (!B.cap[k]) continue;
    const long long cap = (long long)B.cap[k];
    const bool fl = fam_list(k);
    k_bin_hist<<<(unsigned)std::min<long long>((cap + 255) / 256, c->nsm * 4LL), 256, 0, st>>>(
        B.lists[k].as<uint2>(), cap, counts + k, (fl ? c->d_fpairs : c->d_pairs).as<PairDev>(),
        (fl ? c->d_fprims : c->d_prims).as<PrimPair>(), lo, fl ? FAM_IDX_MASK : PAIR_MASK,
        fl ? FAM_IDX_MASK : 0xffffffffu, B.bins[k].as<unsigned char>(), B.hist.as<unsigned long long>() + k * NBIN);
    CK(cudaGetLastError());
    ++nlaunch;
  }
  static_assert(NLIST <= 128, "k_bin_scan runs one thread per list in one 128-thread CTA");
  k_bin_scan<<<1, 128, 0, st>>>(counts, B.caps.as<unsigned long long>(), B.split.as<int>(),
                               B.hist.as<unsigned long long>(), B.cursor.as<unsigned long long>(),
                               B.ranges.as<unsigned long long>(), B.flag.as<unsigned>(), c->nsm,
                               nj + nk <= ADAPTIVE_MAX_DENSITIES ? 1 : 0);
  CK(cudaGetLastError());
  ++nlaunch;
  for (int k = 0; k < NLIST; ++k) {
    if (!B.cap[k]) continue;
    const long long cap = (long long)B.cap[k];
    const bool fl = fam_list(k);
    // family lists: longer blocks per CTA (so each bin's pattern runs are
    // longer) with more threads (so each thread's loops stay as short)
    const long long chunk = fl ? 16384 : 4096;
    k_bin_scatter<<<(unsigned)((cap + chunk - 1) / chunk), fl ? 1024 : 256, 0, st>>>(
        B.lists[k].as<uint2>(), cap, counts + k, (fl ? c->d_fpairs : c->d_pairs).as<PairDev>(),
        fl ? FAM_IDX_MASK : PAIR_MASK, fl ? FAM_IDX_MASK : 0xffffffffu, B.bins[k].as<unsigned char>(),
        B.cursor.as<unsigned long long>() + k * NBIN, B.slists[k].as<uint2>(), chunk, B.flag.as<unsigned>(),
        fl ? c->d_fmem.as<FamMem>() : nullptr);
    CK(cudaGetLastError());
    ++nlaunch;
  }
  if (timing) CK(cudaEventRecord(c->ev[1], st));
  // --- integrals + digestion
  if (nj) CK(cudaMemsetAsync(B.gj.p, 0, sizeof(double) * nj * n2, st));
  if (nk) CK(cudaMemsetAsync(B.gk.p, 0, sizeof(double) * nk * n2, st));
  CK(cudaMemsetAsync(B.primc.p, 0, sizeof(unsigned long long) * NLIST, st));
  CK(cudaMemsetAsync(B.work.p, 0, sizeof(unsigned long long) * 2 * NLIST, st));
  BuildArgs a{};
  a.shells = c->d_shells.as<ShellDev>();
  a.pairs = c->d_pairs.as<PairDev>();
  a.prims = c->d_prims.as<PrimPair>();
  a.primsf = c->d_primsf.as<PrimPairF>();
  a.primsdf = c->d_primsdf.as<PrimPairDF>();
  a.nbf = c->stride;
  a.kstride = n2;
  a.nj = nj;
  a.nk = nk;
  a.prim_cut = 1e-4 * c->tau;
  a.prim_cut2 = a.prim_cut * a.prim_cut;
  set_band(a);
  a.elem_cut = c->tau;
  a.inv_mu2 = job.inv_mu2;
  if (job.gen) {
    const size_t k0 = (size_t)job.gen->k0 * n2;
    a.dj = B.dk.as<double>();
    a.dk = B.dk.as<double>() + k0;
    a.djf = B.dkf.as<float>();
    a.dkf = B.dkf.p ? B.dkf.as<float>() + k0 : nullptr;
    a.djdf = B.dkdf.as<dfl>();
    a.dkdf = B.dkdf.p ? B.dkdf.as<dfl>() + k0 : nullptr;
  } else {
    a.dj = B.dj.as<double>();
    a.dk = (nk == 1) ? B.dj.as<double>() : B.dk.as<double>();
    a.djf = B.djf.as<float>();
    a.dkf = (nk == 1) ? B.djf.as<float>() : B.dkf.as<float>();
    a.djdf = B.djdf.as<dfl>();
    a.dkdf = (nk == 1) ? B.djdf.as<dfl>() : B.dkdf.as<dfl>();
  }
  a.gj = B.gj.as<double>();
  a.gk = B.gk.as<double>();
  a.roots_f32 = (c->precision_mode == 2 || c->precision_mode == 4) ? 1 : 0;
  a.fpairs = c->d_fpairs.as<PairDev>();
  a.fmem = c->d_fmem.as<FamMem>();
  a.fprims = c->d_fprims.as<PrimPair>();
  a.fprimsf = c->d_fprimsf.as<PrimPairF>();
  a.fprimsdf = c->d_fprimsdf.as<PrimPairDF>();
  a.fcoefdf = c->d_fcoefdf.as<FamCoefDF>();
  a.fcoef = c->d_fcoef.as<FamCoef>();
  unsigned long long* ranges = B.ranges.as<unsigned long long>();
  // heaviest classes first
  // family quartets of class cl in precision f32: the heavy head warp per
  // quartet, the rest thread per quartet
  auto launch_fam_list = [&](int cl, int f32) -> int {
    const int fli = fam_list_index(cl, f32);
    if (!B.fam || !B.cap[fli]) return OK;
    a.counters = B.primc.as<unsigned long long>() + fli;
    a.quartets = B.slists[fli].as<uint2>();
    a.nquartets = (long long)B.cap[fli];
    a.range = ranges + 4 * fli;
    a.work = B.work.as<unsigned long long>() + NLIST + fli;
    const int kind = f32 ? FAM_F32 : (df_on(c) ? FAM_DF : FAM_FP64);
    CK(launch_family(cl, c->pure, true, kind, a, c->nsm, st));
    a.range = ranges + 4 * fli + 2;
    a.work = B.work.as<unsigned long long>() + fli;
    CK(launch_family(cl, c->pure, false, kind, a, c->nsm, st));
    nlaunch += 2;
    return OK;
  };
  for (int cl = NCLASS - 1; cl >= 0; --cl) {
    const bool fc = B.fam && fam_class(cl);
    if (!B.cap[cl] && !B.cap[NCLASS + cl] && !(fc && (B.cap[fam_list_index(cl, 0)] || B.cap[fam_list_index(cl, 1)])))
      continue;
    if (timing) CK(cudaEventRecord(c->evc[cl][0], st));
    a.chunk = c->tune.chunk[cl];
    a.ctas_per_sm = c->tune.ctas_per_sm[cl];
    for (int prec = 0; prec < 2; ++prec) {
      const int li = cl + prec * NCLASS;
      if (prec == 1 && fc && (rc = launch_fam_list(cl, 0))) return rc;
      if (timing && prec == 1) CK(cudaEventRecord(c->evc[cl][2], st));   // FP64 launches done
      if (prec == 1 && fc && (rc = launch_fam_list(cl, 1))) return rc;
      if (!B.cap[li]) continue;
      const int fl = prec ? MODE_F32 : (df_on(c) ? MODE_DF : 0);
      a.counters = B.primc.as<unsigned long long>() + li;
      a.quartets = B.slists[li].as<uint2>();
      a.nquartets = (long long)B.cap[li];
      a.team = B.team[li];
      if (class_info(cl).prim && eff_split(c, cl, B.team[li] != 0) < 64) {
        // quartets with >= 2^split primitive quartets (a prefix of the sorted
        // list) go to the warp-per-quartet primitive-parallel kernel
        a.range = ranges + 4 * li;
        a.work = B.work.as<unsigned long long>() + NLIST + li;
        CK(launch_class(cl, c->pure, MODE_PRIM | fl, a, c->nsm, st));
        ++nlaunch;
      }
      a.range = ranges + 4 * li + 2;
      a.work = B.work.as<unsigned long long>() + li;
      CK(launch_class(cl, c->pure, MODE_FOCK | fl, a, c->nsm, st));
      ++nlaunch;
    }
    if (timing) CK(cudaEventRecord(c->evc[cl][1], st));
  }
  if (timing) CK(cudaEventRecord(c->ev[2], st));
  if (job.gen) {
    if ((rc = gen_finalize(c, B, *job.gen, st))) return rc;
  } else if (petite_on(c, job)) {
    if ((rc = petite_finalize(c, B, job, (nk == 1) ? 0.5 * job.se : job.se, st))) return rc;
  } else {
    const double ck = (nk == 1) ? 0.5 * job.se : job.se;
    k_finalize<<<(unsigned)std::min<long long>((c->ntri + 255) / 256, c->nsm * 8LL), 256, 0, st>>>(
        B.gj.as<double>(), B.gk.as<double>(), nk, c->d_mols.as<MolDev>(), c->nmol, c->ntri, c->stride, n2, job.sc,
        ck, job.f, job.f_old, B.flag.as<unsigned>());
    CK(cudaGetLastError());
  }
  ++nlaunch;
  if (timing) CK(cudaEventRecord(c->ev[3], st));
  // readback of the flag, the list lengths and the primitive counts (pinned)
  CK(cudaMemcpyAsync(B.h_rb, B.flag.p, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(B.h_rb + 1, B.counts.p, sizeof(unsigned long long) * NLIST, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(B.h_rb + 1 + NLIST, B.primc.p, sizeof(unsigned long long) * NLIST, cudaMemcpyDeviceToHost,
                     st));
  CK(cudaMemcpyAsync(B.h_rb + 1 + 2 * NLIST, B.counts.as<unsigned long long>() + NLIST,
                     sizeof(unsigned long long) * 2 * NCLASS, cudaMemcpyDeviceToHost, st));
  if (nlaunch_out) *nlaunch_out = nlaunch;
  return OK;
}

void record_stats(oqpg_ctx* c, const BuildBufs& B, int nlaunch, bool timing) {
  const unsigned long long* cnt = B.h_rb + 1;
  const unsigned long long* nprim = B.h_rb + 1 + NLIST;
  for (int k = 0; k < NLIST; ++k) c->counts[k] = cnt[k];
  float t01 = 0, t12 = 0, t03 = 0;
  if (timing) {
    cudaEventElapsedTime(&t01, c->ev[0], c->ev[1]);
    cudaEventElapsedTime(&t12, c->ev[1], c->ev[2]);
    cudaEventElapsedTime(&t03, c->ev[0], c->ev[3]);
  }
  double* S = c->last_stats;
  S[1] = 0;
  double nq = 0, q32 = 0, p32 = 0;
  const unsigned long long* fmq = B.h_rb + 1 + 2 * NLIST;   // member quartets of the family lists (FP64, FP32)
  for (int k = 0; k < NCLASS; ++k) {
    // quartets: the shell quartets evaluated (a family quartet counts its members)
    const bool fl = B.fam && fam_class(k);
    const int f64l = fl ? fam_list_index(k, 0) : 0, f32l = fl ? fam_list_index(k, 1) : 0;
    const unsigned long long q32k = cnt[NCLASS + k] + (fl ? fmq[NCLASS + k] : 0ull);
    const unsigned long long q = cnt[k] + q32k + (fl ? fmq[k] : 0ull);
    const double p32k = (double)nprim[NCLASS + k] + (fl ? (double)nprim[f32l] : 0.0);
    nq += (double)q;
    S[7 + k] = (double)q;
    S[7 + NCLASS + k] = (double)nprim[k] + p32k + (fl ? (double)nprim[f64l] : 0.0);
    q32 += (double)q32k;
    p32 += p32k;
    float tk = 0, t32 = 0;
    if (timing && (B.cap[k] || B.cap[NCLASS + k] || (fl && (B.cap[f64l] || B.cap[f32l])))) {
      cudaEventElapsedTime(&tk, c->evc[k][0], c->evc[k][1]);
      cudaEventElapsedTime(&t32, c->evc[k][2], c->evc[k][1]);
    }
    S[7 + 2 * NCLASS + k] = tk;
    S[10 + 3 * NCLASS + k] = t32;
    S[1] += S[7 + NCLASS + k];
  }
  S[0] = nq;
  S[2] = t01;
  S[3] = t12;
  S[4] = t03;
  S[5] = c->nbf;
  S[6] = c->npair;
  S[7 + 3 * NCLASS] = nlaunch;
  S[8 + 3 * NCLASS] = q32;
  S[9 + 3 * NCLASS] = p32;
}

// Core build on device buffers (synchronous).  dp: packed densities (device),
// f: packed output (device), f_old: optional packed previous Fock (device,
// updated).  The first build of a context runs a count pass to size the
// lists; a later build whose lists outgrow their capacities is redone with
// larger ones (f and f_old untouched in between).
}  // namespace

namespace oqpg {
int ctx_build(oqpg_ctx* c, const Job& job, cudaStream_t st) {
  if (!job.gen && job.nfocks != 1 && job.nfocks != 2) return UNSUPPORTED;
  BuildBufs& B = c->hb;
  int rc;
  if ((rc = ensure_bufs(c, B, job))) return rc;
  if (!B.sized) {
    unsigned long long counts[NLIST];
    if ((rc = count_lists(c, B, job, st, counts))) return rc;
    if ((rc = size_lists(c, B, counts, st))) return rc;
  }
  for (int attempt = 0; attempt < 3; ++attempt) {
    int nlaunch = 0;
    if ((rc = issue_build(c, B, job, st, true, &nlaunch))) return rc;
    CK(cudaStreamSynchronize(st));
    const unsigned flag = (unsigned)(B.h_rb[0] & 0xffffffffu);
    if (flag == 0) {
      record_stats(c, B, nlaunch, true);
      return OK;
    }
    if (flag & 2u) return DEV_ERR;  // sort bookkeeping disagreed with the list lengths
    if ((rc = size_lists(c, B, B.h_rb + 1, st))) return rc;
  }
  return DEV_ERR;  // quartet lists never fitted: nothing was written
}
}  // namespace oqpg

namespace {

// SCF job of packed densities
Job packed_job(const double* dp, double* f, double* f_old, int nfocks, double se, double sc) {
  Job j;
  j.dp = dp; j.f = f; j.f_old = f_old; j.nfocks = nfocks; j.se = se; j.sc = sc;
  return j;
}

// CAM build (int2_run_cam, int2.F90:538-584) of packed densities on device
// buffers: pass 1 over 1/r with cam = {alpha, beta, mu, alpha_c, beta_c}'s
// (alpha, alpha_c) as (se, sc), pass 2 over erf(mu r)/r with (beta, beta_c)
// added to f.
int cam_build(oqpg_ctx* c, const double* dp, double* f, int nfocks, const double* cam, cudaStream_t st) {
  if (!cam || !(cam[2] > 0.0)) return UNSUPPORTED;
  int rc;
  if ((rc = ensure_att(c, cam[2]))) return rc;
  Job j1 = packed_job(dp, f, nullptr, nfocks, cam[0], cam[3]);
  j1.petite = false;   // the petite list serves plain SCF builds only
  if ((rc = ctx_build(c, j1, st))) return rc;
  Job j2 = packed_job(dp, f, f, nfocks, cam[1], cam[4]);
  j2.inv_mu2 = 1.0 / (cam[2] * cam[2]);
  j2.petite = false;
  return ctx_build(c, j2, st);
}

int ctx_build_host(oqpg_ctx* c, const double* d, double* f, double* f_old, int nfocks, double se, double sc,
                   const double* cam = nullptr) {
  if (cam && f_old) return UNSUPPORTED;
  const size_t bytes = sizeof(double) * (size_t)c->ntri * nfocks;
  if (bytes > c->h_bytes) {
    if (c->h_in) cudaFreeHost(c->h_in);
    if (c->h_out) cudaFreeHost(c->h_out);
    c->h_in = c->h_out = nullptr;
    c->h_bytes = 0;
    CK(cudaMallocHost(&c->h_in, bytes));
    CK(cudaMallocHost(&c->h_out, bytes));
    c->h_bytes = bytes;
  }
  CK(c->d_dp.ensure(bytes));
  CK(c->d_f.ensure(bytes));
  if (f_old) CK(c->d_fold.ensure(bytes));
  cudaStream_t st = c->stream;
  std::memcpy(c->h_in, d, bytes);
  CK(cudaMemcpyAsync(c->d_dp.p, c->h_in, bytes, cudaMemcpyHostToDevice, st));
  if (f_old) {
    std::memcpy(c->h_out, f_old, bytes);
    CK(cudaMemcpyAsync(c->d_fold.p, c->h_out, bytes, cudaMemcpyHostToDevice, st));
  }
  int rc = cam ? cam_build(c, c->d_dp.as<double>(), c->d_f.as<double>(), nfocks, cam, st)
               : ctx_build(c, packed_job(c->d_dp.as<double>(), c->d_f.as<double>(),
                                         f_old ? c->d_fold.as<double>() : nullptr, nfocks, se, sc), st);
  if (rc) return rc;
  CK(cudaMemcpyAsync(c->h_out, c->d_f.p, bytes, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  std::memcpy(f, c->h_out, bytes);
  if (f_old) std::memcpy(f_old, c->h_out, bytes);
  return OK;
}

// --- captured builds ---------------------------------------------------------

// Capture the device-driven build on the graph pipeline's buffers (d_gin ->
// d_gout), sized from the lengths of a direct build of the same density.
int graph_capture(oqpg_ctx* c, const double* dp, int nfocks, double se, double sc) {
  if (c->gexec) {
    cudaGraphExecDestroy(c->gexec);
    c->gexec = nullptr;
  }
  if (!c->gstream) CK(cudaStreamCreateWithFlags(&c->gstream, cudaStreamNonBlocking));
  cudaStream_t gs = c->gstream;
  BuildBufs& B = c->gb;
  int rc;
  const size_t bytes = sizeof(double) * (size_t)c->ntri * nfocks;
  CK(c->d_gin.ensure(bytes));
  CK(c->d_gout.ensure(bytes));
  const Job cj = packed_job(dp, nullptr, nullptr, nfocks, se, sc);
  if ((rc = ensure_bufs(c, B, cj))) return rc;
  unsigned long long counts[NLIST];
  if ((rc = count_lists(c, B, cj, gs, counts))) return rc;
  for (int k = 0; k < NLIST; ++k) counts[k] = std::max(counts[k], c->counts[k]);
  if ((rc = size_lists(c, B, counts, gs))) return rc;
  CK(cudaStreamSynchronize(gs));
  cudaGraph_t g = nullptr;
  CK(cudaStreamBeginCapture(gs, cudaStreamCaptureModeRelaxed));
  int nlaunch = 0;
  rc = issue_build(c, B, packed_job(c->d_gin.as<double>(), c->d_gout.as<double>(), nullptr, nfocks, se, sc), gs,
                   false, &nlaunch);
  cudaError_t e = cudaStreamEndCapture(gs, &g);
  if (rc) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  CK(e);
  e = cudaGraphInstantiate(&c->gexec, g, 0);
  cudaGraphDestroy(g);
  CK(e);
  c->g_nfocks = nfocks; c->g_se = se; c->g_sc = sc; c->g_mode = c->precision_mode; c->g_tau32 = c->tau_f32;
  c->g_tau = c->tau;
  c->g_nlaunch = nlaunch;
  ++c->graph_captures;
  return OK;
}

// Build through the captured graph: copy d into the graph's input, replay,
// copy the graph's output to f (all on st), then check the overflow flag.  A
// first call, a change of nfocks / scale factors / precision split, or an
// overflow (the density screens in more quartets than the capture was sized
// for) builds directly and recaptures.
int graph_build(oqpg_ctx* c, const double* d_device, double* f_device, int nfocks, double se, double sc,
                cudaStream_t st) {
  if (nfocks != 1 && nfocks != 2) return UNSUPPORTED;
  const size_t bytes = sizeof(double) * (size_t)c->ntri * nfocks;
  const bool fresh = c->gexec && c->g_nfocks == nfocks && c->g_se == se && c->g_sc == sc &&
                     c->g_mode == c->precision_mode && c->g_tau32 == c->tau_f32 && c->g_tau == c->tau;
  int rc;
  if (fresh) {
    CK(cudaMemcpyAsync(c->d_gin.p, d_device, bytes, cudaMemcpyDeviceToDevice, st));
    CK(cudaGraphLaunch(c->gexec, st));
    CK(cudaMemcpyAsync(f_device, c->d_gout.p, bytes, cudaMemcpyDeviceToDevice, st));
    CK(cudaStreamSynchronize(st));
    if ((c->gb.h_rb[0] & 0xffffffffu) == 0) {
      record_stats(c, c->gb, c->g_nlaunch, false);
      ++c->graph_replays;
      return OK;
    }
  }
  if ((rc = ctx_build(c, packed_job(d_device, f_device, nullptr, nfocks, se, sc), st))) return rc;
  CK(cudaStreamSynchronize(st));
  return graph_capture(c, d_device, nfocks, se, sc);
}

}  // namespace

// ===========================================================================
extern "C" {

int oqpg_create(oqpg_ctx** out, int nshell, const int* am, const int* ncontr, const int* origin, const double* ex,
                const double* cc, const int* harmonic, int natom, const double* xyz, double cutoff) {
  return oqpg_create_batch(out, 1, &nshell, &natom, am, ncontr, origin, ex, cc, harmonic, xyz, cutoff);
}

int oqpg_create_batch(oqpg_ctx** out, int nmol, const int* nshell, const int* natom, const int* am,
                      const int* ncontr, const int* origin, const double* ex, const double* cc, const int* harmonic,
                      const double* xyz, double cutoff) {
  if (!out) return UNSUPPORTED;
  *out = nullptr;
  oqpg_ctx* c = new (std::nothrow) oqpg_ctx;
  if (!c) return NO_MEM;
  const int rc = ctx_init(c, nmol, nshell, natom, am, ncontr, origin, ex, cc, harmonic, xyz, cutoff);
  if (rc) {
    ctx_free(c);
    return rc;
  }
  *out = c;
  return OK;
}

int oqpg_batch_info(const oqpg_ctx* ctx, int* nbf, long long* tri0) {
  if (!ctx) return NOT_INIT;
  for (int m = 0; m < ctx->nmol; ++m) {
    if (nbf) nbf[m] = ctx->mols[m].nbf;
    if (tri0) tri0[m] = ctx->mols[m].tri0;
  }
  return ctx->nmol;
}

int oqpg_destroy(oqpg_ctx* ctx) {
  ctx_free(ctx);
  return OK;
}

int oqpg_nbf(const oqpg_ctx* ctx) { return ctx ? ctx->nbf : -1; }

int oqpg_fock_jk(oqpg_ctx* ctx, const double* d, double* f, int nfocks, double se, double sc) {
  if (!ctx) return NOT_INIT;
  return ctx_build_host(ctx, d, f, nullptr, nfocks, se, sc);
}

int oqpg_fock_jk_device(oqpg_ctx* ctx, const double* d_device, double* f_device, int nfocks, double se, double sc,
                        void* stream) {
  if (!ctx) return NOT_INIT;
  cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
  return ctx_build(ctx, packed_job(d_device, f_device, nullptr, nfocks, se, sc), st);
}

int oqpg_schwarz(const oqpg_ctx* ctx, double* q) {
  if (!ctx) return NOT_INIT;
  if (ctx->nmol != 1) return UNSUPPORTED;
  const int ns = ctx->nshell;
  for (int i = 0; i < ns; ++i)
    for (int j = 0; j <= i; ++j) {
      const double v = ctx->schwarz_pair[(size_t)i * (i + 1) / 2 + j];
      q[(size_t)i * ns + j] = q[(size_t)j * ns + i] = v;
    }
  return OK;
}

int oqpg_fock_jk_graph(oqpg_ctx* ctx, const double* d_device, double* f_device, int nfocks, double se, double sc,
                       void* stream) {
  if (!ctx) return NOT_INIT;
  cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
  return graph_build(ctx, d_device, f_device, nfocks, se, sc, st);
}

int oqpg_graph_info(const oqpg_ctx* ctx, int* captures, int* replays, int* kernels) {
  if (!ctx) return NOT_INIT;
  if (captures) *captures = ctx->graph_captures;
  if (replays) *replays = ctx->graph_replays;
  if (kernels) *kernels = ctx->g_nlaunch;
  return OK;
}

int oqpg_set_tuning(oqpg_ctx* ctx, const int* split_log2, const int* chunk, const int* ctas_per_sm) {
  if (!ctx) return NOT_INIT;
  for (int k = 0; k < NCLASS; ++k) {
    if (split_log2 && (split_log2[k] < -1 || split_log2[k] > 64)) return UNSUPPORTED;
    if (chunk && (chunk[k] < 32 || chunk[k] > 4096 || chunk[k] % 32)) return UNSUPPORTED;
    if (ctas_per_sm && (ctas_per_sm[k] < 0 || ctas_per_sm[k] > 64)) return UNSUPPORTED;
  }
  for (int k = 0; k < NCLASS; ++k) {
    if (split_log2) ctx->tune.split_log2[k] = split_log2[k];
    if (chunk) ctx->tune.chunk[k] = chunk[k];
    if (ctas_per_sm) ctx->tune.ctas_per_sm[k] = ctas_per_sm[k];
  }
  // the split bins live on the device and in the captured graph: redo both
  ctx->hb.sized = false;
  ctx->gb.sized = false;
  if (ctx->gexec) {
    cudaGraphExecDestroy(ctx->gexec);
    ctx->gexec = nullptr;
  }
  return OK;
}

int oqpg_set_kernel_family(oqpg_ctx* ctx, const int* family) {
  if (!ctx) return NOT_INIT;
  if (!family) return UNSUPPORTED;
  for (int k = 0; k < NCLASS; ++k)
    if (family[k] < 0 || family[k] > 2) return UNSUPPORTED;
  for (int k = 0; k < NCLASS; ++k) ctx->tune.family[k] = family[k];
  ctx->hb.sized = false;
  ctx->gb.sized = false;
  if (ctx->gexec) {
    cudaGraphExecDestroy(ctx->gexec);
    ctx->gexec = nullptr;
  }
  return OK;
}

int oqpg_get_kernel_family(const oqpg_ctx* ctx, int* family, int* available) {
  if (!ctx) return NOT_INIT;
  for (int k = 0; k < NCLASS; ++k) {
    if (family) family[k] = ctx->tune.family[k];
    if (available) available[k] = (class_info(k).small ? 1 : 0) | (class_info(k).team ? 2 : 0);
  }
  return OK;
}

int oqpg_get_tuning(const oqpg_ctx* ctx, int* split_log2, int* chunk, int* ctas_per_sm) {
  if (!ctx) return NOT_INIT;
  for (int k = 0; k < NCLASS; ++k) {
    if (split_log2) split_log2[k] = ctx->tune.split_log2[k];
    if (chunk) chunk[k] = ctx->tune.chunk[k];
    if (ctas_per_sm) ctas_per_sm[k] = ctx->tune.ctas_per_sm[k];
  }
  return OK;
}

int oqpg_stats(const oqpg_ctx* ctx, double* out, int n) {
  if (!ctx) return NOT_INIT;
  for (int i = 0; i < n && i < 10 + 4 * NCLASS; ++i) out[i] = ctx->last_stats[i];
  return OK;
}

// FP64 FMA throughput probe: every thread runs 8 independent FMA chains.
__global__ void k_fp64_peak(double* out, int iters, double a, double b) {
  double x[8];
  for (int k = 0; k < 8; ++k) x[k] = threadIdx.x * 1e-3 + k;
  for (int i = 0; i < iters; ++i)
#pragma unroll
    for (int k = 0; k < 8; ++k) x[k] = fma(x[k], a, b);
  double s = 0;
  for (int k = 0; k < 8; ++k) s += x[k];
  if (s == 1234.5) out[0] = s;  // keeps the chains alive
}

int oqpg_measure_fp64_peak(int iters, double* tflops) {
  double* d = nullptr;
  CK(cudaMalloc(&d, sizeof(double)));
  int dev = 0, nsm = 0;
  CK(cudaGetDevice(&dev));
  CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  const int blocks = nsm * 4, threads = 256;
  k_fp64_peak<<<blocks, threads>>>(d, 1000, 0.999999, 1e-9);  // warm-up
  CK(cudaEventRecord(e0));
  k_fp64_peak<<<blocks, threads>>>(d, iters, 0.999999, 1e-9);
  CK(cudaEventRecord(e1));
  CK(cudaEventSynchronize(e1));
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  *tflops = 2.0 * 8.0 * (double)iters * blocks * threads / (ms * 1e-3) / 1e12;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(d);
  return OK;
}

// The library's reciprocal and reciprocal square root (FP64 and double-float)
// beside CUDA's rsqrt() and IEEE division, one argument per thread.
__global__ void k_math_check(const double* __restrict__ x, double* __restrict__ out, long long n) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double v = x[i];
  double* o = out + 6 * i;
  o[0] = oqpg::rsqrt64(v);
  o[1] = rsqrt(v);
  o[2] = oqpg::rcp64(v);
  o[3] = 1.0 / v;
  const float h = (float)v;
  const oqpg::dfl d(h, (float)(v - (double)h));
  o[4] = (double)oqpg::df_rsqrt(d);
  o[5] = (double)oqpg::df_rcp(d);
}

int oqpg_math_check(const double* x_device, double* out_device, long long n) {
  if (!x_device || !out_device || n < 0) return UNSUPPORTED;
  if (n == 0) return OK;
  k_math_check<<<(unsigned)((n + 255) / 256), 256>>>(x_device, out_device, n);
  CK(cudaGetLastError());
  CK(cudaDeviceSynchronize());
  return OK;
}

int oqpg_set_precision(oqpg_ctx* ctx, int mode, double threshold) {
  if (!ctx) return NOT_INIT;
  if (mode < 0 || mode > 4) return UNSUPPORTED;
  const bool split = mode == 1 || mode == 2 || mode == 4;
  if (split && !(threshold > 0.0)) return UNSUPPORTED;
  ctx->precision_mode = mode;
  ctx->tau_f32 = split ? threshold : 0.0;
  ctx->hb.sized = false;  // the FP32 lists are sized by a fresh count pass
  return OK;
}

int routec_fock_set_precision(int mode, double threshold) {
  std::lock_guard<std::mutex> lk(g_mutex);
  if (!g_ctx) return NOT_INIT;
  return oqpg_set_precision(g_ctx, mode, threshold);
}

// int2_compute_t_set_cutoff (int2.F90:480-496): tau, 1e-2 tau and 1e-4 tau of
// the following builds; the exponent cutoff and the Schwarz bounds stay.  At
// or above the cutoff the pair tables were built at, only the primitive counts
// of the shell pairs shrink (the tables are key-ordered, so the pairs the
// reference's tables at this cutoff hold are a prefix); below it the tables
// are rebuilt at the new cutoff.
int oqpg_set_cutoff(oqpg_ctx* ctx, double cutoff) {
  if (!ctx) return NOT_INIT;
  if (!(cutoff > 0.0) || !std::isfinite(cutoff)) return UNSUPPORTED;
  if (cutoff == ctx->tau) return OK;
  int rc;
  if (cutoff < ctx->tau_built) {
    if ((rc = fock_tables(ctx, cutoff))) return rc;
  } else {
    const double qcut = 1e-4 * cutoff;
    std::vector<PairDev> pr = ctx->h_fpairs;
    for (PairDev& p : pr) {
      int n = 0;
      while (n < p.pcnt && !(ctx->h_fkey[p.poff + n] < qcut)) ++n;
      p.pcnt = n;
    }
    if ((rc = upload(ctx->d_pairs, pr, ctx->stream))) return rc;
    CK(cudaStreamSynchronize(ctx->stream));
  }
  if ((rc = family_tables(ctx, cutoff))) return rc;
  if (ctx->gexec) {   // a captured build holds the previous tables
    cudaGraphExecDestroy(ctx->gexec);
    ctx->gexec = nullptr;
  }
  ctx->tau = cutoff;
  ctx->hb.sized = false;  // the lists are sized by a fresh count pass
  return OK;
}

double oqpg_get_cutoff(const oqpg_ctx* ctx) { return ctx ? ctx->tau : -1.0; }

// OpenQP's symmetry data (tagarrays OQP_sym_shell_map, OQP_sym_ao_target,
// OQP_sym_ao_sign: 1-based images, the shell or AO index fastest) for the
// process-global context.
void routec_fock_set_symmetry(const int* nops, const long long* shell_map, const long long* ao_target,
                              const double* ao_sign, int* info) {
  std::lock_guard<std::mutex> lk(g_mutex);
  int rc;
  if (!g_ctx) rc = NOT_INIT;
  else if (!nops) rc = UNSUPPORTED;
  else if (*nops <= 1) rc = oqpg_set_symmetry(g_ctx, 0, nullptr, nullptr, nullptr);
  else if (!shell_map || !ao_target || !ao_sign || *nops > 8) rc = UNSUPPORTED;
  else {
    const int k = *nops, ns = g_ctx->nshell, n = g_ctx->nbf;
    std::vector<int> sm((size_t)k * ns), at((size_t)k * n);
    for (size_t i = 0; i < sm.size(); ++i) sm[i] = (int)shell_map[i] - 1;
    for (size_t i = 0; i < at.size(); ++i) at[i] = (int)ao_target[i] - 1;
    rc = oqpg_set_symmetry(g_ctx, k, sm.data(), at.data(), ao_sign);
  }
  if (info) *info = rc;
}

void routec_fock_set_cutoff(const double* cutoff, int* info) {
  std::lock_guard<std::mutex> lk(g_mutex);
  int rc;
  if (!g_ctx) rc = NOT_INIT;
  else if (!cutoff) rc = UNSUPPORTED;
  else rc = oqpg_set_cutoff(g_ctx, *cutoff);
  if (info) *info = rc;
}

int oqpg_class_l(int c, int* l4) {
  if (c < 0 || c >= NCLASS) return UNSUPPORTED;
  for (int i = 0; i < 4; ++i) l4[i] = class_info(c).l[i];
  return OK;
}

int routec_fock_init(int nshell, const int* am, const int* ncontr, const int* origin, const double* ex,
                     const double* cc, const int* harmonic, int natom, const double* xyz, double cutoff) {
  std::lock_guard<std::mutex> lk(g_mutex);
  sig_release();
  if (g_ctx) {
    ctx_free(g_ctx);
    g_ctx = nullptr;
  }
  return oqpg_create(&g_ctx, nshell, am, ncontr, origin, ex, cc, harmonic, natom, xyz, cutoff);
}

void routec_fock_jk(const double* d, double* f, const int* nbf, const int* nfocks, const double* se,
                    const double* sc, int* info) {
  std::lock_guard<std::mutex> lk(g_mutex);
  int rc;
  if (!g_ctx) rc = NOT_INIT;
  else if (!d || !f || !nbf || !nfocks || !se || !sc) rc = UNSUPPORTED;
  else if (*nbf != g_ctx->nbf || g_ctx->nmol != 1) rc = NOT_INIT;   // registered basis does not match the caller's
  else rc = ctx_build_host(g_ctx, d, f, nullptr, *nfocks, *se, *sc);
  if (info) *info = rc;
}

void routec_fock_jk_inc(const double* dd, double* f, double* f_old, const int* nbf, const int* nfocks,
                        const double* se, const double* sc, int* info) {
  std::lock_guard<std::mutex> lk(g_mutex);
  int rc;
  if (!g_ctx) rc = NOT_INIT;
  else if (!dd || !f || !f_old || !nbf || !nfocks || !se || !sc) rc = UNSUPPORTED;
  else if (*nbf != g_ctx->nbf || g_ctx->nmol != 1) rc = NOT_INIT;
  else rc = ctx_build_host(g_ctx, dd, f, f_old, *nfocks, *se, *sc);
  if (info) *info = rc;
}

int routec_fock_init_batch(int nmol, const int* nshell, const int* natom, const int* am, const int* ncontr,
                           const int* origin, const double* ex, const double* cc, const int* harmonic,
                           const double* xyz, double cutoff) {
  std::lock_guard<std::mutex> lk(g_mutex);
  sig_release();
  if (g_ctx) {
    ctx_free(g_ctx);
    g_ctx = nullptr;
  }
  return oqpg_create_batch(&g_ctx, nmol, nshell, natom, am, ncontr, origin, ex, cc, harmonic, xyz, cutoff);
}

int oqpg_fock_jk_cam(oqpg_ctx* ctx, const double* d, double* f, int nfocks, const double* cam) {
  if (!ctx || !d || !f) return UNSUPPORTED;
  return ctx_build_host(ctx, d, f, nullptr, nfocks, 0.0, 0.0, cam);
}

int oqpg_fock_jk_cam_device(oqpg_ctx* ctx, const double* d_device, double* f_device, int nfocks, const double* cam,
                            void* stream) {
  if (!ctx || !d_device || !f_device) return UNSUPPORTED;
  cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
  int rc = cam_build(ctx, d_device, f_device, nfocks, cam, st);
  if (rc) return rc;
  return cudaStreamSynchronize(st) == cudaSuccess ? OK : DEV_ERR;
}

void routec_fock_jk_cam(const double* d, double* f, const int* nbf, const int* nfocks, const double* cam, int* info) {
  int rc;
  if (!g_ctx) rc = NOT_INIT;
  else if (!d || !f || !nbf || !nfocks || !cam) rc = UNSUPPORTED;
  else if (*nbf != g_ctx->nbf || g_ctx->nmol != 1) rc = NOT_INIT;
  else rc = ctx_build_host(g_ctx, d, f, nullptr, *nfocks, 0.0, 0.0, cam);
  if (info) *info = rc;
}

void routec_fock_td(const double* d2, double* apb, double* amb, const int* nbf, const int* nvec, const int* flags,
                    const double* se, const double* sc, int* info) {
  int rc;
  if (!g_ctx) rc = NOT_INIT;
  else if (!d2 || !apb || !amb || !nbf || !nvec || !flags || !se || !sc) rc = UNSUPPORTED;
  else if (*nbf != g_ctx->nbf) rc = NOT_INIT;
  else rc = oqpg_fock_td(g_ctx, d2, apb, amb, *nvec, *flags, *se, *sc);
  if (info) *info = rc;
}

void routec_fock_mrsf(const double* d3, double* f3, const int* nbf, const int* nvec, const int* nmat,
                      const double* se, const double* sc, int* info) {
  int rc;
  if (!g_ctx) rc = NOT_INIT;
  else if (!d3 || !f3 || !nbf || !nvec || !nmat || !se || !sc) rc = UNSUPPORTED;
  else if (*nbf != g_ctx->nbf) rc = NOT_INIT;
  else rc = oqpg_fock_mrsf(g_ctx, d3, f3, *nvec, *nmat, *se, *sc);
  if (info) *info = rc;
}

void routec_fock_tdgrd(const double* d2, double* apb, double* amb, const int* nbf, const int* flags, const double* se,
                       const double* sc, const double* cam, int* info) {
  int rc;
  if (!g_ctx) rc = NOT_INIT;
  else if (!d2 || !apb || !amb || !nbf || !flags || !se || !sc) rc = UNSUPPORTED;
  else if (*nbf != g_ctx->nbf) rc = NOT_INIT;
  else rc = oqpg_fock_tdgrd(g_ctx, d2, apb, amb, *flags, *se, *sc, cam);
  if (info) *info = rc;
}

void routec_fock_rpagrd(const double* xpy, const int* ldp, const int* np, const double* xmy, const int* ldm,
                        const int* nm, const double* t, const int* ldt, const int* nt, const int* nspin, const int* nbf,
                        double* hpp, double* hpt, double* hmm, const double* se, const double* sc, const double* cam,
                        int* info) {
  int rc;
  if (!g_ctx) rc = NOT_INIT;
  else if (!ldp || !np || !ldm || !nm || !ldt || !nt || !nspin || !nbf || !se || !sc) rc = UNSUPPORTED;
  else if (*nbf != g_ctx->nbf) rc = NOT_INIT;
  else rc = oqpg_fock_rpagrd(g_ctx, xpy, *ldp, *np, xmy, *ldm, *nm, t, *ldt, *nt, *nspin, hpp, hpt, hmm, *se, *sc, cam);
  if (info) *info = rc;
}

void routec_fock_jk_batch(const double* d, double* f, const int* nmol, const int* nfocks, const double* se,
                          const double* sc, int* info) {
  std::lock_guard<std::mutex> lk(g_mutex);
  int rc;
  if (!g_ctx) rc = NOT_INIT;
  else if (!d || !f || !nmol || !nfocks || !se || !sc) rc = UNSUPPORTED;
  else if (*nmol != g_ctx->nmol) rc = NOT_INIT;
  else if (*nfocks != 1 && *nfocks != 2) rc = UNSUPPORTED;
  else {
    oqpg_ctx* c = g_ctx;
    const size_t bytes = sizeof(double) * (size_t)c->ntri * *nfocks;
    rc = OK;
    if (bytes > c->h_bytes) {
      if (c->h_in) cudaFreeHost(c->h_in);
      if (c->h_out) cudaFreeHost(c->h_out);
      c->h_in = c->h_out = nullptr;
      c->h_bytes = 0;
      if (cudaMallocHost(&c->h_in, bytes) != cudaSuccess || cudaMallocHost(&c->h_out, bytes) != cudaSuccess) rc = NO_MEM;
      else c->h_bytes = bytes;
    }
    if (!rc && (c->d_dp.ensure(bytes) != cudaSuccess || c->d_f.ensure(bytes) != cudaSuccess)) rc = NO_MEM;
    if (!rc) {
      std::memcpy(c->h_in, d, bytes);
      if (cudaMemcpyAsync(c->d_dp.p, c->h_in, bytes, cudaMemcpyHostToDevice, c->stream) != cudaSuccess) rc = DEV_ERR;
    }
    if (!rc) rc = graph_build(c, c->d_dp.as<double>(), c->d_f.as<double>(), *nfocks, *se, *sc, c->stream);
    if (!rc) {
      if (cudaMemcpyAsync(c->h_out, c->d_f.p, bytes, cudaMemcpyDeviceToHost, c->stream) != cudaSuccess ||
          cudaStreamSynchronize(c->stream) != cudaSuccess)
        rc = DEV_ERR;
      else
        std::memcpy(f, c->h_out, bytes);
    }
  }
  if (info) *info = rc;
}

void routec_grad2(const double* d, const double* xyz, double* de, const int* nbf, const int* natm,
                  const double* hfscale, const double* coulscale, int* info) {
  std::lock_guard<std::mutex> lk(g_mutex);
  int rc;
  if (!g_ctx) rc = NOT_INIT;
  else if (!d || !xyz || !de || !nbf || !natm || !hfscale || !coulscale) rc = UNSUPPORTED;
  else if (*nbf != g_ctx->nbf || *natm != g_ctx->natom || g_ctx->nmol != 1) rc = NOT_INIT;
  else {
    // the registered geometry must be the caller's
    rc = OK;
    for (int s = 0; s < g_ctx->nshell && rc == OK; ++s) {
      const int at = g_ctx->shell_atom[s];
      const ShellDev& S = g_ctx->shells[s];
      if (std::fabs(S.x - xyz[3 * at]) > 1e-10 || std::fabs(S.y - xyz[3 * at + 1]) > 1e-10 ||
          std::fabs(S.z - xyz[3 * at + 2]) > 1e-10)
        rc = NOT_INIT;
    }
    if (rc == OK) rc = oqpg_grad2(g_ctx, d, 1, *hfscale, *coulscale, de);
  }
  if (info) *info = rc;
}

void routec_grad2_mrsf(const double* d, const double* p, const double* spc, const double* xyz, double* de,
                       const int* nbf, const int* natm, const double* hfscale, const double* hfscale2,
                       const double* coulscale, const double* spcscale, const int* mrst, int* info) {
  std::lock_guard<std::mutex> lk(g_mutex);
  int rc;
  if (!g_ctx) rc = NOT_INIT;
  else if (!d || !p || !spc || !xyz || !de || !nbf || !natm || !hfscale || !hfscale2 || !coulscale || !spcscale ||
           !mrst)
    rc = UNSUPPORTED;
  else if (*nbf != g_ctx->nbf || *natm != g_ctx->natom || g_ctx->nmol != 1) rc = NOT_INIT;
  else {
    rc = OK;
    for (int s = 0; s < g_ctx->nshell && rc == OK; ++s) {
      const int at = g_ctx->shell_atom[s];
      const ShellDev& S = g_ctx->shells[s];
      if (std::fabs(S.x - xyz[3 * at]) > 1e-10 || std::fabs(S.y - xyz[3 * at + 1]) > 1e-10 ||
          std::fabs(S.z - xyz[3 * at + 2]) > 1e-10)
        rc = NOT_INIT;
    }
    if (rc == OK) rc = oqpg_grad2_mrsf(g_ctx, d, p, spc, *hfscale, *hfscale2, *coulscale, spcscale, *mrst, de);
  }
  if (info) *info = rc;
}

void routec_fock_finalize(void) {
  std::lock_guard<std::mutex> lk(g_mutex);
  sig_release();
  ctx_free(g_ctx);
  g_ctx = nullptr;
}

}  // extern "C"
