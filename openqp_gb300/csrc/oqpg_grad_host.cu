// Host side of the two-electron HF gradient: the gradient's pair tables
// (OpenQP's grd2 cutoffs), Cartesian-effective densities, the screened
// quartet lists, class dispatch and the C ABI (oqpg_grad2*, routec_grad2).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <vector>

#include "../../include/openqp_gb300.h"
#include "oqpg_grad.cuh"
#include "oqpg_internal.h"

namespace oqpg {

// Screened gradient quartets, one CTA per bra pair P (OpenQP grd2.F90:306-371):
// Schwarz Q_P Q_Q >= cutoff (a prefix of the Schwarz-sorted pairs), not all
// four shells on one atom (zero by translational invariance), and an upper
// bound of the two-particle density with the shell maxima Dm,
// |cj| Dm_ij Dm_kl + ck (Dm_ik Dm_jl + Dm_il Dm_jk), not below cutoff / 2 /
// (Q_P Q_Q); the kernels apply the exact dabmax test.  With the precision
// split, quartets whose bound Q_P Q_Q x that density bound is below tau32 go
// to the FP32 lists.
struct GListArgs {
  int npair, ns;
  const int2* pair_ij;
  const int* pair_type;
  const PairDev* gpairs;
  const double* q;
  const int* sorted_idx;
  const double* sorted_q;
  const double* dsh;
  const int* atom;
  double cj, ck, cutoff, cutoff2;
  double tau32;                 // bound below tau32: FP32 list (0: none)
  unsigned long long* counts;   // NLIST_SHELL: FP64 lists, then FP32 lists
  uint2* lists[NLIST_SHELL];
  unsigned long long caps[NLIST_SHELL];
  int write;
};

// The classes whose gradient kernels keep the 2D tables in registers
// (grad_lane_class in oqpg_grad.cuh: 3 (la+2)(lb+1)(lc+2)(ld+1) <= 48).
bool grad_lane_class_rt(int c) {
  const ClassInfo& ci = class_info(c);
  return 3 * (ci.l[0] + 2) * (ci.l[1] + 1) * (ci.l[2] + 2) * (ci.l[3] + 1) <= 48;
}

__global__ void __launch_bounds__(256) k_grad_lists(const GListArgs a) {
  __shared__ unsigned cnt[NLIST_SHELL];
  __shared__ unsigned long long base[NLIST_SHELL];
  __shared__ int s_len;
  const int P = blockIdx.x;
  if (a.gpairs[P].pcnt == 0) return;
  const double qP = a.q[P];
  if (!(qP > 0.0)) return;
  if (threadIdx.x == 0) {
    const double thr = a.cutoff / qP * (1.0 - 1e-9);
    int lo = 0, hi = a.npair;
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (a.sorted_q[mid] >= thr) lo = mid + 1;
      else hi = mid;
    }
    s_len = lo;
  }
  __syncthreads();
  const int len = s_len;
  const int2 ij = a.pair_ij[P];
  const int tP = a.pair_type[P];
  const double* di = a.dsh + (long long)ij.x * a.ns;
  const double* dj = a.dsh + (long long)ij.y * a.ns;
  const int ati = a.atom[ij.x], atj = a.atom[ij.y];
  for (int s0 = 0; s0 < len; s0 += blockDim.x) {
    if (threadIdx.x < NLIST_SHELL) cnt[threadIdx.x] = 0;
    __syncthreads();
    const int s = s0 + threadIdx.x;
    const int Q = s < len ? a.sorted_idx[s] : 0x7fffffff;
    int c = -1;
    unsigned slot = 0;
    uint2 ent;
    if (Q <= P && a.gpairs[Q].pcnt > 0) {
      const int2 kl = a.pair_ij[Q];
      const double g = qP * a.q[Q];
      const bool same = ati == atj && ati == a.atom[kl.x] && ati == a.atom[kl.y];
      const double bound = a.cj * di[ij.y] * a.dsh[(long long)kl.x * a.ns + kl.y] +
                           a.ck * (di[kl.x] * dj[kl.y] + di[kl.y] * dj[kl.x]);
      if (!(g < a.cutoff) && !same && !(g * bound < a.cutoff2)) {
        const int tQ = a.pair_type[Q];
        if (tP <= tQ) { c = class_index(tP, tQ); ent = make_uint2(P, Q); }
        else { c = class_index(tQ, tP); ent = make_uint2(Q, P); }
        if (g * bound < a.tau32 && !class_has_f(c)) c += NCLASS;  // f classes: FP64 kernels only
        slot = atomicAdd(&cnt[c], 1u);
      }
    }
    __syncthreads();
    if (threadIdx.x < NLIST_SHELL && cnt[threadIdx.x])
      base[threadIdx.x] = atomicAdd(&a.counts[threadIdx.x], (unsigned long long)cnt[threadIdx.x]);
    __syncthreads();
    if (c >= 0 && a.write) {
      const unsigned long long pos = base[c] + slot;
      if (pos < a.caps[c]) a.lists[c][pos] = ent;
    }
    __syncthreads();
  }
}

}  // namespace oqpg

using namespace oqpg;

namespace oqpg {
cudaError_t launch_grad_f0(int c, const GradArgs& g, int nsm, cudaStream_t st);
cudaError_t launch_grad_f1(int c, const GradArgs& g, int nsm, cudaStream_t st);
cudaError_t launch_grad_f2(int c, const GradArgs& g, int nsm, cudaStream_t st);
cudaError_t launch_grad_f3(int c, const GradArgs& g, int nsm, cudaStream_t st);
cudaError_t launch_grad_f4(int c, const GradArgs& g, int nsm, cudaStream_t st);
cudaError_t launch_grad_f(int c, const GradArgs& g, int nsm, cudaStream_t st) {
  if (c < 30) return launch_grad_f0(c, g, nsm, st);
  if (c < 38) return launch_grad_f1(c, g, nsm, st);
  if (c < 45) return launch_grad_f2(c, g, nsm, st);
  if (c < 50) return launch_grad_f3(c, g, nsm, st);
  return launch_grad_f4(c, g, nsm, st);
}
}  // namespace oqpg

namespace {

int gstatus(cudaError_t e) {
  if (e == cudaSuccess) return OK;
  if (e == cudaErrorMemoryAllocation) return NO_MEM;
  return DEV_ERR;
}

#define GK(x)                                          \
  do {                                                 \
    cudaError_t e_ = (x);                              \
    if (e_ != cudaSuccess) {                           \
      if (std::getenv("OQPG_VERBOSE"))                 \
        std::fprintf(stderr, "openqp_gb300: %s at %s:%d\n", cudaGetErrorString(e_), __FILE__, __LINE__); \
      return gstatus(e_);                              \
    }                                                  \
  } while (0)

template <typename T>
int gupload(DevBuf& b, const std::vector<T>& v, cudaStream_t st) {
  GK(b.ensure(std::max<size_t>(sizeof(T) * v.size(), 16)));
  if (!v.empty()) GK(cudaMemcpyAsync(b.p, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice, st));
  return OK;
}

// Pair tables with the cutoffs of grd2_driver_gen (grd2.F90:231-260): pair
// prefactor 10^-20, exponent 20 ln 10, no |K/p| pre-screen.
int grad_init(oqpg_ctx* c) {
  if (c->grad_ready) return OK;
  cudaStream_t st = c->stream;
  HostPairs gp;
  build_pairs(*c, c->h_am, c->h_ncontr, c->h_poff, c->h_ex.data(), c->h_cc.data(), 1e-20, 20.0 * std::log(10.0),
              false, gp);
  int rc;
  if ((rc = gupload(c->d_gpairs, gp.pairs, st))) return rc;
  if ((rc = gupload(c->d_gprims, gp.prims, st))) return rc;
  if ((rc = gupload(c->d_galpha, gp.alpha, st))) return rc;
  std::vector<PrimPairF> pf(gp.prims.size());
  std::vector<float> af(gp.alpha.size());
  for (size_t i = 0; i < pf.size(); ++i) {
    const PrimPair& q = gp.prims[i];
    pf[i] = PrimPairF{(float)q.p, (float)q.hp, (float)q.px, (float)q.py, (float)q.pz,
                      (float)q.ax, (float)q.ay, (float)q.az, (float)q.sp, 0.0f};
    af[i] = (float)gp.alpha[i];
  }
  if ((rc = gupload(c->d_gprimsf, pf, st))) return rc;
  if ((rc = gupload(c->d_galphaf, af, st))) return rc;
  c->coff.resize(c->nshell);
  int n = 0;
  for (int s = 0; s < c->nshell; ++s) { c->coff[s] = n; n += ncart(c->h_am[s]); }
  c->ncart = n;
  if ((rc = gupload(c->d_coff, c->coff, st))) return rc;
  if ((rc = gupload(c->d_atom, c->shell_atom, st))) return rc;
  GK(cudaStreamSynchronize(st));
  c->grad_ready = true;
  return OK;
}

// Cartesian-effective matrix of one full AO matrix M (nbf x nbf): per shell
// block N T^T M T N (T: pure-d projection, N: Cartesian norms); and its
// screening version (AO values for Cartesian bases).
void cart_effective(const oqpg_ctx* c, const double* M, double* Mc) {
  const int nb = c->nbf, nc = c->ncart;
  for (int si = 0; si < c->nshell; ++si)
    for (int sj = 0; sj < c->nshell; ++sj) {
      const ShellDev& A = c->shells[si];
      const ShellDev& B = c->shells[sj];
      const int na = ncart(A.am), nbc = ncart(B.am);
      const bool pa = A.harm != 0, pb = B.harm != 0;
      for (int x = 0; x < na; ++x)
        for (int y = 0; y < nbc; ++y) {
          double v = 0;
          const int ma = pa ? 2 * A.am + 1 : na, mb = pb ? 2 * B.am + 1 : nbc;
          for (int p = 0; p < ma; ++p) {
            const double tp = pa ? pure_coef(A.am, p, x) : (p == x ? 1.0 : 0.0);
            if (tp == 0.0) continue;
            for (int r = 0; r < mb; ++r) {
              const double tr = pb ? pure_coef(B.am, r, y) : (r == y ? 1.0 : 0.0);
              if (tr == 0.0) continue;
              v += tp * tr * M[(size_t)(A.aoff + p) * nb + B.aoff + r];
            }
          }
          Mc[(size_t)(c->coff[si] + x) * nc + c->coff[sj] + y] = v * cart_norm(A.am, x) * cart_norm(B.am, y);
        }
    }
}

// Two-particle density of a gradient run: the bilinear HF form over
// mats = x, y[, xs, ys], or (mrsf) the MRSF form over the eleven matrices of
// grd2_mrsf_compute_data_t.  cjb / ckb bound |Gamma| by the shell maxima
// for the quartet lists: cjb d_ab d_cd + ckb (d_ac d_bd + d_ad d_bc).
struct GammaSpec {
  bool spin = false, mrsf = false;
  double cj = 0, ckt = 0, cks = 0;
  double mcoul = 0, mx = 0, mx2 = 0, mq[3] = {0, 0, 0};
  double cjb = 0, ckb = 0;
};

int grad_run(oqpg_ctx* c, std::vector<double>& mats, int nmat, const GammaSpec& gs, double cutoff, double* de,
             double inv_mu2 = 0.0);

// dE/dR (accumulated into de[3 natom]) for the two-particle density of the
// full AO matrices x, y (and the spin pair xs, ys, both null or both set).
int grad_build(oqpg_ctx* c, const double* x, const double* y, const double* xs, const double* ys, double cj,
               double ckt, double cks, double cutoff, double* de, double inv_mu2 = 0.0) {
  if (c->nmol != 1) return UNSUPPORTED;
  int rc;
  if ((rc = grad_init(c))) return rc;
  const int nc = c->ncart;
  const size_t n2 = (size_t)nc * nc;
  const int nmat = xs ? 4 : 2;
  std::vector<double> mats(n2 * nmat);
  const double* src[4] = {x, y, xs, ys};
  for (int k = 0; k < nmat; ++k) cart_effective(c, src[k], mats.data() + k * n2);
  GammaSpec gs;
  gs.spin = xs != nullptr;
  gs.cj = cj; gs.ckt = ckt; gs.cks = cks;
  gs.cjb = std::fabs(cj);
  gs.ckb = std::fabs(ckt) + std::fabs(cks);
  return grad_run(c, mats, nmat, gs, cutoff, de, inv_mu2);
}

// inv_mu2 != 0: the erf-attenuated pass (its Schwarz bounds must be current:
// ensure_att).
int grad_run(oqpg_ctx* c, std::vector<double>& mats, int nmat, const GammaSpec& gs, double cutoff, double* de,
             double inv_mu2) {
  int rc;
  cudaStream_t st = c->stream;
  const int nc = c->ncart, ns = c->nshell;
  const size_t n2 = (size_t)nc * nc;
  const bool xs = gs.spin;
  // shell maxima of the screening matrices
  std::vector<double> dsh((size_t)ns * ns, 0.0);
  for (int k = 0; k < nmat; ++k)
    for (int si = 0; si < ns; ++si)
      for (int sj = 0; sj < ns; ++sj) {
        double m = 0;
        const int li = c->shells[si].am, lj = c->shells[sj].am;
        for (int a = 0; a < ncart(li); ++a)
          for (int b = 0; b < ncart(lj); ++b) {
            double v = std::fabs(mats[k * n2 + (size_t)(c->coff[si] + a) * nc + c->coff[sj] + b]);
            if (!c->pure) v /= cart_norm(li, a) * cart_norm(lj, b);
            m = std::max(m, v);
          }
        double& d = dsh[(size_t)si * ns + sj];
        d = std::max(d, m);
      }
  if (gs.mrsf)   // the response matrices are not symmetric and enter transposed too
    for (int si = 0; si < ns; ++si)
      for (int sj = 0; sj < si; ++sj) {
        const double m = std::max(dsh[(size_t)si * ns + sj], dsh[(size_t)sj * ns + si]);
        dsh[(size_t)si * ns + sj] = dsh[(size_t)sj * ns + si] = m;
      }
  cudaEvent_t e0 = c->ev[0], e1 = c->ev[3];
  GK(cudaEventRecord(e0, st));
  // the MRSF form runs in FP64 only (no FP32 copies of its eleven matrices)
  const bool split = !gs.mrsf && (c->precision_mode == 1 || c->precision_mode == 2 || c->precision_mode == 4) &&
                     c->tau_f32 > 0.0;
  if ((rc = gupload(c->d_gmat, mats, st))) return rc;
  if (split) {
    std::vector<float> matsf(mats.size());
    for (size_t k = 0; k < mats.size(); ++k) matsf[k] = (float)mats[k];
    if ((rc = gupload(c->d_gmatf, matsf, st))) return rc;
    GK(cudaStreamSynchronize(st));  // matsf is freed at the end of this scope
  }
  if ((rc = gupload(c->d_dshg, dsh, st))) return rc;
  GK(c->d_gcounts.ensure(sizeof(unsigned long long) * NLIST_SHELL));
  GK(c->d_gwork.ensure(sizeof(unsigned long long) * 2 * NLIST_SHELL));
  GK(c->d_gcnt.ensure(sizeof(unsigned long long) * 2));
  GK(c->d_de.ensure(sizeof(double) * 3 * c->natom));
  GListArgs la{};
  la.npair = c->npair; la.ns = ns;
  la.pair_ij = c->d_pair_ij.as<int2>();
  la.pair_type = c->d_pair_type.as<int>();
  la.gpairs = c->d_gpairs.as<PairDev>();
  const bool att = inv_mu2 != 0.0;
  la.q = (att ? c->d_q_att : c->d_q).as<double>();
  la.sorted_idx = (att ? c->d_sorted_idx_att : c->d_sorted_idx).as<int>();
  la.sorted_q = (att ? c->d_sorted_q_att : c->d_sorted_q).as<double>();
  la.dsh = c->d_dshg.as<double>();
  la.atom = c->d_atom.as<int>();
  la.cj = gs.cjb;
  la.ck = gs.ckb;
  la.cutoff = cutoff;
  la.cutoff2 = 0.5 * cutoff;
  la.tau32 = split ? c->tau_f32 : 0.0;
  la.counts = c->d_gcounts.as<unsigned long long>();
  unsigned long long counts[NLIST_SHELL];
  for (int pass = 0; pass < 3; ++pass) {
    la.write = 1;
    for (int k = 0; k < NLIST_SHELL; ++k) { la.lists[k] = c->d_glists[k].as<uint2>(); la.caps[k] = c->gcaps[k]; }
    GK(cudaMemsetAsync(c->d_gcounts.p, 0, sizeof(unsigned long long) * NLIST_SHELL, st));
    k_grad_lists<<<c->npair, 256, 0, st>>>(la);
    GK(cudaGetLastError());
    GK(cudaMemcpyAsync(counts, c->d_gcounts.p, sizeof(counts), cudaMemcpyDeviceToHost, st));
    GK(cudaStreamSynchronize(st));
    bool ok = true;
    for (int k = 0; k < NLIST_SHELL; ++k)
      if (counts[k] > c->gcaps[k]) {
        ok = false;
        const unsigned long long cap = counts[k] + counts[k] / 8 + 1024;
        GK(c->d_glists[k].ensure(sizeof(uint2) * cap));
        c->gcaps[k] = cap;
      }
    if (ok) break;
    if (pass == 2) return DEV_ERR;
  }
  // the lists of the lane classes sorted by primitive-pair product, heaviest
  // first (counting sort on the device, cursors from the host): quartets of
  // at least 2^8 primitive quartets run warp per quartet (k_grad_lane), the
  // rest thread per quartet (k_grad_small)
  unsigned long long head[NLIST_SHELL] = {0};
  bool sorted[NLIST_SHELL] = {false};
  {
    unsigned long long off[NLIST_SHELL + 1] = {0};
    for (int li = 0; li < NLIST_SHELL; ++li) {
      sorted[li] = counts[li] > 0 && grad_lane_class_rt(li % NCLASS);
      off[li + 1] = off[li] + (sorted[li] ? counts[li] : 0);
    }
    if (off[NLIST_SHELL] > 0) {
      GK(c->d_gbins.ensure(off[NLIST_SHELL]));
      GK(c->d_ghist.ensure(sizeof(unsigned long long) * NLIST_SHELL * NBIN));
      GK(c->d_gcur.ensure(sizeof(unsigned long long) * NLIST_SHELL * NBIN));
      GK(cudaMemsetAsync(c->d_ghist.p, 0, sizeof(unsigned long long) * NLIST_SHELL * NBIN, st));
      unsigned char* bins = c->d_gbins.as<unsigned char>();
      unsigned long long* hist = c->d_ghist.as<unsigned long long>();
      for (int li = 0; li < NLIST_SHELL; ++li) {
        if (!sorted[li]) continue;
        if (c->gscaps[li] < c->gcaps[li]) {
          GK(c->d_gslists[li].ensure(sizeof(uint2) * c->gcaps[li]));
          c->gscaps[li] = c->gcaps[li];
        }
        k_bin_hist<<<(unsigned)std::min<unsigned long long>((counts[li] + 255) / 256, c->nsm * 4ULL), 256, 0, st>>>(
            c->d_glists[li].as<uint2>(), (long long)counts[li], nullptr, c->d_gpairs.as<PairDev>(), nullptr, 0.0f,
            PAIR_MASK, 0xffffffffu, bins + off[li], hist + li * NBIN);
        GK(cudaGetLastError());
      }
      std::vector<unsigned long long> h_hist((size_t)NLIST_SHELL * NBIN), h_cur((size_t)NLIST_SHELL * NBIN);
      GK(cudaMemcpyAsync(h_hist.data(), hist, sizeof(unsigned long long) * h_hist.size(), cudaMemcpyDeviceToHost, st));
      GK(cudaStreamSynchronize(st));
      const int nb_head = head_bins(PRIM_SPLIT_LOG2);
      for (int li = 0; li < NLIST_SHELL; ++li) {
        if (!sorted[li]) continue;
        unsigned long long sum = 0;
        for (int b = 0; b < NBIN; ++b) {
          h_cur[(size_t)li * NBIN + b] = sum;
          sum += h_hist[(size_t)li * NBIN + b];
          if (b < nb_head) head[li] = sum;
        }
        if (sum != counts[li]) return DEV_ERR;
      }
      GK(cudaMemcpyAsync(c->d_gcur.p, h_cur.data(), sizeof(unsigned long long) * h_cur.size(), cudaMemcpyHostToDevice,
                         st));
      const long long chunk = 4096;
      for (int li = 0; li < NLIST_SHELL; ++li) {
        if (!sorted[li]) continue;
        k_bin_scatter<<<(unsigned)((counts[li] + chunk - 1) / chunk), 256, 0, st>>>(
            c->d_glists[li].as<uint2>(), (long long)counts[li], nullptr, c->d_gpairs.as<PairDev>(), PAIR_MASK,
            0xffffffffu, bins + off[li], c->d_gcur.as<unsigned long long>() + li * NBIN,
            c->d_gslists[li].as<uint2>(), chunk, nullptr, nullptr);
        GK(cudaGetLastError());
      }
      GK(cudaStreamSynchronize(st));   // h_cur is freed at the end of this scope
    }
  }
  GK(cudaMemsetAsync(c->d_de.p, 0, sizeof(double) * 3 * c->natom, st));
  GK(cudaMemsetAsync(c->d_gwork.p, 0, sizeof(unsigned long long) * 2 * NLIST_SHELL, st));
  GK(cudaMemsetAsync(c->d_gcnt.p, 0, sizeof(unsigned long long) * 2, st));
  GradArgs g{};
  g.shells = c->d_shells.as<ShellDev>();
  g.pairs = c->d_gpairs.as<PairDev>();
  g.prims = c->d_gprims.as<PrimPair>();
  g.alpha = c->d_galpha.as<double>();
  g.primsf = c->d_gprimsf.as<PrimPairF>();
  g.alphaf = c->d_galphaf.as<float>();
  const double* dm = c->d_gmat.as<double>();
  if (gs.mrsf) {
    g.xt = g.yt = dm;
    g.xs = g.ys = nullptr;
    g.mm = dm;
    g.mrsf = 1;
    g.mcoul = gs.mcoul; g.mx = gs.mx; g.mx2 = gs.mx2;
    g.mq1 = gs.mq[0]; g.mq2 = gs.mq[1]; g.mq3 = gs.mq[2];
  } else {
    g.xt = dm; g.yt = dm + n2;
    g.xs = xs ? dm + 2 * n2 : nullptr;
    g.ys = xs ? dm + 3 * n2 : nullptr;
  }
  if (split) {
    const float* fm = c->d_gmatf.as<float>();
    g.xtf = fm; g.ytf = fm + n2;
    g.xsf = xs ? fm + 2 * n2 : nullptr;
    g.ysf = xs ? fm + 3 * n2 : nullptr;
  }
  g.roots_f32 = (c->precision_mode == 2 || c->precision_mode == 4) ? 1 : 0;
  g.ncart = nc;
  g.coff = c->d_coff.as<int>();
  g.atom = c->d_atom.as<int>();
  g.cj = gs.cj; g.ckt = gs.ckt; g.cks = gs.cks;
  g.pure = c->pure ? 1 : 0;
  g.q = (att ? c->d_q_att : c->d_q).as<double>();
  g.inv_mu2 = inv_mu2;
  g.cutoff2 = 0.5 * cutoff;
  // grd2: dtol = 10^-20 and dabcut = 1e-11 (smaller for very tight exponents), both squared
  double zbig = 0;
  for (double e : c->h_ex) zbig = std::max(zbig, e);
  double dabcut = 1e-11;
  if (zbig > 1e6) dabcut /= 10;
  if (zbig > 1e7) dabcut /= 10;
  g.dtol2 = 1e-40;
  g.dabcut2 = dabcut * dabcut;
  g.sdtol = (float)std::sqrt(g.dtol2);
  g.sdab = (float)std::sqrt(g.dabcut2);
  g.de = c->d_de.as<double>();
  g.counters = c->d_gcnt.as<unsigned long long>();
  double listed = 0, listed32 = 0;
  for (int li = NLIST_SHELL - 1; li >= 0; --li) {
    if (!counts[li]) continue;
    const int cl = li % NCLASS;
    const bool f32 = li >= NCLASS;
    listed += (double)counts[li];
    if (f32) listed32 += (double)counts[li];
    auto launch = [&]() {
      return cl < 15 ? launch_grad_a(cl, g, f32, c->nsm, st)
                     : cl < NCLASS_SD ? launch_grad_b(cl, g, f32, c->nsm, st) : launch_grad_f(cl, g, c->nsm, st);
    };
    if (sorted[li]) {
      const uint2* sl = c->d_gslists[li].as<uint2>();
      g.quartets = sl;                       // heavy head: warp per quartet
      g.nquartets = (long long)head[li];
      g.work = c->d_gwork.as<unsigned long long>() + li;
      g.small = 0;
      GK(launch());
      g.quartets = sl + head[li];            // the rest: thread per quartet
      g.nquartets = (long long)(counts[li] - head[li]);
      g.work = c->d_gwork.as<unsigned long long>() + NLIST_SHELL + li;
      g.small = 1;
      GK(launch());
      g.small = 0;
      continue;
    }
    g.quartets = c->d_glists[li].as<uint2>();
    g.nquartets = (long long)counts[li];
    g.work = c->d_gwork.as<unsigned long long>() + li;
    GK(launch());
  }
  std::vector<double> h_de(3 * c->natom);
  unsigned long long h_cnt[2];
  GK(cudaMemcpyAsync(h_de.data(), c->d_de.p, sizeof(double) * h_de.size(), cudaMemcpyDeviceToHost, st));
  GK(cudaMemcpyAsync(h_cnt, c->d_gcnt.p, sizeof(h_cnt), cudaMemcpyDeviceToHost, st));
  GK(cudaEventRecord(e1, st));
  GK(cudaStreamSynchronize(st));
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  for (size_t k = 0; k < h_de.size(); ++k) de[k] += h_de[k];
  c->grad_stats[0] = listed;
  c->grad_stats[1] = (double)h_cnt[1];
  c->grad_stats[2] = (double)h_cnt[0];
  c->grad_stats[3] = ms;
  c->grad_stats[4] = listed32;
  return OK;
}

void unpack_full(const double* dp, int n, double* D) {
  for (int i = 0; i < n; ++i)
    for (int j = 0; j <= i; ++j) D[(size_t)i * n + j] = D[(size_t)j * n + i] = dp[(size_t)i * (i + 1) / 2 + j];
}

int grad_packed(oqpg_ctx* c, const double* d, int nfocks, double hfscale, double coulscale, double* de) {
  if (nfocks != 1 && nfocks != 2) return UNSUPPORTED;
  const int n = c->nbf;
  const size_t n2 = (size_t)n * n, ntri = (size_t)n * (n + 1) / 2;
  std::vector<double> Dt(n2), Ds;
  unpack_full(d, n, Dt.data());
  if (nfocks == 2) {
    std::vector<double> Db(n2);
    unpack_full(d + ntri, n, Db.data());
    Ds.resize(n2);
    for (size_t k = 0; k < n2; ++k) {
      Ds[k] = Dt[k] - Db[k];
      Dt[k] += Db[k];
    }
  }
  const double* ds = nfocks == 2 ? Ds.data() : nullptr;
  return grad_build(c, Dt.data(), Dt.data(), ds, ds, 4.0 * coulscale, hfscale, hfscale, c->tau, de);
}

// grd2 with the MRSF two-particle density (modules/tdhf_mrsf_gradient.F90:
// 341-355 init, :404-601 get_density): d, p (n, n, 2) raw alpha / beta,
// spc (7, n, n), Fortran column-major.
int grad_mrsf(oqpg_ctx* c, const double* d, const double* p, const double* spc, double hfscale, double hfscale2,
              double coulscale, const double* spcscale, int mrst, double* de, const double* cam5 = nullptr) {
  if (c->nmol != 1) return UNSUPPORTED;
  if (mrst != 1 && mrst != 3) return UNSUPPORTED;
  int rc;
  if ((rc = grad_init(c))) return rc;
  const int n = c->nbf, nc = c->ncart;
  const size_t nn = (size_t)n * n, n2 = (size_t)nc * nc;
  std::vector<double> raw(nn), mats(11 * n2);
  auto make = [&](int m, auto elem) {
    for (int r = 0; r < n; ++r)
      for (int q = 0; q < n; ++q) raw[(size_t)r * n + q] = elem((size_t)r, (size_t)q);
    cart_effective(c, raw.data(), mats.data() + m * n2);
  };
  auto F = [&](const double* M, size_t r, size_t q) { return M[r + n * q]; };
  make(0, [&](size_t r, size_t q) { return F(d, r, q) + F(d + nn, r, q); });
  make(1, [&](size_t r, size_t q) { return F(d, r, q) - F(d + nn, r, q); });
  make(2, [&](size_t r, size_t q) { return F(p, r, q) + F(p + nn, r, q); });
  make(3, [&](size_t r, size_t q) { return F(p, r, q) - F(p + nn, r, q); });
  // spc(1..7) = bo2v, bo1v, bco1, bco2, o21v, co12, ball; kept as ball, bo2v, ..., co12
  const int comp[7] = {6, 0, 1, 2, 3, 4, 5};
  for (int k = 0; k < 7; ++k) make(4 + k, [&](size_t r, size_t q) { return spc[comp[k] + 7 * (r + n * q)]; });
  const double sgnk = mrst == 3 ? -1.0 : 1.0;
  GammaSpec gs;
  gs.mrsf = true;
  gs.mcoul = 4.0 * coulscale;
  gs.mx = hfscale;
  gs.mx2 = hfscale2;
  for (int k = 0; k < 3; ++k) gs.mq[k] = sgnk * spcscale[k];
  // |Gamma| <= cjb d_ab d_cd + ckb (d_ac d_bd + d_ad d_bc) over the shell maxima
  // of all eleven matrices (term counts of the reference's sums)
  gs.cjb = 3.0 * std::fabs(gs.mcoul) + 32.0 * std::fabs(spcscale[2]);
  gs.ckb = 6.0 * std::fabs(hfscale) + 4.0 * std::fabs(hfscale2) + 4.0 * std::fabs(spcscale[0]) +
           4.0 * std::fabs(spcscale[1]) + 16.0 * std::fabs(spcscale[2]);
  if (!cam5) return grad_run(c, mats, 11, gs, c->tau, de);
  // grd2_driver's CAM branch (grd2.F90:104-128): regular pass with the alphas,
  // then the attenuated pass with the betas and no Coulomb; the spin-pair
  // coupling terms enter both passes
  if ((rc = ensure_att(c, cam5[4]))) return rc;
  for (int pass = 0; pass < 2; ++pass) {
    GammaSpec gp = gs;
    gp.mcoul = pass ? 0.0 : 4.0;
    gp.mx = pass ? cam5[1] : cam5[0];
    gp.mx2 = pass ? cam5[3] : cam5[2];
    gp.cjb = 3.0 * std::fabs(gp.mcoul) + 32.0 * std::fabs(spcscale[2]);
    gp.ckb = 6.0 * std::fabs(gp.mx) + 4.0 * std::fabs(gp.mx2) + 4.0 * std::fabs(spcscale[0]) +
             4.0 * std::fabs(spcscale[1]) + 16.0 * std::fabs(spcscale[2]);
    if ((rc = grad_run(c, mats, 11, gp, c->tau, de, pass ? 1.0 / (cam5[4] * cam5[4]) : 0.0))) return rc;
  }
  return OK;
}

// grd2_driver's CAM branch for the SCF densities (packed, nfocks 1 or 2):
// regular pass with coulscale 1 and hfscale alpha, erf(mu r)/r pass with
// coulscale 0 and hfscale beta.
int grad_cam(oqpg_ctx* c, const double* d, int nfocks, double alpha, double beta, double mu, double* de) {
  if (nfocks != 1 && nfocks != 2) return UNSUPPORTED;
  if (!(mu > 0.0)) return UNSUPPORTED;
  int rc;
  if ((rc = ensure_att(c, mu))) return rc;
  const int n = c->nbf;
  const size_t n2 = (size_t)n * n, ntri = (size_t)n * (n + 1) / 2;
  std::vector<double> Dt(n2), Ds;
  unpack_full(d, n, Dt.data());
  if (nfocks == 2) {
    std::vector<double> Db(n2);
    unpack_full(d + ntri, n, Db.data());
    Ds.resize(n2);
    for (size_t k = 0; k < n2; ++k) {
      Ds[k] = Dt[k] - Db[k];
      Dt[k] += Db[k];
    }
  }
  const double* ds = nfocks == 2 ? Ds.data() : nullptr;
  if ((rc = grad_build(c, Dt.data(), Dt.data(), ds, ds, 4.0, alpha, alpha, c->tau, de))) return rc;
  return grad_build(c, Dt.data(), Dt.data(), ds, ds, 0.0, beta, beta, c->tau, de, 1.0 / (mu * mu));
}

}  // namespace

extern "C" {

int oqpg_grad2(oqpg_ctx* ctx, const double* d, int nfocks, double hfscale, double coulscale, double* de) {
  if (!ctx) return NOT_INIT;
  if (!d || !de) return UNSUPPORTED;
  return grad_packed(ctx, d, nfocks, hfscale, coulscale, de);
}

int oqpg_grad2_bilinear(oqpg_ctx* ctx, const double* x, const double* y, const double* xs, const double* ys,
                        double cj, double ckt, double cks, double* de) {
  if (!ctx) return NOT_INIT;
  if (!x || !y || !de || (!xs) != (!ys)) return UNSUPPORTED;
  return grad_build(ctx, x, y, xs, ys, cj, ckt, cks, ctx->tau, de);
}

int oqpg_grad2_mrsf(oqpg_ctx* ctx, const double* d, const double* p, const double* spc, double hfscale,
                    double hfscale2, double coulscale, const double* spcscale, int mrst, double* de) {
  if (!ctx) return NOT_INIT;
  if (!d || !p || !spc || !spcscale || !de) return UNSUPPORTED;
  return grad_mrsf(ctx, d, p, spc, hfscale, hfscale2, coulscale, spcscale, mrst, de);
}

int oqpg_grad2_cam(oqpg_ctx* ctx, const double* d, int nfocks, double alpha, double beta, double mu, double* de) {
  if (!ctx) return NOT_INIT;
  if (!d || !de) return UNSUPPORTED;
  return grad_cam(ctx, d, nfocks, alpha, beta, mu, de);
}

int oqpg_grad2_mrsf_cam(oqpg_ctx* ctx, const double* d, const double* p, const double* spc, const double* cam5,
                        const double* spcscale, int mrst, double* de) {
  if (!ctx) return NOT_INIT;
  if (!d || !p || !spc || !cam5 || !spcscale || !de || !(cam5[4] > 0.0)) return UNSUPPORTED;
  return grad_mrsf(ctx, d, p, spc, cam5[0], cam5[2], 1.0, spcscale, mrst, de, cam5);
}

int oqpg_grad2_sf(oqpg_ctx* ctx, const double* d, const double* p, const double* v, double hfscale, double hfscale2,
                  double coulscale, double* de) {
  if (!ctx) return NOT_INIT;
  if (!d || !p || !v || !de) return UNSUPPORTED;
  // grd2_sf_compute_data_t's density is the MRSF one with ball = v and every
  // spin-pair coupling term off (modules/tdhf_sf_gradient.F90:423-502)
  const size_t n = (size_t)ctx->nbf;
  std::vector<double> spc(7 * n * n, 0.0);
  for (size_t q = 0; q < n * n; ++q) spc[6 + 7 * q] = v[q];
  const double zero[3] = {0.0, 0.0, 0.0};
  return grad_mrsf(ctx, d, p, spc.data(), hfscale, hfscale2, coulscale, zero, 1, de);
}

int oqpg_grad_stats(const oqpg_ctx* ctx, double* out, int n) {
  if (!ctx) return NOT_INIT;
  for (int i = 0; i < n && i < 5; ++i) out[i] = ctx->grad_stats[i];
  return OK;
}

}  // extern "C"
