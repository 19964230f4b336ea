// Response-type Fock builds on the same screened quartet pipeline: general
// square (not necessarily symmetric) densities, many at once.
//
// Consumers in OpenQP (each replaced by one call here):
//  * int2_td_data_t (tdhf_lib.F90:140-224, parallel_stop :89-111): TDHF / TDDFT
//    A+B and A-B products, CPHF (modules/cphf.F90:193), NMR shielding
//    (modules/nmr_shielding.F90:454-487);
//  * int2_tdgrd_data_t (tdhf_lib.F90:228-295): the spin-adapted A+B / A-B of
//    the SF and MRSF Z-vector equations (modules/tdhf_sf_z_vector.F90:252,
//    modules/tdhf_mrsf_z_vector.F90:1009, 1737);
//  * int2_rpagrd_data_t (tdhf_lib.F90:1068-1322): H+[X+Y], H+[T], H-[X-Y] of
//    the TDHF / TDDFT gradient (modules/tdhf_z_vector.F90:341, 484);
//  * int2_mrsf_data_t (tdhf_mrsf_lib.F90:218-333, pass 1) and
//    int2_umrsf_data_t (tdhf_mrsf_lib.F90:337-426, pass 1): MRSF / UMRSF
//    sigma vectors.
// All of them are sums of J[X] and K[X] with full permutational sums over the
// caller's matrices X; the GenJob recipe built here says which slices
// (X + X^T)/2 or (X - X^T)/2 are staged, which accumulators they feed and how
// each output matrix is assembled from the accumulators.
#include <cstring>

#include "oqpg_common.cuh"
#include "oqpg_internal.h"
#include "../../include/openqp_gb300.h"

namespace oqpg {

// Staged slice s: S[s][r][c] = (X(r, c) + sign X(c, r)) / 2 in the stacked
// row-major layout (columns beyond nbf zeroed).
__global__ void k_stage_gen(const double* __restrict__ in, long long rs, long long cs,
                            const GenSlice* __restrict__ sl, int nsl, int n, int stride, double* out) {
  const long long per = (long long)n * stride, tot = per * nsl;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < tot;
       t += (long long)gridDim.x * blockDim.x) {
    const int s = (int)(t / per);
    const long long u = t - (long long)s * per;
    const int r = (int)(u / stride), c = (int)(u % stride);
    double v = 0.0;
    if (c < n) {
      const GenSlice S = sl[s];
      const double x = in[S.base + r * rs + c * cs], y = in[S.base + c * rs + r * cs];
      v = 0.5 * (x + (double)S.sign * y);
    }
    out[t] = v;
  }
}

// shltd (tdhf_lib.F90:300-325) / shell_den_screen_mrsf (tdhf_mrsf_lib.F90:189-214):
// for the pair (i >= j) the maximum |X(r, c)| over r in shell j, c in shell i
// (that orientation of the block only) and over the screening inputs.
__global__ void k_dsh_gen(const double* __restrict__ in, long long rs, long long cs,
                          const long long* __restrict__ scr, int nscr, const int2* __restrict__ pair_ij, int npair,
                          const int* __restrict__ aoff, const int* __restrict__ nao, int ns, double* dsh, float* dshf,
                          unsigned long long* dmax_bits) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < npair;
       t += (long long)gridDim.x * blockDim.x) {
    const int2 ij = pair_ij[t];
    const int hi = ij.x > ij.y ? ij.x : ij.y, lo = ij.x > ij.y ? ij.y : ij.x;
    const int r0 = aoff[lo], r1 = r0 + nao[lo], c0 = aoff[hi], c1 = c0 + nao[hi];
    double m = 0.0;
    for (int q = 0; q < nscr; ++q) {
      const double* x = in + scr[q];
      for (int c = c0; c < c1; ++c)
        for (int r = r0; r < r1; ++r) m = fmax(m, fabs(x[r * rs + c * cs]));
    }
    dsh[(long long)ij.x * ns + ij.y] = m;
    dsh[(long long)ij.y * ns + ij.x] = m;
    dshf[(long long)ij.x * ns + ij.y] = (float)m;
    dshf[(long long)ij.y * ns + ij.x] = (float)m;
    atomicMax(dmax_bits, (unsigned long long)__double_as_longlong(m));
  }
}

// out_o(r, c) = sum over the terms of o of coef (G[r][c] + sign G[c][r]),
// G the term's Coulomb or exchange accumulator (added to out_o with
// accumulate).  Nothing is written when a quartet list overflowed (the build
// is then redone).
__global__ void k_finalize_gen(const double* __restrict__ gj, const double* __restrict__ gk, size_t kstride,
                               int stride, int n, const GenOut* __restrict__ outs, int nout,
                               const GenTerm* __restrict__ terms, long long ors, long long ocs, int accumulate,
                               const unsigned* __restrict__ flag) {
  if (flag && *flag) return;
  const long long per = (long long)n * n, tot = per * nout;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < tot;
       t += (long long)gridDim.x * blockDim.x) {
    const int o = (int)(t / per);
    const long long u = t - (long long)o * per;
    const int c = (int)(u / n), r = (int)(u % n);
    const GenOut O = outs[o];
    double v = 0.0;
    for (int k = 0; k < O.nterm; ++k) {
      const GenTerm T = terms[O.term0 + k];
      const double* G = (T.kind ? gk : gj) + (size_t)T.idx * kstride;
      v += T.coef * (G[(size_t)r * stride + c] + (double)T.sign * G[(size_t)c * stride + r]);
    }
    double* d = O.dst + (r * ors + c * ocs);
    *d = accumulate ? *d + v : v;
  }
}

namespace {

#define CKR(x)                                         \
  do {                                                 \
    cudaError_t e_ = (x);                              \
    if (e_ != cudaSuccess) return e_ == cudaErrorMemoryAllocation ? NO_MEM : DEV_ERR; \
  } while (0)

size_t align16(size_t b) { return (b + 15) & ~(size_t)15; }

struct TabLayout {
  size_t slices, screen, outs, terms, total;
};

TabLayout tab_layout(const GenJob& g) {
  TabLayout L;
  L.slices = 0;
  L.screen = align16(L.slices + sizeof(GenSlice) * g.slices.size());
  L.outs = align16(L.screen + sizeof(long long) * g.screen.size());
  L.terms = align16(L.outs + sizeof(GenOut) * g.outs.size());
  L.total = align16(L.terms + sizeof(GenTerm) * g.terms.size()) + 16;
  return L;
}

unsigned grid_for(long long n, int nsm) { return (unsigned)std::min<long long>((n + 255) / 256, nsm * 8LL); }

}  // namespace

int gen_densities(oqpg_ctx* c, BuildBufs& B, const GenJob& g, cudaStream_t st) {
  const TabLayout L = tab_layout(g);
  CKR(B.gtab.ensure(L.total));
  unsigned char* tab = B.gtab.as<unsigned char>();
  if (!g.slices.empty())
    CKR(cudaMemcpyAsync(tab + L.slices, g.slices.data(), sizeof(GenSlice) * g.slices.size(), cudaMemcpyHostToDevice,
                        st));
  if (!g.screen.empty())
    CKR(cudaMemcpyAsync(tab + L.screen, g.screen.data(), sizeof(long long) * g.screen.size(),
                        cudaMemcpyHostToDevice, st));
  if (!g.outs.empty())
    CKR(cudaMemcpyAsync(tab + L.outs, g.outs.data(), sizeof(GenOut) * g.outs.size(), cudaMemcpyHostToDevice, st));
  if (!g.terms.empty())
    CKR(cudaMemcpyAsync(tab + L.terms, g.terms.data(), sizeof(GenTerm) * g.terms.size(), cudaMemcpyHostToDevice,
                        st));
  const int nsl = (int)g.slices.size();
  const long long n2 = (long long)c->nbf * c->stride;
  if (nsl) {
    k_stage_gen<<<grid_for(n2 * nsl, c->nsm), 256, 0, st>>>(g.in, g.in_rs, g.in_cs, (const GenSlice*)(tab + L.slices),
                                                            nsl, c->nbf, c->stride, B.dk.as<double>());
    CKR(cudaGetLastError());
    if (split_on(c)) {
      k_to_f32<<<grid_for(n2 * nsl, c->nsm), 256, 0, st>>>(B.dk.as<double>(), n2 * nsl, B.dkf.as<float>());
      CKR(cudaGetLastError());
    }
    if (df_on(c)) {
      k_to_df<<<grid_for(n2 * nsl, c->nsm), 256, 0, st>>>(B.dk.as<double>(), n2 * nsl, B.dkdf.as<dfl>());
      CKR(cudaGetLastError());
    }
  }
  CKR(cudaMemsetAsync(B.dmax.p, 0, sizeof(unsigned long long), st));
  CKR(cudaMemsetAsync(B.dsh.p, 0, sizeof(double) * std::max<long long>(c->dsh_elems, 1), st));
  k_dsh_gen<<<(unsigned)std::min<long long>((c->npair + 127) / 128, c->nsm * 8LL), 128, 0, st>>>(
      g.in, g.in_rs, g.in_cs, (const long long*)(tab + L.screen), (int)g.screen.size(), c->d_pair_ij.as<int2>(),
      c->npair, c->d_aoff.as<int>(), c->d_naos.as<int>(), c->nshell, B.dsh.as<double>(), B.dshf.as<float>(),
      B.dmax.as<unsigned long long>());
  CKR(cudaGetLastError());
  return OK;
}

int gen_finalize(oqpg_ctx* c, BuildBufs& B, const GenJob& g, cudaStream_t st) {
  const TabLayout L = tab_layout(g);
  const unsigned char* tab = B.gtab.as<unsigned char>();
  const long long n2 = (long long)c->nbf * c->nbf;
  if (g.outs.empty()) return OK;
  k_finalize_gen<<<grid_for(n2 * (long long)g.outs.size(), c->nsm), 256, 0, st>>>(
      B.gj.as<double>(), B.gk.as<double>(), (size_t)c->nbf * c->stride, c->stride, c->nbf,
      (const GenOut*)(tab + L.outs), (int)g.outs.size(), (const GenTerm*)(tab + L.terms), g.out_rs, g.out_cs,
      g.accumulate ? 1 : 0, B.flag.as<unsigned>());
  CKR(cudaGetLastError());
  return OK;
}

namespace {

GenTerm term(double coef, int kind, int idx, int sign) {
  GenTerm t;
  t.coef = coef; t.kind = kind; t.idx = idx; t.sign = sign; t.pad = 0;
  return t;
}

// int2_td_data_t recipe.  d2 (n, n, nvec) and apb / amb (n, n, nvec), Fortran
// column-major; with the full sums J, K and D = d2(:, :, v):
//   A+B (after the symmetrisation of parallel_stop): 4 sc J[D] - 2 se K[Ds]
//   A-B:                                             -2 se K[Da]
//   Tamm-Dancoff, into amb:                 2 sc J[D] (if Coulomb) - se K[D]
void td_job(const oqpg_ctx* c, const double* d2, double* apb, double* amb, int nvec, int flags, double se,
            double sc, GenJob& g) {
  const long long n = c->nbf, nn = n * n;
  const bool tda = flags & OQPG_TD_TDA;
  const bool want_apb = !tda && (flags & OQPG_TD_APB), want_amb = !tda && (flags & OQPG_TD_AMB);
  const bool need_j = want_apb || (tda && (flags & OQPG_TD_TDA_COULOMB));
  const bool need_ks = want_apb || tda, need_ka = want_amb || tda;
  g.in = d2;
  g.in_rs = 1; g.in_cs = n;
  g.out_rs = 1; g.out_cs = n;
  const int nsym = need_ks ? nvec : 0;
  for (int v = 0; v < nsym; ++v) g.slices.push_back(GenSlice{v * nn, +1, 0});
  if (need_ka)
    for (int v = 0; v < nvec; ++v) g.slices.push_back(GenSlice{v * nn, -1, 0});
  g.nj = need_j ? nvec : 0;
  g.k0 = 0;
  g.nk = (int)g.slices.size();
  for (int v = 0; v < nvec; ++v) g.screen.push_back(v * nn);
  const int ka0 = nsym;
  for (int v = 0; v < nvec; ++v) {
    GenOut o{apb + v * nn, (int)g.terms.size(), 0};
    if (want_apb) {
      g.terms.push_back(term(4.0 * sc, 0, v, +1));
      g.terms.push_back(term(-2.0 * se, 1, v, +1));
    }
    o.nterm = (int)g.terms.size() - o.term0;
    g.outs.push_back(o);
  }
  for (int v = 0; v < nvec; ++v) {
    GenOut o{amb + v * nn, (int)g.terms.size(), 0};
    if (tda) {
      if (need_j) g.terms.push_back(term(2.0 * sc, 0, v, +1));
      g.terms.push_back(term(-se, 1, v, +1));
      g.terms.push_back(term(-se, 1, ka0 + v, -1));
    } else if (want_amb) {
      g.terms.push_back(term(-2.0 * se, 1, ka0 + v, -1));
    }
    o.nterm = (int)g.terms.size() - o.term0;
    g.outs.push_back(o);
  }
}

}  // namespace

// int2_mrsf_data_t (nmat 7) / int2_umrsf_data_t (nmat 11) recipe, pass 1.
// Component m of vector v: element (r, c) at base + r rs + c cs with
// base = m sm + v sv (MrsfLayout); with X that matrix:
//   MRSF:  m < 4: sc J[X] - se K[X];  m = 4..6: -se K[X]
//   UMRSF: m < 8: sc J[X] - se K[X];  m = 8, 9: -se K[X^T];  m = 10: -se K[X]
// neg_lead negates the outputs of components 0..5 (the MRSF triplet sign of
// tdhf_mrsf_energy.F90:762-766).  Screening density: component nmat - 1 of
// every vector.
void mrsf_job_layout(const oqpg_ctx* c, const double* in, double* out, int nvec, int nmat, double se, double sc,
                     const MrsfLayout& L, bool neg_lead, GenJob& g) {
  const bool um = nmat == 11;
  const int ncoul = um ? 8 : 4;
  g.in = in;
  g.in_rs = L.rs; g.in_cs = L.cs;
  g.out_rs = L.rs; g.out_cs = L.cs;
  auto base = [&](int m, int v) { return (long long)m * L.sm + (long long)v * L.sv; };
  for (int m = 0; m < nmat; ++m)
    for (int v = 0; v < nvec; ++v) g.slices.push_back(GenSlice{base(m, v), +1, 0});
  for (int m = 0; m < nmat; ++m)
    for (int v = 0; v < nvec; ++v) g.slices.push_back(GenSlice{base(m, v), -1, 0});
  g.nj = ncoul * nvec;
  g.k0 = 0;
  g.nk = 2 * nmat * nvec;
  for (int v = 0; v < nvec; ++v) g.screen.push_back(base(nmat - 1, v));
  for (int m = 0; m < nmat; ++m)
    for (int v = 0; v < nvec; ++v) {
      const int s = m * nvec + v, a = nmat * nvec + s;
      const double sg = neg_lead && m < 6 ? -1.0 : 1.0;
      GenOut o{out + base(m, v), (int)g.terms.size(), 0};
      if (m < ncoul) g.terms.push_back(term(sg * sc, 0, s, +1));
      const bool transposed = um && (m == 8 || m == 9);
      g.terms.push_back(term(-sg * se, 1, s, +1));
      g.terms.push_back(term(sg * (transposed ? se : -se), 1, a, -1));
      o.nterm = (int)g.terms.size() - o.term0;
      g.outs.push_back(o);
    }
}

namespace {

// d3 / f3 (nvec, nmat, n, n) Fortran column-major, the data types' layout.
MrsfLayout fortran_mrsf(const oqpg_ctx* c, int nvec, int nmat) {
  const long long n = c->nbf;
  return MrsfLayout{(long long)nmat * nvec, n * nmat * nvec, nvec, 1};
}

void mrsf_job(const oqpg_ctx* c, const double* d3, double* f3, int nvec, int nmat, double se, double sc,
              GenJob& g) {
  mrsf_job_layout(c, d3, f3, nvec, nmat, se, sc, fortran_mrsf(c, nvec, nmat), false, g);
}

// Second (erf-attenuated) CAM pass of int2_mrsf_data_t / int2_umrsf_data_t
// (tdhf_mrsf_lib.F90:314-328, 409-420): only the last component, -beta K[X],
// added to f3.
void mrsf_cam2_job(const oqpg_ctx* c, const double* d3, double* f3, int nvec, int nmat, double beta, GenJob& g) {
  const long long n = c->nbf;
  g.in = d3;
  g.in_rs = (long long)nmat * nvec; g.in_cs = n * nmat * nvec;
  g.out_rs = g.in_rs; g.out_cs = g.in_cs;
  const int m = nmat - 1;
  for (int v = 0; v < nvec; ++v) g.slices.push_back(GenSlice{(long long)m * nvec + v, +1, 0});
  for (int v = 0; v < nvec; ++v) g.slices.push_back(GenSlice{(long long)m * nvec + v, -1, 0});
  g.nj = 0;
  g.k0 = 0;
  g.nk = 2 * nvec;
  for (int v = 0; v < nvec; ++v) g.screen.push_back((long long)m * nvec + v);
  for (int v = 0; v < nvec; ++v) {
    GenOut o{f3 + (long long)m * nvec + v, (int)g.terms.size(), 2};
    g.terms.push_back(term(-beta, 1, v, +1));
    g.terms.push_back(term(-beta, 1, nvec + v, -1));
    g.outs.push_back(o);
  }
  g.accumulate = true;
}

// int2_tdgrd_data_t recipe (tdhf_lib.F90:228-295 with the int2_td_data_t
// parallel_stop): d2 / apb / amb (n, n, 2) Fortran column-major, D1, D2 the two
// spin densities:
//   A+B, spin s (after the symmetrisation): 2 sc J[D1 + D2] - 2 se K[Ds_s]
//   A-B, spin 1: -2 se K[D1a];  spin 2: zero
void tdgrd_job(const oqpg_ctx* c, const double* d2, double* apb, double* amb, int flags, double se, double sc,
               GenJob& g) {
  const long long n = c->nbf, nn = n * n;
  const bool want_apb = flags & OQPG_TD_APB, want_amb = flags & OQPG_TD_AMB;
  g.in = d2;
  g.in_rs = 1; g.in_cs = n;
  g.out_rs = 1; g.out_cs = n;
  if (want_apb)
    for (int v = 0; v < 2; ++v) g.slices.push_back(GenSlice{v * nn, +1, 0});
  const int ka = (int)g.slices.size();
  if (want_amb) g.slices.push_back(GenSlice{0, -1, 0});
  g.nj = want_apb ? 2 : 0;
  g.k0 = 0;
  g.nk = (int)g.slices.size();
  for (int v = 0; v < 2; ++v) g.screen.push_back(v * nn);
  for (int v = 0; v < 2; ++v) {
    GenOut o{apb + v * nn, (int)g.terms.size(), 0};
    if (want_apb) {
      g.terms.push_back(term(2.0 * sc, 0, 0, +1));
      g.terms.push_back(term(2.0 * sc, 0, 1, +1));
      g.terms.push_back(term(-2.0 * se, 1, v, +1));
    }
    o.nterm = (int)g.terms.size() - o.term0;
    g.outs.push_back(o);
  }
  for (int v = 0; v < 2; ++v) {
    GenOut o{amb + v * nn, (int)g.terms.size(), 0};
    if (want_amb && v == 0) g.terms.push_back(term(-2.0 * se, 1, ka, -1));
    o.nterm = (int)g.terms.size() - o.term0;
    g.outs.push_back(o);
  }
}

// Operand layout of an int2_rpagrd_data_t build in one device block: xpy
// (n, n, ldp, np), then xmy (n, n, ldm, nm), then t (n, n, ldt, nt); outputs
// hpp (n, n, nspin, np), hpt (n, n, nspin, nt), hmm (n, n, nspin, nm).
struct RpaDims {
  int np, ldp, nm, ldm, nt, ldt, nspin;
  long long xpy_off() const { return 0; }
  long long xmy_off(long long nn) const { return nn * ldp * np; }
  long long t_off(long long nn) const { return xmy_off(nn) + nn * ldm * nm; }
  long long in_elems(long long nn) const { return t_off(nn) + nn * ldt * nt; }
  long long out_elems(long long nn) const { return nn * nspin * (np + nt + nm); }
};

// int2_rpagrd_data_t recipe (tdhf_lib.F90:1177-1322 with parallel_stop
// :1113-1145).  With V a vector of xpy or t and S = spin component:
//   nspin 1: H+[V] = 4 sc J[V1] - 2 se K[V1]
//   nspin 2: H+[V]_s = 2 sc J[V1 + V2] - 2 se K[V_s]
//   H-[V]: spin 1 -2 se K[V1a], other spin zero
// H+ is taken of the symmetric part of V: every caller passes symmetric
// matrices (modules/tdhf_z_vector.F90:325-331, 439-447), and for a
// non-symmetric V the reference's sum depends on its quartet ordering.  The
// shell density is the maximum over every component of xpy and xmy (both
// only when np > 0) and of t (init_screen, tdhf_lib.F90:1161-1173).
void rpagrd_job(const oqpg_ctx* c, const double* in, const RpaDims& R, double* out, double se, double sc, GenJob& g) {
  const long long n = c->nbf, nn = n * n;
  g.in = in;
  g.in_rs = 1; g.in_cs = n;
  g.out_rs = 1; g.out_cs = n;
  const int ns = R.nspin;
  // symmetric slices of the H+ operands first (they feed J and K), then the
  // antisymmetric ones of H-
  auto plus_base = [&](int set, int v, int s) {
    return set == 0 ? R.xpy_off() + nn * ((long long)v * R.ldp + s) : R.t_off(nn) + nn * ((long long)v * R.ldt + s);
  };
  const int nplus = R.np + R.nt;
  for (int u = 0; u < nplus; ++u) {
    const int set = u < R.np ? 0 : 1, v = u < R.np ? u : u - R.np;
    for (int s = 0; s < ns; ++s) g.slices.push_back(GenSlice{plus_base(set, v, s), +1, 0});
  }
  const int km = (int)g.slices.size();
  for (int v = 0; v < R.nm; ++v) g.slices.push_back(GenSlice{R.xmy_off(nn) + nn * (long long)v * R.ldm, -1, 0});
  g.nj = km;
  g.k0 = 0;
  g.nk = (int)g.slices.size();
  if (R.np > 0) {
    for (long long q = 0; q < (long long)R.ldp * R.np; ++q) g.screen.push_back(R.xpy_off() + q * nn);
    for (long long q = 0; q < (long long)R.ldm * R.nm; ++q) g.screen.push_back(R.xmy_off(nn) + q * nn);
  }
  for (long long q = 0; q < (long long)R.ldt * R.nt; ++q) g.screen.push_back(R.t_off(nn) + q * nn);
  const double cj = ns == 1 ? 4.0 * sc : 2.0 * sc;
  for (int u = 0; u < nplus; ++u)
    for (int s = 0; s < ns; ++s) {
      GenOut o{out + nn * ((long long)u * ns + s), (int)g.terms.size(), 0};
      for (int s2 = 0; s2 < ns; ++s2) g.terms.push_back(term(cj, 0, u * ns + s2, +1));
      g.terms.push_back(term(-2.0 * se, 1, u * ns + s, +1));
      o.nterm = (int)g.terms.size() - o.term0;
      g.outs.push_back(o);
    }
  for (int v = 0; v < R.nm; ++v)
    for (int s = 0; s < ns; ++s) {
      GenOut o{out + nn * ((long long)(nplus + v) * ns + s), (int)g.terms.size(), 0};
      if (s == 0) g.terms.push_back(term(-2.0 * se, 1, km + v, -1));
      o.nterm = (int)g.terms.size() - o.term0;
      g.outs.push_back(o);
    }
}

int run_job(oqpg_ctx* c, const GenJob& g, cudaStream_t st, double inv_mu2 = 0.0) {
  Job j;
  j.gen = &g;
  j.inv_mu2 = inv_mu2;
  return ctx_build(c, j, st);
}

// cam = {alpha, beta, mu, alpha_coulomb, beta_coulomb} (int2_run_cam,
// int2.F90:538-584): pass 1 with scale_exchange alpha and scale_coulomb
// alpha_coulomb over 1/r, pass 2 with beta and beta_coulomb over erf(mu r)/r.
bool cam_ok(const double* cam) { return cam && cam[2] > 0.0; }

// host-buffer build: the input is copied to the context's d_dp, the job writes
// its outputs into d_f (nout_buf consecutive blocks), which are copied back
int host_job(oqpg_ctx* c, const double* in, size_t in_elems, double* const* host_out, const size_t* out_elems,
             int nout_buf, const GenJob& g, const GenJob* g2 = nullptr, double inv_mu2 = 0.0) {
  cudaStream_t st = c->stream;
  CKR(cudaMemcpyAsync(c->d_dp.p, in, sizeof(double) * in_elems, cudaMemcpyHostToDevice, st));
  int rc = run_job(c, g, st);
  if (rc) return rc;
  if (g2 && (rc = run_job(c, *g2, st, inv_mu2))) return rc;
  size_t off = 0;
  for (int b = 0; b < nout_buf; ++b) {
    if (host_out[b])
      CKR(cudaMemcpyAsync(host_out[b], c->d_f.as<double>() + off, sizeof(double) * out_elems[b],
                          cudaMemcpyDeviceToHost, st));
    off += out_elems[b];
  }
  CKR(cudaStreamSynchronize(st));
  return OK;
}

// One build, or the two CAM passes (cam = {alpha, beta, mu, alpha_coulomb,
// beta_coulomb}), of the recipe make(se, sc, job) on stream st.
template <class Make>
int run_scaled(oqpg_ctx* c, const double* cam, double se, double sc, cudaStream_t st, Make make) {
  if (!cam) {
    GenJob g;
    make(se, sc, g);
    return run_job(c, g, st);
  }
  int rc;
  if ((rc = ensure_att(c, cam[2]))) return rc;
  GenJob g1, g2;
  make(cam[0], cam[3], g1);
  make(cam[1], cam[4], g2);
  g2.accumulate = true;
  if ((rc = run_job(c, g1, st))) return rc;
  return run_job(c, g2, st, 1.0 / (cam[2] * cam[2]));
}

bool rpa_dims_ok(const RpaDims& R, const double* xpy, const double* xmy, const double* t) {
  if (R.nspin != 1 && R.nspin != 2) return false;
  if (R.np < 0 || R.nm < 0 || R.nt < 0) return false;
  if ((R.np && (!xpy || R.ldp < R.nspin)) || (R.nm && (!xmy || R.ldm < R.nspin)) || (R.nt && (!t || R.ldt < R.nspin)))
    return false;
  return true;
}

bool td_args_ok(const oqpg_ctx* c, int nvec, int flags) {
  return c && c->nmol == 1 && nvec >= 1 && (flags & ~(OQPG_TD_APB | OQPG_TD_AMB | OQPG_TD_TDA | OQPG_TD_TDA_COULOMB)) == 0;
}

}  // namespace
}  // namespace oqpg

using namespace oqpg;

extern "C" {

int oqpg_fock_td_device(oqpg_ctx* ctx, const double* d2, double* apb, double* amb, int nvec, int flags, double se,
                        double sc, void* stream) {
  if (!td_args_ok(ctx, nvec, flags) || !d2 || !apb || !amb) return UNSUPPORTED;
  GenJob g;
  td_job(ctx, d2, apb, amb, nvec, flags, se, sc, g);
  cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
  int rc = run_job(ctx, g, st);
  if (rc) return rc;
  return cudaStreamSynchronize(st) == cudaSuccess ? OK : DEV_ERR;
}

int oqpg_fock_td(oqpg_ctx* ctx, const double* d2, double* apb, double* amb, int nvec, int flags, double se,
                 double sc) {
  if (!td_args_ok(ctx, nvec, flags) || !d2) return UNSUPPORTED;
  const size_t tot = (size_t)ctx->nbf * ctx->nbf * nvec;
  if (ctx->d_dp.ensure(sizeof(double) * tot) != cudaSuccess) return NO_MEM;
  if (ctx->d_f.ensure(sizeof(double) * 2 * tot) != cudaSuccess) return NO_MEM;
  GenJob g;
  td_job(ctx, ctx->d_dp.as<double>(), ctx->d_f.as<double>(), ctx->d_f.as<double>() + tot, nvec, flags, se, sc, g);
  double* outs[2] = {apb, amb};
  const size_t elems[2] = {tot, tot};
  return host_job(ctx, d2, tot, outs, elems, 2, g);
}

int oqpg_fock_mrsf_device(oqpg_ctx* ctx, const double* d3, double* f3, int nvec, int nmat, double se, double sc,
                          void* stream) {
  if (!ctx || ctx->nmol != 1 || nvec < 1 || (nmat != 7 && nmat != 11) || !d3 || !f3) return UNSUPPORTED;
  GenJob g;
  mrsf_job(ctx, d3, f3, nvec, nmat, se, sc, g);
  cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
  int rc = run_job(ctx, g, st);
  if (rc) return rc;
  return cudaStreamSynchronize(st) == cudaSuccess ? OK : DEV_ERR;
}

int oqpg_fock_mrsf(oqpg_ctx* ctx, const double* d3, double* f3, int nvec, int nmat, double se, double sc) {
  if (!ctx || ctx->nmol != 1 || nvec < 1 || (nmat != 7 && nmat != 11) || !d3) return UNSUPPORTED;
  const size_t tot = (size_t)ctx->nbf * ctx->nbf * nmat * nvec;
  if (ctx->d_dp.ensure(sizeof(double) * tot) != cudaSuccess) return NO_MEM;
  if (ctx->d_f.ensure(sizeof(double) * tot) != cudaSuccess) return NO_MEM;
  GenJob g;
  mrsf_job(ctx, ctx->d_dp.as<double>(), ctx->d_f.as<double>(), nvec, nmat, se, sc, g);
  double* outs[1] = {f3};
  const size_t elems[1] = {tot};
  return host_job(ctx, d3, tot, outs, elems, 1, g);
}

int oqpg_fock_td_cam(oqpg_ctx* ctx, const double* d2, double* apb, double* amb, int nvec, int flags,
                     const double* cam) {
  if (!td_args_ok(ctx, nvec, flags) || !d2 || !cam_ok(cam)) return UNSUPPORTED;
  int rc;
  if ((rc = ensure_att(ctx, cam[2]))) return rc;
  const size_t tot = (size_t)ctx->nbf * ctx->nbf * nvec;
  if (ctx->d_dp.ensure(sizeof(double) * tot) != cudaSuccess) return NO_MEM;
  if (ctx->d_f.ensure(sizeof(double) * 2 * tot) != cudaSuccess) return NO_MEM;
  GenJob g1, g2;
  double* pa = ctx->d_f.as<double>();
  td_job(ctx, ctx->d_dp.as<double>(), pa, pa + tot, nvec, flags, cam[0], cam[3], g1);
  td_job(ctx, ctx->d_dp.as<double>(), pa, pa + tot, nvec, flags, cam[1], cam[4], g2);
  g2.accumulate = true;
  double* outs[2] = {apb, amb};
  const size_t elems[2] = {tot, tot};
  return host_job(ctx, d2, tot, outs, elems, 2, g1, &g2, 1.0 / (cam[2] * cam[2]));
}

int oqpg_fock_mrsf_cam(oqpg_ctx* ctx, const double* d3, double* f3, int nvec, int nmat, const double* cam) {
  if (!ctx || ctx->nmol != 1 || nvec < 1 || (nmat != 7 && nmat != 11) || !d3 || !cam_ok(cam)) return UNSUPPORTED;
  int rc;
  if ((rc = ensure_att(ctx, cam[2]))) return rc;
  const size_t tot = (size_t)ctx->nbf * ctx->nbf * nmat * nvec;
  if (ctx->d_dp.ensure(sizeof(double) * tot) != cudaSuccess) return NO_MEM;
  if (ctx->d_f.ensure(sizeof(double) * tot) != cudaSuccess) return NO_MEM;
  GenJob g1, g2;
  mrsf_job(ctx, ctx->d_dp.as<double>(), ctx->d_f.as<double>(), nvec, nmat, cam[0], cam[3], g1);
  mrsf_cam2_job(ctx, ctx->d_dp.as<double>(), ctx->d_f.as<double>(), nvec, nmat, cam[1], g2);
  double* outs[1] = {f3};
  const size_t elems[1] = {tot};
  return host_job(ctx, d3, tot, outs, elems, 1, g1, &g2, 1.0 / (cam[2] * cam[2]));
}

int oqpg_fock_tdgrd_device(oqpg_ctx* ctx, const double* d2, double* apb, double* amb, int flags, double se,
                           double sc, const double* cam, void* stream) {
  if (!ctx || ctx->nmol != 1 || (flags & ~(OQPG_TD_APB | OQPG_TD_AMB)) || !d2 || !apb || !amb) return UNSUPPORTED;
  if (cam && !cam_ok(cam)) return UNSUPPORTED;
  cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
  int rc = run_scaled(ctx, cam, se, sc, st, [&](double x, double y, GenJob& g) {
    tdgrd_job(ctx, d2, apb, amb, flags, x, y, g);
  });
  if (rc) return rc;
  return cudaStreamSynchronize(st) == cudaSuccess ? OK : DEV_ERR;
}

int oqpg_fock_tdgrd(oqpg_ctx* ctx, const double* d2, double* apb, double* amb, int flags, double se, double sc,
                    const double* cam) {
  if (!ctx || ctx->nmol != 1 || (flags & ~(OQPG_TD_APB | OQPG_TD_AMB)) || !d2 || !apb || !amb) return UNSUPPORTED;
  if (cam && !cam_ok(cam)) return UNSUPPORTED;
  const size_t tot = (size_t)ctx->nbf * ctx->nbf * 2;
  if (ctx->d_dp.ensure(sizeof(double) * tot) != cudaSuccess) return NO_MEM;
  if (ctx->d_f.ensure(sizeof(double) * 2 * tot) != cudaSuccess) return NO_MEM;
  cudaStream_t st = ctx->stream;
  double* dp = ctx->d_dp.as<double>();
  double* f = ctx->d_f.as<double>();
  CKR(cudaMemcpyAsync(dp, d2, sizeof(double) * tot, cudaMemcpyHostToDevice, st));
  int rc = run_scaled(ctx, cam, se, sc, st, [&](double x, double y, GenJob& g) {
    tdgrd_job(ctx, dp, f, f + tot, flags, x, y, g);
  });
  if (rc) return rc;
  CKR(cudaMemcpyAsync(apb, f, sizeof(double) * tot, cudaMemcpyDeviceToHost, st));
  CKR(cudaMemcpyAsync(amb, f + tot, sizeof(double) * tot, cudaMemcpyDeviceToHost, st));
  CKR(cudaStreamSynchronize(st));
  return OK;
}

// Shared body of the host and device RPA-gradient forms: the three operand
// arrays are gathered into the context's d_dp (copy kind `kind`), the outputs
// come back from d_f (to hpp / hpt / hmm with kind `back`).
static int rpagrd_body(oqpg_ctx* ctx, const double* xpy, int ldp, int np, const double* xmy, int ldm, int nm,
                       const double* t, int ldt, int nt, int nspin, double* hpp, double* hpt, double* hmm, double se,
                       double sc, const double* cam, cudaStream_t st, cudaMemcpyKind kind, cudaMemcpyKind back) {
  const RpaDims R{np, ldp, nm, ldm, nt, ldt, nspin};
  if (!ctx || ctx->nmol != 1 || !rpa_dims_ok(R, xpy, xmy, t)) return UNSUPPORTED;
  if ((np && !hpp) || (nt && !hpt) || (nm && !hmm)) return UNSUPPORTED;
  if (cam && !cam_ok(cam)) return UNSUPPORTED;
  const long long nn = (long long)ctx->nbf * ctx->nbf;
  if (ctx->d_dp.ensure(sizeof(double) * std::max<long long>(R.in_elems(nn), 1)) != cudaSuccess) return NO_MEM;
  if (ctx->d_f.ensure(sizeof(double) * std::max<long long>(R.out_elems(nn), 1)) != cudaSuccess) return NO_MEM;
  double* dp = ctx->d_dp.as<double>();
  double* f = ctx->d_f.as<double>();
  if (np) CKR(cudaMemcpyAsync(dp + R.xpy_off(), xpy, sizeof(double) * nn * ldp * np, kind, st));
  if (nm) CKR(cudaMemcpyAsync(dp + R.xmy_off(nn), xmy, sizeof(double) * nn * ldm * nm, kind, st));
  if (nt) CKR(cudaMemcpyAsync(dp + R.t_off(nn), t, sizeof(double) * nn * ldt * nt, kind, st));
  int rc = run_scaled(ctx, cam, se, sc, st, [&](double x, double y, GenJob& g) { rpagrd_job(ctx, dp, R, f, x, y, g); });
  if (rc) return rc;
  const long long blk = nn * nspin;
  if (np) CKR(cudaMemcpyAsync(hpp, f, sizeof(double) * blk * np, back, st));
  if (nt) CKR(cudaMemcpyAsync(hpt, f + blk * np, sizeof(double) * blk * nt, back, st));
  if (nm) CKR(cudaMemcpyAsync(hmm, f + blk * (np + nt), sizeof(double) * blk * nm, back, st));
  CKR(cudaStreamSynchronize(st));
  return OK;
}

int oqpg_fock_rpagrd(oqpg_ctx* ctx, const double* xpy, int ldp, int np, const double* xmy, int ldm, int nm,
                     const double* t, int ldt, int nt, int nspin, double* hpp, double* hpt, double* hmm, double se,
                     double sc, const double* cam) {
  return rpagrd_body(ctx, xpy, ldp, np, xmy, ldm, nm, t, ldt, nt, nspin, hpp, hpt, hmm, se, sc, cam,
                     ctx ? ctx->stream : nullptr, cudaMemcpyHostToDevice, cudaMemcpyDeviceToHost);
}

int oqpg_fock_rpagrd_device(oqpg_ctx* ctx, const double* xpy, int ldp, int np, const double* xmy, int ldm, int nm,
                            const double* t, int ldt, int nt, int nspin, double* hpp, double* hpt, double* hmm,
                            double se, double sc, const double* cam, void* stream) {
  cudaStream_t st = stream ? (cudaStream_t)stream : (ctx ? ctx->stream : nullptr);
  return rpagrd_body(ctx, xpy, ldp, np, xmy, ldm, nm, t, ldt, nt, nspin, hpp, hpt, hmm, se, sc, cam, st,
                     cudaMemcpyDeviceToDevice, cudaMemcpyDeviceToDevice);
}

}  // extern "C"
