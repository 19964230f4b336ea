// Petite list: the symmetry reduction of OpenQP's SCF Fock build
// (int2.F90:411-469, 781-795; scf_addons.F90:1100-1137, 1205, 1250-1337,
// 1563-1615), abelian tier.
//
// With an abelian point group G given as signed AO permutations (every
// operation maps each shell onto a shell of the same kind and each AO onto +/-
// an AO), a totally symmetric density gives a Fock matrix with the same
// symmetry.  The build then computes only one canonical quartet per orbit of
// G, the lexicographically largest, weighted by the orbit size (k_lists,
// petite_wlog2); the result is a skeleton matrix whose projection onto the
// totally symmetric component, F <- (1/|G|) sum_op T_op F T_op^T, is the
// complete Fock matrix.  As in the reference the element cutoff applies to the
// unweighted integral (the abelian tier), and an incremental build projects
// the increment before it is added to F_old.
//
// The reduction applies to plain SCF builds of packed densities on a
// single-molecule context, and only while the density is invariant: every
// build measures max |P(D) - D| / max |D| on the device (the reference's
// petite_density_asymmetry) and runs the complete build when it exceeds 1e-6,
// so the result is the complete Fock matrix either way.  Response builds,
// CAM builds and gradients never use it (the reference opts only the SCF in).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/openqp_gb300.h"
#include "oqpg_internal.h"

namespace oqpg {

bool petite_on(const oqpg_ctx* c, const Job& job) {
  return c->sym_nops > 1 && job.petite && !job.gen && job.inv_mu2 == 0.0 && c->nmol == 1;
}

namespace {

__device__ __forceinline__ void tri_rc(long long u, int& a, int& b) {   // packed u = a(a+1)/2 + b, a >= b
  a = (int)((sqrt(8.0 * (double)u + 1.0) - 1.0) * 0.5);
  while ((long long)a * (a + 1) / 2 > u) --a;
  while ((long long)(a + 1) * (a + 2) / 2 <= u) ++a;
  b = (int)(u - (long long)a * (a + 1) / 2);
}

// (1/|G|) sum_op s_op(a') s_op(b') M(a', b'), a' = T_op^-1(a): the totally
// symmetric component of the packed symmetric matrix m at (a, b)
__device__ __forceinline__ double project(const double* __restrict__ m, const int* __restrict__ inv,
                                         const double* __restrict__ sgn, int nops, int nbf, int a, int b) {
  double v = 0.0;
  for (int op = 0; op < nops; ++op) {
    const int ia = __ldg(inv + op * nbf + a), ib = __ldg(inv + op * nbf + b);
    const int hi = ia > ib ? ia : ib, lo = ia > ib ? ib : ia;
    v = fma(__ldg(sgn + op * nbf + a) * __ldg(sgn + op * nbf + b), __ldg(m + (long long)hi * (hi + 1) / 2 + lo), v);
  }
  return v / (double)nops;
}

// bits[0] = max |P(D) - D|, bits[1] = max |D| over all densities (FP64 bit
// patterns of non-negative values compare as integers)
__global__ void k_sym_check(const double* __restrict__ dp, int nfocks, long long ntri, int nbf,
                            const int* __restrict__ inv, const double* __restrict__ sgn, int nops,
                            unsigned long long* bits) {
  unsigned long long r = 0, s = 0;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < nfocks * ntri;
       t += (long long)gridDim.x * blockDim.x) {
    const long long comp = t / ntri, u = t - comp * ntri;
    int a, b;
    tri_rc(u, a, b);
    const double v = dp[t];
    const double p = project(dp + comp * ntri, inv, sgn, nops, nbf, a, b);
    r = max(r, (unsigned long long)__double_as_longlong(fabs(p - v)));
    s = max(s, (unsigned long long)__double_as_longlong(fabs(v)));
  }
  for (int o = 16; o > 0; o >>= 1) {
    r = max(r, __shfl_xor_sync(0xffffffffu, r, o));
    s = max(s, __shfl_xor_sync(0xffffffffu, s, o));
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMax(bits, r);
    atomicMax(bits + 1, s);
  }
}

// dst = P(src) (+ f_old; f_old <- dst) when the density passed the check,
// else dst = src (+ f_old): the lists then held every quartet.  Nothing is
// written after a list overflow (the host rebuilds).
__global__ void k_symmetrize(const double* __restrict__ src, double* __restrict__ dst, double* f_old, int nfocks,
                             long long ntri, int nbf, const int* __restrict__ inv, const double* __restrict__ sgn,
                             int nops, const unsigned long long* __restrict__ bits, const unsigned* __restrict__ flag) {
  if (flag && *flag) return;
  const bool on = __longlong_as_double((long long)bits[0]) <= 1e-6 * __longlong_as_double((long long)bits[1]);
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < nfocks * ntri;
       t += (long long)gridDim.x * blockDim.x) {
    const long long comp = t / ntri, u = t - comp * ntri;
    double v;
    if (on) {
      int a, b;
      tri_rc(u, a, b);
      v = project(src + comp * ntri, inv, sgn, nops, nbf, a, b);
    } else {
      v = src[t];
    }
    if (f_old) {
      v += f_old[t];
      f_old[t] = v;
    }
    dst[t] = v;
  }
}

#define CKP(x)                                    \
  do {                                            \
    cudaError_t e_ = (x);                         \
    if (e_ != cudaSuccess) return e_ == cudaErrorMemoryAllocation ? NO_MEM : DEV_ERR; \
  } while (0)

}  // namespace

int petite_check(oqpg_ctx* c, BuildBufs& B, const Job& job, cudaStream_t st) {
  CKP(cudaMemsetAsync(B.sym.p, 0, 2 * sizeof(unsigned long long), st));
  const long long n = (long long)job.nfocks * c->ntri;
  k_sym_check<<<(unsigned)std::min<long long>((n + 255) / 256, c->nsm * 8LL), 256, 0, st>>>(
      job.dp, job.nfocks, c->ntri, c->nbf, c->d_sym_inv.as<int>(), c->d_sym_sgn.as<double>(), c->sym_nops,
      B.sym.as<unsigned long long>());
  CKP(cudaGetLastError());
  return OK;
}

int petite_finalize(oqpg_ctx* c, BuildBufs& B, const Job& job, double ck, cudaStream_t st) {
  const size_t n2 = (size_t)c->nbf * c->stride;
  const int nk = job.nk();
  k_finalize<<<(unsigned)std::min<long long>((c->ntri + 255) / 256, c->nsm * 8LL), 256, 0, st>>>(
      B.gj.as<double>(), B.gk.as<double>(), nk, c->d_mols.as<MolDev>(), c->nmol, c->ntri, c->stride, n2, job.sc, ck,
      B.fsk.as<double>(), nullptr, B.flag.as<unsigned>());
  CKP(cudaGetLastError());
  const long long n = (long long)job.nfocks * c->ntri;
  k_symmetrize<<<(unsigned)std::min<long long>((n + 255) / 256, c->nsm * 8LL), 256, 0, st>>>(
      B.fsk.as<double>(), job.f, job.f_old, job.nfocks, c->ntri, c->nbf, c->d_sym_inv.as<int>(),
      c->d_sym_sgn.as<double>(), c->sym_nops, B.sym.as<unsigned long long>(), B.flag.as<unsigned>());
  CKP(cudaGetLastError());
  return OK;
}

}  // namespace oqpg

using namespace oqpg;

extern "C" int oqpg_set_symmetry(oqpg_ctx* c, int nops, const int* shell_map, const int* ao_target,
                                 const double* ao_sign) {
  if (!c) return NOT_INIT;
  if (c->gexec) {   // a captured build holds the previous reduction
    cudaGraphExecDestroy(c->gexec);
    c->gexec = nullptr;
  }
  c->hb.sized = false;
  if (nops <= 1) {
    c->sym_nops = 0;
    return OK;
  }
  c->sym_nops = 0;
  if (c->nmol != 1 || !shell_map || !ao_target || !ao_sign || nops > 8 || (nops & (nops - 1))) return UNSUPPORTED;
  const int ns = c->nshell, n = c->nbf;
  std::vector<int> inv((size_t)nops * n, -1);
  std::vector<double> sgn((size_t)nops * n, 0.0);
  for (int op = 0; op < nops; ++op) {
    std::vector<char> seen(ns, 0);
    for (int s = 0; s < ns; ++s) {
      const int t = shell_map[(size_t)op * ns + s];
      if (t < 0 || t >= ns || seen[t] || c->h_am[t] != c->h_am[s] || c->naos[t] != c->naos[s]) return UNSUPPORTED;
      seen[t] = 1;
      // AO i of shell s goes to AO i of its image, with a sign +-1
      for (int i = 0; i < c->naos[s]; ++i) {
        const int mu = c->aoff[s] + i;
        const int a = ao_target[(size_t)op * n + mu];
        const double sg = ao_sign[(size_t)op * n + mu];
        if (a != c->aoff[t] + i || !(sg == 1.0 || sg == -1.0)) return UNSUPPORTED;
        inv[(size_t)op * n + a] = mu;
        sgn[(size_t)op * n + a] = sg;
      }
    }
  }
  // the operations must form a group: closed under composition
  for (int p = 0; p < nops; ++p)
    for (int q = 0; q < nops; ++q) {
      bool found = false;
      for (int r = 0; r < nops && !found; ++r) {
        bool same = true;
        for (int mu = 0; mu < n && same; ++mu) {
          const int a = ao_target[(size_t)q * n + mu];
          same = ao_target[(size_t)r * n + mu] == ao_target[(size_t)p * n + a] &&
                 ao_sign[(size_t)r * n + mu] == ao_sign[(size_t)q * n + mu] * ao_sign[(size_t)p * n + a];
        }
        found = same;
      }
      if (!found) return UNSUPPORTED;
    }
  std::vector<int> map(shell_map, shell_map + (size_t)nops * ns);
  cudaStream_t st = c->stream;
  CKP(c->d_sym_map.ensure(sizeof(int) * map.size()));
  CKP(c->d_sym_inv.ensure(sizeof(int) * inv.size()));
  CKP(c->d_sym_sgn.ensure(sizeof(double) * sgn.size()));
  CKP(cudaMemcpyAsync(c->d_sym_map.p, map.data(), sizeof(int) * map.size(), cudaMemcpyHostToDevice, st));
  CKP(cudaMemcpyAsync(c->d_sym_inv.p, inv.data(), sizeof(int) * inv.size(), cudaMemcpyHostToDevice, st));
  CKP(cudaMemcpyAsync(c->d_sym_sgn.p, sgn.data(), sizeof(double) * sgn.size(), cudaMemcpyHostToDevice, st));
  CKP(cudaStreamSynchronize(st));
  c->sym_nops = nops;
  return OK;
}

extern "C" int oqpg_symmetry_info(const oqpg_ctx* c, int* nops, int* reduced) {
  if (!c) return NOT_INIT;
  if (nops) *nops = c->sym_nops > 1 ? c->sym_nops : 1;
  if (reduced) {
    // whether the last direct build used the reduction (its density passed the check)
    *reduced = 0;
    if (c->sym_nops > 1 && c->hb.sym.p) {
      unsigned long long b[2] = {0, 0};
      if (cudaMemcpy(b, c->hb.sym.p, sizeof(b), cudaMemcpyDeviceToHost) != cudaSuccess) return DEV_ERR;
      double r, s;
      std::memcpy(&r, &b[0], sizeof r);
      std::memcpy(&s, &b[1], sizeof s);
      *reduced = r <= 1e-6 * s ? 1 : 0;
    }
  }
  return OK;
}
