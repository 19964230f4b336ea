// MRSF Davidson sigma session: the routec_sig_* seam of OpenQP
// (source/modules/routec_sig.F90:1-140, called from
// source/modules/tdhf_mrsf_energy.F90:638-690).  One routec_sig_iter call
// replaces, for every new trial vector, the native triple
//   iatogen + mrsfcbc (tdhf_lib.F90:480-498, tdhf_mrsf_lib.F90:940-1273)
//   int2_mrsf_data_t build (the screened quartet pipeline, nmat 7)
//   triplet sign (tdhf_mrsf_energy.F90:762-766), mrsfmntoia + mrsfesum
//   (tdhf_mrsf_lib.F90:1463-1735, 1918-2036)
// on the device of the routec_fock_init context.  All vectors of a call go
// through one integral pass; the MO <-> AO transforms are cuBLAS DGEMMs
// (column-major, the reference's own layout) and three elementwise kernels.
//
// Indices are 0-based: open shells lr1 = nocca - 2, lr2 = nocca - 1; the
// trial space is X(i, j), i < nocca, j >= noccb, packed i fastest.
#include <cublas_v2.h>

#include <mutex>

#include "oqpg_common.cuh"
#include "oqpg_internal.h"
#include "../../include/openqp_gb300.h"

namespace oqpg {
namespace {

constexpr double kIsqrt2 = 0.70710678118654752440;

struct SigSession {
  oqpg_ctx* ctx = nullptr;
  int n = 0, na = 0, nb = 0, mrst = 1;
  double scale = 1.0;
  cublasHandle_t blas = nullptr;
  DevBuf va, vb, fa, fb;                       // (n, n) column-major
  DevBuf bv, x, d3, f3, t12, c12, y, w, sc, e, tv, sig;
};

std::mutex g_sig_mutex;
SigSession* g_sig = nullptr;

// X_v(r, c) = bvec(r + na (c - nb), v) inside the (na, n - nb) block, else 0.
__global__ void k_sig_unpack(const double* __restrict__ bv, int nv, int n, int na, int nb, double* __restrict__ x) {
  const long long nn = (long long)n * n, tot = nn * nv, ntrial = (long long)na * (n - nb);
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < tot; t += (long long)gridDim.x * blockDim.x) {
    const int v = (int)(t / nn);
    const long long u = t - v * nn;
    const int r = (int)(u % n), c = (int)(u / n);
    x[t] = (r < na && c >= nb) ? bv[r + (long long)na * (c - nb) + ntrial * v] : 0.0;
  }
}

// mrsfcbc's rank-1 / rank-2 components and the OO corrections of ball:
// t12 = (t1, t2) = vb_virt X(lr1 | lr2, virt)^T, c12 = (c1, c2) =
// va_closed X(closed, lr1 | lr2); ball already holds the CV block when have_cv.
__global__ void k_sig_cbc(const double* __restrict__ x, const double* __restrict__ t12,
                          const double* __restrict__ c12, const double* __restrict__ va, const double* __restrict__ vb,
                          int nv, int n, int na, int mrst, int have_cv, double* __restrict__ d3) {
  const long long nn = (long long)n * n, tot = nn * nv;
  const int lr1 = na - 2, lr2 = na - 1;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < tot; t += (long long)gridDim.x * blockDim.x) {
    const int v = (int)(t / nn);
    const long long u = t - v * nn;
    const int r = (int)(u % n), c = (int)(u / n);
    const double* xv = x + v * nn;
    const double* tv = t12 + (long long)v * 2 * n;
    const double* cv = c12 + (long long)v * 2 * n;
    const double a1r = va[r + (long long)n * lr1], a2r = va[r + (long long)n * lr2];
    const double a1c = va[c + (long long)n * lr1], a2c = va[c + (long long)n * lr2];
    const double b1r = vb[r + (long long)n * lr1], b2r = vb[r + (long long)n * lr2];
    const double b1c = vb[c + (long long)n * lr1], b2c = vb[c + (long long)n * lr2];
    const double t1r = tv[r], t2r = tv[n + r], t1c = tv[c], t2c = tv[n + c];
    const double c1r = cv[r], c2r = cv[n + r], c1c = cv[c], c2c = cv[n + c];
    double* o = d3 + (long long)v * 7 * nn + u;
    const double f0 = a2r * t2c, f1 = a1r * t1c, f2 = c1r * b1c, f3 = c2r * b2c;
    o[0] = f0;
    o[nn] = f1;
    o[2 * nn] = f2;
    o[3 * nn] = f3;
    o[4 * nn] = t2r * a1c - t1r * a2c;
    o[5 * nn] = b2r * c1c - b1r * c2c;
    double ball = (have_cv ? o[6 * nn] : 0.0) + f0 + f1 + f2 + f3;
    const double x11 = xv[lr1 + (long long)n * lr1] * kIsqrt2;
    if (mrst == 1)
      ball += xv[lr2 + (long long)n * lr1] * a2r * b1c + xv[lr1 + (long long)n * lr2] * a1r * b2c +
              x11 * (a1r * b1c - a2r * b2c);
    else
      ball += x11 * (a1r * b1c + a2r * b2c);
    o[6 * nn] = ball;
  }
}

// mrsfesum's scr: X with its two open-open diagonal elements cleared.
__global__ void k_sig_clear_oo(double* x, int nv, int n, int na) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nv) return;
  const long long nn = (long long)n * n;
  x[v * nn + (na - 2) + (long long)n * (na - 2)] = 0.0;
  x[v * nn + (na - 1) + (long long)n * (na - 1)] = 0.0;
}

// sigma(:, v) = pack(mrsfmntoia wrk) + pack(mrsfesum wrk1), one CTA per vector.
__global__ void k_sig_final(const double* __restrict__ bv, const double* __restrict__ xs,
                            const double* __restrict__ scr, const double* __restrict__ e,
                            const double* __restrict__ fa, const double* __restrict__ fb, int n, int na, int nb,
                            int mrst, double* __restrict__ sig) {
  const int v = blockIdx.x;
  const long long nn = (long long)n * n, ntrial = (long long)na * (n - nb);
  const int lr1 = na - 2, lr2 = na - 1;
  const double s2 = mrst == 1 ? -1.0 : 1.0;
  const double* X = xs + v * nn;
  const double* S = scr + v * nn;
  const double* E = e + v * nn;
  __shared__ double red[32];
  double part = 0.0;
  for (int k = threadIdx.x; k < na; k += blockDim.x)
    part += -fa[lr1 + (long long)n * k] * X[k + (long long)n * lr1] - s2 * fa[lr2 + (long long)n * k] * X[k + (long long)n * lr2];
  for (int j = nb + threadIdx.x; j < n; j += blockDim.x)
    part += fb[lr1 + (long long)n * j] * X[lr1 + (long long)n * j] + s2 * fb[lr2 + (long long)n * j] * X[lr2 + (long long)n * j];
  for (int o = 16; o; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = part;
  __syncthreads();
  if (threadIdx.x < 32) {
    double q = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
    for (int o = 16; o; o >>= 1) q += __shfl_xor_sync(0xffffffffu, q, o);
    if (threadIdx.x == 0) red[0] = q;
  }
  __syncthreads();
  const double dumn = red[0];
  const double x11 = bv[lr1 + (long long)na * (lr1 - nb) + ntrial * v], xlr = x11 * kIsqrt2;
  for (long long k = threadIdx.x; k < ntrial; k += blockDim.x) {
    const int i = (int)(k % na), j = nb + (int)(k / na);
    double out;
    if (i == lr2 && j == lr2) {
      out = 0.0;
    } else if (mrst == 3 && ((i == lr1 && j == lr2) || (i == lr2 && j == lr1))) {
      out = 0.0;
    } else if (i == lr1 && j == lr1) {
      const double m = (S[lr1 + (long long)n * lr1] + s2 * S[lr2 + (long long)n * lr2]) * kIsqrt2;
      const double es = dumn * kIsqrt2 + x11 * (fb[lr1 + (long long)n * lr1] + fb[lr2 + (long long)n * lr2] -
                                                fa[lr1 + (long long)n * lr1] - fa[lr2 + (long long)n * lr2]) * 0.5;
      out = m + es;
    } else {
      double es = E[i + (long long)n * j];
      if (i == lr1) es += fb[j + (long long)n * lr1] * xlr;
      if (i == lr2) es += s2 * fb[j + (long long)n * lr2] * xlr;
      if (j == lr1) es -= fa[i + (long long)n * lr1] * xlr;
      if (j == lr2) es -= s2 * fa[i + (long long)n * lr2] * xlr;
      out = S[i + (long long)n * j] + es;
    }
    sig[k + ntrial * v] = out;
  }
}

#define CKS(x)                                                                       \
  do {                                                                               \
    cudaError_t e_ = (x);                                                            \
    if (e_ != cudaSuccess) return e_ == cudaErrorMemoryAllocation ? NO_MEM : DEV_ERR; \
  } while (0)
#define CKB(x)                                         \
  do {                                                 \
    if ((x) != CUBLAS_STATUS_SUCCESS) return DEV_ERR;  \
  } while (0)

unsigned grid_of(long long work, int nsm) { return (unsigned)std::max<long long>(1, std::min<long long>((work + 255) / 256, nsm * 8LL)); }

// C(m, n) = alpha op(A) op(B) + beta C for nv strided batches.
cublasStatus_t gemm(cublasHandle_t h, bool ta, bool tb, int m, int n, int k, double alpha, const double* A, int lda,
                    long long sa, const double* B, int ldb, long long sb, double beta, double* C, int ldc, long long sc,
                    int nv) {
  return cublasDgemmStridedBatched(h, ta ? CUBLAS_OP_T : CUBLAS_OP_N, tb ? CUBLAS_OP_T : CUBLAS_OP_N, m, n, k, &alpha,
                                   A, lda, sa, B, ldb, sb, &beta, C, ldc, sc, nv);
}

// bvec / sigma are host buffers, or device buffers with device_io (then st
// is the caller's stream).
int sig_run(SigSession& S, const double* bvec_in, int nv, double* sigma_out, bool device_io, cudaStream_t st) {
  oqpg_ctx* c = S.ctx;
  const int n = S.n, na = S.na, nb = S.nb, nvir = n - na, nvb = n - nb, lr1 = na - 2, lr2 = na - 1;
  const long long nn = (long long)n * n, ntrial = (long long)na * nvb;
  const size_t D = sizeof(double);
  CKS(S.bv.ensure(D * ntrial * nv));
  CKS(S.sig.ensure(D * ntrial * nv));
  CKS(S.x.ensure(D * nn * nv));
  CKS(S.d3.ensure(D * 7 * nn * nv));
  CKS(S.f3.ensure(D * 7 * nn * nv));
  CKS(S.t12.ensure(D * 2 * n * nv));
  CKS(S.c12.ensure(D * 2 * n * nv));
  CKS(S.y.ensure(D * std::max(1, n * nb) * nv));
  CKS(S.w.ensure(D * (long long)na * n * nv));
  CKS(S.sc.ensure(D * nn * nv));
  CKS(S.e.ensure(D * nn * nv));
  CKS(S.tv.ensure(D * 4 * n * nv));
  const double* bv = device_io ? bvec_in : S.bv.as<double>();
  double *x = S.x.as<double>(), *d3 = S.d3.as<double>(), *f3 = S.f3.as<double>();
  double *t12 = S.t12.as<double>(), *c12 = S.c12.as<double>(), *y = S.y.as<double>(), *w = S.w.as<double>();
  double *scr = S.sc.as<double>(), *e = S.e.as<double>(), *tv = S.tv.as<double>();
  double* sig = device_io ? sigma_out : S.sig.as<double>();
  const double *va = S.va.as<double>(), *vb = S.vb.as<double>(), *fa = S.fa.as<double>(), *fb = S.fb.as<double>();
  cublasHandle_t h = S.blas;
  CKB(cublasSetStream(h, st));

  if (!device_io) CKS(cudaMemcpyAsync(S.bv.p, bvec_in, D * ntrial * nv, cudaMemcpyHostToDevice, st));
  k_sig_unpack<<<grid_of(nn * nv, c->nsm), 256, 0, st>>>(bv, nv, n, na, nb, x);
  CKS(cudaGetLastError());
  // mrsfcbc
  CKS(cudaMemsetAsync(t12, 0, D * 2 * n * nv, st));
  CKS(cudaMemsetAsync(c12, 0, D * 2 * n * nv, st));
  if (nvir > 0)
    CKB(gemm(h, false, true, n, 2, nvir, 1.0, vb + (long long)n * na, n, 0, x + lr1 + (long long)n * na, n, nn, 0.0,
             t12, n, 2LL * n, nv));
  const bool have_cv = nb > 0 && nvir > 0;
  if (nb > 0)
    CKB(gemm(h, false, false, n, 2, nb, 1.0, va, n, 0, x + (long long)n * lr1, n, nn, 0.0, c12, n, 2LL * n, nv));
  if (have_cv) {
    CKB(gemm(h, false, true, n, nb, nvir, 1.0, vb + (long long)n * na, n, 0, x + (long long)n * na, n, nn, 0.0, y, n,
             (long long)n * nb, nv));
    CKB(gemm(h, false, true, n, n, nb, 1.0, va, n, 0, y, n, (long long)n * nb, 0.0, d3 + 6 * nn, n, 7 * nn, nv));
  }
  k_sig_cbc<<<grid_of(nn * nv, c->nsm), 256, 0, st>>>(x, t12, c12, va, vb, nv, n, na, S.mrst, have_cv ? 1 : 0, d3);
  CKS(cudaGetLastError());
  // int2_mrsf_data_t build, scale_exchange = scale_coulomb = scale, triplet sign folded in
  {
    GenJob g;
    mrsf_job_layout(c, d3, f3, nv, 7, S.scale, S.scale, MrsfLayout{1, n, nn, 7 * nn}, S.mrst == 3, g);
    Job j;
    j.gen = &g;
    const int rc = ctx_build(c, j, st);
    if (rc) return rc;
  }
  // mrsfmntoia: scr block = va_occ^T agdlr vb_(noccb:), then the rank-1 updates
  CKB(gemm(h, true, false, na, n, n, 1.0, va, n, 0, f3 + 6 * nn, n, 7 * nn, 0.0, w, na, (long long)na * n, nv));
  CKB(gemm(h, false, false, na, nvb, n, 1.0, w, na, (long long)na * n, vb + (long long)n * nb, n, 0, 0.0,
           scr + (long long)n * nb, n, nn, nv));
  const double* vb1 = vb + (long long)n * lr1;
  const double* vb2 = vb + (long long)n * lr2;
  const double* va1 = va + (long long)n * lr1;
  const double* va2 = va + (long long)n * lr2;
  CKB(gemm(h, false, false, n, 1, n, 1.0, f3 + 1 * nn, n, 7 * nn, vb2, n, 0, 0.0, tv, n, 4LL * n, nv));
  CKB(gemm(h, false, false, n, 1, n, 1.0, f3 + 5 * nn, n, 7 * nn, vb1, n, 0, 1.0, tv, n, 4LL * n, nv));
  CKB(gemm(h, false, false, n, 1, n, 1.0, f3 + 0 * nn, n, 7 * nn, vb1, n, 0, 0.0, tv + n, n, 4LL * n, nv));
  CKB(gemm(h, false, false, n, 1, n, -1.0, f3 + 5 * nn, n, 7 * nn, vb2, n, 0, 1.0, tv + n, n, 4LL * n, nv));
  CKB(gemm(h, true, false, n, 1, n, 1.0, f3 + 3 * nn, n, 7 * nn, va1, n, 0, 0.0, tv + 2 * n, n, 4LL * n, nv));
  CKB(gemm(h, true, false, n, 1, n, 1.0, f3 + 4 * nn, n, 7 * nn, va2, n, 0, 1.0, tv + 2 * n, n, 4LL * n, nv));
  CKB(gemm(h, true, false, n, 1, n, 1.0, f3 + 2 * nn, n, 7 * nn, va2, n, 0, 0.0, tv + 3 * n, n, 4LL * n, nv));
  CKB(gemm(h, true, false, n, 1, n, -1.0, f3 + 4 * nn, n, 7 * nn, va1, n, 0, 1.0, tv + 3 * n, n, 4LL * n, nv));
  if (na > 2) {
    CKB(gemm(h, true, false, na - 2, 1, n, 1.0, va, n, 0, tv, n, 4LL * n, 1.0, scr + (long long)n * lr2, n, nn, nv));
    CKB(gemm(h, true, false, na - 2, 1, n, 1.0, va, n, 0, tv + n, n, 4LL * n, 1.0, scr + (long long)n * lr1, n, nn,
             nv));
  }
  if (nvir > 0) {
    CKB(gemm(h, true, false, 1, nvir, n, 1.0, tv + 2 * n, n, 4LL * n, vb + (long long)n * na, n, 0, 1.0,
             scr + lr1 + (long long)n * na, n, nn, nv));
    CKB(gemm(h, true, false, 1, nvir, n, 1.0, tv + 3 * n, n, 4LL * n, vb + (long long)n * na, n, 0, 1.0,
             scr + lr2 + (long long)n * na, n, nn, nv));
  }
  // mrsfesum on X with the open-open diagonal cleared
  k_sig_clear_oo<<<(nv + 127) / 128, 128, 0, st>>>(x, nv, n, na);
  CKS(cudaGetLastError());
  CKB(gemm(h, false, true, na, nvb, nvb, 1.0, x + (long long)n * nb, n, nn, fb + nb + (long long)n * nb, n, 0, 0.0,
           e + (long long)n * nb, n, nn, nv));
  CKB(gemm(h, false, false, na, nvb, na, -1.0, fa, n, 0, x + (long long)n * nb, n, nn, 1.0, e + (long long)n * nb, n,
           nn, nv));
  k_sig_final<<<nv, 256, 0, st>>>(bv, x, scr, e, fa, fb, n, na, nb, S.mrst, sig);
  CKS(cudaGetLastError());
  if (!device_io) CKS(cudaMemcpyAsync(sigma_out, sig, D * ntrial * nv, cudaMemcpyDeviceToHost, st));
  CKS(cudaStreamSynchronize(st));
  return OK;
}

void sig_free_locked() {
  if (!g_sig) return;
  SigSession* S = g_sig;
  g_sig = nullptr;
  if (S->blas) cublasDestroy(S->blas);
  for (DevBuf* b : {&S->va, &S->vb, &S->fa, &S->fb, &S->bv, &S->x, &S->d3, &S->f3, &S->t12, &S->c12, &S->y, &S->w,
                    &S->sc, &S->e, &S->tv, &S->sig})
    b->release();
  delete S;
}

}  // namespace

void sig_release() {
  std::lock_guard<std::mutex> lk(g_sig_mutex);
  sig_free_locked();
}

}  // namespace oqpg

using namespace oqpg;

extern "C" {

int routec_sig_init(const int* nbf, const double* mo_a, const double* mo_b, const double* fmo_a, const double* fmo_b,
                    const int* nocca, const int* noccb, const int* kind) {
  std::lock_guard<std::mutex> lk(g_sig_mutex);
  sig_free_locked();
  oqpg_ctx* c = routec_context();
  if (!c) return NOT_INIT;
  if (!nbf || !mo_a || !mo_b || !fmo_a || !fmo_b || !nocca || !noccb || !kind) return UNSUPPORTED;
  if (*nbf != c->nbf || c->nmol != 1) return NOT_INIT;
  const int n = *nbf, na = *nocca, nb = *noccb;
  if ((*kind != 1 && *kind != 3) || nb < 0 || na != nb + 2 || na > n) return UNSUPPORTED;
  SigSession* S = new SigSession;
  S->ctx = c;
  S->n = n;
  S->na = na;
  S->nb = nb;
  S->mrst = *kind;
  const size_t bytes = sizeof(double) * (size_t)n * n;
  int rc = OK;
  if (cublasCreate(&S->blas) != CUBLAS_STATUS_SUCCESS) {
    S->blas = nullptr;
    rc = DEV_ERR;
  }
  const double* src[4] = {mo_a, mo_b, fmo_a, fmo_b};
  DevBuf* dst[4] = {&S->va, &S->vb, &S->fa, &S->fb};
  for (int i = 0; i < 4 && rc == OK; ++i) {
    cudaError_t e = dst[i]->ensure(bytes);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dst[i]->p, src[i], bytes, cudaMemcpyHostToDevice, c->stream);
    if (e != cudaSuccess) rc = e == cudaErrorMemoryAllocation ? NO_MEM : DEV_ERR;
  }
  if (rc == OK && cudaStreamSynchronize(c->stream) != cudaSuccess) rc = DEV_ERR;
  g_sig = S;
  if (rc != OK) sig_free_locked();
  return rc;
}

void routec_sig_set_scale(const double* s) {
  std::lock_guard<std::mutex> lk(g_sig_mutex);
  if (g_sig && s) g_sig->scale = *s;
}

void routec_sig_iter(const double* bvec_mo, const int* nv_new, double* sigma_mo, int* info) {
  std::lock_guard<std::mutex> lk(g_sig_mutex);
  int rc;
  if (!g_sig || g_sig->ctx != routec_context()) rc = NOT_INIT;
  else if (!bvec_mo || !nv_new || !sigma_mo || *nv_new < 0) rc = UNSUPPORTED;
  else if (*nv_new == 0) rc = OK;
  else rc = sig_run(*g_sig, bvec_mo, *nv_new, sigma_mo, false, g_sig->ctx->stream);
  if (info) *info = rc;
}

int oqpg_sig_iter_device(const double* bvec, int nv, double* sigma, void* stream) {
  std::lock_guard<std::mutex> lk(g_sig_mutex);
  if (!g_sig || g_sig->ctx != routec_context()) return NOT_INIT;
  if (!bvec || !sigma || nv < 0) return UNSUPPORTED;
  if (nv == 0) return OK;
  return sig_run(*g_sig, bvec, nv, sigma, true, stream ? (cudaStream_t)stream : g_sig->ctx->stream);
}

void routec_sig_free(void) { sig_release(); }

}  // extern "C"
