// Fock build that allocates no device memory.
//
// Some callers cannot call cudaMalloc at build time: a host program whose own
// pool allocator owns every byte of device memory (a PyTorch process with its
// caching allocator, an application that reserves its memory up front) gets
// out-of-memory or fragmentation from allocations made behind its back, and a
// latency-critical SCF loop cannot afford the device-wide synchronisation a
// cudaMalloc/cudaFree pair may cause.  For them oqpg_fock_jk_noalloc runs the
// plain-FP64 build of oqpg_fock_jk_device (precision mode 0, fixed launch
// parameters: the primitive-parallel head at 2^8 primitive quartets and no
// tuned grid caps, whatever the context's precision split and tuning say; the
// context's cutoff applies), with every per-build buffer (densities, J/K
// accumulators, shell densities, quartet lists, counters) carved out of one
// file-scope device array of fixed size, so it calls no cudaMalloc, cudaFree
// or allocating library routine.  The read-only tables of the molecule
// (shells, primitive pairs, Schwarz bounds) are the context's, made once by
// oqpg_create.
//
// Limits: nbf <= 128 and nshell <= 128, checked before any kernel runs; the
// screened quartets of all classes must fit the rest of the array (an
// unsorted and a sorted 8-byte entry each: about 1.5 million at nbf = 128),
// which the screening pass finds out.  Either limit returns status 5 with
// the caller's output untouched (only the scratch array has been written).
#include <cstring>
#include <mutex>

#include "../../include/openqp_gb300.h"
#include "oqpg_internal.h"

namespace {

constexpr int NOALLOC_MAX_NBF = 128;
constexpr int NOALLOC_MAX_SHELLS = 128;
constexpr size_t NOALLOC_BYTES = 24u << 20;   // 24 MiB per device
constexpr int NOALLOC_TOO_LARGE = 5;
constexpr int MAX_DEVICES = 64;

// The scratch array.  Every GPU that loads the library holds it until the
// process exits.  All calls on a device share it and it keeps the last call's
// contents; each call clears what must start at zero.  Calls that overlap on
// the GPU (two streams, two host threads) race on it.
static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_BYTES];

std::mutex g_noalloc_mutex;
void* g_scratch_addr[MAX_DEVICES] = {nullptr};

// Device address of g_noalloc_scratch on the current device.  In host code
// the array's name is a host-side stand-in, not a device address, so the
// address is looked up once per device (with that device current) and cached.
// Under lazy module loading the first lookup may load the module and reserve
// the array's device memory at that moment, so the first call on a device
// should come before any stream capture and before a pool allocator takes
// the rest of the device memory.
int scratch_address(void** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= MAX_DEVICES) return oqpg::DEV_ERR;
  std::lock_guard<std::mutex> lk(g_noalloc_mutex);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return oqpg::DEV_ERR;
    g_scratch_addr[dev] = p;
  }
  *out = g_scratch_addr[dev];
  return oqpg::OK;
}

struct Carver {
  unsigned char* base;
  size_t used = 0;
  template <typename T>
  T* take(size_t count) {
    used = (used + 255) & ~size_t(255);
    T* p = reinterpret_cast<T*>(base + used);
    used += sizeof(T) * count;
    return p;
  }
};

}  // namespace

using namespace oqpg;

extern "C" int oqpg_fock_jk_noalloc(oqpg_ctx* c, const double* d_device, double* f_device, int nfocks, double se,
                                    double sc, void* stream) {
  if (!c) return NOT_INIT;
  if (nfocks != 1 && nfocks != 2) return UNSUPPORTED;
  if (c->nmol != 1) return UNSUPPORTED;
  if (c->nbf > NOALLOC_MAX_NBF || c->nshell > NOALLOC_MAX_SHELLS) return NOALLOC_TOO_LARGE;
  void* sp = nullptr;
  if (int rc = scratch_address(&sp)) return rc;
  cudaStream_t st = stream ? (cudaStream_t)stream : c->stream;
  const int n = c->nbf, ns = c->nshell, nk = nfocks;
  const size_t n2 = (size_t)n * n;
  Carver cv{static_cast<unsigned char*>(sp)};
  double* dj = cv.take<double>(n2);
  double* dk = cv.take<double>(2 * n2);
  double* gj = cv.take<double>(n2);
  double* gk = cv.take<double>(2 * n2);
  double* dsh = cv.take<double>((size_t)ns * ns);
  float* dshf = cv.take<float>((size_t)ns * ns);
  unsigned long long* dmax = cv.take<unsigned long long>(1);
  unsigned long long* counts = cv.take<unsigned long long>(NCLASS);
  unsigned long long* hist = cv.take<unsigned long long>(NCLASS * NBIN);
  unsigned long long* cursor = cv.take<unsigned long long>(NCLASS * NBIN);
  unsigned long long* primc = cv.take<unsigned long long>(NCLASS);
  unsigned long long* work = cv.take<unsigned long long>(2 * NCLASS);
  cv.used = (cv.used + 255) & ~size_t(255);
  // unsorted + sorted copies; a multiple of 32 entries (256 bytes), so the
  // second copy starts aligned and both end inside the array
  const size_t qcap = ((NOALLOC_BYTES - cv.used) / (2 * sizeof(uint2))) & ~size_t(31);
  uint2* lists = cv.take<uint2>(qcap);
  uint2* slists = cv.take<uint2>(qcap);
  if (cv.used > NOALLOC_BYTES) return DEV_ERR;

// A failed launch or copy waits for the work already queued on the stream
// (it uses the shared array) before the call returns.
#define NK(x)                                      \
  do {                                             \
    cudaError_t e_ = (x);                          \
    if (e_ != cudaSuccess) {                       \
      cudaStreamSynchronize(st);                   \
      return DEV_ERR;                              \
    }                                              \
  } while (0)

  NK(cudaMemsetAsync(dmax, 0, sizeof(unsigned long long), st));
  k_unpack<<<(unsigned)((n2 + 255) / 256), 256, 0, st>>>(d_device, nfocks, c->d_mols.as<MolDev>(),
                                                         c->d_row_mol.as<int>(), n, n, dj, dk);
  NK(cudaGetLastError());
  const long long npair = c->npair;
  k_dsh<<<(unsigned)((npair + 127) / 128), 128, 0, st>>>(d_device, nfocks, c->d_mols.as<MolDev>(),
                                                         c->d_pair_mol.as<int>(), c->d_pair_ij.as<int2>(),
                                                         c->npair, c->d_aoff.as<int>(), c->d_naos.as<int>(), dsh,
                                                         dshf, dmax);
  NK(cudaGetLastError());
  ListArgs la{};
  la.npair = c->npair;
  la.mols = c->d_mols.as<MolDev>();
  la.pair_mol = c->d_pair_mol.as<int>();
  la.pair_ij = c->d_pair_ij.as<int2>();
  la.pair_type = c->d_pair_type.as<int>();
  la.q = c->d_q.as<double>();
  la.qf = c->d_qf.as<float>();
  la.sorted_idx = c->d_sorted_idx.as<int>();
  la.sorted_q = c->d_sorted_q.as<double>();
  la.dsh = dsh;
  la.dshf = dshf;
  la.dmax_bits = dmax;
  la.tau = c->tau;
  la.counts = counts;
  // pass 1: counts only
  la.write = 0;
  NK(cudaMemsetAsync(counts, 0, sizeof(unsigned long long) * NCLASS, st));
  k_lists<<<c->npair, 256, 0, st>>>(la);
  NK(cudaGetLastError());
  unsigned long long h_counts[NCLASS];
  NK(cudaMemcpyAsync(h_counts, counts, sizeof(h_counts), cudaMemcpyDeviceToHost, st));
  NK(cudaStreamSynchronize(st));
  unsigned long long off[NCLASS], total = 0;
  for (int k = 0; k < NCLASS; ++k) { off[k] = total; total += h_counts[k]; }
  if (total > qcap) return NOALLOC_TOO_LARGE;
  // pass 2: fill each class into its exact range
  la.write = 1;
  for (int k = 0; k < NCLASS; ++k) { la.lists[k] = lists + off[k]; la.caps[k] = h_counts[k]; }
  NK(cudaMemsetAsync(counts, 0, sizeof(unsigned long long) * NCLASS, st));
  k_lists<<<c->npair, 256, 0, st>>>(la);
  NK(cudaGetLastError());
  // order each class by primitive-quartet count
  NK(cudaMemsetAsync(hist, 0, sizeof(unsigned long long) * NCLASS * NBIN, st));
  for (int k = 0; k < NCLASS; ++k) {
    if (!h_counts[k]) continue;
    k_bin_hist<<<(unsigned)((h_counts[k] + 255) / 256), 256, 0, st>>>(lists + off[k], (long long)h_counts[k], nullptr,
                                                                      c->d_pairs.as<PairDev>(), nullptr, 0.0f,
                                                                      PAIR_MASK, 0xffffffffu, nullptr,
                                                                      hist + k * NBIN);
    NK(cudaGetLastError());
  }
  unsigned long long h_hist[NCLASS * NBIN], h_cur[NCLASS * NBIN];
  NK(cudaMemcpyAsync(h_hist, hist, sizeof(h_hist), cudaMemcpyDeviceToHost, st));
  NK(cudaStreamSynchronize(st));
  for (int k = 0; k < NCLASS; ++k) {
    unsigned long long s = 0;
    for (int b = 0; b < NBIN; ++b) { h_cur[k * NBIN + b] = s; s += h_hist[k * NBIN + b]; }
    if (s != h_counts[k]) return DEV_ERR;
  }
  NK(cudaMemcpyAsync(cursor, h_cur, sizeof(h_cur), cudaMemcpyHostToDevice, st));
  for (int k = 0; k < NCLASS; ++k) {
    if (!h_counts[k]) continue;
    const long long chunk = 4096;
    k_bin_scatter<<<(unsigned)((h_counts[k] + chunk - 1) / chunk), 256, 0, st>>>(
        lists + off[k], (long long)h_counts[k], nullptr, c->d_pairs.as<PairDev>(), PAIR_MASK, 0xffffffffu, nullptr,
        cursor + k * NBIN, slists + off[k], chunk, nullptr, nullptr);
    NK(cudaGetLastError());
  }
  // integrals and digestion
  NK(cudaMemsetAsync(gj, 0, sizeof(double) * n2, st));
  NK(cudaMemsetAsync(gk, 0, sizeof(double) * nk * n2, st));
  NK(cudaMemsetAsync(primc, 0, sizeof(unsigned long long) * NCLASS, st));
  NK(cudaMemsetAsync(work, 0, sizeof(unsigned long long) * 2 * NCLASS, st));
  BuildArgs a{};
  a.shells = c->d_shells.as<ShellDev>();
  a.pairs = c->d_pairs.as<PairDev>();
  a.prims = c->d_prims.as<PrimPair>();
  a.nbf = n;
  a.kstride = n2;
  a.nj = 1;
  a.nk = nk;
  a.prim_cut = 1e-4 * c->tau;
  a.prim_cut2 = a.prim_cut * a.prim_cut;
  set_band(a);
  a.elem_cut = c->tau;
  a.dj = dj;
  a.dk = (nk == 1) ? dj : dk;
  a.gj = gj;
  a.gk = gk;
  for (int cl = NCLASS - 1; cl >= 0; --cl) {
    if (!h_counts[cl]) continue;
    a.counters = primc + cl;
    long long head = 0;
    if (class_info(cl).prim && class_info(cl).small) {   // thread per quartet where the class has it
      for (int b = 0; b < head_bins(PRIM_SPLIT_LOG2); ++b) head += (long long)h_hist[cl * NBIN + b];
      if (head > 0) {
        a.quartets = slists + off[cl];
        a.nquartets = head;
        a.work = work + NCLASS + cl;
        NK(launch_class(cl, c->pure, MODE_PRIM, a, c->nsm, st));
      }
    }
    if ((long long)h_counts[cl] > head) {
      a.quartets = slists + off[cl] + head;
      a.nquartets = (long long)h_counts[cl] - head;
      a.work = work + cl;
      NK(launch_class(cl, c->pure, MODE_FOCK, a, c->nsm, st));
    }
  }
  const long long ntri = (long long)n * (n + 1) / 2;
  const double ck = (nk == 1) ? 0.5 * se : se;
  k_finalize<<<(unsigned)((ntri + 255) / 256), 256, 0, st>>>(gj, gk, nk, c->d_mols.as<MolDev>(), 1, ntri, n, n2,
                                                             sc, ck, f_device, nullptr, nullptr);
  NK(cudaGetLastError());
  NK(cudaStreamSynchronize(st));
#undef NK
  return OK;
}
