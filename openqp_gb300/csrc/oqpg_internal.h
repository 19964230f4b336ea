// Definitions shared by the host translation units: the context of one
// registered molecule, the device-buffer helper, and the build-pipeline
// kernels defined in oqpg_host.cu.
#pragma once
#include <cuda_runtime.h>

#include <vector>

#include "oqpg_classes.h"

namespace oqpg {

enum Status { OK = 0, NOT_INIT = 1, NO_MEM = 2, UNSUPPORTED = 3, DEV_ERR = 4 };

constexpr int NBIN = 64;            // primitive-count bins of the class-list sort
constexpr int PRIM_SPLIT_LOG2 = 8;  // >= 256 primitive quartets: warp per quartet

struct ListArgs {
  int npair, ns;
  const int2* pair_ij;      // shells (i >= j) of each pair, canonical order
  const int* pair_type;
  const double* q;          // Schwarz bound per pair
  const float* qf;
  const int* sorted_idx;    // pairs by descending Schwarz bound
  const double* sorted_q;
  const double* dsh;
  const float* dshf;
  const unsigned long long* dmax_bits;
  double tau;
  double tau_f32;               // quartets with bound < tau_f32 go to the FP32 lists (0: none)
  unsigned long long* counts;   // 2 NCLASS: FP64 lists, then FP32 lists
  uint2* lists[2 * NCLASS];
  unsigned long long caps[2 * NCLASS];
  int write;
};

struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  cudaError_t ensure(size_t b) {
    if (b <= bytes) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
    cudaError_t e = cudaMalloc(&p, b);
    if (e == cudaSuccess) bytes = b;
    return e;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
  template <typename T> T* as() const { return (T*)p; }
};

// Build-pipeline kernels (oqpg_host.cu).
__global__ void k_unpack(const double* __restrict__ dp, int nfocks, int nbf, double* dj, double* dk);
__global__ void k_to_f32(const double* __restrict__ x, long long n, float* y);
__global__ void k_dsh(const double* __restrict__ dp, int nfocks, int nbf, int ns, const int* __restrict__ aoff,
                      const int* __restrict__ nao, double* dsh, float* dshf, unsigned long long* dmax_bits);
__global__ void k_lists(const ListArgs a);
__global__ void k_bin_hist(const uint2* __restrict__ list, long long n, const PairDev* __restrict__ pairs,
                           unsigned long long* hist);
__global__ void k_bin_scatter(const uint2* __restrict__ list, long long n, const PairDev* __restrict__ pairs,
                              unsigned long long* cursors, uint2* out, long long chunk);
__global__ void k_finalize(const double* __restrict__ gj, const double* __restrict__ gk, int nk, int nbf, double sc,
                           double ck, double* f, double* f_old);
void set_band(BuildArgs& a);

}  // namespace oqpg

struct oqpg_ctx {
  int dev = 0, nsm = 152;
  cudaStream_t stream = nullptr;
  int nshell = 0, nbf = 0, natom = 0, npair = 0;
  bool pure = false;
  double tau = 1e-10;
  std::vector<oqpg::ShellDev> shells;
  std::vector<int> aoff, naos;
  std::vector<double> schwarz_pair;   // per pair (canonical index)
  // precision split: 0 = every quartet in FP64, 1 = bound < tau_f32 in FP32
  int precision_mode = 0;
  double tau_f32 = 0.0;
  // device tables
  oqpg::DevBuf d_shells, d_pairs, d_prims, d_primsf, d_pair_ij, d_pair_type, d_q, d_qf, d_aoff, d_naos;
  // per-build buffers
  oqpg::DevBuf d_dp, d_dj, d_dk, d_djf, d_dkf, d_gj, d_gk, d_f, d_fold, d_dsh, d_dshf, d_dmax, d_counts,
      d_prim_counter;
  oqpg::DevBuf d_lists[2 * oqpg::NCLASS], d_slists[2 * oqpg::NCLASS];
  oqpg::DevBuf d_sorted_idx, d_sorted_q, d_hist, d_cursor, d_work;
  unsigned long long caps[2 * oqpg::NCLASS] = {0};
  unsigned long long counts[2 * oqpg::NCLASS] = {0};
  bool have_caps = false;
  // pinned staging
  double* h_in = nullptr;
  double* h_out = nullptr;
  size_t h_bytes = 0;
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  cudaEvent_t evc[oqpg::NCLASS][2] = {};
  double last_stats[10 + 3 * oqpg::NCLASS] = {0};
};
