// Definitions shared by the host translation units: the context of one
// registered molecule, the device-buffer helper, and the build-pipeline
// kernels defined in oqpg_host.cu.
#pragma once
#include <cuda_runtime.h>

#include <vector>

#include "oqpg_classes.h"
#include "oqpg_df.cuh"

namespace oqpg {

enum Status { OK = 0, NOT_INIT = 1, NO_MEM = 2, UNSUPPORTED = 3, DEV_ERR = 4 };

// Primitive-count bins of the class-list sort, heaviest first: a quartet with
// n surviving primitive quartets goes to bin NBIN - 1 - b(n), b(n) = n - 1 for
// n < BIN_EXACT (exact counts, so the lanes of a warp run equal trip counts)
// and 4 log2(n) + BIN_EXACT - 25 above (quarter octaves).
constexpr int NBIN = 128;
constexpr int BIN_EXACT = 64;
// Bins 0 .. head_bins(s) - 1 hold the quartets with at least 2^s primitive quartets.
__host__ __device__ inline int head_bins(int s) {
  if (s < 0) return NBIN;
  if (s > 30) return 0;
  const int b = (1 << s) < BIN_EXACT ? (1 << s) - 1 : 4 * s + BIN_EXACT - 25;
  return b > NBIN - 1 ? 0 : NBIN - b;
}
constexpr int PRIM_SPLIT_LOG2 = 8;  // >= 256 primitive quartets: warp per quartet
// split_bins entry of a list whose head the device sizes from the list itself
// (k_bin_scan: the default of thread-per-quartet lists)
constexpr int SPLIT_ADAPTIVE = -1;

// One molecule of a context (a context holds a batch of one or more).  Its
// shells, pairs and AO rows are contiguous ranges of the context's tables;
// its matrices are rows [row0, row0 + nbf) of the stacked nrows x stride
// matrices (columns 0 .. nbf-1); its packed densities / Fock matrices start
// at nfocks * tri0 of the caller's arrays, one nbf(nbf+1)/2 triangle per density.
struct MolDev {
  int nbf, ns, shell0, pair0, npair, row0;
  long long tri0;  // packed elements (per density) of the molecules before it
  long long dsh0;  // first element of its ns x ns shell-density block
};

// Quartet lists of a build: the FP64 shell-quartet list of every class, the
// FP32 lists of the precision split, then the family-quartet lists of the
// shell-family classes (FP64, then FP32).
constexpr int NLIST_SHELL = 2 * NCLASS;
constexpr int NLIST = NLIST_SHELL + 2 * NFAMCLS;
__host__ __device__ inline int fam_list_index(int c, int f32 = 0) { return NLIST_SHELL + f32 * NFAMCLS + fam_slot(c); }
// the class of list k
__host__ __device__ inline int list_class(int k) {
  return k < NLIST_SHELL ? k % NCLASS : fam_slot_class((k - NLIST_SHELL) % NFAMCLS);
}

struct ListArgs {
  int npair;                // pairs of the whole batch (one CTA each)
  const MolDev* mols;
  const int* pair_mol;      // molecule of each pair
  const int2* pair_ij;      // shells (i >= j, molecule-local) of each pair, canonical order
  const int* pair_type;
  const double* q;          // Schwarz bound per pair
  const float* qf;
  const int* sorted_idx;    // per molecule: its pairs by descending Schwarz bound (segment at pair0)
  const double* sorted_q;
  const double* dsh;        // per molecule ns x ns blocks at dsh0
  const float* dshf;
  const unsigned long long* dmax_bits;  // per molecule
  double tau;
  double tau_f32;               // quartets with bound < tau_f32 go to the FP32 lists (0: none)
  unsigned long long* counts;   // NLIST: FP64 lists, FP32 lists, family lists
  uint2* lists[NLIST];
  unsigned long long caps[NLIST];
  int write;
  // petite list (one molecule): shell images of the symmetry operations,
  // map[op ns + s]; sym_bits = (density asymmetry, density scale) as FP64 bits,
  // the reduction applies when asymmetry <= 1e-6 scale
  const int* sym_map;
  int sym_nops;
  int sym_ns;
  const unsigned long long* sym_bits;
  // shell families: k_lists leaves the quartets of the family classes with a
  // member-sharing side (pair_fam_multi) to k_lists_fam, which lists family
  // quartets into the family lists
  int fam;
  const unsigned char* pair_fam_multi;   // per pair: its family pair has more than one member
  int nfpair;
  const PairDev* fpairs;
  const FamMem* fmem;
  const int* fpair_mol;
  const int* fpair_type;
  const double* fq;                      // family Schwarz bound: the largest member bound
  const int* fsorted_idx;                // per molecule: its family pairs by descending bound
  const double* fsorted_q;
  const int* fmol0;                      // first family pair of each molecule
  const int* fmoln;                      // and their number
  const int* fmsorted_idx;               // per molecule: the family pairs with more than one member,
  const double* fmsorted_q;              // by descending bound (segment at fmmol0, fmmoln entries)
  const int* fmmol0;
  const int* fmmoln;
  unsigned long long* fam_members;       // per class: member quartets listed, FP64 then FP32 (statistics)
};

// The quartet screen of k_lists (int2.F90:975-986) for bra pair (shells ij,
// bound qP) and ket pair Q (shells kl): the FP32 test value
// Q_P Q_Q max(4D_ij, 4D_kl, D_jl, D_jk, D_il, D_ik) and, with the reference's
// operation order, the FP64 one.  di, dj: the shell-density rows of i and j.
__device__ __forceinline__ float quartet_value_f32(const ListArgs& a, int ns, const float* dshf, const float* di,
                                                   const float* dj, float dij4, float qPf, int Q, int2 kl) {
  const float m = fmaxf(fmaxf(fmaxf(dij4, 4.0f * dshf[(long long)kl.x * ns + kl.y]), fmaxf(dj[kl.y], dj[kl.x])),
                        fmaxf(di[kl.y], di[kl.x]));
  return qPf * a.qf[Q] * m;
}
__device__ __forceinline__ double quartet_value(const ListArgs& a, int ns, const double* dshd, int2 ij, double qP,
                                                int Q, int2 kl) {
  const double* Di = dshd + (long long)ij.x * ns;
  const double* Dj = dshd + (long long)ij.y * ns;
  double v = qP * a.q[Q];
  v *= fmax(fmax(fmax(4.0 * Di[ij.y], 4.0 * dshd[(long long)kl.x * ns + kl.y]), fmax(Dj[kl.y], Dj[kl.x])),
            fmax(Di[kl.y], Di[kl.x]));
  return v;
}

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
__global__ void k_unpack(const double* __restrict__ dp, int nfocks, const MolDev* __restrict__ mols,
                         const int* __restrict__ row_mol, int nrows, int stride, double* dj, double* dk);
__global__ void k_to_f32(const double* __restrict__ x, long long n, float* y);
__global__ void k_to_df(const double* __restrict__ x, long long n, dfl* y);
__global__ void k_dsh(const double* __restrict__ dp, int nfocks, const MolDev* __restrict__ mols,
                      const int* __restrict__ pair_mol, const int2* __restrict__ pair_ij, int npair,
                      const int* __restrict__ aoff, const int* __restrict__ nao, double* dsh, float* dshf,
                      unsigned long long* dmax_bits);
__global__ void k_lists(const ListArgs a);
// family quartets (oqpg_family.cu), one CTA per family pair
__global__ void k_lists_fam(const ListArgs a);
// n entries, or with n_dev the device count min(*n_dev, n) (n is then the capacity)
// prims null: bins by the product of the pair primitive counts; else by the
// primitive quartets passing the FP32 pre-screen at lo (bins[t] stores each bin)
// (xmask, ymask: the bits of an entry's x and y that hold the pair indices)
__global__ void k_bin_hist(const uint2* __restrict__ list, long long n, const unsigned long long* n_dev,
                           const PairDev* __restrict__ pairs, const PrimPair* __restrict__ prims, float lo,
                           unsigned xmask, unsigned ymask, unsigned char* bins, unsigned long long* hist);
__global__ void k_bin_scatter(const uint2* __restrict__ list, long long n, const unsigned long long* n_dev,
                              const PairDev* __restrict__ pairs, unsigned xmask, unsigned ymask,
                              const unsigned char* __restrict__ bins, unsigned long long* cursors, uint2* out,
                              long long chunk, const unsigned* flag, const FamMem* __restrict__ fmem);
__global__ void k_bin_scan(const unsigned long long* counts, const unsigned long long* caps, const int* split_bins,
                           const unsigned long long* hist, unsigned long long* cursors, unsigned long long* ranges,
                           unsigned* overflow, int nsm, int adaptive);
// (does nothing when *flag != 0: a list overflowed and the build is redone)
__global__ void k_finalize(const double* __restrict__ gj, const double* __restrict__ gk, int nk,
                           const MolDev* __restrict__ mols, int nmol, long long ntri_total, int stride,
                           size_t kstride, double sc, double ck, double* f, double* f_old,
                           const unsigned* __restrict__ flag);
void set_band(BuildArgs& a);

// --- general (square, not necessarily symmetric) densities -----------------
// A response-type build (TDHF / CPHF A+B and A-B, MRSF sigma vectors) needs,
// per input matrix X, J[X] and K[X] with the full permutational sums
//   J[X]_ij = sum_kl (ij|kl) X_kl,   K[X]_ik = sum_jl (ij|kl) X_jl.
// J only sees Xs = (X + X^T)/2; K[X] = K[Xs] + K[Xa] with Xa = (X - X^T)/2.
// The kernels digest symmetric-storage densities: for a density S staged as a
// full square matrix they accumulate G with J_full = G + G^T, and for K
// K_full = G + G^T when S is symmetric, G - G^T when it is antisymmetric.
// A job is a list of staged slices (Xs or Xa of one input), the Coulomb
// slices [0, nj) and exchange slices [k0, k0 + nk) of that list, and per
// output matrix a short sum of coef * (G + sign G^T) terms.
struct GenSlice {
  long long base;  // input matrix: element (r, c) at in[base + r in_rs + c in_cs]
  int sign;        // +1: (X + X^T)/2, -1: (X - X^T)/2
  int pad;
};
struct GenTerm {
  double coef;
  int kind;  // 0: Coulomb accumulator idx, 1: exchange accumulator idx
  int idx;
  int sign;  // +1 / -1: G + sign G^T
  int pad;
};
struct GenOut {
  double* dst;     // device: element (r, c) at dst[r out_rs + c out_cs]
  int term0, nterm;
};
struct GenJob {
  const double* in = nullptr;  // device
  long long in_rs = 1, in_cs = 0, out_rs = 1, out_cs = 0;
  std::vector<GenSlice> slices;
  int nj = 0, k0 = 0, nk = 0;
  std::vector<long long> screen;  // bases of the inputs that form the shell density
  std::vector<GenOut> outs;
  std::vector<GenTerm> terms;
  bool accumulate = false;  // add into the outputs (second CAM pass) instead of overwriting
};

// One build: packed SCF densities (gen == nullptr) or a general job.
struct Job {
  const double* dp = nullptr;
  int nfocks = 0;
  double* f = nullptr;
  double* f_old = nullptr;
  double se = 1.0, sc = 1.0;
  const GenJob* gen = nullptr;
  double inv_mu2 = 0.0;  // erf(mu r)/r pass of a CAM build (needs ensure_att(mu) first)
  bool petite = true;    // the context's petite list may apply (plain SCF builds of packed densities)
  int nj() const { return gen ? gen->nj : 1; }
  int nk() const { return gen ? gen->nk : nfocks; }
};

// Host-side primitive-pair tables of a context (oqpg_host.cu).
struct HostPairs {
  std::vector<PairDev> pairs;
  std::vector<PrimPair> prims;
  std::vector<double> alpha;  // exponent of the pair's first shell, per primitive pair
  // screening key min(|K|, |K/p|) of each primitive pair (pre-screened tables:
  // a shell pair's primitive pairs are in decreasing key order, so the pairs
  // that a looser cutoff keeps are a prefix of its range)
  std::vector<double> key;
  std::vector<int2> ij;       // molecule-local shells of each pair
  std::vector<int> type;
  std::vector<int> mol;
};

struct GradArgs;
struct BuildBufs;
}  // namespace oqpg
struct oqpg_ctx;
namespace oqpg {
void build_pairs(const oqpg_ctx& c, const std::vector<int>& am, const std::vector<int>& ncontr,
                 const std::vector<int>& poff, const double* ex, const double* cc, double qcut, double ecut,
                 bool sp_screen, HostPairs& out, bool key_order = false, bool s_on_b = false);
// general-job density staging / shell density and result assembly (oqpg_response.cu)
int gen_densities(oqpg_ctx* c, BuildBufs& B, const GenJob& g, cudaStream_t st);
int gen_finalize(oqpg_ctx* c, BuildBufs& B, const GenJob& g, cudaStream_t st);
bool split_on(const oqpg_ctx* c);
bool df_on(const oqpg_ctx* c);
int ctx_build(oqpg_ctx* c, const Job& job, cudaStream_t st);
// petite list (oqpg_petite.cu): whether it applies to a job, the density
// invariance check (before the lists) and the symmetrisation of the skeleton
// Fock matrix (in place of the plain finalize)
bool petite_on(const oqpg_ctx* c, const Job& job);
int petite_check(oqpg_ctx* c, BuildBufs& B, const Job& job, cudaStream_t st);
int petite_finalize(oqpg_ctx* c, BuildBufs& B, const Job& job, double ck, cudaStream_t st);
int ensure_att(oqpg_ctx* c, double mu);
// shell families (oqpg_family.cu): the family tables at a cutoff (after the
// Schwarz bounds), and whether a job's build lists family quartets
int family_tables(oqpg_ctx* c, double cutoff);
bool fam_on(const oqpg_ctx* c, const Job& job);

// Layout of an MRSF-type operand: component m of vector v, element (r, c) at
// m sm + v sv + r rs + c cs.
struct MrsfLayout {
  long long rs, cs, sm, sv;
};
void mrsf_job_layout(const oqpg_ctx* c, const double* in, double* out, int nvec, int nmat, double se, double sc,
                     const MrsfLayout& L, bool neg_lead, GenJob& g);
// The process-global context of the routec_* seam (null before routec_fock_init)
// and the end of the MRSF sigma session bound to it.
oqpg_ctx* routec_context();
void sig_release();
cudaError_t launch_grad_a(int c, const GradArgs& g, bool f32, int nsm, cudaStream_t st);
cudaError_t launch_grad_b(int c, const GradArgs& g, bool f32, int nsm, cudaStream_t st);
cudaError_t launch_grad_f(int c, const GradArgs& g, int nsm, cudaStream_t st);  // classes with f, FP64


// Per-build device buffers of one build pipeline (a context has one for its
// direct builds and one owned by its captured graph).
struct BuildBufs {
  DevBuf dj, dk, djf, dkf, djdf, dkdf, gj, gk, dsh, dshf, dmax, counts, primc, hist, cursor, work, ranges, caps,
      split, flag, gtab, sym, fsk;
  DevBuf lists[NLIST], slists[NLIST], bins[NLIST];
  unsigned long long cap[NLIST] = {0};
  unsigned char team[NLIST] = {0};     // list runs the warp-per-quartet kernels (set with the sizes)
  bool sized = false;
  bool fam = false;                    // the last build issued listed family quartets
  // pinned readback: [0] flag, [1, 1+NLIST) counts, then NLIST primitive
  // counts, then the member quartets of the family lists (NCLASS FP64, NCLASS FP32)
  unsigned long long* h_rb = nullptr;
  void release() {
    DevBuf* b[] = {&dj, &dk, &djf, &dkf, &djdf, &dkdf, &gj, &gk, &dsh, &dshf, &dmax, &counts, &primc, &hist,
                   &cursor, &work, &ranges, &caps, &split, &flag, &gtab, &sym, &fsk};
    for (DevBuf* x : b) x->release();
    for (auto& x : lists) x.release();
    for (auto& x : slists) x.release();
    for (auto& x : bins) x.release();
    if (h_rb) cudaFreeHost(h_rb);
    h_rb = nullptr;
    sized = false;
    for (auto& x : cap) x = 0;
    for (auto& x : team) x = 0;
  }
};

}  // namespace oqpg

// Per-class launch parameters picked by the autotuner.
struct oqpg_tuning {
  int split_log2[oqpg::NCLASS];  // quartets with >= 2^k primitive quartets run primitive-parallel (-1: 8, 4 warp per quartet)
  int family[oqpg::NCLASS];      // classes with both kernel families: 0 by list size, 1 thread, 2 warp per quartet
  int chunk[oqpg::NCLASS];       // small classes: quartets a warp takes per grab (multiple of 32)
  int ctas_per_sm[oqpg::NCLASS]; // grid cap per SM (0: as many as fit)
};

struct oqpg_ctx {
  int dev = 0, nsm = 152;
  cudaStream_t stream = nullptr;
  // nbf: AO rows of the whole batch (sum over molecules); stride: largest nbf
  int nshell = 0, nbf = 0, natom = 0, npair = 0, nmol = 1, stride = 0;
  long long ntri = 0, dsh_elems = 0;  // packed elements per density, shell-density elements (whole batch)
  bool pure = false;
  bool has_f = false;   // an f shell is registered
  double tau = 1e-10;      // run-time cutoff of the Fock-type builds (oqpg_set_cutoff)
  double tau_built = 1e-10;  // cutoff the Fock pair tables were built at (tau >= tau_built)
  std::vector<oqpg::PairDev> h_fpairs;  // those tables' shell pairs with their full primitive counts
  std::vector<double> h_fkey;           // and the screening key of every primitive pair
  std::vector<oqpg::ShellDev> shells;
  std::vector<int> aoff, naos;
  std::vector<oqpg::MolDev> mols;
  std::vector<double> schwarz_pair;   // per pair (canonical index within each molecule, molecules in order)
  // the registered basis (host copies; the gradient builds its own pair tables from them)
  std::vector<int> h_am, h_ncontr, h_poff, shell_atom;
  std::vector<double> h_ex, h_cc;
  oqpg_tuning tune;
  // petite list: nops >= 2 symmetry operations (abelian: signed AO permutations)
  int sym_nops = 0;
  oqpg::DevBuf d_sym_map, d_sym_inv, d_sym_sgn;   // shell images; AO preimages and their signs
  // shell families (oqpg_family.cu): on by default; tables at the current cutoff
  bool fam_enabled = true;
  int nfpair = 0, nfam_multi = 0;   // family pairs; those with more than one member
  oqpg::DevBuf d_fpairs, d_fmem, d_fprims, d_fprimsf, d_fprimsdf, d_fcoef, d_fcoefdf, d_fpair_mol, d_fpair_type, d_fq, d_fsorted_idx, d_fsorted_q,
      d_fmol0, d_fmoln, d_pair_fam_multi, d_fmsorted_idx, d_fmsorted_q, d_fmmol0, d_fmmoln;
  // precision split: 0 = every quartet in FP64, 1 = bound < tau_f32 in FP32
  int precision_mode = 0;
  double tau_f32 = 0.0;
  // device tables
  oqpg::DevBuf d_shells, d_pairs, d_prims, d_primsf, d_primsdf, d_pair_ij, d_pair_type, d_q, d_qf, d_aoff, d_naos, d_mols,
      d_pair_mol, d_row_mol;
  oqpg::DevBuf d_sorted_idx, d_sorted_q;
  // screening tables of the erf-attenuated operator (CAM pass 2) for att_mu
  double att_mu = 0.0;
  std::vector<double> schwarz_pair_att;
  oqpg::DevBuf d_q_att, d_qf_att, d_sorted_idx_att, d_sorted_q_att;
  // per-build buffers: direct builds, and the captured graph's own set
  oqpg::BuildBufs hb, gb;
  oqpg::DevBuf d_dp, d_f, d_fold;     // device copies of host-buffer builds
  unsigned long long counts[oqpg::NLIST] = {0};
  // pinned staging
  double* h_in = nullptr;
  double* h_out = nullptr;
  size_t h_bytes = 0;
  // captured device-driven build (graph replay)
  cudaGraphExec_t gexec = nullptr;
  cudaStream_t gstream = nullptr;
  int g_nfocks = 0, g_mode = -1;
  double g_se = 0, g_sc = 0, g_tau32 = 0, g_tau = 0;
  oqpg::DevBuf d_gin, d_gout;        // the graph's packed input / output
  int graph_replays = 0, graph_captures = 0, g_nlaunch = 0;
  // two-electron gradient: pair tables with the gradient cutoffs (built on first use)
  bool grad_ready = false;
  int ncart = 0;
  std::vector<int> coff;
  oqpg::DevBuf d_gpairs, d_gprims, d_galpha, d_gprimsf, d_galphaf, d_coff, d_atom, d_gmat, d_gmatf, d_dshg,
      d_gcounts, d_gwork, d_de, d_gcnt;
  oqpg::DevBuf d_glists[oqpg::NLIST_SHELL];   // FP64 lists, then the FP32 lists of the precision split
  unsigned long long gcaps[oqpg::NLIST_SHELL] = {0};
  oqpg::DevBuf d_gslists[oqpg::NLIST_SHELL];  // the lane classes' lists sorted by primitive-pair product
  unsigned long long gscaps[oqpg::NLIST_SHELL] = {0};
  oqpg::DevBuf d_gbins, d_ghist, d_gcur;
  double grad_stats[5] = {0, 0, 0, 0, 0};  // quartets listed, evaluated, primitive quartets, ms, FP32 listed
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  cudaEvent_t evc[oqpg::NCLASS][3] = {};   // class start, after its FP64 launches, end
  double last_stats[10 + 4 * oqpg::NCLASS] = {0};
};
