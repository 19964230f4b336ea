// The 55 (la lb | lc ld) classes of s-f quartets in kernel orientation and
// the launchers of their kernels (one translation unit per group of classes).
#pragma once
#include <cuda_runtime.h>

#include "oqpg_common.cuh"

namespace oqpg {

// Pair types (la <= lb): the six s-d ones, then the four with an f shell.
constexpr int NPAIRTYPE = 10;  // ss sp sd pp pd dd | sf pf df ff
constexpr int NPAIRTYPE_SD = 6;
constexpr int NCLASS_SD = 21;  // classes of two s-d pair types
constexpr int NCLASS = 55;     // pair type of bra <= pair type of ket
constexpr int PAIR_L[NPAIRTYPE][2] = {{0, 0}, {0, 1}, {0, 2}, {1, 1}, {1, 2}, {2, 2},
                                      {0, 3}, {1, 3}, {2, 3}, {3, 3}};

__host__ __device__ inline int pair_type(int la, int lb) {  // la <= lb
  return lb == 3 ? 6 + la : (la == 0 ? lb : (la == 1 ? 2 + lb : 5));
}
// Classes of two s-d pair types keep the indices 0..20; a class with an f
// pair (ket type tk >= 6, bra type tb <= tk) follows at 21 + (tk(tk+1) - 42)/2 + tb.
__host__ __device__ inline int class_index(int tbra, int tket) {  // tbra <= tket
  if (tket < NPAIRTYPE_SD) return tbra * NPAIRTYPE_SD - tbra * (tbra - 1) / 2 + (tket - tbra);
  return NCLASS_SD + (tket * (tket + 1) - 42) / 2 + tbra;
}
// classes 21.. involve an f shell: FP64 kernels only
__host__ __device__ constexpr bool class_has_f(int c) { return c >= NCLASS_SD; }

struct ClassInfo {
  int l[4];
  int small;       // 1: has the thread-per-quartet kernels (k_small, k_prim)
  int team;        // 1: has the warp-per-quartet kernels (k_team, k_prim_team)
  int prim;        // 1: has the primitive-parallel kernel for its heavily contracted quartets
};

// Classes whose Cartesian block and one root's 2D tables fit in registers get a
// primitive-parallel kernel (lanes split the primitive quartets).
__host__ __device__ constexpr bool prim_parallel(int la, int lb, int lc, int ld) {
  return ncart(la) * ncart(lb) * ncart(lc) * ncart(ld) <= 27 ||
         ncart(la) * ncart(lb) * ncart(lc) * ncart(ld) + 3 * (la + 1) * (lb + 1) * (lc + 1) * (ld + 1) <= 100;
}
const ClassInfo& class_info(int c);
// Kernel families of a class.  Thread per quartet keeps the whole block in
// registers (up to 108 Cartesian elements, 27 with an f shell; beyond 54 with
// some spilling, cheap next to the FP64 work); warp per quartet shares one
// quartet among 32 lanes (above 27 elements).  A class with both (28-108
// elements, no f shell) picks per list at launch: thread per quartet needs
// enough quartets to fill the GPU.  Measured on (H2O)32 cc-pVDZ, thread per
// quartet ran (sp|pd) 2.3x, (sd|pd) 2.2x, (sp|dd) 1.8x, (pp|pp) 1.2x faster;
// on (H2O)16 6-31G(d), with ~1e4-1e5 quartets per list, warp per quartet ran
// (sp|pd) 1.5x, (sd|pp) 2.3x, (pp|pp) 5x faster.
__host__ __device__ constexpr bool has_small(int la, int lb, int lc, int ld) {
  return ncart(la) * ncart(lb) * ncart(lc) * ncart(ld) <= ((la == 3 || lb == 3 || lc == 3 || ld == 3) ? 27 : 108);
}
__host__ __device__ constexpr bool has_team(int la, int lb, int lc, int ld) {
  return ncart(la) * ncart(lb) * ncart(lc) * ncart(ld) > 27;
}
// Shell families (oqpg_common.cuh): the most member shell pairs a pair of
// type (la <= lb) can have (families are s shells, two at most), and the
// classes built as family quartets: members on some side, and a block of
// members x elements small enough for registers ((ss|ss), (ss|sp), (ss|sd),
// (ss|pp), (ss|pd), (sp|sp), (sp|sd), (sp|pp)).
__host__ __device__ constexpr int fam_members_max(int la, int lb) {
  return la == 0 ? (lb == 0 ? 4 : 2) : 1;
}
__host__ __device__ constexpr bool fam_class_l(int la, int lb, int lc, int ld) {
  return la <= 2 && lb <= 2 && lc <= 2 && ld <= 2 && fam_members_max(la, lb) * fam_members_max(lc, ld) > 1 &&
         ncart(la) * ncart(lb) * ncart(lc) * ncart(ld) * fam_members_max(la, lb) * fam_members_max(lc, ld) <= 72;
}
__host__ __device__ inline bool fam_class(int c) { return c <= 4 || (c >= 6 && c <= 8); }
constexpr bool fam_class_table_ok() {   // the list above is fam_class_l over the s-d classes
  for (int tb = 0; tb < NPAIRTYPE_SD; ++tb)
    for (int tk = tb; tk < NPAIRTYPE_SD; ++tk) {
      const int c = tb * NPAIRTYPE_SD - tb * (tb - 1) / 2 + (tk - tb);
      const bool listed = c <= 4 || (c >= 6 && c <= 8);
      if (listed != fam_class_l(PAIR_L[tb][0], PAIR_L[tb][1], PAIR_L[tk][0], PAIR_L[tk][1])) return false;
    }
  return true;
}
static_assert(fam_class_table_ok(), "family classes: 0-4 (ss|ss..pd), 6-8 (sp|sp), (sp|sd), (sp|pp)");
// The family classes in order (list slots of their family-quartet lists).
constexpr int NFAMCLS = 8;
__host__ __device__ inline int fam_slot(int c) { return c <= 4 ? c : c - 1; }
__host__ __device__ inline int fam_slot_class(int j) { return j <= 4 ? j : j + 1; }
// Family-pair types: the pair types of the family classes (ss, sp, sd, pp, pd).
__host__ __device__ inline bool fam_pair_type(int t) { return t <= 4; }
// kind: FAM_FP64, FAM_F32 (FP32 family quartets of the split) or FAM_DF
// (double-float, the df modes)
constexpr int FAM_FP64 = 0, FAM_F32 = 1, FAM_DF = 2;
cudaError_t launch_family(int c, bool pure, bool warp, int kind, const BuildArgs& a, int nsm, cudaStream_t st);
cudaError_t launch_family_df(int c, bool pure, bool warp, const BuildArgs& a, int nsm, cudaStream_t st);

// Thread per quartet by default from this many quartets per SM in a list
// (four waves of 128-thread CTAs at two CTAs per SM, the occupancy at 255
// registers per thread).
constexpr long long SMALL_MIN_PER_SM = 4 * 256;

// Kernel variants of a class.
constexpr int MODE_FOCK = 0;     // Fock build
constexpr int MODE_SCHWARZ = 1;  // Schwarz bounds of diagonal quartets
constexpr int MODE_PRIM = 2;     // Fock build, one warp per heavily contracted quartet, lanes split primitives
constexpr int MODE_F32 = 8;      // flag: FP32 quartets of the precision-split build
constexpr int MODE_DF = 16;      // flag: double-float kernels for the thread-per-quartet classes

// Launch the kernel of class c in the given mode.
cudaError_t launch_class(int c, bool pure, int mode, const BuildArgs& a, int nsm, cudaStream_t st);

// group launchers (defined in oqpg_cls_*.cu)
cudaError_t launch_group0(int c, bool pure, int mode, const BuildArgs& a, int nsm, cudaStream_t st);
cudaError_t launch_group1(int c, bool pure, int mode, const BuildArgs& a, int nsm, cudaStream_t st);
cudaError_t launch_group2(int c, bool pure, int mode, const BuildArgs& a, int nsm, cudaStream_t st);
cudaError_t launch_group3(int c, bool pure, int mode, const BuildArgs& a, int nsm, cudaStream_t st);
cudaError_t launch_group4(int c, bool pure, int mode, const BuildArgs& a, int nsm, cudaStream_t st);
cudaError_t launch_group5(int c, bool pure, int mode, const BuildArgs& a, int nsm, cudaStream_t st);
cudaError_t launch_group6(int c, bool pure, int mode, const BuildArgs& a, int nsm, cudaStream_t st);
cudaError_t launch_group7(int c, bool pure, int mode, const BuildArgs& a, int nsm, cudaStream_t st);
cudaError_t launch_group8(int c, bool pure, int mode, const BuildArgs& a, int nsm, cudaStream_t st);
cudaError_t launch_group9(int c, bool pure, int mode, const BuildArgs& a, int nsm, cudaStream_t st);
cudaError_t launch_group10(int c, bool pure, int mode, const BuildArgs& a, int nsm, cudaStream_t st);
cudaError_t launch_group11(int c, bool pure, int mode, const BuildArgs& a, int nsm, cudaStream_t st);
cudaError_t launch_group12(int c, bool pure, int mode, const BuildArgs& a, int nsm, cudaStream_t st);
cudaError_t launch_group13(int c, bool pure, int mode, const BuildArgs& a, int nsm, cudaStream_t st);
cudaError_t launch_group14(int c, bool pure, int mode, const BuildArgs& a, int nsm, cudaStream_t st);
cudaError_t launch_group15(int c, bool pure, int mode, const BuildArgs& a, int nsm, cudaStream_t st);
cudaError_t launch_group16(int c, bool pure, int mode, const BuildArgs& a, int nsm, cudaStream_t st);
cudaError_t launch_group17(int c, bool pure, int mode, const BuildArgs& a, int nsm, cudaStream_t st);
cudaError_t launch_group18(int c, bool pure, int mode, const BuildArgs& a, int nsm, cudaStream_t st);

}  // namespace oqpg
