// Launch helpers shared by the per-group translation units.
#pragma once
#include "oqpg_classes.h"
#include "oqpg_eri.cuh"

namespace oqpg {

// Persistent launch: as many 128-thread CTAs as fit on the device at once
// (never more than the work needs); the kernels pull work from a.work.
template <typename Kern>
cudaError_t launch_persistent(Kern kern, size_t smem, long long per_block_items, const BuildArgs& a, int nsm,
                              cudaStream_t st) {
  if (a.nquartets <= 0) return cudaSuccess;
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  int per_sm = 1;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 128, smem);
  if (per_sm < 1) per_sm = 1;
  long long blocks = (a.nquartets + per_block_items - 1) / per_block_items;
  const long long cap = (long long)nsm * per_sm;
  if (blocks > cap) blocks = cap;
  kern<<<(unsigned)blocks, 128, smem, st>>>(a);
  return cudaGetLastError();
}

template <int LA, int LB, int LC, int LD, bool PURE, bool SCH>
cudaError_t launch_small(const BuildArgs& a, int nsm, cudaStream_t st) {
  return launch_persistent(k_small<LA, LB, LC, LD, PURE, SCH>, 0, 128, a, nsm, st);
}

template <int LA, int LB, int LC, int LD, bool PURE, bool SCH>
cudaError_t launch_team(const BuildArgs& a, int nsm, cudaStream_t st) {
  const size_t smem = sizeof(double) * 4 * TeamSmem<LA, LB, LC, LD, PURE>::PER_WARP;
  return launch_persistent(k_team<LA, LB, LC, LD, PURE, SCH>, smem, 4, a, nsm, st);
}

// Classes with more than 27 Cartesian elements run one warp per quartet.
template <int LA, int LB, int LC, int LD>
constexpr bool is_team() { return Cls<LA, LB, LC, LD>::NE > 27; }

// mode: MODE_FOCK, MODE_SCHWARZ (diagonal classes only), MODE_PRIM (small
// classes only: the heavily contracted head of a sorted list).
template <int LA, int LB, int LC, int LD>
cudaError_t launch_cls(bool pure, int mode, const BuildArgs& a, int nsm, cudaStream_t st) {
  constexpr bool DIAG = (LA == LC && LB == LD);
  const bool sch = mode == MODE_SCHWARZ;
  if (sch && !DIAG) return cudaErrorInvalidValue;
  if (mode == MODE_PRIM) {
    if constexpr (is_team<LA, LB, LC, LD>()) {
      return cudaErrorInvalidValue;
    } else {
      return pure ? launch_persistent(k_prim<LA, LB, LC, LD, true>, 0, 4, a, nsm, st)
                  : launch_persistent(k_prim<LA, LB, LC, LD, false>, 0, 4, a, nsm, st);
    }
  }
  if constexpr (is_team<LA, LB, LC, LD>()) {
    if constexpr (DIAG) {
      if (sch) return pure ? launch_team<LA, LB, LC, LD, true, true>(a, nsm, st)
                           : launch_team<LA, LB, LC, LD, false, true>(a, nsm, st);
    }
    return pure ? launch_team<LA, LB, LC, LD, true, false>(a, nsm, st)
                : launch_team<LA, LB, LC, LD, false, false>(a, nsm, st);
  } else {
    if constexpr (DIAG) {
      if (sch) return pure ? launch_small<LA, LB, LC, LD, true, true>(a, nsm, st)
                           : launch_small<LA, LB, LC, LD, false, true>(a, nsm, st);
    }
    return pure ? launch_small<LA, LB, LC, LD, true, false>(a, nsm, st)
                : launch_small<LA, LB, LC, LD, false, false>(a, nsm, st);
  }
}

}  // namespace oqpg
