// Launch helpers shared by the per-group translation units.
#pragma once
#include "oqpg_classes.h"
#include "oqpg_eri.cuh"

namespace oqpg {

template <int LA, int LB, int LC, int LD, bool PURE, bool SCH>
cudaError_t launch_small(const BuildArgs& a, int nsm, cudaStream_t st) {
  if (a.nquartets <= 0) return cudaSuccess;
  long long blocks = (a.nquartets + 127) / 128;
  const long long cap = (long long)nsm * 16;
  if (blocks > cap) blocks = cap;
  k_small<LA, LB, LC, LD, PURE, SCH><<<(unsigned)blocks, 128, 0, st>>>(a);
  return cudaGetLastError();
}

template <int LA, int LB, int LC, int LD, bool PURE, bool SCH>
cudaError_t launch_team(const BuildArgs& a, int nsm, cudaStream_t st) {
  if (a.nquartets <= 0) return cudaSuccess;
  const size_t smem = sizeof(double) * 4 * TeamSmem<LA, LB, LC, LD, PURE>::PER_WARP;
  auto kern = k_team<LA, LB, LC, LD, PURE, SCH>;
  static bool attr_set = false;
  if (!attr_set) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    attr_set = true;
  }
  int per_sm = 1;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 128, smem);
  if (per_sm < 1) per_sm = 1;
  long long blocks = (a.nquartets + 3) / 4;
  const long long cap = (long long)nsm * per_sm * 4;
  if (blocks > cap) blocks = cap;
  kern<<<(unsigned)blocks, 128, smem, st>>>(a);
  return cudaGetLastError();
}

// Classes with more than 27 Cartesian elements run one warp per quartet.
template <int LA, int LB, int LC, int LD>
constexpr bool is_team() { return Cls<LA, LB, LC, LD>::NE > 27; }

template <int LA, int LB, int LC, int LD>
cudaError_t launch_cls(bool pure, bool sch, const BuildArgs& a, int nsm, cudaStream_t st) {
  constexpr bool DIAG = (LA == LC && LB == LD);
  if (sch && !DIAG) return cudaErrorInvalidValue;
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
