// Launch helpers shared by the per-group translation units.
#pragma once
#include "oqpg_classes.h"
#include "oqpg_eri.cuh"

namespace oqpg {

// Persistent launch: as many 128-thread CTAs as fit on the device at once
// (or a.ctas_per_sm per SM; never more than a.nquartets needs); the kernels
// pull work from a.work.
template <typename Kern>
cudaError_t launch_persistent(Kern kern, size_t smem, long long per_block_items, const BuildArgs& a, int nsm,
                              cudaStream_t st, int threads = 128) {
  if (a.nquartets <= 0) return cudaSuccess;
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  int per_sm = 1;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem);
  if (a.ctas_per_sm > 0 && a.ctas_per_sm < per_sm) per_sm = a.ctas_per_sm;
  if (per_sm < 1) per_sm = 1;
  long long blocks = (a.nquartets + per_block_items - 1) / per_block_items;
  const long long cap = (long long)nsm * per_sm;
  if (blocks > cap) blocks = cap;
  kern<<<(unsigned)blocks, threads, smem, st>>>(a);
  return cudaGetLastError();
}

// Warps per CTA of a warp-per-quartet kernel: 4 unless the per-warp shared
// memory of the class (the largest f classes) leaves room for fewer.
template <int LA, int LB, int LC, int LD, bool PURE, typename T>
constexpr int team_warps() {
  constexpr size_t per_warp = sizeof(T) * TeamSmem<LA, LB, LC, LD, PURE>::PER_WARP;
  constexpr size_t budget = 220 * 1024 - sizeof(int) * Cls<LA, LB, LC, LD>::NE;  // s_offs is static
  return per_warp * 4 <= budget ? 4 : (per_warp * 2 <= budget ? 2 : 1);
}

// The kernel family a launch uses: a class with both runs warp per quartet
// when a.team is set (the host decides per list), thread per quartet otherwise.
template <int LA, int LB, int LC, int LD>
__host__ __device__ constexpr bool only_team() { return !has_small(LA, LB, LC, LD); }

template <int LA, int LB, int LC, int LD, bool PURE, typename T>
cudaError_t launch_team(int kind, const BuildArgs& a, int nsm, cudaStream_t st) {
  if constexpr (has_team(LA, LB, LC, LD)) {
    constexpr int W = team_warps<LA, LB, LC, LD, PURE, T>();
    const size_t smem = sizeof(T) * W * TeamSmem<LA, LB, LC, LD, PURE>::PER_WARP;
    if (kind == MODE_PRIM) {
      if constexpr (prim_parallel(LA, LB, LC, LD))
        return launch_persistent(k_prim_team<LA, LB, LC, LD, PURE, T>, smem, W, a, nsm, st, 32 * W);
      else
        return cudaErrorInvalidValue;
    }
    return launch_persistent(k_team<LA, LB, LC, LD, PURE, false, T>, smem, W, a, nsm, st, 32 * W);
  } else {
    return cudaErrorInvalidValue;
  }
}

// The FP64 thread-per-quartet (pp|pp) kernel (81 block elements beside the
// 2D tables: 255 registers and a 368-byte stack frame) runs one CTA of four
// warps per SM unless a grid cap is tuned.  Measured against two CTAs per SM
// (its register limit): (H2O)32 cc-pVDZ 10.1 -> 6.9 ms, (H2O)16 6-31G(d)
// 0.48 -> 0.42 ms.  The same cap for the other thread-per-quartet kernels
// with a stack frame was slower on C40H82 6-31G(d): (sp|sd) 19.0 -> 21.9 ms,
// (sd|pd) 8.7 -> 9.5 ms, (sp|dd) 4.4 -> 4.8 ms.
template <int LA, int LB, int LC, int LD, typename T>
constexpr bool small_one_cta() {
  return LA == 1 && LB == 1 && LC == 1 && LD == 1 && std::is_same<T, double>::value;
}

template <int LA, int LB, int LC, int LD, bool PURE, typename T>
cudaError_t launch_fock(int kind, const BuildArgs& a, int nsm, cudaStream_t st) {
  if constexpr (only_team<LA, LB, LC, LD>()) {
    return launch_team<LA, LB, LC, LD, PURE, T>(kind, a, nsm, st);
  } else {
    if constexpr (has_team(LA, LB, LC, LD)) {
      if (a.team) return launch_team<LA, LB, LC, LD, PURE, T>(kind, a, nsm, st);
    }
    if (kind == MODE_PRIM) return launch_persistent(k_prim<LA, LB, LC, LD, PURE, T>, 0, 4, a, nsm, st);
    if (small_one_cta<LA, LB, LC, LD, T>() && a.ctas_per_sm == 0) {
      BuildArgs b = a;
      b.ctas_per_sm = 1;
      return launch_persistent(k_small<LA, LB, LC, LD, PURE, false, T>, 0, 128, b, nsm, st);
    }
    return launch_persistent(k_small<LA, LB, LC, LD, PURE, false, T>, 0, 128, a, nsm, st);
  }
}

// Schwarz bounds of the diagonal quartets: thread per quartet where the class
// has it.
template <int LA, int LB, int LC, int LD, bool PURE>
cudaError_t launch_schwarz(const BuildArgs& a, int nsm, cudaStream_t st) {
  if constexpr (LA == LC && LB == LD) {
    if constexpr (only_team<LA, LB, LC, LD>()) {
      constexpr int W = team_warps<LA, LB, LC, LD, PURE, double>();
      const size_t smem = sizeof(double) * W * TeamSmem<LA, LB, LC, LD, PURE>::PER_WARP;
      return launch_persistent(k_team<LA, LB, LC, LD, PURE, true, double>, smem, W, a, nsm, st, 32 * W);
    } else {
      return launch_persistent(k_small<LA, LB, LC, LD, PURE, true, double>, 0, 128, a, nsm, st);
    }
  } else {
    return cudaErrorInvalidValue;
  }
}

// mode: MODE_FOCK, MODE_SCHWARZ (diagonal classes only), MODE_PRIM (the
// heavily contracted head of a sorted list), each optionally with MODE_F32
// (FP32 quartets of the precision-split build; not Schwarz).
template <int LA, int LB, int LC, int LD, bool PURE>
cudaError_t launch_df(int kind, const BuildArgs& a, int nsm, cudaStream_t st) {
  if constexpr (only_team<LA, LB, LC, LD>()) {
    return launch_fock<LA, LB, LC, LD, PURE, dfl>(kind, a, nsm, st);
  } else {
    if constexpr (has_team(LA, LB, LC, LD)) {
      if (a.team) return launch_team<LA, LB, LC, LD, PURE, dfl>(kind, a, nsm, st);
    }
    if (kind == MODE_PRIM) return launch_persistent(k_prim_df<LA, LB, LC, LD, PURE>, 0, 4, a, nsm, st);
    return launch_persistent(k_small_df<LA, LB, LC, LD, PURE>, 0, 128, a, nsm, st);
  }
}

template <int LA, int LB, int LC, int LD>
cudaError_t launch_cls(bool pure, int mode, const BuildArgs& a, int nsm, cudaStream_t st) {
  if constexpr (LA == 3 || LB == 3 || LC == 3 || LD == 3) {
    // f classes: FP64 kernels only (never on the FP32 lists; FP64 in the df modes)
    if (mode & MODE_F32) return cudaErrorInvalidValue;
    const int kind = mode & ~MODE_DF;
    if (kind == MODE_SCHWARZ)
      return pure ? launch_schwarz<LA, LB, LC, LD, true>(a, nsm, st) : launch_schwarz<LA, LB, LC, LD, false>(a, nsm, st);
    return pure ? launch_fock<LA, LB, LC, LD, true, double>(kind, a, nsm, st)
                : launch_fock<LA, LB, LC, LD, false, double>(kind, a, nsm, st);
  }
  const bool f32 = (mode & MODE_F32) != 0;
  if (mode & MODE_DF) {
    const int kind = mode & ~(MODE_DF | MODE_F32);
    return pure ? launch_df<LA, LB, LC, LD, true>(kind, a, nsm, st) : launch_df<LA, LB, LC, LD, false>(kind, a, nsm, st);
  }
  const int kind = mode & ~MODE_F32;
  if (kind == MODE_SCHWARZ) {
    if (f32) return cudaErrorInvalidValue;
    return pure ? launch_schwarz<LA, LB, LC, LD, true>(a, nsm, st) : launch_schwarz<LA, LB, LC, LD, false>(a, nsm, st);
  }
  if (f32)
    return pure ? launch_fock<LA, LB, LC, LD, true, float>(kind, a, nsm, st)
                : launch_fock<LA, LB, LC, LD, false, float>(kind, a, nsm, st);
  return pure ? launch_fock<LA, LB, LC, LD, true, double>(kind, a, nsm, st)
              : launch_fock<LA, LB, LC, LD, false, double>(kind, a, nsm, st);
}

}  // namespace oqpg
