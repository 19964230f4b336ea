// Double-float arithmetic for the "df" precision mode: a value is an
// unevaluated sum hi + lo of two FP32 numbers (about 44 significant bits), and
// every operation is a short sequence of FP32 instructions.  GB300 issues
// FP32 at 64x its FP64 rate, so an FMA built from ~15 FP32 instructions still
// costs about a quarter of one FP64 FMA.  Algorithms: Knuth's two-sum,
// Dekker's fast two-sum, the FMA-based exact product, and Newton steps for
// the reciprocal and reciprocal square root (one step from the FP32 hardware
// approximation doubles its ~23 bits).
#pragma once
#include <cuda_runtime.h>

namespace oqpg {

// the double-float fma and __ldg below must not hide the FP64 / FP32 ones
using ::fma;
using ::__ldg;

struct dfl {
  float hi, lo;
  __host__ __device__ constexpr dfl() : hi(0.f), lo(0.f) {}
  __host__ __device__ constexpr dfl(float h, float l) : hi(h), lo(l) {}
  // exact for the small integers and powers of two the kernels use as constants
  __host__ __device__ constexpr dfl(int v) : hi((float)v), lo(0.f) {}
  __host__ __device__ constexpr explicit dfl(double v) : hi((float)v), lo((float)(v - (double)(float)v)) {}
  __host__ __device__ explicit operator double() const { return (double)hi + (double)lo; }
};

__device__ __forceinline__ dfl df_two_sum(float a, float b) {
  const float s = a + b;
  const float bb = s - a;
  return dfl(s, (a - (s - bb)) + (b - bb));
}
__device__ __forceinline__ dfl df_fast_two_sum(float a, float b) {  // |a| >= |b|
  const float s = a + b;
  return dfl(s, b - (s - a));
}
__device__ __forceinline__ dfl operator+(dfl x, dfl y) {
  dfl s = df_two_sum(x.hi, y.hi);
  return df_fast_two_sum(s.hi, s.lo + (x.lo + y.lo));
}
__device__ __forceinline__ dfl operator-(dfl x) { return dfl(-x.hi, -x.lo); }
__device__ __forceinline__ dfl operator-(dfl x, dfl y) { return x + (-y); }
__device__ __forceinline__ dfl operator*(dfl x, dfl y) {
  const float p = x.hi * y.hi;
  float e = fmaf(x.hi, y.hi, -p);
  e = fmaf(x.hi, y.lo, fmaf(x.lo, y.hi, e));
  return df_fast_two_sum(p, e);
}
__device__ __forceinline__ dfl& operator+=(dfl& x, dfl y) { return x = x + y; }
__device__ __forceinline__ dfl& operator*=(dfl& x, dfl y) { return x = x * y; }
__device__ __forceinline__ dfl fma(dfl x, dfl y, dfl z) {
  const float p = x.hi * y.hi;
  float e = fmaf(x.hi, y.hi, -p);
  e = fmaf(x.hi, y.lo, fmaf(x.lo, y.hi, e));
  dfl s = df_two_sum(p, z.hi);
  return df_fast_two_sum(s.hi, s.lo + (e + z.lo));
}
__device__ __forceinline__ double df_to_double(dfl x) { return (double)x.hi + (double)x.lo; }

// 1/x and 1/sqrt(x) (x > 0): FP32 approximation, one Newton step in double-float
__device__ __forceinline__ dfl df_rcp(dfl x) {
  const float y0 = 1.0f / x.hi;
  // e = 1 - x y0 in double-float, then y = y0 + y0 e
  const dfl xy = x * dfl(y0, 0.f);
  const float e = (1.0f - xy.hi) - xy.lo;
  return df_fast_two_sum(y0, y0 * e);
}
__device__ __forceinline__ dfl df_rsqrt(dfl x) {
  const float y0 = rsqrtf(x.hi);
  const dfl xy = x * dfl(y0, 0.f);
  const dfl xyy = xy * dfl(y0, 0.f);
  const float e = (1.0f - xyy.hi) - xyy.lo;
  return df_fast_two_sum(y0, 0.5f * y0 * e);
}

// Primitive pair in double-float (80 bytes like PrimPair): p, 0.5/p, P, P - A,
// K/p, and the FP32 screening pair (K/p, p).
struct PrimPairDF {
  dfl p, hp, px, py, pz, ax, ay, az, sp;
  float spf, pf;
};

__device__ __forceinline__ dfl df_ld(const dfl* p) {
  const float2 v = __ldg(reinterpret_cast<const float2*>(p));
  return dfl(v.x, v.y);
}
__device__ __forceinline__ dfl __ldg(const dfl* p) { return df_ld(p); }

// element cutoff |v| < cut -> 0 on the leading word (cut > 0)
__device__ __forceinline__ dfl cut_elem(dfl v, dfl cut) {
  return (__float_as_int(v.hi) & 0x7fffffff) < __float_as_int(cut.hi) ? dfl() : v;
}

__device__ __forceinline__ double shfl_xor_t(double v, int off) { return __shfl_xor_sync(0xffffffffu, v, off); }
__device__ __forceinline__ float shfl_xor_t(float v, int off) { return __shfl_xor_sync(0xffffffffu, v, off); }
__device__ __forceinline__ dfl shfl_xor_t(dfl v, int off) {
  return dfl(__shfl_xor_sync(0xffffffffu, v.hi, off), __shfl_xor_sync(0xffffffffu, v.lo, off));
}

}  // namespace oqpg
