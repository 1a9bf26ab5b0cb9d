// dfloat.cuh -- double-float arithmetic on the FP32 pipes.
//
// A value is the unevaluated sum hi + lo of two floats with |lo| <= ulp(hi) / 2: about 48
// significant bits, near FP64's 53, with every operation on the FP32 units.  GB300 issues
// FP32 at about 64 times its FP64 rate, so an FP64-accurate transform runs faster in
// double-float than in native FP64.
//
// Algorithms (published error-free transformations):
//   two_sum   Knuth's TwoSum: s + e = a + b exactly, no ordering assumption;
//   fast2sum  Dekker's Fast2Sum: the same for |a| >= |b|;
//   product   the exact product a * b = p + e with e = fma(a, b, -p);
//   add       the "sloppy" double-double addition: TwoSum of the high parts, the low
//             parts added to the error term, renormalised (absolute error about
//             2^-46 (|a| + |b|): enough for transforms, whose error is measured in norm);
//   div       one Newton correction of the float quotient (Dekker 1971).
// T. J. Dekker, "A floating-point technique for extending the available precision",
// Numer. Math. 18 (1971); D. E. Knuth, TAOCP vol. 2, sec. 4.2.2.
// Every float operation is an explicitly rounded intrinsic, so the compiler cannot fuse
// or reorder the steps the error terms depend on.
#pragma once
#include <cuda_runtime.h>

struct dfl {
  float hi, lo;
  dfl() = default;
  __host__ __device__ constexpr dfl(float h, float l) : hi(h), lo(l) {}
  __host__ __device__ constexpr dfl(int i) : hi((float)i), lo(0.0f) {}
  __host__ __device__ constexpr dfl(float f) : hi(f), lo(0.0f) {}
  __host__ __device__ constexpr dfl(double d) : hi((float)d), lo((float)(d - (double)(float)d)) {}
  __host__ __device__ explicit operator double() const { return (double)hi + (double)lo; }
};

struct __align__(16) dfl2 {
  dfl x, y;
};

namespace dfops {
__device__ __forceinline__ dfl two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return dfl(s, e);
}
__device__ __forceinline__ dfl fast2sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return dfl(s, __fsub_rn(b, __fsub_rn(s, a)));
}
}  // namespace dfops

__device__ __forceinline__ dfl operator+(dfl a, dfl b) {
  const dfl s = dfops::two_sum(a.hi, b.hi);
  return dfops::fast2sum(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}
__device__ __forceinline__ dfl operator-(dfl a) { return dfl(-a.hi, -a.lo); }
__device__ __forceinline__ dfl operator-(dfl a, dfl b) { return a + (-b); }
__device__ __forceinline__ dfl operator*(dfl a, dfl b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return dfops::fast2sum(p, e);
}
__device__ __forceinline__ dfl operator/(dfl a, dfl b) {
  const float q1 = __fdiv_rn(a.hi, b.hi);
  const dfl r = a - dfl(q1) * b;
  return dfops::fast2sum(q1, __fdiv_rn(r.hi, b.hi));
}
__device__ __forceinline__ dfl& operator+=(dfl& a, dfl b) { return a = a + b; }
__device__ __forceinline__ dfl& operator-=(dfl& a, dfl b) { return a = a - b; }
__device__ __forceinline__ dfl& operator*=(dfl& a, dfl b) { return a = a * b; }

__device__ __forceinline__ dfl shfl_xor_val(dfl v, int m) {
  return dfl(__shfl_xor_sync(0xffffffffu, v.hi, m), __shfl_xor_sync(0xffffffffu, v.lo, m));
}
__device__ __forceinline__ float shfl_xor_val(float v, int m) { return __shfl_xor_sync(0xffffffffu, v, m); }
__device__ __forceinline__ double shfl_xor_val(double v, int m) { return __shfl_xor_sync(0xffffffffu, v, m); }

// field values in and out of the transform's arithmetic type
template <typename T, typename TIO>
__device__ __forceinline__ T from_io(TIO v) { return (T)v; }
template <>
__device__ __forceinline__ dfl from_io<dfl, double>(double v) {
  const float h = __double2float_rn(v);
  return dfl(h, __double2float_rn(v - (double)h));
}
template <typename TIO, typename T>
__device__ __forceinline__ TIO to_io(T v) { return (TIO)v; }
template <>
__device__ __forceinline__ double to_io<double, dfl>(dfl v) { return (double)v.hi + (double)v.lo; }
