// Double-word ("float-float") arithmetic for the FP64-accurate float32 step.
//
// GB300 issues about 2 FP64 fused multiply-adds per clock per SM against 128 FP32
// ones, so the float64 step is bound by its FP64 instructions. A double-word value
// x = hi + lo is the unevaluated sum of two float32 numbers (|lo| <= ulp(hi) / 2
// once normalised): 48 significand bits, unit roundoff u^2 = 2^-48 ~ 3.6e-15,
// the float32 exponent range. It occupies 8 bytes, like a double, so the state and
// coefficient arrays keep the float64 layout and traffic.
//
// Building blocks (all with round-to-nearest intrinsics, which are never
// contracted or reassociated by the compiler):
//   two_sum  (Knuth): s + e == a + b exactly, 6 operations;
//   two_prod (with FMA): p + e == a * b exactly, 2 operations.
// fma(x, y, c) is one step of the compensated dot product (Ogita, Rump and Oishi,
// "Accurate sum and dot product", SIAM J. Sci. Comput. 26(6), 2005, Algorithm
// Dot2) over double-word operands: the high parts are summed with two_sum, every
// rounding error and the cross terms x.hi*y.lo + x.lo*y.hi are gathered in the low
// word. The result is left unnormalised so that a chain of fma's costs 12
// operations per term; settle() normalises it (two_sum of the two words) at the
// end of a chain, before the value is stored or multiplied. The dropped term
// x.lo*y.lo and the float32 roundings of the low word give an error of a few u^2
// times the sum of the magnitudes of the terms, the same form as one float64 FMA
// chain (with u^2 in place of 2^-53).
//
// The other operators follow the double-word algorithms of Joldes, Muller and
// Popescu ("Tight and rigorous error bounds for basic building blocks of
// double-word arithmetic", ACM TOMS 44(2), 2017): product with FMA (DWTimesDW),
// sum with a final normalisation (SloppyDWPlusDW, normalised by two_sum), and a
// quotient refined by one Newton correction of the float32 quotient.
#pragma once

#include <cuda_runtime.h>

namespace fds {

// the float and double overloads stay visible next to the double-word one below
using ::fma;

struct __align__(8) dw {
  float hi, lo;
  dw() = default;
  __host__ __device__ constexpr dw(float h, float l) : hi(h), lo(l) {}
  __host__ __device__ explicit constexpr dw(int z) : hi((float)z), lo(0.0f) {}
  // split of a double: hi = fl32(x), lo = fl32(x - hi) (x - hi is exact in double)
  __device__ explicit dw(double x) {
    hi = __double2float_rn(x);
    lo = __double2float_rn(__dsub_rn(x, (double)hi));
  }
  __device__ explicit operator double() const { return __dadd_rn((double)hi, (double)lo); }
};

__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// normalised pair of a + b (exact)
__device__ __forceinline__ dw settle(const dw& x) {
  float s, e;
  two_sum(x.hi, x.lo, s, e);
  return dw(s, e);
}
template <typename T>
__device__ __forceinline__ T settle(const T& x) {
  return x;
}

__device__ __forceinline__ dw operator-(const dw& x) { return dw(-x.hi, -x.lo); }

// c + x*y, unnormalised (one compensated dot-product step)
__device__ __forceinline__ dw fma(const dw& x, const dw& y, const dw& c) {
  const float p = __fmul_rn(x.hi, y.hi);
  const float pe = __fmaf_rn(x.hi, y.hi, -p);
  float s, se;
  two_sum(c.hi, p, s, se);
  float lo = __fadd_rn(c.lo, __fadd_rn(se, pe));
  lo = __fmaf_rn(x.hi, y.lo, lo);
  lo = __fmaf_rn(x.lo, y.hi, lo);
  return dw(s, lo);
}

__device__ __forceinline__ dw operator*(const dw& x, const dw& y) {
  const float p = __fmul_rn(x.hi, y.hi);
  float e = __fmaf_rn(x.hi, y.hi, -p);
  e = __fmaf_rn(x.hi, y.lo, e);
  e = __fmaf_rn(x.lo, y.hi, e);
  const float s = __fadd_rn(p, e);  // Fast2Sum: |p| >= |e|
  return dw(s, __fsub_rn(e, __fsub_rn(s, p)));
}

__device__ __forceinline__ dw operator+(const dw& x, const dw& y) {
  float s, e;
  two_sum(x.hi, y.hi, s, e);
  e = __fadd_rn(e, __fadd_rn(x.lo, y.lo));
  return settle(dw(s, e));
}

__device__ __forceinline__ dw operator-(const dw& x, const dw& y) { return x + (-y); }

__device__ __forceinline__ dw operator/(const dw& x, const dw& y) {
  const float q1 = __fdiv_rn(x.hi, y.hi);
  const dw r = x - dw(q1, 0.0f) * y;  // remainder of the float32 quotient
  const float q2 = __fdiv_rn(r.hi, y.hi);
  return settle(dw(q1, q2));
}

// read-only global load of 4- or 8-byte values and of double words
template <typename T>
__device__ __forceinline__ T ldg_t(const T* p) {
  return __ldg(p);
}
template <>
__device__ __forceinline__ dw ldg_t<dw>(const dw* p) {
  const float2 v = __ldg(reinterpret_cast<const float2*>(p));
  return dw(v.x, v.y);
}

// Load from L2 (not L1): state written by other CTAs of a running kernel.
template <typename T>
__device__ __forceinline__ T ldcg_t(const T* p) {
  return __ldcg(p);
}
template <>
__device__ __forceinline__ dw ldcg_t<dw>(const dw* p) {
  const float2 v = __ldcg(reinterpret_cast<const float2*>(p));
  return dw(v.x, v.y);
}

}  // namespace fds
