// Shared device/host helpers for the microLC GB300 library.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdio>
#include <stdexcept>
#include <string>

#include "microlc_gb300.h"

namespace mlc {

// Error carried from the depths of the library to the C-ABI boundary, where it
// becomes a status code and the context's last-error text.
struct Error : public std::runtime_error {
  int code;
  Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

#define MLC_CUDA(call)                                                                         \
  do {                                                                                         \
    cudaError_t e_ = (call);                                                                   \
    if (e_ != cudaSuccess)                                                                     \
      throw ::mlc::Error(e_ == cudaErrorMemoryAllocation ? MLC_ERR_OOM : MLC_ERR_CUDA,         \
                         std::string(#call) + ": " + cudaGetErrorString(e_) + " at " +         \
                             __FILE__ + ":" + std::to_string(__LINE__));                       \
  } while (0)

#define MLC_CHECK_LAUNCH() MLC_CUDA(cudaGetLastError())

#define MLC_REQUIRE(cond, code, msg)                   \
  do {                                                 \
    if (!(cond)) throw ::mlc::Error((code), (msg));    \
  } while (0)

template <typename T>
struct alignas(2 * sizeof(T)) C2 {
  T x, y;
};

// Float-float number: hi + lo, about 48 significant bits.  GB300 issues FP32 about sixty
// times faster than FP64, so FFTs run several times faster in it than in FP64 at about
// 1e-14 relative accuracy.  Every step uses explicitly rounded intrinsics (no contraction or
// reassociation can break the error-free transforms).  The sum is the two-sum of the high
// parts plus the low parts (8 FP32 operations), the product the FMA two-product plus the
// cross terms (4 operations).  Neither renormalises its result: the pair stays an exact
// two-term representation, |lo| grows to at most a few ulp(hi) over a chain of butterflies,
// and the error of every operation stays below a few 2^-47 of its operands' magnitude --
// the bound the FFT's norm-wise error analysis needs.  ff_norm restores |lo| <= ulp(hi)/2
// where a caller needs hi alone (divisions, values stored between passes).
struct ff {
  float hi, lo;
  ff() = default;
  __host__ __device__ constexpr ff(float h, float l) : hi(h), lo(l) {}
  __host__ __device__ constexpr ff(double d) : hi((float)d), lo((float)(d - (double)(float)d)) {}
  __host__ __device__ constexpr ff(int i) : ff((double)i) {}
};

__device__ __forceinline__ ff ff_renorm(float s, float e) {
  const float h = __fadd_rn(s, e);
  return ff(h, __fsub_rn(e, __fsub_rn(h, s)));
}
__device__ __forceinline__ ff ff_norm(ff a) { return ff_renorm(a.hi, a.lo); }
__device__ __forceinline__ ff operator+(ff a, ff b) {
  const float s = __fadd_rn(a.hi, b.hi);
  const float bb = __fsub_rn(s, a.hi);
  const float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(b.hi, bb));
  return ff(s, __fadd_rn(e, __fadd_rn(a.lo, b.lo)));
}
__device__ __forceinline__ ff operator-(ff a) { return ff(-a.hi, -a.lo); }
__device__ __forceinline__ ff operator-(ff a, ff b) { return a + (-b); }
__device__ __forceinline__ ff operator*(ff a, ff b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return ff(p, e);
}
__device__ __forceinline__ ff& operator+=(ff& a, ff b) { return a = a + b; }

// x times a power of two s: exact (barring underflow), two FP32 products for float-float.
template <typename T>
__device__ __forceinline__ T scale2(T x, float s) {
  return x * (T)s;
}
__device__ __forceinline__ ff scale2(ff x, float s) { return ff(__fmul_rn(x.hi, s), __fmul_rn(x.lo, s)); }
__device__ __forceinline__ double ff_to_double(ff a) { return __dadd_rn((double)a.hi, (double)a.lo); }

// a / b to float-float accuracy: the FP32 quotient of the normalised operands, then one
// correction from the float-float residual.
__device__ __forceinline__ ff ff_div(ff a, ff b) {
  a = ff_norm(a);
  b = ff_norm(b);
  const float q1 = __fdiv_rn(a.hi, b.hi);
  const ff r = ff_norm(a - ff(q1, 0.f) * b);
  return ff_renorm(q1, __fdiv_rn(r.hi, b.hi));
}

// Values stored between the passes of a forward transform are renormalised (3 operations per
// value) so that the low parts cannot keep growing from pass to pass; the inverse column
// passes (P1, P2) store theirs as they are, since only the last row pass follows them and it
// rounds every pixel from both parts.  FP32 and FP64 values pass unchanged.
template <typename T>
__device__ __forceinline__ T fin(T v) { return v; }
__device__ __forceinline__ ff fin(ff v) { return ff_norm(v); }

// log10 of an FP64 value in float-float arithmetic (our own evaluation, from the series
// log m = 2 atanh(s) = 2 (s + s^3/3 + s^5/5 + ...), s = (m - 1)/(m + 1)): x = 2^e m with m
// in [sqrt(1/2), sqrt(2)), so |s| <= 0.172 and eleven terms reach 2^-48; m is split into
// its high 24 and low 29 significand bits with integer operations; log10 x =
// (e ln 2 + log m) / ln 10.  About 1e-14 relative (FP64 magnitudes within 1e-13), at a
// few FP64 operations where the FP64 library call needs a few dozen (GB300 runs FP64 at a
// small fraction of its FP32 rate).  Zero, negative, subnormal, infinite and NaN inputs
// take the library's log10.
__device__ __forceinline__ double log10_f32x2(double x) {
  if (!(x >= 2.2250738585072014e-308) || !(x <= 1.7976931348623157e308)) return log10(x);
  unsigned long long bits = (unsigned long long)__double_as_longlong(x);
  int e = (int)(bits >> 52) - 1023;
  unsigned long long mb = (bits & 0x000FFFFFFFFFFFFFull) | 0x3FF0000000000000ull;  // m in [1, 2)
  if (mb > 0x3FF6A09E667F3BCDull) {                                               // m > sqrt(2): m / 2
    mb -= 0x0010000000000000ull;
    e += 1;
  }
  const int em = (int)(mb >> 52) - 1023;  // -1 or 0
  const unsigned long long mant = mb & 0x000FFFFFFFFFFFFFull;
  const float mh = __int_as_float(((em + 127) << 23) | (int)(mant >> 29));           // top 24 bits, exact
  const float ml = (float)(unsigned)(mant & 0x1FFFFFFFull) * (em ? 0x1p-53f : 0x1p-52f);  // the rest
  const ff m(mh, ml);
  const ff one(1.0f, 0.0f);
  const ff s = ff_div(m - one, m + one);
  const ff z = s * s;
  ff p(1.0 / 23.0);
  p = ff(1.0 / 21.0) + z * p;
  p = ff(1.0 / 19.0) + z * p;
  p = ff(1.0 / 17.0) + z * p;
  p = ff(1.0 / 15.0) + z * p;
  p = ff(1.0 / 13.0) + z * p;
  p = ff(1.0 / 11.0) + z * p;
  p = ff(1.0 / 9.0) + z * p;
  p = ff(1.0 / 7.0) + z * p;
  p = ff(1.0 / 5.0) + z * p;
  p = ff(1.0 / 3.0) + z * p;
  const ff logm = (s + s * (z * p)) * ff(2.0f, 0.0f);
  const ff ln = ff((float)e, 0.0f) * ff(0.69314718055994530942) + logm;
  const ff r = ln * ff(0.43429448190325182765);
  return __dadd_rn((double)r.hi, (double)r.lo);
}

// The element type a real transform writes by default: FP32 and FP64 transforms their own,
// float-float transforms FP64 (FP64 maps); FP32 maps with float-float transforms instantiate
// the inverse row passes with float output instead.
template <typename T>
struct RealOut {
  using type = T;
};
template <>
struct RealOut<ff> {
  using type = double;
};
// One transform value rounded to the output element type.
template <typename TO>
__device__ __forceinline__ TO out_cvt(float v) { return (TO)v; }
template <typename TO>
__device__ __forceinline__ TO out_cvt(double v) { return (TO)v; }
template <typename TO>
__device__ __forceinline__ TO out_cvt(ff v);
template <>
__device__ __forceinline__ double out_cvt<double>(ff v) { return ff_to_double(v); }
template <>
__device__ __forceinline__ float out_cvt<float>(ff v) { return __fadd_rn(v.hi, v.lo); }

// read-only (non-coherent) load of a complex value
__device__ __forceinline__ C2<float> ldc(const C2<float>* p) {
  const float2 v = __ldg(reinterpret_cast<const float2*>(p));
  return C2<float>{v.x, v.y};
}
__device__ __forceinline__ C2<double> ldc(const C2<double>* p) {
  const double2 v = __ldg(reinterpret_cast<const double2*>(p));
  return C2<double>{v.x, v.y};
}
__device__ __forceinline__ C2<ff> ldc(const C2<ff>* p) {
  const float4 v = __ldg(reinterpret_cast<const float4*>(p));
  return C2<ff>{ff(v.x, v.y), ff(v.z, v.w)};
}

template <typename T>
__host__ __device__ __forceinline__ C2<T> cmul(C2<T> a, C2<T> b) {
  return C2<T>{a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x};
}
// a * conj(b)
template <typename T>
__host__ __device__ __forceinline__ C2<T> cmulc(C2<T> a, C2<T> b) {
  return C2<T>{a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y};
}
template <typename T>
__host__ __device__ __forceinline__ C2<T> cadd(C2<T> a, C2<T> b) {
  return C2<T>{a.x + b.x, a.y + b.y};
}
template <typename T>
__host__ __device__ __forceinline__ C2<T> csub(C2<T> a, C2<T> b) {
  return C2<T>{a.x - b.x, a.y - b.y};
}
template <typename T>
__host__ __device__ __forceinline__ C2<T> cscale(C2<T> a, T s) {
  return C2<T>{a.x * s, a.y * s};
}
template <typename T>
__host__ __device__ __forceinline__ C2<T> cconj(C2<T> a) {
  return C2<T>{a.x, -a.y};
}
template <typename T>
__device__ __forceinline__ C2<T> cfin(C2<T> a) {
  return C2<T>{fin(a.x), fin(a.y)};
}
// multiply by -i (forward) or +i (inverse)
template <typename T, bool INV>
__host__ __device__ __forceinline__ C2<T> mul_mi(C2<T> a) {
  return INV ? C2<T>{-a.y, a.x} : C2<T>{a.y, -a.x};
}

inline int ceil_div(long a, long b) { return (int)((a + b - 1) / b); }
inline long round_up(long a, long b) { return ((a + b - 1) / b) * b; }

}  // namespace mlc
