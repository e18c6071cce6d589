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

// read-only (non-coherent) load of a complex value
__device__ __forceinline__ C2<float> ldc(const C2<float>* p) {
  const float2 v = __ldg(reinterpret_cast<const float2*>(p));
  return C2<float>{v.x, v.y};
}
__device__ __forceinline__ C2<double> ldc(const C2<double>* p) {
  const double2 v = __ldg(reinterpret_cast<const double2*>(p));
  return C2<double>{v.x, v.y};
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
// multiply by -i (forward) or +i (inverse)
template <typename T, bool INV>
__host__ __device__ __forceinline__ C2<T> mul_mi(C2<T> a) {
  return INV ? C2<T>{-a.y, a.x} : C2<T>{a.y, -a.x};
}

inline int ceil_div(long a, long b) { return (int)((a + b - 1) / b); }
inline long round_up(long a, long b) { return ((a + b - 1) / b) * b; }

}  // namespace mlc
