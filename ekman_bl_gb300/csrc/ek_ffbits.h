// double <-> float conversions on the integer pipes.  GB300's FP64 pipe,
// which also executes the F2F conversions, is narrow (~1/64 of FP32), so
// kernels that compute in FP32 or float-float on FP64 fields must not
// convert through it.
//
//   d2f_bits(x)   RN(x) to float
//   f2d_bits(f)   f widened exactly to double
//
// Both equal the hardware conversion bit for bit in the float normal range
// and for infinities; values below it become zero, and a NaN stays a quiet
// NaN of the same sign.  Nothing falls back to the hardware conversion: a
// compiler may turn such a branch into a select and issue the conversion for
// every value.  (Splitting a double into a float-float pair, or joining one,
// in 64-bit integer arithmetic was measured to cost as much as the one FP64
// add it saves, so those stay FP64.)  The header compiles as plain C++ too,
// so the CPU tests can check it.
#pragma once

#include <cstdint>
#include <cstring>

#ifdef __CUDACC__
#define EK_HD __host__ __device__ __forceinline__
#else
#define EK_HD inline
#endif

namespace ek {

EK_HD uint64_t dbits(double x) {
#ifdef __CUDA_ARCH__
  return (uint64_t)__double_as_longlong(x);
#else
  uint64_t u;
  std::memcpy(&u, &x, 8);
  return u;
#endif
}
EK_HD double dfrom(uint64_t u) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)u);
#else
  double x;
  std::memcpy(&x, &u, 8);
  return x;
#endif
}
EK_HD uint32_t fbits(float x) {
#ifdef __CUDA_ARCH__
  return __float_as_uint(x);
#else
  uint32_t u;
  std::memcpy(&u, &x, 4);
  return u;
#endif
}
EK_HD float ffrom(uint32_t u) {
#ifdef __CUDA_ARCH__
  return __uint_as_float(u);
#else
  float x;
  std::memcpy(&x, &u, 4);
  return x;
#endif
}

EK_HD float d2f_bits(double x) {
  const uint64_t u = dbits(x);
  const uint32_t uh = (uint32_t)(u >> 32), ul = (uint32_t)u;
  const uint32_t sign = uh & 0x80000000u;
  const int e = (int)((uh >> 20) & 0x7ffu);
  if (e == 0x7ff) {  // infinity, or NaN (quiet, with the payload's top bits)
    const bool nan = ((uh & 0xfffffu) | ul) != 0u;
    return ffrom(sign | 0x7f800000u | (nan ? (0x400000u | ((uh & 0xfffffu) << 2) | (ul >> 30)) : 0u));
  }
  const int fe = e - 896;
  if (fe <= 0) return ffrom(sign);
  if (fe >= 0xff) return ffrom(sign | 0x7f800000u);
  const uint32_t mant = ((uh & 0xfffffu) << 3) | (ul >> 29);
  uint32_t r = sign | ((uint32_t)fe << 23) | mant;
  const uint32_t dropped = ul & 0x1fffffffu;
  if (dropped > 0x10000000u || (dropped == 0x10000000u && (mant & 1u))) r += 1u;
  return ffrom(r);
}

EK_HD double f2d_bits(float f) {
  const uint32_t u = fbits(f);
  const uint32_t sign = u & 0x80000000u;
  const uint32_t e = (u >> 23) & 0xffu;
  if (e == 0) return dfrom((uint64_t)sign << 32);
  const uint32_t mant = u & 0x7fffffu;
  const uint32_t de = (e == 0xff) ? 0x7ffu : e + 896u;  // infinity and NaN keep their class and payload
  return dfrom(((uint64_t)(sign | (de << 20) | (mant >> 3)) << 32) | ((uint64_t)(mant << 29)));
}

}  // namespace ek
