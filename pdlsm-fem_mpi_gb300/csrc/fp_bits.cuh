// Float <-> double conversions on the integer pipe, shared by the step
// kernels and the Krylov solves.
#pragma once

#include <cstdint>

namespace pdx {

// Conversions between float and double on the integer pipe.  GB300 issues
// FP64 arithmetic and FP64 conversions at 2 lanes per clock per SM (FP32
// FMA: 128; both measured on the GB300), so the mixed kernels keep them off
// the per-DOF update: only the FP64 accumulation
// u_{n+1} = (2 u_n - u_{n-1}) + dt^2 F / m runs on the FP64 pipe.  Both
// conversions give the bits of cvt.f64.f32 / cvt.rn.f32.f64; the rare inputs
// outside the plain normal range (float subnormals, infinities, NaN) take
// the hardware conversion.
__device__ __forceinline__ double f2d_bits(float f) {
  const uint32_t b = __float_as_uint(f);
  const uint32_t em = b & 0x7fffffffu;
  if (em == 0u) return __hiloint2double((int)(b & 0x80000000u), 0);
  if (em < 0x00800000u || em >= 0x7f800000u) return (double)f;
  // exponent bias 127 -> 1023 (+896 << 20 in the high word); 23 -> 52 mantissa bits
  const uint32_t hi = (b & 0x80000000u) | ((em >> 3) + (896u << 20));
  return __hiloint2double((int)hi, (int)(em << 29));
}

__device__ __forceinline__ float d2f_bits(double d) {
  const uint32_t hi = (uint32_t)__double2hiint(d), lo = (uint32_t)__double2loint(d);
  const uint32_t sgn = hi & 0x80000000u;
  const uint32_t e = (hi >> 20) & 0x7ffu;
  if (e == 0u && (hi & 0xfffffu) == 0u && lo == 0u) return __uint_as_float(sgn);
  if (e <= 896u || e >= 1151u) return (float)d;
  uint32_t r = ((e - 896u) << 23) | ((hi & 0xfffffu) << 3) | (lo >> 29);
  const uint32_t rest = lo & 0x1fffffffu;   // the 29 bits rounded away
  if (rest > 0x10000000u || (rest == 0x10000000u && (r & 1u))) r += 1u;   // nearest, ties to even
  return __uint_as_float(sgn | r);
}

}  // namespace pdx
