// Two FP32 values in one 64-bit register pair, evaluated by the packed
// FP32x2 instructions of sm_100+ (__fadd2_rn, __fmul2_rn, __ffma2_rn: one
// issue for both lanes, per-lane rounding identical to the scalar
// instructions).  Used as the scalar type R of the radix kernels of
// vk_fft.cuh, a C2<f2> holds two independent complex values (lane 0 and lane
// 1), so one call of dft<f2, ...> transforms two butterflies -- two lines at
// the same positions -- with about half the FP32 instructions of two scalar
// calls.  Only the FP32-bulk form uses it.
#pragma once

#include "vk_fft.cuh"

namespace vk {

struct f2 {
  float2 v;
  f2() = default;
  __device__ __forceinline__ f2(float2 a) : v(a) {}
  __device__ __forceinline__ f2(float a, float b) : v(make_float2(a, b)) {}
  // broadcast constant (R(c) in the radix kernels)
  __device__ __forceinline__ explicit f2(double c) : v(make_float2((float)c, (float)c)) {}
  __device__ __forceinline__ explicit f2(int c) : v(make_float2((float)c, (float)c)) {}
};

__device__ __forceinline__ f2 operator+(f2 a, f2 b) { return f2(__fadd2_rn(a.v, b.v)); }
// a - b = (-1) b + a, exact in one fused operation
__device__ __forceinline__ f2 operator-(f2 a, f2 b) { return f2(__ffma2_rn(b.v, make_float2(-1.f, -1.f), a.v)); }
__device__ __forceinline__ f2 operator-(f2 a) { return f2(__fmul2_rn(a.v, make_float2(-1.f, -1.f))); }
__device__ __forceinline__ f2 operator*(f2 a, f2 b) { return f2(__fmul2_rn(a.v, b.v)); }
__device__ __forceinline__ f2 fma(f2 a, f2 b, f2 c) { return f2(__ffma2_rn(a.v, b.v, c.v)); }

struct C2f2 {
  f2 x, y;
};
template <> struct CplxOf<f2> { using T = C2f2; };

// lanes <-> complex values
__device__ __forceinline__ C2f2 cpack(float2 a, float2 b) {
  C2f2 r;
  r.x = f2(a.x, b.x);
  r.y = f2(a.y, b.y);
  return r;
}
__device__ __forceinline__ float2 clane0(const C2f2& c) { return make_float2(c.x.v.x, c.y.v.x); }
__device__ __forceinline__ float2 clane1(const C2f2& c) { return make_float2(c.x.v.y, c.y.v.y); }
// the same complex value in both lanes (a twiddle shared by both butterflies)
__device__ __forceinline__ C2f2 cbcast(float2 a) { return cpack(a, a); }

}  // namespace vk
