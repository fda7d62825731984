// pack2.cuh - two FP32 lanes in one 64-bit register.
//
// Blackwell executes add/sub/mul/fma on a pair of FP32 values held in a
// register pair as one instruction (PTX .f32x2, sm_100 and later), so
// identical arithmetic on two cells issues half the instructions.  The
// operations here are hand-written inline PTX, IEEE round-to-nearest, one
// rounding each (fma is fused); lane-wise operations the instruction set
// has no packed form for (min, max, abs, copysign, reciprocal, square root)
// work on the two halves separately.
#pragma once
#include <cuda_runtime.h>

namespace vacgpu {

struct f2 {
  unsigned long long v;
};

__device__ __forceinline__ f2 f2m(float lo, float hi) {
  f2 r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r.v) : "f"(lo), "f"(hi));
  return r;
}
__device__ __forceinline__ f2 f2s(float a) { return f2m(a, a); }
__device__ __forceinline__ void f2u(f2 a, float& lo, float& hi) {
  asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(a.v));
}
__device__ __forceinline__ float f2lo(f2 a) {
  float l, h;
  f2u(a, l, h);
  return l;
}
__device__ __forceinline__ float f2hi(f2 a) {
  float l, h;
  f2u(a, l, h);
  return h;
}

__device__ __forceinline__ f2 operator+(f2 a, f2 b) {
  f2 r;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
  return r;
}
__device__ __forceinline__ f2 operator-(f2 a, f2 b) {
  f2 r;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
  return r;
}
__device__ __forceinline__ f2 operator*(f2 a, f2 b) {
  f2 r;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
  return r;
}
// a*b + c with one rounding
__device__ __forceinline__ f2 ffma(f2 a, f2 b, f2 c) {
  f2 r;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r.v) : "l"(a.v), "l"(b.v), "l"(c.v));
  return r;
}
__device__ __forceinline__ f2& operator+=(f2& a, f2 b) { return a = a + b; }
__device__ __forceinline__ f2& operator-=(f2& a, f2 b) { return a = a - b; }

// -a: flip both sign bits (exact, also for zeros)
__device__ __forceinline__ f2 fneg(f2 a) {
  f2 r;
  r.v = a.v ^ 0x8000000080000000ull;
  return r;
}

// lane-wise operations
__device__ __forceinline__ f2 vmin(f2 a, f2 b) {
  float al, ah, bl, bh;
  f2u(a, al, ah);
  f2u(b, bl, bh);
  return f2m(fminf(al, bl), fminf(ah, bh));
}
__device__ __forceinline__ f2 vmax(f2 a, f2 b) {
  float al, ah, bl, bh;
  f2u(a, al, ah);
  f2u(b, bl, bh);
  return f2m(fmaxf(al, bl), fmaxf(ah, bh));
}
__device__ __forceinline__ f2 vabs(f2 a) {
  f2 r;
  r.v = a.v & 0x7fffffff7fffffffull;
  return r;
}
// |a| with the sign of b, per lane
__device__ __forceinline__ f2 vcopysign(f2 a, f2 b) {
  f2 r;
  r.v = (a.v & 0x7fffffff7fffffffull) | (b.v & 0x8000000080000000ull);
  return r;
}
// a with its sign flipped where b is negative (a * sign(b) for b != 0)
__device__ __forceinline__ f2 vxorsign(f2 a, f2 b) {
  f2 r;
  r.v = a.v ^ (b.v & 0x8000000080000000ull);
  return r;
}
// 1/a: the build's FP32 reciprocal per lane
__device__ __forceinline__ f2 vrcp(f2 a) {
  float l, h;
  f2u(a, l, h);
  return f2m(1.0f / l, 1.0f / h);
}
__device__ __forceinline__ f2 vsqrt(f2 a) {
  float l, h;
  f2u(a, l, h);
  return f2m(sqrtf(l), sqrtf(h));
}
// x >= lo ? x : lo per lane (the reference's max(p, smallp): NaN kept)
__device__ __forceinline__ f2 vclamp_lo(f2 a, float lo) {
  float l, h;
  f2u(a, l, h);
  return f2m(l >= lo ? l : lo, h >= lo ? h : lo);
}

// two adjacent floats of shared or global memory (8-byte aligned)
__device__ __forceinline__ f2 ld2(const float* p) {
  const float2 t = *reinterpret_cast<const float2*>(p);
  return f2m(t.x, t.y);
}
__device__ __forceinline__ void st2(float* p, f2 a) {
  float2 t;
  f2u(a, t.x, t.y);
  *reinterpret_cast<float2*>(p) = t;
}

}  // namespace vacgpu
