// Two FP32 values in one 64-bit register pair, computed with the packed FP32
// instructions of sm_100 and later (add / sub / mul / fma .rn.f32x2). Each
// half of a packed operation is the IEEE round-to-nearest result of the same
// float operation on that half's operands, so an update written once for
// float and instantiated for F2 gives, per half, the bits of the float
// update: two lattice cells for the issue cost of one.
#pragma once

namespace imx {

struct F2 {
  unsigned long long v;
  F2() = default;
  __device__ __forceinline__ explicit F2(float a) {
    asm("mov.b64 %0, {%1, %1};" : "=l"(v) : "f"(a));
  }
  __device__ __forceinline__ F2(float a, float b) {
    asm("mov.b64 %0, {%1, %2};" : "=l"(v) : "f"(a), "f"(b));
  }
  __device__ __forceinline__ float lo() const {
    float a, b;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(v));
    return a;
  }
  __device__ __forceinline__ float hi() const {
    float a, b;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(v));
    return b;
  }
};

__device__ __forceinline__ F2 operator+(F2 a, F2 b) {
  F2 r;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
  return r;
}
__device__ __forceinline__ F2 operator-(F2 a, F2 b) {
  F2 r;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
  return r;
}
__device__ __forceinline__ F2& operator+=(F2& a, F2 b) { return a = a + b; }
__device__ __forceinline__ F2& operator-=(F2& a, F2 b) { return a = a - b; }

__device__ __forceinline__ F2 r_add(F2 a, F2 b) { return a + b; }
__device__ __forceinline__ F2 r_mul(F2 a, F2 b) {
  F2 r;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
  return r;
}
__device__ __forceinline__ F2 r_fma(F2 a, F2 b, F2 c) {
  F2 r;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r.v) : "l"(a.v), "l"(b.v), "l"(c.v));
  return r;
}
// per half: the float square root (IEEE round-to-nearest)
__device__ __forceinline__ F2 r_sqrt(F2 a) { return F2(sqrtf(a.lo()), sqrtf(a.hi())); }

}  // namespace imx
