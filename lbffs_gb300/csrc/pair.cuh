// Two FP32 lanes in one 64-bit register pair, computed with the packed FP32x2 instructions of
// sm_100+ (PTX add/sub/mul/fma .f32x2).  The bulk kernel keeps two cells per thread, so running
// their collision arithmetic as pairs issues one instruction where two scalar ones were needed.
// add / sub / mul carry no rounding modifier, which leaves the code generator free to contract a
// multiply and an add into one fused multiply-add, as it does for the scalar expressions; every
// lane still rounds exactly as a scalar FP32 operation would.
#pragma once
#include <cuda_runtime.h>

namespace lbffs {

struct F2 {
    unsigned long long u;
};

__device__ __forceinline__ F2 pk(float x, float y)
{
    F2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r.u) : "f"(x), "f"(y));
    return r;
}
__device__ __forceinline__ F2 splat(float x) { return pk(x, x); }
__device__ __forceinline__ float lane0(F2 a) { return __uint_as_float((unsigned)(a.u & 0xffffffffull)); }
__device__ __forceinline__ float lane1(F2 a) { return __uint_as_float((unsigned)(a.u >> 32)); }
__device__ __forceinline__ float lane(F2 a, int v) { return v == 0 ? lane0(a) : lane1(a); }

__device__ __forceinline__ F2 operator+(F2 a, F2 b)
{
    F2 r;
    asm("add.f32x2 %0, %1, %2;" : "=l"(r.u) : "l"(a.u), "l"(b.u));
    return r;
}
__device__ __forceinline__ F2 operator-(F2 a, F2 b)
{
    F2 r;
    asm("sub.f32x2 %0, %1, %2;" : "=l"(r.u) : "l"(a.u), "l"(b.u));
    return r;
}
__device__ __forceinline__ F2 operator*(F2 a, F2 b)
{
    F2 r;
    asm("mul.f32x2 %0, %1, %2;" : "=l"(r.u) : "l"(a.u), "l"(b.u));
    return r;
}
__device__ __forceinline__ F2 fma2(F2 a, F2 b, F2 c)
{
    F2 r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r.u) : "l"(a.u), "l"(b.u), "l"(c.u));
    return r;
}
__device__ __forceinline__ F2 operator+(F2 a, float b) { return a + splat(b); }
__device__ __forceinline__ F2 operator+(float a, F2 b) { return splat(a) + b; }
__device__ __forceinline__ F2 operator-(F2 a, float b) { return a - splat(b); }
__device__ __forceinline__ F2 operator-(float a, F2 b) { return splat(a) - b; }
__device__ __forceinline__ F2 operator*(F2 a, float b) { return a * splat(b); }
__device__ __forceinline__ F2 operator*(float a, F2 b) { return splat(a) * b; }
__device__ __forceinline__ F2& operator+=(F2& a, F2 b) { return a = a + b; }
__device__ __forceinline__ F2& operator-=(F2& a, F2 b) { return a = a - b; }
__device__ __forceinline__ F2& operator*=(F2& a, F2 b) { return a = a * b; }
__device__ __forceinline__ F2& operator*=(F2& a, float b) { return a = a * b; }

}  // namespace lbffs
