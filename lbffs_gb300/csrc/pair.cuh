// Two FP32 lanes in one 64-bit register pair, computed with the packed FP32x2 instructions of
// sm_100+ (PTX add/sub/mul/fma .f32x2).  The bulk kernel keeps two cells per thread, so running
// their collision arithmetic as pairs issues one instruction where two scalar ones were needed.
// Every operation carries an explicit round-to-nearest modifier, so the code generator never
// contracts a multiply and an add on its own: fused multiply-adds are written out (fma2 / mad),
// and a lane's result is the same in every kernel that inlines the arithmetic, whatever the
// surrounding code.
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
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r.u) : "l"(a.u), "l"(b.u));
    return r;
}
__device__ __forceinline__ F2 operator-(F2 a, F2 b)
{
    F2 r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r.u) : "l"(a.u), "l"(b.u));
    return r;
}
__device__ __forceinline__ F2 operator*(F2 a, F2 b)
{
    F2 r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r.u) : "l"(a.u), "l"(b.u));
    return r;
}
__device__ __forceinline__ F2 fma2(F2 a, F2 b, F2 c)
{
    F2 r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r.u) : "l"(a.u), "l"(b.u), "l"(c.u));
    return r;
}
// a * b + c rounded once, for one lane (float) or two (F2)
__device__ __forceinline__ float mad(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ F2 mad(F2 a, F2 b, F2 c) { return fma2(a, b, c); }
__device__ __forceinline__ F2 mad(F2 a, float b, F2 c) { return fma2(a, splat(b), c); }
__device__ __forceinline__ F2 mad(float a, F2 b, F2 c) { return fma2(splat(a), b, c); }
__device__ __forceinline__ F2 mad(F2 a, F2 b, float c) { return fma2(a, b, splat(c)); }
// -a (exact)
__device__ __forceinline__ float neg(float a) { return -a; }
__device__ __forceinline__ F2 neg(F2 a)
{
    F2 r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r.u) : "l"(a.u), "l"(splat(-1.f).u));
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
