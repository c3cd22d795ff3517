// Packed FP32 arithmetic for the mixed-precision force loops: two FP32 lanes in one 64-bit
// register, operated on by one f32x2 instruction (add/sub/mul/fma.rn.f32x2), which halves
// the issue slots of FP32 work on sm_103a.  One pair record (BodyPair) holds the same
// quantity of two source bodies per 8-byte slot, so one instruction serves both bodies.
#pragma once
#include "ddx_internal.cuh"

namespace ddx {
namespace {

typedef unsigned long long f2;   // two FP32 lanes of one f32x2 instruction

__device__ __forceinline__ f2 f2_dup(float a) {
    f2 r; asm("mov.b64 %0, {%1, %1};" : "=l"(r) : "f"(a)); return r;
}
__device__ __forceinline__ void f2_split(f2 v, float& lo, float& hi) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}
__device__ __forceinline__ f2 f2_join(float lo, float hi) {
    f2 r; asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi)); return r;
}
__device__ __forceinline__ f2 add2(f2 a, f2 b) {
    f2 r; asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b)); return r;
}
__device__ __forceinline__ f2 sub2(f2 a, f2 b) {
    f2 r; asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b)); return r;
}
__device__ __forceinline__ f2 mul2(f2 a, f2 b) {
    f2 r; asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b)); return r;
}
__device__ __forceinline__ f2 fma2(f2 a, f2 b, f2 c) {
    f2 r; asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c)); return r;
}
__device__ __forceinline__ float rsqrt_approx(float x) {
    float r; asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x)); return r;
}
__device__ __forceinline__ void kahan2(f2& S, f2& C, f2 v) {
    const f2 y = sub2(v, C);
    const f2 t = add2(S, y);
    C = sub2(sub2(t, S), y);
    S = t;
}
// Compensated sum of both lanes of (S, C), in FP64.
__device__ __forceinline__ double f2_total(f2 S, f2 C) {
    float s0, s1, c0, c1;
    f2_split(S, s0, s1);
    f2_split(C, c0, c1);
    return ((double)s0 - (double)c0) + ((double)s1 - (double)c1);
}

}  // namespace
}  // namespace ddx
