// Packed FP32 pair arithmetic (add/sub/mul/fma .rn.f32x2, sm_100 family): one instruction does
// the same round-to-nearest operation on two lanes, halving the FP32 instruction count of a
// kernel that updates two points per thread.  The code generator contracts a pair multiply that
// feeds a pair add into one pair FMA (measured on sm_103a, with or without -fmad=false, even
// when the multiply is written as an FMA with a -0 addend), so a chain of them rounds like the
// FMA form: kernels that must round exactly like separate scalar operations use the scalar
// __fmul_rn / __fadd_rn intrinsics instead.
#pragma once

#include <cuda_fp16.h>

namespace gb {
namespace f2 {

__device__ __forceinline__ unsigned long long pack(float2 v)
{
    unsigned long long r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(v.x), "f"(v.y));
    return r;
}

__device__ __forceinline__ float2 unpack(unsigned long long r)
{
    float2 v;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(v.x), "=f"(v.y) : "l"(r));
    return v;
}

__device__ __forceinline__ float2 add(float2 a, float2 b)
{
    unsigned long long r;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(pack(a)), "l"(pack(b)));
    return unpack(r);
}

__device__ __forceinline__ float2 sub(float2 a, float2 b)
{
    unsigned long long r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(pack(a)), "l"(pack(b)));
    return unpack(r);
}

__device__ __forceinline__ float2 mul(float2 a, float2 b)
{
    unsigned long long r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(pack(a)), "l"(pack(b)));
    return unpack(r);
}

// a * b + c, one rounding per lane
__device__ __forceinline__ float2 fma(float2 a, float2 b, float2 c)
{
    unsigned long long r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(pack(a)), "l"(pack(b)), "l"(pack(c)));
    return unpack(r);
}

__device__ __forceinline__ float2 splat(float s) { return make_float2(s, s); }

__device__ __forceinline__ float2 from_half2(__half2 h) { return __half22float2(h); }

}  // namespace f2
}  // namespace gb
