// swgb_numeric.cuh -- device restatement of the Reactor numeric primitives the
// draw path depends on (src/Reactor/LLVMReactor.cpp, src/Reactor/Reactor.cpp).
//
// The translation unit is compiled with -ftz=true -prec-div=true
// -prec-sqrt=true -fmad=false, so:
//   * every f32 add/sub/mul/div flushes subnormal inputs and results to a zero
//     of the same sign, as the reference's worker threads do (FTZ+DAZ,
//     src/System/SwiftConfig.cpp:136-139);
//   * a / b is the IEEE-rounded quotient (Rcp with relaxedPrecision = false is
//     1.0f / x on x86, src/Reactor/Reactor.cpp:4812-4851);
//   * no multiply-add is contracted unless written as mul_add() below, which
//     stands for Reactor's MulAdd / ShaderCore mulAdd (llvm.fmuladd, fused when
//     the JIT host has FMA; src/Pipeline/ShaderCore.cpp:714-722).
#pragma once

#include <stdint.h>

namespace swgb {

__device__ __forceinline__ float mul_add(float a, float b, float c) { return __fmaf_rn(a, b, c); }

// Max(x, y) = x > y ? x : y, Min(x, y) = x < y ? x : y
// (src/Reactor/Reactor.cpp:3980-3988, LLVMReactor.cpp:4443-4453).
__device__ __forceinline__ float rmax(float x, float y) { return x > y ? x : y; }
__device__ __forceinline__ float rmin(float x, float y) { return x < y ? x : y; }

// RoundInt: cvtss2si / cvtps2dq -- round half to even, 0x80000000 when the
// value does not fit (LLVMReactor.cpp:2373-2381,2684-2692).
__device__ __forceinline__ int32_t round_int(float x)
{
    return (x >= -2147483648.0f && x < 2147483648.0f) ? __float2int_rn(x) : INT32_MIN;
}

// RoundIntClamped on SIMD::Float: nearbyint + fptosi.sat (LLVMReactor.cpp:4264-4281).
// cvt.rni.s32.f32 saturates and maps NaN to 0, which is fptosi.sat.
__device__ __forceinline__ int32_t round_int_clamped(float x) { return __float2int_rn(x); }

// Int(Float) / Int4(Float4): cvttss2si / cvttps2dq -- truncation, 0x80000000
// when the value does not fit.
__device__ __forceinline__ int32_t trunc_int(float x)
{
    return (x >= -2147483648.0f && x < 2147483648.0f) ? __float2int_rz(x) : INT32_MIN;
}

// MulHigh (pmulhuw, LLVMReactor.cpp:2229-2237).
__device__ __forceinline__ uint32_t mulhi_u16(uint32_t a, uint32_t b) { return ((a & 0xFFFFu) * (b & 0xFFFFu)) >> 16; }

__device__ __forceinline__ uint32_t addsat_u16(uint32_t a, uint32_t b)
{
    uint32_t s = a + b;
    return s > 0xFFFFu ? 0xFFFFu : s;
}
__device__ __forceinline__ uint32_t subsat_u16(uint32_t a, uint32_t b) { return a > b ? a - b : 0u; }

// log2(sqrt(x)) by the exponent-bit trick of SamplerCore (src/Pipeline/SamplerCore.cpp:1333-1341).
__device__ __forceinline__ float log2sqrt(float lod)
{
    lod = lod * lod;
    lod = __int2float_rn(__float_as_int(lod)) - 1065353216.0f;  // Float(As<Int>(lod)) - Float(0x3F800000)
    lod = lod * __int_as_float(0x33000000);                     // * 0.25 * 2^-23
    return lod;
}

// halfToFloatBits (src/Pipeline/ShaderCore.cpp:627-645): texel conversion of
// R16G16B16A16_SFLOAT textures.
__device__ __forceinline__ float half_bits_to_float(uint32_t h)
{
    uint32_t sign16 = h & 0x8000u, man16 = h & 0x03FFu, exp16 = h & 0x7C00u;
    uint32_t sign32 = sign16 << 16, man32 = man16 << 13, exp32 = (exp16 + 0x1C000u) << 13;
    uint32_t norm32 = (man32 | exp32) | (exp16 == 0x7C00u ? 0x7F800000u : 0u);
    const uint32_t magic = 126u << 23;
    uint32_t denorm32 = __float_as_uint(__uint_as_float(magic + man16) - __uint_as_float(magic));
    return __uint_as_float(sign32 | (exp16 == 0 ? denorm32 : norm32));
}

// Reactor's Float(Half) (src/Reactor/Reactor.cpp:3787-3815), used when the
// blend reads an R16G16B16A16_SFLOAT attachment (a half inf/NaN reads as 65536+).
// For a nonzero exponent the reference builds ((e + 112) << 23) | (m << 13),
// which is the half's low 15 bits shifted by 13 plus 112 << 23 (exponent 31
// included: it stays finite); for a zero exponent it normalises m, giving the
// exact value m * 2^-24, a normal float (zero for m = 0).
__device__ __forceinline__ float reactor_half_to_float(uint32_t h)
{
    const uint32_t em = h & 0x7FFFu, sgn = (h & 0x8000u) << 16;
    const uint32_t mag = em >= 0x400u ? (em << 13) + (112u << 23) : __float_as_uint((float)em * 5.9604644775390625e-8f);
    return __uint_as_float(sgn | mag);
}

// Reactor's Half(Float) (src/Reactor/Reactor.cpp:3744-3770), used by
// writeColor for R16G16B16A16_SFLOAT attachments.
__device__ __forceinline__ uint32_t reactor_float_to_half(float f)
{
    uint32_t fp32i = __float_as_uint(f);
    uint32_t ab = fp32i & 0x7FFFFFFFu;
    uint32_t fp16i = (fp32i & 0x80000000u) >> 16;
    if(ab > 0x47FFEFFFu)
        fp16i |= 0x7FFFu;
    else if(ab < 0x38800000u)
    {
        int32_t mantissa = (int32_t)((ab & 0x007FFFFFu) | 0x00800000u);
        int32_t e = 113 - (int32_t)(ab >> 23);
        uint32_t a2 = e < 24 ? (uint32_t)(mantissa >> e) : 0u;
        fp16i |= ((a2 + 0x00000FFFu + ((a2 >> 13) & 1u)) >> 13) & 0xFFFFu;
    }
    else
        fp16i |= ((ab + 0xC8000000u + 0x00000FFFu + ((ab >> 13) & 1u)) >> 13) & 0xFFFFu;
    return fp16i & 0xFFFFu;
}

// Log2 and Exp2 at relaxed (mediump) precision, the forms Pow<Mediump> uses
// (src/Pipeline/ShaderCore.cpp:336-386,406-470,472-477; the CMake build's
// SWIFTSHADER_LEGACY_PRECISION is false).  Log2: the float's bits read as an
// integer give a piecewise-linear log2; a quadratic in the unnormalised
// mantissa corrects it.  Exp2: the clamped input split into floor and
// fraction, a quadratic correction, and the sum scaled into the exponent
// field (Malossi et al., "Fast Exponential Computation on SIMD
// Architectures").
__device__ __forceinline__ float log2_mediump(float x)
{
    const int32_t im = __float_as_int(x);
    float y = mul_add(__int2float_rn(im), 1.0f / (1 << 23), -127.0f);
    if(im == 0x7F800000) y = __int_as_float(__float_as_int(y) | 0x7F800000);  // log2(inf) = inf
    const float m = __int2float_rn(im & 0x007FFFFF);
    const float f = mul_add(mul_add(2.8017103e-22f, m, -8.373131e-15f), m, 5.0615534e-8f);
    return mul_add(f, m, y);
}
__device__ __forceinline__ float exp2_mediump(float x)
{
    float x0 = rmin(x, 128.0f);
    x0 = rmax(x0, __int_as_float((int32_t)0xC2FDFFFF));  // -126.999992
    const float f = x0 - floorf(x0);
    const float r = mul_add(mul_add(7.8145574e-2f, f, 2.2617357e-1f), f, -3.0444314e-1f);
    const float y = mul_add(r, f, x0);
    return __int_as_float(trunc_int(mul_add((float)(1 << 23), y, (float)(127 << 23))));
}
__device__ __forceinline__ float pow_mediump(float x, float y) { return exp2_mediump(log2_mediump(x) * y); }

// sRGB transfer functions of colour attachments (ShaderCore.cpp:914-930):
// linear below the knee, else the mediump power.
__device__ __forceinline__ float linear_to_srgb(float c)
{
    const float lc = c * 12.92f;
    const float ec = mul_add(1.055f, pow_mediump(c, 1.0f / 2.4f), -0.055f);
    return c < 0.0031308f ? lc : ec;
}
__device__ __forceinline__ float srgb_to_linear(float c)
{
    const float lc = c * (1.0f / 12.92f);
    const float ec = pow_mediump(mul_add(c, 1.0f / 1.055f, 0.055f / 1.055f), 2.4f);
    return c < 0.04045f ? lc : ec;
}

}  // namespace swgb
