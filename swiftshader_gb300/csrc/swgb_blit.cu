// swgb_blit.cu -- the Blitter steps either side of a draw on the GPU: clears,
// multisample resolves and scaled blits (mip generation is one LINEAR blit per
// level) of the draw path's attachment and texture formats
// (sw::Blitter, src/Device/Blitter.cpp).
//
// This unit is compiled WITHOUT flush-to-zero.  The reference runs blit
// routines on the queue thread, which keeps IEEE subnormals: only the marl
// worker threads that run draws set FTZ/DAZ (src/System/SwiftConfig.cpp:
// 136-139).  Otherwise the arithmetic follows the routine Blitter::generate
// emits: unfused multiplies and adds, Reactor's RoundInt / Half conversions
// and its mediump sRGB transfer functions.
//
// Every kernel is HBM-bound byte work: clears write, resolves read four
// sample planes and write one, blits read up to four texels per pixel.  One
// thread per pixel (per 16-byte chunk for clears, per four pixels for the
// byte-averaging resolve); indices are clamped to the source so that no read
// leaves it whatever the region.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

#include "swgb_blit.h"
#include "swgb_numeric.cuh"

using namespace swgb;

namespace swgbb {

namespace {

__host__ __device__ constexpr bool kind_unorm8(int k) { return k == BK_RGBA8 || k == BK_BGRA8; }
__host__ __device__ constexpr bool kind_float(int k) { return k == BK_RGBA16F || k == BK_RGBA32F; }
__host__ __device__ constexpr int kind_bytes(int k) { return kind_unorm8(k) ? 4 : (k == BK_RGBA16F ? 8 : 16); }

// readFloat4 (Blitter.cpp:312-550): 8-bit formats as their byte values,
// B8G8R8A8 swizzled to R, G, B, A (.zyxw); half floats through Reactor's
// Float(Half).
__device__ __forceinline__ float4 read_texel(const uint8_t *p, int kind)
{
    switch(kind)
    {
    case BK_RGBA8:
    {
        const uint32_t v = *(const uint32_t *)p;
        return make_float4((float)(v & 0xFFu), (float)((v >> 8) & 0xFFu), (float)((v >> 16) & 0xFFu), (float)(v >> 24));
    }
    case BK_BGRA8:
    {
        const uint32_t v = *(const uint32_t *)p;
        return make_float4((float)((v >> 16) & 0xFFu), (float)((v >> 8) & 0xFFu), (float)(v & 0xFFu), (float)(v >> 24));
    }
    case BK_RGBA16F:
    {
        const uint2 v = *(const uint2 *)p;
        return make_float4(reactor_half_to_float(v.x & 0xFFFFu), reactor_half_to_float(v.x >> 16),
                           reactor_half_to_float(v.y & 0xFFFFu), reactor_half_to_float(v.y >> 16));
    }
    default: return *(const float4 *)p;
    }
}

// RoundShort4 then PackUnsigned: RoundInt, saturate to int16, then to 0..255
// (Reactor.cpp:1947-1951, Blitter.cpp:674-692).
__device__ __forceinline__ uint32_t pack_unorm8(float c)
{
    int32_t r = round_int(c);
    r = r < -32768 ? -32768 : (r > 32767 ? 32767 : r);
    return r < 0 ? 0u : (r > 255 ? 255u : (uint32_t)r);
}

// The same for a value known to lie in [0, 256): RoundInt in range, the
// 16-bit saturation a no-op, only the clamp at 255 left.
__device__ __forceinline__ uint32_t pack_unorm8_bounded(float c) { return (uint32_t)min(__float2int_rn(c), 255); }

// write (Blitter.cpp:553-1180), all four components written.  BOUNDED: the
// colour came from 8-bit texels (blends and sRGB round trips of values in
// [0, 255] stay in [0, 256)).
template<bool BOUNDED = false>
__device__ __forceinline__ void write_texel(uint8_t *p, int kind, float4 c)
{
    auto pk = [](float v) { return BOUNDED ? pack_unorm8_bounded(v) : pack_unorm8(v); };
    switch(kind)
    {
    case BK_RGBA8: *(uint32_t *)p = pk(c.x) | (pk(c.y) << 8) | (pk(c.z) << 16) | (pk(c.w) << 24); break;
    case BK_BGRA8: *(uint32_t *)p = pk(c.z) | (pk(c.y) << 8) | (pk(c.x) << 16) | (pk(c.w) << 24); break;
    case BK_RGBA16F:
        *(uint2 *)p = make_uint2(reactor_float_to_half(c.x) | (reactor_float_to_half(c.y) << 16),
                                 reactor_float_to_half(c.z) | (reactor_float_to_half(c.w) << 16));
        break;
    default: *(float4 *)p = c; break;
    }
}

__device__ __forceinline__ float4 mul4(float4 a, float m) { return make_float4(a.x * m, a.y * m, a.z * m, a.w * m); }

// ApplyScaleAndClamp (Blitter.cpp:1427-1485) for the formats here: 8-bit
// formats scale 255, float formats 1; sRGB conversions when allowed and one
// side is sRGB; float into 8-bit clamps to [0, 255].
__device__ __forceinline__ float4 scale_and_clamp(float4 v, int srcKind, bool srcSRGB, int dstKind, bool dstSRGB, bool allowSRGB,
                                                  bool preScaled)
{
    const float unscale = kind_unorm8(srcKind) ? 255.0f : 1.0f;
    const float scale = kind_unorm8(dstKind) ? 255.0f : 1.0f;
    if(allowSRGB && ((srcSRGB && !preScaled) || dstSRGB))
    {
        v = mul4(v, preScaled ? 1.0f / scale : 1.0f / unscale);  // unapply scale / apply unscale
        if(srcSRGB && !preScaled)
        {
            v.x = srgb_to_linear(v.x);
            v.y = srgb_to_linear(v.y);
            v.z = srgb_to_linear(v.z);
        }
        else
        {
            v.x = linear_to_srgb(v.x);
            v.y = linear_to_srgb(v.y);
            v.z = linear_to_srgb(v.z);
        }
        v = mul4(v, scale);
    }
    else if(unscale != scale)
        v = mul4(v, scale / unscale);
    if(kind_float(srcKind) && !kind_float(dstKind))
    {
        v = make_float4(rmin(v.x, scale), rmin(v.y, scale), rmin(v.z, scale), rmin(v.w, scale));
        v = make_float4(rmax(v.x, 0.0f), rmax(v.y, 0.0f), rmax(v.z, 0.0f), rmax(v.w, 0.0f));
    }
    if(kind_float(srcKind) && kind_unorm8(dstKind))  // !isUnsigned(src) && isUnsigned(dst)
        v = make_float4(rmax(v.x, 0.0f), rmax(v.y, 0.0f), rmax(v.z, 0.0f), rmax(v.w, 0.0f));
    return v;
}

__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

// The bilinear branch of Blitter::sample after its four reads
// (Blitter.cpp:1625-1653): sRGB texels decoded when allowed, the blend
// (c00 ix + c01 fx) iy + (c10 ix + c11 fx) fy, then ApplyScaleAndClamp.
template<int SK, int DK>
__device__ __forceinline__ float4 bilinear(const BlitParams &P, float4 c00, float4 c01, float4 c10, float4 c11, float fx, float fy)
{
    const bool convertSrc = P.allowSRGB && P.srcSRGB;
    if(convertSrc)
    {
        c00 = scale_and_clamp(c00, SK, P.srcSRGB, DK, P.dstSRGB, P.allowSRGB, false);
        c01 = scale_and_clamp(c01, SK, P.srcSRGB, DK, P.dstSRGB, P.allowSRGB, false);
        c10 = scale_and_clamp(c10, SK, P.srcSRGB, DK, P.dstSRGB, P.allowSRGB, false);
        c11 = scale_and_clamp(c11, SK, P.srcSRGB, DK, P.dstSRGB, P.allowSRGB, false);
    }
    const float ix = 1.0f - fx, iy = 1.0f - fy;
    float4 color;
    color.x = (c00.x * ix + c01.x * fx) * iy + (c10.x * ix + c11.x * fx) * fy;
    color.y = (c00.y * ix + c01.y * fx) * iy + (c10.y * ix + c11.y * fx) * fy;
    color.z = (c00.z * ix + c01.z * fx) * iy + (c10.z * ix + c11.z * fx) * fy;
    color.w = (c00.w * ix + c01.w * fx) * iy + (c10.w * ix + c11.w * fx) * fy;
    return scale_and_clamp(color, SK, P.srcSRGB, DK, P.dstSRGB, P.allowSRGB, convertSrc);
}

// Blitter::sample (Blitter.cpp:1497-1657), 2D: nearest texel (its samples
// averaged for a resolve) or the bilinear blend of four.
template<int SK, int DK, bool FILTER>
__device__ __forceinline__ float4 sample(const BlitParams &P, float x, float y)
{
    const bool convertSrc = P.allowSRGB && P.srcSRGB;
    bool preScaled = false;
    float4 color;
    if(!FILTER)
    {
        int X = trunc_int(x), Y = trunc_int(y);
        if(P.clampToEdge)
        {
            X = clampi(X, 0, P.sW - 1);
            Y = clampi(Y, 0, P.sH - 1);
        }
        X = clampi(X, 0, P.sW - 1);  // in range already unless the region is malformed
        Y = clampi(Y, 0, P.sH - 1);
        const uint8_t *s = P.src + (int64_t)Y * P.sPitch + (int64_t)X * kind_bytes(SK);
        color = read_texel(s, SK);
        if(P.srcSamples > 1)
        {
            if(convertSrc)
            {
                color = scale_and_clamp(color, SK, P.srcSRGB, DK, P.dstSRGB, P.allowSRGB, false);
                preScaled = true;
            }
            float4 accum = color;
            for(int q = 1; q < P.srcSamples; q++)
            {
                s += P.sSlice;
                color = read_texel(s, SK);
                if(convertSrc) color = scale_and_clamp(color, SK, P.srcSRGB, DK, P.dstSRGB, P.allowSRGB, false);
                accum = make_float4(accum.x + color.x, accum.y + color.y, accum.z + color.z, accum.w + color.w);
            }
            color = mul4(accum, 1.0f / (float)P.srcSamples);
        }
    }
    else
    {
        float X = x, Y = y;
        if(P.clampToEdge)
        {
            X = rmin(rmax(x, 0.5f), (float)P.sW - 0.5f);
            Y = rmin(rmax(y, 0.5f), (float)P.sH - 0.5f);
        }
        const float x0 = X - 0.5f, y0 = Y - 0.5f;
        int X0 = max(trunc_int(x0), 0), Y0 = max(trunc_int(y0), 0);
        int X1 = X0 + 1, Y1 = Y0 + 1;
        X1 = X1 >= P.sW ? X0 : X1;
        Y1 = Y1 >= P.sH ? Y0 : Y1;
        const int rx0 = clampi(X0, 0, P.sW - 1), rx1 = clampi(X1, 0, P.sW - 1);
        const int ry0 = clampi(Y0, 0, P.sH - 1), ry1 = clampi(Y1, 0, P.sH - 1);
        const float4 c00 = read_texel(P.src + (int64_t)ry0 * P.sPitch + (int64_t)rx0 * kind_bytes(SK), SK);
        const float4 c01 = read_texel(P.src + (int64_t)ry0 * P.sPitch + (int64_t)rx1 * kind_bytes(SK), SK);
        const float4 c10 = read_texel(P.src + (int64_t)ry1 * P.sPitch + (int64_t)rx0 * kind_bytes(SK), SK);
        const float4 c11 = read_texel(P.src + (int64_t)ry1 * P.sPitch + (int64_t)rx1 * kind_bytes(SK), SK);
        return bilinear<SK, DK>(P, c00, c01, c10, c11, x0 - (float)X0, y0 - (float)Y0);
    }
    return scale_and_clamp(color, SK, P.srcSRGB, DK, P.dstSRGB, P.allowSRGB, preScaled);
}

// The blit routine's pixel loop (Blitter.cpp:1714-1786): one thread per
// destination pixel of the box, a warp per 32 pixels of a row; one kernel per
// (source format, destination format, filter), so the per-texel format
// switches fold away.
template<int SK, int DK, bool FILTER>
__global__ void __launch_bounds__(256) k_blit(BlitParams P)
{
    const int i = P.x0d + (int)(blockIdx.x * 32 + (threadIdx.x & 31));
    const int j = P.y0d + (int)(blockIdx.y * 8 + (threadIdx.x >> 5));
    if(i >= P.x1d || j >= P.y1d) return;
    const float x = P.x0 + (float)i * P.w;
    const float y = P.y0 + (float)j * P.h;
    const float4 c = sample<SK, DK, FILTER>(P, x, y);
    write_texel<kind_unorm8(SK)>(P.dst + (int64_t)j * P.dPitch + (int64_t)i * kind_bytes(DK), DK, c);
}

// A LINEAR blit of src box (0, 0, 2W, 2H) onto dst box (0, 0, W, H) inside
// both images -- one mip level from the one above.  There the routine's
// positions are exact: x = 1 + 2i, X0 = 2i, X1 = 2i + 1, fx = fy = 1/2, so the
// blend above is evaluated on texels 2i, 2i + 1 of rows 2j, 2j + 1.  Each
// thread makes PX destination pixels from a 2PX x 2 texel block: four for
// 8-bit texels (two 16-byte loads per row when the rows are 16-byte
// aligned), two for float texels.
template<int SK, int DK>
__global__ void __launch_bounds__(256) k_blit_half(BlitParams P)
{
    constexpr int PX = kind_unorm8(SK) ? 4 : 2;
    constexpr int B = kind_bytes(SK);
    const int i0 = PX * (int)(blockIdx.x * 32 + (threadIdx.x & 31));
    const int j = (int)(blockIdx.y * 8 + (threadIdx.x >> 5));
    if(i0 >= P.x1d || j >= P.y1d) return;
    const int n = min(PX, P.x1d - i0);  // destination pixels of this thread
    const uint8_t *r0 = P.src + (int64_t)(2 * j) * P.sPitch + (int64_t)(2 * i0) * B;
    const uint8_t *r1 = r0 + P.sPitch;
    float4 a[2 * PX], b[2 * PX];
    if(kind_unorm8(SK) && n == PX && P.vec16)
    {
#pragma unroll
        for(int h = 0; h < PX / 2; h++)
        {
            const uint4 u = *(const uint4 *)(r0 + 16 * h), v = *(const uint4 *)(r1 + 16 * h);
            const uint32_t uu[4] = {u.x, u.y, u.z, u.w}, vv[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
            for(int k = 0; k < 4; k++)
            {
                a[4 * h + k] = read_texel((const uint8_t *)&uu[k], SK);
                b[4 * h + k] = read_texel((const uint8_t *)&vv[k], SK);
            }
        }
    }
    else
    {
#pragma unroll
        for(int k = 0; k < 2 * PX; k++)
            if(k < 2 * n)
            {
                a[k] = read_texel(r0 + k * B, SK);
                b[k] = read_texel(r1 + k * B, SK);
            }
    }
    uint8_t *d = P.dst + (int64_t)j * P.dPitch + (int64_t)i0 * kind_bytes(DK);
#pragma unroll
    for(int p = 0; p < PX; p++)
        if(p < n)
            write_texel<kind_unorm8(SK)>(d + p * kind_bytes(DK), DK,
                                         bilinear<SK, DK>(P, a[2 * p], a[2 * p + 1], b[2 * p], b[2 * p + 1], 0.5f, 0.5f));
}

// The NEAREST blit a float-format resolve is (Blitter.cpp:1508-1545): at
// scale 1 the sample position of destination pixel i is source texel
// i + (srcOffset - dstOffset) exactly; its four samples are read, summed in
// order, scaled by 1/4 and written -- no scale, clamp or sRGB step applies to
// float formats.  Two pixels per thread for half floats, each sample of each
// pixel read with its own texel-sized load.
template<int SK>
__global__ void __launch_bounds__(256) k_resolve_float(BlitParams P, int dx, int dy)
{
    constexpr int PX = SK == BK_RGBA16F ? 2 : 1;
    constexpr int B = kind_bytes(SK);
    const int i0 = P.x0d + PX * (int)(blockIdx.x * 32 + (threadIdx.x & 31));
    const int j = P.y0d + (int)(blockIdx.y * 8 + (threadIdx.x >> 5));
    if(i0 >= P.x1d || j >= P.y1d) return;
    const int n = min(PX, P.x1d - i0);
    const uint8_t *s = P.src + (int64_t)(j + dy) * P.sPitch + (int64_t)(i0 + dx) * B;
    uint8_t *d = P.dst + (int64_t)j * P.dPitch + (int64_t)i0 * B;
#pragma unroll
    for(int p = 0; p < PX; p++)
        if(p < n)
        {
            float4 acc = read_texel(s + p * B, SK);
#pragma unroll
            for(int q = 1; q < 4; q++)
            {
                const float4 c = read_texel(s + p * B + q * P.sSlice, SK);
                acc = make_float4(acc.x + c.x, acc.y + c.y, acc.z + c.z, acc.w + c.w);
            }
            write_texel(d + p * B, SK, mul4(acc, 1.0f / 4.0f));
        }
}

// fastResolve (Blitter.cpp:2079-2205): per byte, the rounding-up average of
// samples 0 and 1, of 2 and 3, then of the two (averageByte4 /
// _mm_avg_epu8; __vavgu4 computes the same (a + b + 1) >> 1 per byte).
__device__ __forceinline__ void resolve_bytes_quad(const ResolveParams &R, int x, int y)
{
    const uint8_t *s = R.src + (int64_t)y * R.sPitch + (int64_t)x * 4;
    uint8_t *d = R.dst + (int64_t)y * R.dPitch + (int64_t)x * 4;
    if(R.vec16 && x + 3 < R.width)
    {
        const uint4 c0 = *(const uint4 *)s, c1 = *(const uint4 *)(s + R.sSlice);
        const uint4 c2 = *(const uint4 *)(s + 2 * R.sSlice), c3 = *(const uint4 *)(s + 3 * R.sSlice);
        uint4 o;
        o.x = __vavgu4(__vavgu4(c0.x, c1.x), __vavgu4(c2.x, c3.x));
        o.y = __vavgu4(__vavgu4(c0.y, c1.y), __vavgu4(c2.y, c3.y));
        o.z = __vavgu4(__vavgu4(c0.z, c1.z), __vavgu4(c2.z, c3.z));
        o.w = __vavgu4(__vavgu4(c0.w, c1.w), __vavgu4(c2.w, c3.w));
        *(uint4 *)d = o;
        return;
    }
    for(int k = 0; k < 4 && x + k < R.width; k++)
    {
        const uint32_t c0 = *(const uint32_t *)(s + 4 * k), c1 = *(const uint32_t *)(s + 4 * k + R.sSlice);
        const uint32_t c2 = *(const uint32_t *)(s + 4 * k + 2 * R.sSlice), c3 = *(const uint32_t *)(s + 4 * k + 3 * R.sSlice);
        *(uint32_t *)(d + 4 * k) = __vavgu4(__vavgu4(c0, c1), __vavgu4(c2, c3));
    }
}

__global__ void __launch_bounds__(256) k_resolve_bytes(ResolveParams R)
{
    const int x = 4 * (int)(blockIdx.x * blockDim.x + threadIdx.x);  // four pixels per thread
    if(x >= R.width) return;
    for(int y = (int)blockIdx.y; y < R.height; y += (int)gridDim.y) resolve_bytes_quad(R, x, y);
}

// The texel a clear writes (Blitter::clear, Blitter.cpp:55-168): the value
// clamped to [0, 1] for normalized formats, then fastClear's packing
// (:170-244) for R8G8B8A8_UNORM, B8G8R8A8_UNORM, D32_SFLOAT and S8_UINT, or
// the blit routine's constant colour (readFloat4 of the value,
// ApplyScaleAndClamp, write; :1700-1712) for the other formats.
__device__ void clear_texel(const ClearParams &C, uint8_t out[16])
{
    float v[4] = {C.value[0], C.value[1], C.value[2], C.value[3]};
    if(C.normalized)
        for(int k = 0; k < 4; k++)
        {
            if(v[k] < 0.0f) v[k] = 0.0f;  // sw::clamp
            if(v[k] > 1.0f) v[k] = 1.0f;
        }
    uint32_t w = 0;
    switch(C.dstFormat)
    {
    case SWGB_FORMAT_R8G8B8A8_UNORM:
    case SWGB_FORMAT_B8G8R8A8_UNORM:
    {
        uint32_t c[4];
        for(int k = 0; k < 4; k++) c[k] = (uint32_t)__float2uint_rz(255.0f * v[k] + 0.5f);  // (uint32_t)(255 * c + 0.5f)
        w = C.dstFormat == SWGB_FORMAT_R8G8B8A8_UNORM ? (c[0] | (c[1] << 8) | (c[2] << 16) | (c[3] << 24))
                                                      : (c[2] | (c[1] << 8) | (c[0] << 16) | (c[3] << 24));
        for(int k = 0; k < 4; k++) out[k] = (uint8_t)(w >> (8 * k));
        return;
    }
    case SWGB_FORMAT_D32_SFLOAT:
        w = __float_as_uint(C.value[0]);  // the float's bits, unclamped
        for(int k = 0; k < 4; k++) out[k] = (uint8_t)(w >> (8 * k));
        return;
    case SWGB_FORMAT_S8_UINT: out[0] = (uint8_t)C.stencil; return;
    case SWGB_FORMAT_D16_UNORM:
    {
        // D32_SFLOAT source (scale 1) into D16_UNORM (scale 0xFFFF): multiply,
        // clamp to [0, 0xFFFF], UShort(RoundInt(x))
        float x = v[0] * 65535.0f;
        x = rmax(rmin(x, 65535.0f), 0.0f);
        const uint32_t h = (uint32_t)round_int(x) & 0xFFFFu;
        out[0] = (uint8_t)h;
        out[1] = (uint8_t)(h >> 8);
        return;
    }
    default:
    {
        const float4 c = scale_and_clamp(make_float4(v[0], v[1], v[2], v[3]), BK_RGBA32F, false, C.dstKind, C.dstSRGB, true, false);
        write_texel(out, C.dstKind, c);
        return;
    }
    }
}

// Fills one row of the area in one sample plane with the clear texel:
// 16-byte aligned chunks, the unaligned head and tail bytewise.  The texel
// pattern repeats every bpp bytes from any texel-aligned address.
__device__ __forceinline__ void clear_row(const ClearParams &C, const uint8_t *tex, int row, int plane)
{
    uint8_t *base = C.dst + (int64_t)plane * C.slice + (int64_t)(C.y + row) * C.pitch + (int64_t)C.x * C.bpp;
    const uintptr_t b0 = (uintptr_t)base, b1 = b0 + (uintptr_t)C.rowBytes;
    const uintptr_t a0 = (b0 + 15) & ~(uintptr_t)15, a1 = b1 & ~(uintptr_t)15;
    const uintptr_t tid = threadIdx.x;
    if(a0 >= a1)
    {
        // the row fits between two boundaries: bytewise
        for(uintptr_t a = b0 + tid; a < b1; a += blockDim.x) *(uint8_t *)a = tex[a & 15];
        return;
    }
    if(b0 + tid < a0) *(uint8_t *)(b0 + tid) = tex[(b0 + tid) & 15];
    if(a1 + tid < b1) *(uint8_t *)(a1 + tid) = tex[(a1 + tid) & 15];
    const uint4 pat = *(const uint4 *)tex;
    for(uintptr_t a = a0 + tid * 16; a < a1; a += (uintptr_t)blockDim.x * 16) *(uint4 *)a = pat;
}

// One block per run of rows (grid-stride over rows x sample planes), its
// threads striding each row in 16-byte chunks.
__global__ void __launch_bounds__(256) k_clear(ClearParams C)
{
    __shared__ __align__(16) uint8_t tex[16];
    if(threadIdx.x == 0)
    {
        uint8_t t[16];
        clear_texel(C, t);
        for(int k = 0; k < 16; k++) tex[k] = t[k % C.bpp];
    }
    __syncthreads();
    for(int ry = (int)blockIdx.x; ry < C.rows * C.planes; ry += (int)gridDim.x) clear_row(C, tex, ry % C.rows, ry / C.rows);
}

using BlitKernel = void (*)(BlitParams);
template<int SK, int DK>
constexpr BlitKernel blit_kernel(bool filter) { return filter ? k_blit<SK, DK, true> : k_blit<SK, DK, false>; }
template<int SK>
BlitKernel blit_kernel(int dk, bool filter)
{
    switch(dk)
    {
    case BK_RGBA8: return blit_kernel<SK, BK_RGBA8>(filter);
    case BK_BGRA8: return blit_kernel<SK, BK_BGRA8>(filter);
    case BK_RGBA16F: return blit_kernel<SK, BK_RGBA16F>(filter);
    default: return blit_kernel<SK, BK_RGBA32F>(filter);
    }
}

}  // namespace

cudaError_t launch_blit(const BlitParams &P, cudaStream_t st)
{
    const int w = P.x1d - P.x0d, h = P.y1d - P.y0d;
    if(w <= 0 || h <= 0) return cudaSuccess;
    const bool f = P.filter != 0;
    // the exact 2:1 reduction from the origin (mip generation), same format kinds
    const bool half = f && !P.clampToEdge && P.x0 == 1.0f && P.y0 == 1.0f && P.w == 2.0f && P.h == 2.0f && P.x0d == 0 &&
                      P.y0d == 0 && 2 * P.x1d <= P.sW && 2 * P.y1d <= P.sH && P.srcKind == P.dstKind;
    if(half)
    {
        BlitKernel k = P.srcKind == BK_RGBA8 ? k_blit_half<BK_RGBA8, BK_RGBA8>
                       : P.srcKind == BK_BGRA8 ? k_blit_half<BK_BGRA8, BK_BGRA8>
                       : P.srcKind == BK_RGBA16F ? k_blit_half<BK_RGBA16F, BK_RGBA16F>
                                                 : k_blit_half<BK_RGBA32F, BK_RGBA32F>;
        const int px = (P.srcKind == BK_RGBA8 || P.srcKind == BK_BGRA8) ? 4 : 2;  // destination pixels per thread
        k<<<dim3((w + 32 * px - 1) / (32 * px), (h + 7) / 8), 256, 0, st>>>(P);
        return cudaGetLastError();
    }
    // a float-format 4-sample resolve at scale 1
    if(!f && P.srcSamples == 4 && P.w == 1.0f && P.h == 1.0f && P.srcKind == P.dstKind && kind_float(P.srcKind))
    {
        const int dx = (int)floorf(P.x0), dy = (int)floorf(P.y0);  // srcOffset - dstOffset
        const int px = P.srcKind == BK_RGBA16F ? 2 : 1;
        const dim3 g((w + 32 * px - 1) / (32 * px), (h + 7) / 8);
        if(P.srcKind == BK_RGBA16F)
            k_resolve_float<BK_RGBA16F><<<g, 256, 0, st>>>(P, dx, dy);
        else
            k_resolve_float<BK_RGBA32F><<<g, 256, 0, st>>>(P, dx, dy);
        return cudaGetLastError();
    }
    BlitKernel k = P.srcKind == BK_RGBA8     ? blit_kernel<BK_RGBA8>(P.dstKind, f)
                   : P.srcKind == BK_BGRA8   ? blit_kernel<BK_BGRA8>(P.dstKind, f)
                   : P.srcKind == BK_RGBA16F ? blit_kernel<BK_RGBA16F>(P.dstKind, f)
                                             : blit_kernel<BK_RGBA32F>(P.dstKind, f);
    k<<<dim3((w + 31) / 32, (h + 7) / 8), 256, 0, st>>>(P);
    return cudaGetLastError();
}

cudaError_t launch_resolve_bytes(const ResolveParams &R, cudaStream_t st)
{
    if(R.width <= 0 || R.height <= 0) return cudaSuccess;
    const int quads = (R.width + 3) / 4;
    k_resolve_bytes<<<dim3((quads + 255) / 256, (unsigned)std::min(R.height, 65535)), 256, 0, st>>>(R);
    return cudaGetLastError();
}

cudaError_t launch_clear(const ClearParams &C, cudaStream_t st)
{
    if(C.rows <= 0 || C.rowBytes <= 0 || C.planes <= 0) return cudaSuccess;
    // 152 SMs x 8 resident blocks of 256 threads
    k_clear<<<(unsigned)std::min(C.rows * C.planes, 152 * 8), 256, 0, st>>>(C);
    return cudaGetLastError();
}

}  // namespace swgbb
